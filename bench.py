"""Benchmark: logdet(1-M) matrices per second and time-to-E for the CaPS
plane-sphere free energy at R/L=150 (Drude gold, T=300 K, ldim=1050, matrices
of dimension 2100), on the GPU through the library's C-ABI.

One step = one complete free-energy evaluation (Matsubara sum with the
reference's m cutoff 1e-9 and xi truncation 1e-6, ~980 matrices), i.e. the
call caps_free_energy() a user of the library makes.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--precision fp64|mixed]
  python bench.py --impl reference ...   # CPU restatement of the reference on host cores

Multi-GPU (torchrun, one process per GPU) runs independent replicas: every
rank evaluates the whole workload; value = all ranks' matrices / max time.
Prints one JSON line on rank 0.
"""
import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "logdetD/s and time-to-E at R/L=150: mixed+learned vs FP64 GPU, |ΔE/E|≤1e-6"
UNIT = "logdetD/s"
# workload: Drude gold, R/L=150, L=1um, T=300K, ldim=1050
R, L, T, LDIM = 150e-6, 1e-6, 300.0, 1050
OMEGAP_EV, GAMMA_EV = 9.0, 0.035
CUTOFF, EPSREL = 1e-9, 1e-6
WORKLOAD = ("Drude gold (wp=9 eV, gamma=0.035 eV), R/L=150, L=1e-6 m, T=300 K, ldim=1050 (matrix dim 2100), "
            "full Matsubara sum (cutoff 1e-9, epsrel 1e-6)")
E_REFERENCE = None  # filled from tests/golden when present


def rank_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("LOCAL_RANK", 0)), int(os.environ.get("WORLD_SIZE", 1))


class ClockSampler:
    """samples nvidia-smi clocks and throttle reasons while running"""
    FIELDS = "index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown," \
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap"

    def __init__(self, gpu_index):
        self.idx = gpu_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.idx), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append(ln.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons, power = [], [], set(), []
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
                power.append(float(f[3]))
            except ValueError:
                continue
            for k, name in enumerate(names):
                if f[5 + k].lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm), "power_w_max": max(power) if power else None}


def barrier(dist):
    if dist is not None:
        dist.barrier()


def allmax(dist, x):
    if dist is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def allsum(dist, x):
    if dist is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def load_reference_energy():
    p = os.path.join(ROOT, "tests", "golden", "energy_drude_RbyL150_ldim1050_T300.json")
    if os.path.exists(p):
        return json.load(open(p))
    return None


def cpu_sample_tasks(n, seed=0):
    """a fixed sample of (xi, m) of the workload: Matsubara n in 1..9, m in 0..109"""
    import numpy as np
    rng = np.random.default_rng(seed)
    Ts = 2 * math.pi * 1.38064852e-23 * (R + L) * T / (1.0545718e-34 * 299792458.0)
    ns = rng.integers(1, 10, n)
    ms = rng.integers(0, 110, n)
    return [k * Ts for k in ns], [int(m) for m in ms]


def cpu_baseline(nmat, threads):
    """the CPU restatement of the reference (oracle port) on host threads: det/s on a bounded sample"""
    from oracle import binding as ob
    xi, m = cpu_sample_tasks(nmat)
    t = time.time()
    ob.logdetD_batch(R, L, LDIM, xi, m, (OMEGAP_EV, GAMMA_EV), threads=threads)
    dt = time.time() - t
    return nmat / dt, dt


def run_reference(args, dist, rank, world):
    threads = os.cpu_count() or 1
    per_step = args.cpu_sample or threads  # default: one matrix per host thread per step
    if rank != 0:
        return
    for _ in range(args.warmup):
        cpu_baseline(per_step, threads)
    t0 = time.time()
    total = 0
    for k in range(args.steps):
        cpu_baseline(per_step, threads)
        total += per_step
    dt = time.time() - t0
    value = total / dt
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": dt / args.steps * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic (inputs fully set by the geometry/material scalars)", "impl": "reference",
        "config": {"workload": WORKLOAD, "sample_per_step": "%d (xi,m) matrices of the workload, fixed seed" % per_step},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": "%d matrices per step (dim 2100), oracle restatement of the reference (C, dense LU) on %d host threads" % (per_step, threads)},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# DRAM bytes per algorithmic byte of the trailing update (k_syrk_pipe, all four launch kinds
# of a 256-column panel), from the ncu capture summarised in profiles/k_syrk_pipe_c3.md
SYRK_DRAM_PER_ALGORITHMIC = 1.14


def measured_hbm_peak():
    """HBM copy bandwidth of the GB300s (GB/s) from MEASURED_PEAKS.json, else the fallback"""
    p = os.path.join(os.path.dirname(os.path.abspath(__file__)), "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            v = json.load(f)["hbm_gbs"]
        return float(v), "of measured (MEASURED_PEAKS.json hbm_gbs: STREAM-style copy)"
    except (OSError, KeyError, ValueError):
        return 6800.0, "of fallback (6.8 TB/s, one earlier GB300 measurement)"


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--precision", default="mixed", choices=["fp64", "mixed"])
    ap.add_argument("--cpu-sample", type=int, default=0, help="matrices in the CPU-baseline sample (0: 2 per host thread)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--plain", action="store_true",
                    help="plain truncation schedule instead of the learned proposal")
    ap.add_argument("--no-fp64-reference", action="store_true",
                    help="skip the side measurement of the plain FP64 form")
    ap.add_argument("--ncu-case", action="store_true",
                    help="profiling case: one batch of 8 matrices of the workload (n in {1,5}, m in {0,20,40,60})")
    ap.add_argument("--ncu-matrices", type=int, default=8,
                    help="matrices in the profiling case; other than 8: n = 1..4, m = 0, 4, 8, ... (all factored), "
                         "e.g. 48 for a trailing-matrix working set above L2")
    args = ap.parse_args()
    if args.ncu_case:
        import caps_gb300 as cg
        Ts = 2 * math.pi * 1.38064852e-23 * (R + L) * T / (1.0545718e-34 * 299792458.0)
        caps = cg.Caps(R, L, ldim=LDIM)
        caps.set_drude(OMEGAP_EV, GAMMA_EV)
        caps.set_precision(cg.PREC_MIXED if args.precision == "mixed" else cg.PREC_FP64)
        if args.ncu_matrices == 8:
            xi = [n * Ts for n in (1, 5) for m in (0, 20, 40, 60)]
            ms = [m for n in (1, 5) for m in (0, 20, 40, 60)]
        else:  # n = 1..4, m = 0, 4, 8, ...: every matrix large enough to be factored
            per = (args.ncu_matrices + 3) // 4
            xi = [n * Ts for n in (1, 2, 3, 4) for k in range(per)][:args.ncu_matrices]
            ms = [4 * k for n in (1, 2, 3, 4) for k in range(per)][:args.ncu_matrices]
        out, st = caps.logdetD_batch(xi, ms)
        print(json.dumps({"logdetD": list(out), "status": [int(s) for s in st], "phases_ms": cg.timings()}))
        return

    rank, local_rank, world = rank_env()
    dist = None
    if world > 1:
        import torch.distributed as dist_mod
        dist_mod.init_process_group("gloo", init_method="env://")
        dist = dist_mod
    if args.impl == "reference":
        run_reference(args, dist, rank, world)
        if dist is not None:
            dist.barrier()
        return
    if world > 1 and "CUDA_VISIBLE_DEVICES" not in os.environ:
        os.environ["CUDA_VISIBLE_DEVICES"] = str(local_rank)

    import caps_gb300 as cg

    fp64_peak = cg.fp64_peak()
    fp32_peak = cg.fp32_peak()
    caps = cg.Caps(R, L, ldim=LDIM)
    caps.set_drude(OMEGAP_EV, GAMMA_EV)
    caps.set_precision(cg.PREC_MIXED if args.precision == "mixed" else cg.PREC_FP64)

    net, train_info = None, None
    args.learned = not args.plain
    if args.learned:
        from caps_gb300 import learned
        t_tr = time.time()
        net, train_info = learned.train(seed=0)
        train_info["seconds"] = time.time() - t_tr

    E = None
    for _ in range(args.warmup):
        E, info = caps.free_energy(T, CUTOFF, EPSREL, mlp=net)

    clocks = ClockSampler(local_rank if "CUDA_VISIBLE_DEVICES" not in os.environ else os.environ["CUDA_VISIBLE_DEVICES"].split(",")[0])
    barrier(dist)
    cg.counters(reset=True)
    cg.reset_timings()
    cg.kernel_timing(True)
    clocks.start()
    t0 = time.time()
    infos = []
    for _ in range(args.steps):
        E, info = caps.free_energy(T, CUTOFF, EPSREL, mlp=net)
        infos.append(info)
    wall = time.time() - t0
    clk = clocks.stop()
    barrier(dist)
    ctr = cg.counters()
    wk = cg.work()
    ph = cg.timings(cumulative=True)   # device ms per phase, summed over the timed steps
    syrk_ms, syrk_bytes, syrk_n = cg.kernel_stats()
    cg.kernel_timing(False)

    ndet = sum(i["ndet"] for i in infos)
    dev_s = ph[5] * 1e-3

    # the plain FP64 GPU form on the same workload (1 warm-up + 2 timed calls), for the
    # mixed+learned vs FP64 ratio of the metric
    fp64 = None
    if not args.no_fp64_reference and (args.learned or args.precision != "fp64"):
        c64 = cg.Caps(R, L, ldim=LDIM)
        c64.set_drude(OMEGAP_EV, GAMMA_EV)
        c64.free_energy(T, CUTOFF, EPSREL)
        cg.reset_timings()
        t64 = time.time()
        E64 = None
        for _ in range(2):
            E64, i64 = c64.free_energy(T, CUTOFF, EPSREL)
        t64 = (time.time() - t64) / 2
        d64 = cg.timings(cumulative=True)[5] * 1e-3 / 2
        fp64 = {"time_to_E_s": t64, "value": i64["ndet"] / d64, "matrices": i64["ndet"], "E": E64,
                "phases_ms": dict(zip(["setup_mie", "K", "I", "elements", "factor", "total"], [x / 2 for x in cg.timings(cumulative=True)]))}
    wall_max = allmax(dist, wall)
    dev_max = allmax(dist, dev_s)
    ndet_all = allsum(dist, ndet)
    if rank != 0:
        return

    value = ndet_all / dev_max          # device time (CUDA events on the launching stream)
    e2e = ndet_all / wall_max           # wall time of the public API call, host work and copies included
    fac_s = ph[4] * 1e-3
    achieved = wk["factor_flops"] / fac_s / 1e12 if fac_s > 0 else None
    hbm_peak, hbm_src = measured_hbm_peak()
    syrk_gbs = syrk_bytes / (syrk_ms * 1e-3) / 1e9 if syrk_ms > 0 else None
    ref = load_reference_energy()
    err = abs(E - ref["E"]) / abs(ref["E"]) if ref else None

    cpu = None
    if not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        nm = args.cpu_sample or 2 * threads
        v, dt = cpu_baseline(nm, threads)
        cpu = {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": "%d (xi,m) matrices of the workload (dim 2100, fixed seed), %.1f s on %d host threads" % (nm, dt, threads)}

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": wall_max / args.steps * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64" if args.precision == "fp64" else
                 "f64 (Mie, K, log-factorials, exponents, pivot logs, correction) + float-float q-sums + f32 delta-Cholesky",
        "data": "synthetic (inputs fully set by the geometry/material scalars)",
        "config": {"workload": WORKLOAD, "matrices_per_step": ndet / args.steps, "precision": args.precision,
                   "truncation": "learned (MLP proposal, reference rules verify)" if args.learned else "plain (extrapolating schedule)",
                   "wasted_matrices_per_step": sum(i["nwasted"] for i in infos) / args.steps,
                   "parallelism": "replicas" if world > 1 else "single GPU",
                   "l2": "no flush needed: every matrix (35 MB) and the per-chunk working set (>10 GB) exceed L2"},
        "time_to_E_s": wall_max / args.steps,
        "E": E, "E_reference": ref["E"] if ref else None, "E_rel_err": err,
        "phases_ms_per_step": {k: v / args.steps for k, v in zip(["setup_mie", "K", "I", "elements", "factor", "total"], ph)},
        "roofline": ({"bound": "fp64", "kernel": "FP64 Cholesky (potf2+trsm+syrk), n^3/3 flops per factored matrix",
                      "achieved": achieved, "peak": fp64_peak, "unit": "TFLOP/s",
                      "frac": achieved / fp64_peak if achieved else None,
                      "peak_source": "measured live: DFMA-chain probe kernel (caps_gpu_fp64_peak); MEASURED_PEAKS.json has no FP64 figure",
                      "traffic": None} if args.precision == "fp64" else
                     {"bound": "hbm",
                      "kernel": "k_syrk_pipe: persistent warp-specialised tcgen05 trailing update of the FP32 delta-form "
                                "Cholesky (256-column panels, split TF32, TMEM accumulators; the whole-trailing-matrix "
                                "launches fed by bulk copies of split-TF32 panel images that the panel solves write); "
                                "algorithmic bytes = target block read + written once and the panel rows read once, "
                                "per factored matrix",
                      "achieved": syrk_gbs, "peak": hbm_peak, "unit": "GB/s",
                      "frac": syrk_gbs / hbm_peak if syrk_gbs else None,
                      "traffic": syrk_bytes / syrk_n * SYRK_DRAM_PER_ALGORITHMIC if syrk_n else None,
                      "peak_source": hbm_src,
                      "launches": syrk_n, "avg_launch_ms": syrk_ms / syrk_n if syrk_n else None,
                      "algorithmic_bytes_per_launch": syrk_bytes / syrk_n if syrk_n else None,
                      "traffic_source": "DRAM bytes per algorithmic byte of the k_syrk_pipe launches from one ncu "
                                        "capture (profiles/k_syrk_pipe_c3.md), times this run's algorithmic bytes per "
                                        "launch (the images are written by the panel solves, outside these launches)",
                      "fp32_accurate_tflops_factorisation": achieved}),
        "dominant_kernel": None if args.precision == "fp64" else {
            "kernel": "k_itab_grp<3> (float-float q-sums)", "phase_share_of_step": ph[2] / ph[5] if ph[5] else None,
            "bound": "FP32/ALU instruction issue; no HBM or tensor roofline applies (DRAM idle)",
            "evidence": "profiles/k_itab_grp_c3_small.md"},
        "cpu_baseline": cpu,
        "learned_training": train_info,
        "fp64_plain_form": fp64,
        "time_to_E_speedup_vs_fp64_plain": (fp64["time_to_E_s"] / (wall_max / args.steps)) if fp64 else None,
        "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": ctr["h2d"] / args.steps, "d2h_bytes_per_step": ctr["d2h"] / args.steps},
        "gpu_launches": ctr["launches"],
        "clocks": clk,
    }
    print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
