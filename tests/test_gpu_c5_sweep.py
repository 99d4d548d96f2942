"""The learned-truncation sweep over the 64 fixed-seed random geometries (log-uniform R/L in
[10, 500], T uniform in [0, 350] K, Drude omega_p in [7, 10] eV, gamma in [0.02, 0.05] eV,
ldim = ceil(7 R/L); draws as in test_gpu_c5.py): per geometry the mixed form's free energy with
the learned proposal (network trained on the plane-sphere benchmark geometries, learned.CONFIGS,
none of the 64 among them) against the same form with the plain schedule.  The reference's
rules decide which terms enter, so the two energies are equal; the sweep records the matrices
each computed, those beyond the cutoffs and the time.

Heavy (about ten GPU-minutes): it runs only when CAPS_C5_SWEEP is set, and writes its
summary as JSON to the file CAPS_C5_SWEEP names."""
import json
import os
import time

import pytest

from test_gpu_c5 import draws

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(not os.environ.get("CAPS_C5_SWEEP"), reason="opt-in sweep (set CAPS_C5_SWEEP=<summary.json>)")]


def test_learned_sweep_64_geometries():
    import caps_gb300 as cg
    from caps_gb300 import learned
    net, tinfo = learned.train(seed=0, which=learned.CONFIGS)
    rows = []
    for RbyL, T, wp, ga, ldim in draws():
        L = 1e-6
        c = cg.Caps(RbyL * L, L, ldim=ldim)
        c.set_drude(wp, ga)
        c.set_precision(cg.PREC_MIXED)
        t = time.time()
        E0, i0 = c.free_energy(T)
        t0 = time.time() - t
        t = time.time()
        E1, i1 = c.free_energy(T, mlp=net)
        t1 = time.time() - t
        rows.append(dict(RbyL=RbyL, T=T, omegap_eV=wp, gamma_eV=ga, ldim=ldim, E_plain=E0, E_learned=E1, nxi=i0["nxi"],
                         plain=dict(matrices=i0["ndet"], beyond=i0["nwasted"], seconds=t0),
                         learned=dict(matrices=i1["ndet"], beyond=i1["nwasted"], seconds=t1)))
        print("R/L %6.1f T %6.1f ldim %5d: E %.10g | plain %6d (%5d beyond) %7.2f s | learned %6d (%5d beyond) %7.2f s" %
              (RbyL, T, ldim, E1, i0["ndet"], i0["nwasted"], t0, i1["ndet"], i1["nwasted"], t1), flush=True)
    summary = dict(training=tinfo, geometries=rows,
                   equal=sum(r["E_plain"] == r["E_learned"] for r in rows),
                   plain_seconds=sum(r["plain"]["seconds"] for r in rows),
                   learned_seconds=sum(r["learned"]["seconds"] for r in rows),
                   plain_matrices=sum(r["plain"]["matrices"] for r in rows),
                   learned_matrices=sum(r["learned"]["matrices"] for r in rows),
                   plain_beyond=sum(r["plain"]["beyond"] for r in rows),
                   learned_beyond=sum(r["learned"]["beyond"] for r in rows))
    json.dump(summary, open(os.environ["CAPS_C5_SWEEP"], "w"), indent=1)
    assert summary["equal"] == len(rows), [(r["RbyL"], r["T"]) for r in rows if r["E_plain"] != r["E_learned"]]
