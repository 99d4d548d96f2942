"""Training data and training of the learned-truncation network.

The samples are log|logdetD(xi, m)| values computed by the library's plain FP64
method, for perfect reflectors and Drude metals, on a log grid of the decay
variable 2 xi L / c and a grid of m / sqrt(R/L).  Training runs on the GPU
through the library's own kernels (caps_mlp_train).

Two training sets:
  HELD_OUT  (the default): small geometries, R/L = 10 .. 50, and Drude metals other
            than gold (omega_p = 9 eV, gamma = 0.035 eV).  Neither the R/L = 150
            geometry of the benchmark nor its material is in it, so the benchmark
            measures the network on a workload it has not seen.
  CONFIGS   R/L = 20, 50, 150 (the plane-sphere benchmark geometries) with gold and
            two other Drude metals: the network for sweeps over random geometries,
            none of which it has seen either.
"""
import math
import time

import numpy as np

from . import MLP, PREC_FP64, Caps

HBAR, KB, CL = 1.0545718e-34, 1.38064852e-23, 299792458.0
PERFECT_OMEGAP_EV = 50.0   # feature value that encodes a perfect reflector
TAIL_FLOOR = 1e-16         # smallest |logdetD| kept as a training target

HELD_OUT = dict(geometries=[(10e-6, 1e-6, 70), (20e-6, 1e-6, 140), (35e-6, 1e-6, 245), (50e-6, 1e-6, 350)],
                materials=[None, (7.0, 0.02), (10.0, 0.05), (8.0, 0.045)])
CONFIGS = dict(geometries=[(20e-6, 1e-6, 140), (50e-6, 1e-6, 350), (150e-6, 1e-6, 1050)],
               materials=[None, (9.0, 0.035), (7.0, 0.02), (10.0, 0.05)])


def training_set(geometries=HELD_OUT["geometries"], materials=HELD_OUT["materials"], nxi=12, ms=None,
                 precision=PREC_FP64):
    """features X (n,5), targets y = log|logdetD| and the number of matrices computed"""
    X, y, count = [], [], 0
    for R, L, ldim in geometries:
        RbyL = R / L
        # decay variable 2 xi L / c from 0.01 to 14 (the first Matsubara frequency at 300 K,
        # L = 1 um, is 0.82; at 5 K it is 0.014), not on any Matsubara grid
        decay = np.exp(np.linspace(np.log(0.01), np.log(14.0), nxi))
        xis = decay * (1 + RbyL) / 2
        mlist = ms if ms is not None else sorted(set(int(round(v)) for v in np.linspace(0, 2.2 * math.sqrt(RbyL) * 8, 14)))
        for mat in materials:
            c = Caps(R, L, ldim=ldim)
            c.set_precision(precision)
            if mat:
                c.set_drude(*mat)
            wp, ga = (mat if mat else (PERFECT_OMEGAP_EV, 0.0))
            bx = [x for x in xis for _ in mlist]
            bm = [m for _ in xis for m in mlist]
            out, st = c.logdetD_batch(bx, bm)
            count += len(bx)
            for xi_, m, v, s in zip(bx, bm, out, st):
                # the truncation rules only look at values within ~1e-15 of the leading
                # term (m cutoff 1e-9 of v_0, v_0 >= 1e-6): a deeper tail is left out
                if s >= 16 or not (v < -TAIL_FLOOR):
                    continue
                X.append(MLP.features(RbyL, xi_, m, wp, ga))
                y.append(math.log(-v))
    return np.array(X, dtype=np.float32), np.array(y, dtype=np.float32), count


def train(seed=0, epochs=4000, lr=3e-3, data=None, which=HELD_OUT):
    """a trained MLP and (loss, samples, matrices computed for the data, seconds of data
    generation and of training)"""
    t0 = time.time()
    X, y, count = data if data is not None else training_set(which["geometries"], which["materials"])
    t1 = time.time()
    net = MLP(seed)
    loss = net.train(X, y, epochs=epochs, lr=lr)
    t2 = time.time()
    info = dict(loss=loss, samples=len(y), matrices=count, data_seconds=t1 - t0, train_seconds=t2 - t1)
    if data is None:
        info.update(geometries_RbyL=[g[0] / g[1] for g in which["geometries"]],
                    materials=[m if m else "perfect" for m in which["materials"]])
    return net, info
