"""Training data and training of the learned-truncation network.

The samples are log|logdetD(xi, m)| values computed by the library's plain FP64
method on the benchmark geometries (R/L = 20, 50, 100, 150 with ldim = 7 R/L),
for perfect reflectors and Drude metals, on a log grid of frequencies and a
grid of m.  Training runs on the GPU through the library's own kernels.
"""
import math

import numpy as np

from . import MLP, PREC_FP64, Caps

HBAR, KB, CL = 1.0545718e-34, 1.38064852e-23, 299792458.0
GEOMETRIES = [(20e-6, 1e-6, 140), (50e-6, 1e-6, 350), (100e-6, 1e-6, 700), (150e-6, 1e-6, 1050)]
MATERIALS = [None, (9.0, 0.035), (7.0, 0.02), (10.0, 0.05)]
PERFECT_OMEGAP_EV = 50.0   # feature value that encodes a perfect reflector
TAIL_FLOOR = 1e-16         # smallest |logdetD| kept as a training target


def training_set(geometries=GEOMETRIES, materials=MATERIALS, nxi=9, ms=None, precision=PREC_FP64):
    """features X (n,5), targets y = log|logdetD| and the number of matrices computed"""
    X, y, count = [], [], 0
    for R, L, ldim in geometries:
        RbyL = R / L
        Ts = 2 * math.pi * KB * (R + L) * 300.0 / (HBAR * CL)          # Matsubara spacing at 300 K
        xis = Ts * np.exp(np.linspace(np.log(0.35), np.log(14.0), nxi))  # not on the Matsubara grid
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


def train(seed=0, epochs=4000, lr=3e-3, data=None):
    """a trained MLP and (loss, samples, matrices computed for the data)"""
    X, y, count = data if data is not None else training_set()
    net = MLP(seed)
    loss = net.train(X, y, epochs=epochs, lr=lr)
    return net, dict(loss=loss, samples=len(y), matrices=count)
