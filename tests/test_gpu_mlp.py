"""Learned truncation: GPU forward/backward kernels against the NumPy reference,
training on plain-method data, and the learned free-energy driver against the
plain one (same E, fewer matrices)."""
import numpy as np
import pytest

import mlp_reference as ref

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def cg():
    import caps_gb300
    return caps_gb300


def test_gpu_gradient_matches_reference(cg):
    net = cg.MLP(seed=3)
    rng = np.random.default_rng(2)
    X = rng.normal(0, 1, (777, 5)).astype(np.float32)
    y = rng.normal(-5, 3, 777).astype(np.float32)
    loss, g = net.loss_grad(X, y)
    lr, gr, _ = ref.loss_grad(net.params().astype(np.float64), X.astype(np.float64), y.astype(np.float64))
    assert abs(loss - lr) <= 1e-5 * abs(lr)
    scale = np.abs(gr).max()
    assert np.abs(g - gr).max() <= 1e-4 * scale, np.abs(g - gr).max() / scale


def test_gpu_predict_matches_reference(cg):
    net = cg.MLP(seed=5)
    X = np.random.default_rng(4).normal(0, 1, (300, 5)).astype(np.float32)
    _, _, yr = ref.loss_grad(net.params().astype(np.float64), X.astype(np.float64), np.zeros(300))
    assert np.abs(net.predict(X) - yr).max() <= 1e-4 * max(1.0, np.abs(yr).max())


@pytest.fixture(scope="module")
def trained(cg):
    from caps_gb300 import learned
    data = learned.training_set(geometries=[(10e-6, 1e-6, 70), (20e-6, 1e-6, 140)], materials=[None, (9.0, 0.035)], nxi=7)
    net, info = learned.train(seed=0, epochs=3000, data=data)
    return net, info, data


def test_training_reduces_loss(cg, trained):
    net, info, (X, y, _) = trained
    fresh = cg.MLP(seed=0)
    l0, _ = fresh.loss_grad(X, y)
    assert info["loss"] < 0.05 * l0, (info["loss"], l0)


def test_learned_free_energy_equals_plain_with_fewer_matrices(cg, trained):
    """what the trained network gains: the same E from fewer matrices in fewer batches"""
    net = trained[0]
    for R, L, ldim, drude in [(20e-6, 1e-6, 140, (9.0, 0.035)), (15e-6, 1e-6, 105, None)]:
        c = cg.Caps(R, L, ldim=ldim)
        if drude:
            c.set_drude(*drude)
        E0, i0 = c.free_energy(300.0)
        E1, i1 = c.free_energy(300.0, mlp=net)
        assert E1 == E0, (E1, E0)            # same terms, same values: the reference rules decide
        assert i1["ndet"] <= i0["ndet"], (i1, i0)
        assert i1["nwasted"] < i0["nwasted"] or i0["nwasted"] == 0, (i1, i0)


def test_learned_sweep_random_geometries(cg, trained):
    """the learned-truncation sweep over random geometries (fixed seed; log-uniform R/L,
    T in (0, 350] K, Drude omega_p in [7, 10] eV, gamma in [0.02, 0.05] eV, ldim = 7 R/L;
    R/L <= 30 here to keep the plain runs short): in both precisions the learned E equals
    the plain E exactly -- the reference's rules decide which terms enter -- and the matrices
    beyond the cutoffs stay a small share of those needed"""
    import math
    net = trained[0]
    rng = np.random.default_rng(1)
    done = 0
    while done < 4:
        RbyL = math.exp(rng.uniform(math.log(10), math.log(500)))
        T, wp, ga = rng.uniform(0, 350), rng.uniform(7, 10), rng.uniform(0.02, 0.05)
        if RbyL > 30 or T < 1:
            continue
        L = 1e-6
        for prec in (cg.PREC_FP64, cg.PREC_MIXED):
            c = cg.Caps(RbyL * L, L, ldim=int(math.ceil(7 * RbyL)))
            c.set_drude(wp, ga)
            c.set_precision(prec)
            E0, i0 = c.free_energy(T)
            E1, i1 = c.free_energy(T, mlp=net)
            assert E1 == E0, (RbyL, T, prec, E1, E0)
            needed = i0["ndet"] - i0["nwasted"]
            assert i1["nwasted"] <= max(8, 0.5 * needed), (RbyL, T, prec, i1, i0)
        done += 1
