"""The NumPy reference of the network, checked by central finite differences
(it is the CPU reference for the GPU gradients in test_gpu_mlp.py)."""
import numpy as np

import mlp_reference as ref


def test_reference_gradient_finite_differences():
    rng = np.random.default_rng(1)
    p = rng.normal(0, 0.3, ref.NPARAM)
    X = rng.normal(0, 1, (40, 5))
    y = rng.normal(0, 1, 40)
    loss, g, _ = ref.loss_grad(p, X, y)
    idx = rng.choice(ref.NPARAM, 60, replace=False)
    for i in idx:
        e = np.zeros_like(p); e[i] = 1e-6
        fd = (ref.loss_grad(p + e, X, y)[0] - ref.loss_grad(p - e, X, y)[0]) / 2e-6
        assert abs(fd - g[i]) <= 1e-6 + 1e-5 * abs(g[i]), (i, fd, g[i])
