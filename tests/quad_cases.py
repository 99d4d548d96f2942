"""Test integrands for the quadrature restatements (shared by the tests and by
tests/golden/make_golden_quad.py, which records the reference's results for them)."""
import math

# name -> (f, bound, inf)
QAGI = {
    "exp": (lambda x: math.exp(-x), 0.0, 1),
    "lorentz": (lambda x: 1.0 / (1.0 + x * x), 0.0, 1),
    "sqrt_sing": (lambda x: math.exp(-x) / math.sqrt(x) if x > 0 else 0.0, 0.0, 1),
    "log_sing": (lambda x: math.log(x) * math.exp(-x) if x > 0 else 0.0, 0.0, 1),
    "slow": (lambda x: 1.0 / ((1.0 + x) * math.sqrt(x)) if x > 0 else 0.0, 0.0, 1),
    "osc": (lambda x: math.sin(x) ** 2 * math.exp(-x / 3), 0.0, 1),
    "bose": (lambda x: x ** 3 / math.expm1(x) if 0 < x < 700 else 0.0, 0.0, 1),
    "casimir": (lambda x: -x * math.log1p(-math.exp(-x)) if x > 0 else 0.0, 0.0, 1),
    "powertail": (lambda x: 1.0 / (1.0 + x) ** 1.1, 0.0, 1),
    "shifted": (lambda x: math.exp(-(x - 2.0)) * math.cos(x), 2.0, 1),
    "left": (lambda x: math.exp(x) / (1.0 + x * x), 0.5, -1),
    "gauss": (lambda x: math.exp(-x * x), 0.0, 2),
}
EPSRELS = [1e-6, 1e-10]

# name -> (f, L)
FCQS = {
    "exp": (lambda x: math.exp(-x), 1.0),
    "lorentz": (lambda x: 1.0 / (1.0 + x * x), 1.0),
    "casimir": (lambda x: -x * math.log1p(-math.exp(-x)) if x > 0 else 0.0, 2.0),
    "gauss": (lambda x: math.exp(-x * x), 0.5),
}
