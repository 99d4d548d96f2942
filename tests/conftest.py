import json
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300)")


@pytest.fixture(scope="session")
def unit_vectors():
    return json.load(open(os.path.join(GOLDEN, "reference_unit_tests.json")))


@pytest.fixture(scope="session")
def ref_values():
    return json.load(open(os.path.join(GOLDEN, "reference_values.json")))


SMALL_ENERGIES = ["pr_RbyL10_ldim70_T300", "drude_RbyL10_ldim70_T300", "plasma_RbyL10_ldim70_T300",
                  "t0_drude_RbyL20_ldim100", "psd_drude_RbyL10_ldim70_T300", "material_RbyL10_ldim70_T300"]


@pytest.fixture(scope="session")
def energy_golden():
    """free energies from the unmodified reference library (tests/golden/make_golden_energy.py)"""
    return {n: json.load(open(os.path.join(GOLDEN, "energy_%s.json" % n))) for n in SMALL_ENERGIES}


def rel(a, b):
    return abs(a - b) / max(1.0, abs(b))


def relx(a, b):
    """relative error in the reference's AssertAlmostEqual sense (unittest.c:64)"""
    return 0.0 if a == b else abs(1 - a / b)
