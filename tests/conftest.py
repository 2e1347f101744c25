import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libzandgpu.so")
    # kernel choices measured during the tests stay in a file of this session
    if "ZG_TUNE_CACHE" not in os.environ:
        import tempfile
        os.environ["ZG_TUNE_CACHE"] = os.path.join(tempfile.mkdtemp(prefix="zg_tune_"), "tune.json")


def load_golden(case):
    import json
    z = np.load(os.path.join(GOLDEN, case + ".npz"))
    d = {k: z[k] for k in z.files}
    d["params"] = json.loads(str(z["params"]))
    return d


def golden_callbacks(p):
    """bias(t, a) and dH(t, sig) of a golden case, as its Bias.py defines them."""
    from zandpack_gb300.workloads import bias_value
    U = p["hubbard_U"]

    def dH(t, sig):
        if U is None:
            return 0.0
        d = np.einsum("kii->ki", sig).real
        out = np.zeros(sig.shape, complex)
        i = np.arange(sig.shape[-1])
        out[:, i, i] = U * (d - 0.5)
        return out
    return (lambda t, a: bias_value(p["bias"], t, a)), dH


@pytest.fixture(params=["mini2", "mini3", "c1"])
def golden(request):
    path = os.path.join(GOLDEN, request.param + ".npz")
    if not os.path.exists(path):
        pytest.skip("fixture %s missing" % request.param)
    return request.param, load_golden(request.param)


@pytest.fixture(params=["nz_mini2", "nz_mini3"])
def golden_nz(request):
    """Fixtures of the reference ``nozand`` (non-orthogonal basis)."""
    path = os.path.join(GOLDEN, request.param + ".npz")
    if not os.path.exists(path):
        pytest.skip("fixture %s missing" % request.param)
    return request.param, load_golden(request.param)
