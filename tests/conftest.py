import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the libgxcorr kernels)")


def _ensure_built():
    from oracle import oracle as O
    if not os.path.exists(O.ORACLE_SO) or \
            os.path.getmtime(O.ORACLE_SO) < os.path.getmtime(os.path.join(ROOT, "oracle", "fxoracle.c")):
        subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), O.ORACLE_SO], check=True)
    from gcorr_gb300 import buildlib
    buildlib.build()


_ensure_built()


def gpu_available() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def golden_cases():
    import numpy as np
    out = {}
    for f in sorted(os.listdir(GOLDEN)):
        if f.endswith(".npz"):
            out[f[:-4]] = dict(np.load(os.path.join(GOLDEN, f)))
    return out
