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


def _load_golden(prefix_shape: bool):
    import numpy as np
    out = {}
    for f in sorted(os.listdir(GOLDEN)):
        if f.endswith(".npz") and f.startswith("shape_") == prefix_shape:
            out[f[:-4]] = dict(np.load(os.path.join(GOLDEN, f)))
    return out


@pytest.fixture(scope="session")
def golden_cases():
    """Small fixtures: the reference's full output, the FP64 oracle's, geometry."""
    return _load_golden(False)


@pytest.fixture(scope="session")
def shape_cases():
    """Benchmark-shaped fixtures (6 antennas x nchan 1024; 16 antennas x nchan 4096): the
    reference's output whole (ref_vis) or on every ch_step-th channel (ref_vis_sub) with each
    (baseline, product)'s channel sum (ref_sum) and power (ref_pow); counts and geometry."""
    return _load_golden(True)


def reference_checks(vis, d):
    """Relative errors of crosses vis [nbl][4][nchan] against a benchmark-shaped fixture: per
    (baseline, product) rel RMS on the stored channels, and the rel errors of the channel sums and
    powers over all channels."""
    import numpy as np
    from oracle import oracle as O
    nx = int(d["nant"]) * (int(d["nant"]) - 1) // 2
    v = np.asarray(vis)[:nx]
    if "ref_vis" in d:
        return {"per_product": O.rel_rms_per_product(v, d["ref_vis"]).max()}
    step = int(d["ch_step"])
    per = O.rel_rms_per_product(v[:, :, ::step], d["ref_vis_sub"]).max()
    v64 = v.astype(np.complex128)
    sums = np.abs(v64.sum(axis=-1) - d["ref_sum"]) / np.sqrt(d["ref_pow"] * v.shape[-1])
    pw = np.abs((np.abs(v64) ** 2).sum(axis=-1) - d["ref_pow"]) / d["ref_pow"]
    return {"per_product": per, "sum": float(sums.max()), "power": float(pw.max())}
