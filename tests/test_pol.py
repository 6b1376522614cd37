"""CPU checks of the polarisation-conversion oracle: the voltage-domain transform
(examples/chris/bench/gpubench.cu:145-160) equals J_j V J_k^H on visibilities."""
import numpy as np

from oracle import oracle as O


def _jvj(vis, gains, nant, autos=True):
    nchan = vis.shape[-1]
    pairs = [(j, k) for j in range(nant - 1) for k in range(j + 1, nant)] + ([(j, j) for j in range(nant)] if autos else [])
    out = np.empty_like(vis)
    for b, (j, k) in enumerate(pairs):
        for c in range(nchan):
            Jj = np.array([[gains[j, 0, c], -gains[j, 1, c]], [gains[j, 0, c], gains[j, 1, c]]])
            Jk = np.array([[gains[k, 0, c], -gains[k, 1, c]], [gains[k, 0, c], gains[k, 1, c]]])
            V = vis[b, :, c].reshape(2, 2)
            out[b, :, c] = (Jj @ V @ Jk.conj().T).reshape(4)
    return out


def test_voltage_and_visibility_forms_agree():
    rng = np.random.default_rng(5)
    nant, nfft, nchan = 4, 7, 6
    x = rng.normal(size=(nant, 2, nfft, nchan)) + 1j * rng.normal(size=(nant, 2, nfft, nchan))
    g = rng.normal(size=(nant, 2, nchan)) + 1j * rng.normal(size=(nant, 2, nchan))
    want = O.correlate_voltages(O.lin2circ_voltages(x, g))
    got = _jvj(O.correlate_voltages(x), g, nant)
    assert np.allclose(got, want, rtol=1e-12, atol=1e-12)


def test_ideal_feeds_circular_of_pure_linear():
    # X-only linear signal -> equal power in R and L, RL = RR
    nant, nfft, nchan = 2, 5, 3
    x = np.zeros((nant, 2, nfft, nchan), np.complex128)
    x[:, 0] = 1.0
    v = O.correlate_voltages(O.lin2circ_voltages(x))
    assert np.allclose(v[..., 0, :], 0.5) and np.allclose(v[..., 3, :], 0.5) and np.allclose(v[..., 1, :], 0.5)
