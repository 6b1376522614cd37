"""GPU tests of the VDIF depacketiser (gxc_vdif_depacketize) and of frame-validity
flagging in the correlator, against the FP64 oracle with the same flags."""
import numpy as np
import pytest
import torch

from gcorr_gb300 import FxKernel, synth, vdif
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _stream(data, payload, fps, s0, f0, drop=(), extra=True, **kw):
    fr = vdif.packetize(data, payload, fps, s0, f0, **kw)
    keep = [k for k in range(len(fr)) if k not in set(drop)]
    frames = [fr[k] for k in keep]
    if extra:
        alien = fr[0].copy()
        alien[:32] = vdif.header_words(s0, f0, fr.shape[1], thread=5).view(np.uint8)  # other thread
        alien[32:] = 0xAA
        late = fr[0].copy()
        late[:32] = vdif.header_words(s0 - 1, f0, fr.shape[1]).view(np.uint8)  # before the window
        bad = fr[1].copy()
        w0 = bad[:4].view("<u4")
        w0 |= np.uint32(1 << 31)  # marked invalid
        frames += [alien, late, bad]
    rng = np.random.default_rng(len(frames))
    order = rng.permutation(len(frames))
    return np.stack([frames[k] for k in order]).reshape(-1), fr.shape[1]


@pytest.mark.parametrize("payload", [256, 200])
def test_depacketize_round_trip(payload):
    rng = np.random.default_rng(payload)
    nslots = 61
    data = rng.integers(0, 256, nslots * payload, dtype=np.uint8)
    drop = (0, 10, 11, 60)
    stream, fb = _stream(data, payload, fps=25, s0=1000, f0=3, drop=drop)
    out, valid, stats = vdif.depacketize(torch.from_numpy(stream).cuda(), fb, payload, 1000, 3, 25, nslots,
                                         thread_id=0, fill=0x55)
    torch.cuda.synchronize()
    out, valid, stats = out.cpu().numpy(), valid.cpu().numpy(), stats.cpu().numpy()
    want = np.ones(nslots, np.uint8)
    want[list(drop)] = 0  # frame 1's invalid-marked duplicate is skipped; its good copy fills the slot
    assert np.array_equal(valid, want)
    o, d = out.reshape(nslots, payload), data.reshape(nslots, payload)
    assert np.array_equal(o[want == 1], d[want == 1])
    assert (o[want == 0] == 0x55).all()
    assert list(stats) == [nslots - len(drop), 2, 1]


def test_depacketize_8bit_offset_binary():
    rng = np.random.default_rng(8)
    payload, nslots = 512, 9
    signed = rng.integers(-128, 128, nslots * payload).astype(np.int8).view(np.uint8)
    stream, fb = _stream(signed, payload, fps=1000, s0=7, f0=0, bits=8, is_complex=True,
                         signed_to_offset_binary=True, extra=False)
    out, valid, _ = vdif.depacketize(torch.from_numpy(stream).cuda(), fb, payload, 7, 0, 1000, nslots,
                                     offset_binary_8bit=True)
    assert valid.all().item()
    assert np.array_equal(out.cpu().numpy(), signed)


def test_correlation_with_dropped_frames_vs_masked_oracle():
    w = synth.Workload(nant=3, nchan=256, nfft=60, bw_hz=32e6, rho=0.2, seed=33)
    d = synth.generate(w)
    F = w.fft_len
    payload = 256
    spf = vdif.samples_per_frame(payload, 2)  # 512 samples per frame
    nbytes = w.bytes_per_antenna
    nslots = -(-nbytes // payload)
    drops = {0: (10,), 1: (20, 21), 2: ()}
    outs, valids = [], []
    for a in range(w.nant):
        raw = np.zeros(nslots * payload, np.uint8)
        raw[:nbytes] = d["inputs"][a].numpy()
        stream, fb = _stream(raw, payload, fps=100, s0=50, f0=0, drop=drops[a])
        o, v, _ = vdif.depacketize(torch.from_numpy(stream).cuda(), fb, payload, 50, 0, 100, nslots, thread_id=0)
        outs.append(o)
        valids.append(v)
    fx = FxKernel(w.nant, w.nchan, w.nfft, 2, w.lo_hz, w.bw_hz, False, rotator="exact", autos=True)
    fx.setInputData(outs)
    fx.setDelays(d["poly"], d["fso"])
    fx.setFrameValidity(valids, spf)
    fx.process()
    vis, counts = fx.visibilities(), fx.baseline_counts()
    cfg = O.config_from_workload(w, O.ROT_EXACT, True)
    mask = np.ones((w.nant, w.nfft), np.uint8)
    for a in range(w.nant):
        for i in range(w.nfft):
            g = O.geometry(cfg, d["poly"][a], d["fso"][a], i)
            if g.valid and any(f in drops[a] for f in range(g.offset // spf, (g.offset + F - 1) // spf + 1)):
                mask[a, i] = 0
    assert (mask == 0).sum() >= 5
    ref, rc = O.exact_process(cfg, [x.numpy() for x in d["inputs"]], d["poly"], d["fso"], mask=mask)
    assert np.array_equal(counts, rc)
    assert O.rel_rms_per_product(vis, ref).max() < 1e-5
    # clearing the flags restores the unflagged result
    fx.setFrameValidity(None)
    fx.process()
    ref2, rc2 = O.exact_process(cfg, [x.numpy() for x in d["inputs"]], d["poly"], d["fso"])
    assert np.array_equal(fx.baseline_counts(), rc2)
    fx.close()
