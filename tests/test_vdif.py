"""CPU tests of the VDIF header codec: the library's parser against the header
writer, with the bit fields of the VDIF standard (as the reference's
examples/mark/dump_vdif.py:40-55 reads them)."""
import numpy as np
import pytest

from gcorr_gb300 import vdif


@pytest.mark.parametrize("legacy", [False, True])
def test_header_round_trip(legacy):
    w = vdif.header_words(seconds=123456789, frame=4321, frame_bytes=8032, nchan=2, bits=2, is_complex=False,
                          thread=17, station=0x4142, ref_epoch=45, legacy=legacy, invalid=False, version=1)
    h = vdif.parse_header(w.view(np.uint8))
    assert h["seconds"] == 123456789 and h["frame"] == 4321 and h["frame_bytes"] == 8032
    assert h["nchan"] == 2 and h["bits"] == 2 and h["is_complex"] == 0 and h["thread"] == 17
    assert h["station"] == 0x4142 and h["ref_epoch"] == 45 and h["legacy"] == int(legacy) and h["version"] == 1
    assert h["header_bytes"] == (16 if legacy else 32) and h["invalid"] == 0


def test_header_fields_by_hand():
    # w0: invalid + 5 s; w1: epoch 3, frame 7; w2: 4 channels, 1000 * 8 bytes; w3: complex, 8 bits, thread 2, station 9
    words = np.array([(1 << 31) | 5, (3 << 24) | 7, (2 << 24) | 1000, (1 << 31) | (7 << 26) | (2 << 16) | 9], "<u4")
    h = vdif.parse_header(words.view(np.uint8))
    assert (h["invalid"], h["seconds"], h["ref_epoch"], h["frame"]) == (1, 5, 3, 7)
    assert (h["nchan"], h["frame_bytes"], h["is_complex"], h["bits"], h["thread"], h["station"]) == (4, 8000, 1, 8, 2, 9)


def test_packetize_layout():
    data = np.arange(3 * 64, dtype=np.uint8)
    fr = vdif.packetize(data, 64, frames_per_second=2, seconds0=10, frame0=1)
    assert fr.shape == (3, 96)
    hs = [vdif.parse_header(f) for f in fr]
    assert [(h["seconds"], h["frame"]) for h in hs] == [(10, 1), (11, 0), (11, 1)]
    assert np.array_equal(fr[:, 32:].reshape(-1), data)
    assert vdif.samples_per_frame(64, 2) == 128 and vdif.samples_per_frame(64, 8, is_complex=True) == 16
