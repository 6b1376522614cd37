"""CPU tests of the PSRDADA stream reader (csrc/dada_io.cpp): the ASCII header format the
reference's ingest writes (ingest/src/ingest.c:185-330: HDR_SIZE bytes of "KEY value  # comment"
lines, UTC_START / MJD_START / PICOSECONDS filled in, unset template fields) and the data that
follows it, read per antenna in sub-integration-sized pieces."""
import numpy as np
import pytest

from gcorr_gb300 import _lib as L
from gcorr_gb300 import dada

FIELDS = {"UTC_START": "2024-05-01-12:00:00", "MJD_START": "60431.5", "PICOSECONDS": 250000,
          "SOURCE": "unset", "FREQ": 8432.0, "BW": 64.0, "TSAMP": 0.0078125, "NBIT": 2, "NPOL": 2,
          "NDIM": 1, "NCHAN": 1, "BYTES_PER_SECOND": 32000000, "OBS_OFFSET": 0}


def test_header_fields_and_lookup():
    text = dada.make_header(dict(FIELDS, TELESCOPE="ATCA      # with a comment"))
    h = dada.parse_header(text)
    assert h.hdr_size == 4096 and (h.nbit, h.npol, h.ndim, h.nchan) == (2, 2, 1, 1)
    assert (h.bw_mhz, h.freq_mhz, h.tsamp_us) == (64.0, 8432.0, 0.0078125)
    assert (h.bytes_per_second, h.obs_offset, h.picoseconds) == (32000000, 0, 250000)
    assert h.mjd_start == 60431.5 and h.utc_start == b"2024-05-01-12:00:00" and h.source == b""
    assert dada.header_value(text, "TELESCOPE") == "ATCA"
    with pytest.raises(L.GxcError):
        dada.header_value(text, "RECEIVER")
    # absent fields: HDR_SIZE defaults to 4096, numbers to -1, reals to 0
    h2 = dada.parse_header(b"NBIT 8\n")
    assert h2.hdr_size == 4096 and h2.nbit == 8 and h2.npol == -1 and h2.bw_mhz == 0.0


def test_config_from_header():
    r_cfg = L.GxcConfig()
    h = dada.parse_header(dada.make_header(FIELDS))
    import ctypes as C
    assert L.lib().gxc_dada_config(C.byref(h), C.byref(r_cfg)) == L.GXC_OK
    assert r_cfg.nbit == 2 and r_cfg.is_complex == 0 and r_cfg.bw_hz == 64e6 and r_cfg.lo_hz == 8400e6
    h1 = dada.parse_header(dada.make_header(dict(FIELDS, NPOL=1)))
    assert L.lib().gxc_dada_config(C.byref(h1), C.byref(r_cfg)) == L.GXC_ERR_UNSUPPORTED


@pytest.mark.parametrize("hdr_size", [4096, 8192])
def test_reader_streams_per_antenna(tmp_path, hdr_size):
    rng = np.random.default_rng(hdr_size)
    data = [rng.integers(0, 256, 10000, dtype=np.uint8) for _ in range(3)]
    paths = [str(tmp_path / f"ant{a}.dada") for a in range(3)]
    for p, d in zip(paths, data):
        dada.write_stream(p, FIELDS, d, hdr_size=hdr_size)
    r = dada.DadaReader(paths, 4000)
    assert r.header(1).hdr_size == hdr_size and r.header(2).nbit == 2
    bufs = [np.zeros(4000, dtype=np.uint8) for _ in range(3)]
    for k in range(2):
        assert r.read(bufs)
        for a in range(3):
            assert np.array_equal(bufs[a], data[a][4000 * k:4000 * (k + 1)])
    assert not r.read(bufs)  # 2000 bytes left: end of data
    r.close()


def test_reader_offset_binary_and_errors(tmp_path):
    d = np.arange(256, dtype=np.uint8)
    p = str(tmp_path / "a.dada")
    dada.write_stream(p, dict(FIELDS, NBIT=8, NDIM=2), d)
    r = dada.DadaReader([p], 256, offset_binary_8bit=True)
    buf = np.zeros(256, dtype=np.uint8)
    assert r.read([buf])
    assert np.array_equal(buf.view(np.int8), (d.astype(np.int16) - 128).astype(np.int8))
    r.close()
    with pytest.raises(L.GxcError):
        dada.DadaReader([str(tmp_path / "missing.dada")], 16)
    short = tmp_path / "short.dada"
    short.write_bytes(dada.make_header(dict(FIELDS), hdr_size=8192)[:5000])
    with pytest.raises(L.GxcError):
        dada.DadaReader([str(short)], 16)
