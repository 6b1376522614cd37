"""ctypes declarations for libgxcorr.so (the C ABI in include/gxc.h)."""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libgxcorr.so")

GXC_OK = 0
GXC_ERR_INVALID_ARGUMENT = 1
GXC_ERR_UNSUPPORTED = 2
GXC_ERR_CUDA = 3
GXC_ERR_OUT_OF_MEMORY = 4
GXC_ERR_STATE = 5
GXC_ERR_TIMEOUT = 6
GXC_END_OF_DATA = 7
GXC_PRECISION_FP32, GXC_PRECISION_FP16, GXC_PRECISION_FP8 = 0, 1, 2
# size of gxc_xcorr_noalloc's fixed device scratch array (include/gxc.h)
GXC_XCORR_NOALLOC_SCRATCH_BYTES = 16 << 20
GXC_ROTATOR_EXACT, GXC_ROTATOR_FXKERNEL = 0, 1
GXC_XENGINE_AUTO, GXC_XENGINE_CUDA_CORE, GXC_XENGINE_TENSOR = 0, 1, 2
GXC_FFT_AUTO, GXC_FFT_CUDA_CORE, GXC_FFT_TENSOR = 0, 1, 2
GXC_XSPLIT_AUTO, GXC_XSPLIT_OFF, GXC_XSPLIT_ON = 0, 1, 2
GXC_FP8_SCALE_CHANNEL, GXC_FP8_SCALE_HANDLE = 0, 1
_STATUS = {0: "ok", 1: "invalid argument", 2: "unsupported", 3: "CUDA error", 4: "out of memory",
           5: "bad call order", 6: "device wait timed out", 7: "end of data"}

# every function include/gxc.h declares (the CPU tests check the export list against the header)
EXPORTS = [
    "gxc_config_init", "gxc_validate_config", "gxc_input_bytes_per_antenna", "gxc_input_bytes_for_ffts",
    "gxc_num_baselines",
    "gxc_status_string", "gxc_create", "gxc_destroy", "gxc_set_input", "gxc_set_delays", "gxc_process",
    "gxc_sync", "gxc_accumulate", "gxc_get_visibilities", "gxc_device_visibilities", "gxc_get_baseline_counts",
    "gxc_get_valid_flags", "gxc_last_error", "gxc_last_launch_count", "gxc_fft_block", "gxc_num_blocks", "gxc_fft_engine", "gxc_enable_stage_timing",
    "gxc_stage_times", "gxc_xcorr", "gxc_xcorr_noalloc", "gxc_batch_create", "gxc_batch_launch", "gxc_batch_size",
    "gxc_batch_job", "gxc_batch_launch_count", "gxc_batch_destroy", "gxc_pipeline_create", "gxc_pipeline_submit",
    "gxc_pipeline_wait", "gxc_pipeline_sync", "gxc_pipeline_integration", "gxc_pipeline_set_lin2circ",
    "gxc_pipeline_handle", "gxc_pipeline_last_error", "gxc_pipeline_destroy", "gxc_lin2circ",
    "gxc_conf_read", "gxc_conf_config", "gxc_conf_int", "gxc_conf_double", "gxc_conf_antenna_name",
    "gxc_conf_antenna_file", "gxc_conf_delays", "gxc_conf_free", "gxc_reader_open", "gxc_reader_read",
    "gxc_reader_close", "gxc_save_visibilities", "gxc_host_alloc", "gxc_host_free", "gxc_set_frame_validity",
    "gxc_vdif_parse_header", "gxc_vdif_depacketize", "gxc_probe_unpack",
    "gxc_dada_parse_header", "gxc_dada_header_value", "gxc_dada_config", "gxc_dada_open", "gxc_dada_header_of",
    "gxc_dada_read", "gxc_dada_close",
]


class GxcConfig(C.Structure):
    _fields_ = [("nant", C.c_int), ("nchan", C.c_int), ("nfft", C.c_int), ("nbit", C.c_int),
                ("is_complex", C.c_int), ("lo_hz", C.c_double), ("bw_hz", C.c_double), ("precision", C.c_int),
                ("rotator", C.c_int), ("autos", C.c_int), ("x_engine", C.c_int), ("fft_block", C.c_int),
                ("device", C.c_int), ("fft_engine", C.c_int), ("x_split", C.c_int), ("fp8_scaling", C.c_int)]


class GxcVdifHeader(C.Structure):
    _fields_ = [("invalid", C.c_int), ("legacy", C.c_int), ("seconds", C.c_int64), ("ref_epoch", C.c_int),
                ("frame", C.c_int), ("version", C.c_int), ("nchan", C.c_int), ("frame_bytes", C.c_int),
                ("is_complex", C.c_int), ("bits", C.c_int), ("thread", C.c_int), ("station", C.c_int),
                ("header_bytes", C.c_int)]


class GxcDadaHeader(C.Structure):
    _fields_ = [("hdr_size", C.c_longlong), ("nbit", C.c_int), ("npol", C.c_int), ("ndim", C.c_int),
                ("nchan", C.c_int), ("bw_mhz", C.c_double), ("freq_mhz", C.c_double), ("tsamp_us", C.c_double),
                ("bytes_per_second", C.c_longlong), ("obs_offset", C.c_longlong), ("picoseconds", C.c_longlong),
                ("mjd_start", C.c_double), ("utc_start", C.c_char * 32), ("source", C.c_char * 64)]


class GxcJob(C.Structure):
    _fields_ = [("cfg", GxcConfig), ("inputs", C.c_void_p), ("poly", C.c_void_p), ("fso", C.c_void_p)]


class GxcError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(msg)
        self.status = status


_lib = None


def status_name(st: int) -> str:
    return _STATUS.get(int(st), f"status {st}")


def lib():
    """Load libgxcorr.so; raises if it has not been built (no fallback path exists)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is missing: build it with gcorr_gb300.build()")
        l = C.CDLL(LIB_PATH)
        P, V = C.POINTER, C.c_void_p
        l.gxc_config_init.argtypes = [P(GxcConfig)]
        l.gxc_config_init.restype = None
        l.gxc_validate_config.argtypes = [P(GxcConfig)]
        l.gxc_validate_config.restype = C.c_int
        l.gxc_input_bytes_per_antenna.argtypes = [P(GxcConfig)]
        l.gxc_input_bytes_per_antenna.restype = C.c_size_t
        l.gxc_input_bytes_for_ffts.argtypes = [P(GxcConfig), P(C.c_double), P(C.c_double), C.c_int, C.c_int]
        l.gxc_input_bytes_for_ffts.restype = C.c_longlong
        l.gxc_num_baselines.argtypes = [P(GxcConfig)]
        l.gxc_num_baselines.restype = C.c_int
        l.gxc_status_string.argtypes = [C.c_int]
        l.gxc_status_string.restype = C.c_char_p
        l.gxc_create.argtypes = [P(GxcConfig), P(V)]
        l.gxc_create.restype = C.c_int
        l.gxc_destroy.argtypes = [V]
        l.gxc_destroy.restype = C.c_int
        l.gxc_set_input.argtypes = [V, V, C.c_size_t]
        l.gxc_set_input.restype = C.c_int
        l.gxc_set_delays.argtypes = [V, V, V]
        l.gxc_set_delays.restype = C.c_int
        l.gxc_process.argtypes = [V, V]
        l.gxc_process.restype = C.c_int
        l.gxc_sync.argtypes = [V]
        l.gxc_sync.restype = C.c_int
        l.gxc_accumulate.argtypes = [V, V]
        l.gxc_accumulate.restype = C.c_int
        l.gxc_get_visibilities.argtypes = [V, V]
        l.gxc_get_visibilities.restype = C.c_int
        l.gxc_device_visibilities.argtypes = [V]
        l.gxc_device_visibilities.restype = V
        l.gxc_get_baseline_counts.argtypes = [V, V]
        l.gxc_get_baseline_counts.restype = C.c_int
        l.gxc_get_valid_flags.argtypes = [V, V]
        l.gxc_get_valid_flags.restype = C.c_int
        l.gxc_last_error.argtypes = [V]
        l.gxc_last_error.restype = C.c_char_p
        l.gxc_last_launch_count.argtypes = [V]
        l.gxc_last_launch_count.restype = C.c_int
        l.gxc_dada_parse_header.argtypes = [C.c_char_p, C.c_size_t, P(GxcDadaHeader)]
        l.gxc_dada_parse_header.restype = C.c_int
        l.gxc_dada_header_value.argtypes = [C.c_char_p, C.c_size_t, C.c_char_p, C.c_char_p, C.c_size_t]
        l.gxc_dada_header_value.restype = C.c_int
        l.gxc_dada_config.argtypes = [P(GxcDadaHeader), P(GxcConfig)]
        l.gxc_dada_config.restype = C.c_int
        l.gxc_dada_open.argtypes = [V, C.c_int, C.c_size_t, C.c_int, P(V)]
        l.gxc_dada_open.restype = C.c_int
        l.gxc_dada_header_of.argtypes = [V, C.c_int, P(GxcDadaHeader)]
        l.gxc_dada_header_of.restype = C.c_int
        l.gxc_dada_read.argtypes = [V, V]
        l.gxc_dada_read.restype = C.c_int
        l.gxc_dada_close.argtypes = [V]
        l.gxc_dada_close.restype = C.c_int
        l.gxc_probe_unpack.argtypes = [V, V]
        l.gxc_probe_unpack.restype = C.c_int
        l.gxc_fft_block.argtypes = [V]
        l.gxc_fft_block.restype = C.c_int
        l.gxc_num_blocks.argtypes = [V]
        l.gxc_num_blocks.restype = C.c_int
        l.gxc_fft_engine.argtypes = [V]
        l.gxc_fft_engine.restype = C.c_int
        l.gxc_enable_stage_timing.argtypes = [V, C.c_int]
        l.gxc_enable_stage_timing.restype = C.c_int
        l.gxc_stage_times.argtypes = [V, V, V, V]
        l.gxc_stage_times.restype = C.c_int
        l.gxc_xcorr.argtypes = [V, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, V, V]
        l.gxc_xcorr.restype = C.c_int
        l.gxc_xcorr_noalloc.argtypes = [V, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, V, V]
        l.gxc_xcorr_noalloc.restype = C.c_int
        l.gxc_batch_create.argtypes = [V, C.c_int, P(V)]
        l.gxc_batch_create.restype = C.c_int
        l.gxc_batch_launch.argtypes = [V, V]
        l.gxc_batch_launch.restype = C.c_int
        l.gxc_batch_size.argtypes = [V]
        l.gxc_batch_size.restype = C.c_int
        l.gxc_batch_job.argtypes = [V, C.c_int]
        l.gxc_batch_job.restype = V
        l.gxc_batch_launch_count.argtypes = [V]
        l.gxc_batch_launch_count.restype = C.c_int
        l.gxc_batch_destroy.argtypes = [V]
        l.gxc_batch_destroy.restype = C.c_int
        l.gxc_pipeline_create.argtypes = [P(GxcConfig), C.c_int, C.c_int, P(V)]
        l.gxc_pipeline_create.restype = C.c_int
        l.gxc_pipeline_submit.argtypes = [V, V, V, V, V, P(C.c_int64)]
        l.gxc_pipeline_submit.restype = C.c_int
        l.gxc_pipeline_wait.argtypes = [V, C.c_int64]
        l.gxc_pipeline_wait.restype = C.c_int
        l.gxc_pipeline_sync.argtypes = [V]
        l.gxc_pipeline_sync.restype = C.c_int
        l.gxc_pipeline_integration.argtypes = [V, V, C.c_int, P(C.c_int)]
        l.gxc_pipeline_integration.restype = C.c_int
        l.gxc_pipeline_set_lin2circ.argtypes = [V, C.c_int, V]
        l.gxc_pipeline_set_lin2circ.restype = C.c_int
        l.gxc_pipeline_handle.argtypes = [V]
        l.gxc_pipeline_handle.restype = V
        l.gxc_pipeline_last_error.argtypes = [V]
        l.gxc_pipeline_last_error.restype = C.c_char_p
        l.gxc_pipeline_destroy.argtypes = [V]
        l.gxc_pipeline_destroy.restype = C.c_int
        l.gxc_lin2circ.argtypes = [V, V, C.c_int, C.c_int, C.c_int, V]
        l.gxc_lin2circ.restype = C.c_int
        l.gxc_conf_read.argtypes = [C.c_char_p, P(V)]
        l.gxc_conf_read.restype = C.c_int
        l.gxc_conf_config.argtypes = [V, P(GxcConfig)]
        l.gxc_conf_config.restype = C.c_int
        l.gxc_conf_int.argtypes = [V, C.c_char_p]
        l.gxc_conf_int.restype = C.c_int
        l.gxc_conf_double.argtypes = [V, C.c_char_p]
        l.gxc_conf_double.restype = C.c_double
        l.gxc_conf_antenna_name.argtypes = [V, C.c_int]
        l.gxc_conf_antenna_name.restype = C.c_char_p
        l.gxc_conf_antenna_file.argtypes = [V, C.c_int]
        l.gxc_conf_antenna_file.restype = C.c_char_p
        l.gxc_conf_delays.argtypes = [V, V, V]
        l.gxc_conf_delays.restype = C.c_int
        l.gxc_conf_free.argtypes = [V]
        l.gxc_conf_free.restype = None
        l.gxc_reader_open.argtypes = [V, C.c_int, C.c_size_t, P(V)]
        l.gxc_reader_open.restype = C.c_int
        l.gxc_reader_read.argtypes = [V, V]
        l.gxc_reader_read.restype = C.c_int
        l.gxc_reader_close.argtypes = [V]
        l.gxc_reader_close.restype = C.c_int
        l.gxc_save_visibilities.argtypes = [C.c_char_p, V, C.c_int, C.c_int, C.c_double]
        l.gxc_save_visibilities.restype = C.c_int
        l.gxc_host_alloc.argtypes = [C.c_size_t, P(V)]
        l.gxc_host_alloc.restype = C.c_int
        l.gxc_host_free.argtypes = [V]
        l.gxc_host_free.restype = C.c_int
        l.gxc_set_frame_validity.argtypes = [V, V, C.c_size_t, C.c_int64]
        l.gxc_set_frame_validity.restype = C.c_int
        l.gxc_vdif_parse_header.argtypes = [V, P(GxcVdifHeader)]
        l.gxc_vdif_parse_header.restype = C.c_int
        l.gxc_vdif_depacketize.argtypes = [V, C.c_size_t, C.c_int, C.c_int, C.c_int64, C.c_int, C.c_int, C.c_int,
                                           C.c_int, C.c_uint8, V, C.c_size_t, V, V, V]
        l.gxc_vdif_depacketize.restype = C.c_int
        _lib = l
    return _lib


def check(st: int, handle, what: str):
    if st != GXC_OK:
        msg = ""
        if handle is not None:
            m = lib().gxc_last_error(handle)
            msg = m.decode() if m else ""
        raise GxcError(st, f"{what}: {status_name(st)}" + (f": {msg}" if msg else ""))
