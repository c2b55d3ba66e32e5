"""ctypes binding of libvhsdecode_gb300 (include/vhsdecode_gb300.h).

Mirrors the reference's managed-to-native layer for the cuda-fast backend
(Core/Dsp/CudaFast/CudaFastNativeRuntime.cs:73-119, 180-185, 491-621):
the library is loaded by path, the ABI version is checked, struct layouts
carry ``struct_size``, and every non-zero status raises -- CANCELLED as
``OperationCanceled``, CUDA_UNAVAILABLE as ``BackendUnavailable``, anything
else as ``NativeError`` (CudaFastNativeRuntime.cs:595-618).  There is no CPU
fallback: a missing library or device raises.
"""
import ctypes
import os

import numpy as np

ABI_VERSION = 0x00010005
STATUS_OK = 0
STATUS_NULL_POINTER = -20000
STATUS_INVALID_ARGUMENT = -20001
STATUS_CUDA_UNAVAILABLE = -20002
STATUS_INPUT_ERROR = -20003
STATUS_OUTPUT_ERROR = -20004
STATUS_DECODE_ERROR = -20005
STATUS_CANCELLED = -20006
STATUS_INTERNAL_ERROR = -20007

PROFILE_NTSC, PROFILE_PAL, PROFILE_PAL_M = 0, 1, 2
TAPE_SP, TAPE_LP, TAPE_EP = 0, 1, 2
FORMAT_VHS, FORMAT_SVHS = 0, 1
INPUT_FLOAT32, INPUT_INT16, INPUT_FLAC = 0, 1, 2
PRECISION_FP32_FUSED, PRECISION_FP64_PLAIN = 0, 1
DECODE_DEVICE_INPUT = 0x1
DECODE_DEMOD_ONLY = 0x2
DECODE_FLOAT_INPUT = 0x4
DECODE_CHROMA = 0x8

LIB_PATH = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "lib",
                        "libvhsdecode_gb300.so")

EXPORTS = [
    "vhsdecode_gb300_flac_info", "vhsdecode_gb300_flac_decode",
    "vhsdecode_gb300_get_abi_version", "vhsdecode_gb300_get_runtime_info", "vhsdecode_gb300_run",
    "vhsdecode_gb300_get_last_error", "vhsdecode_gb300_session_create",
    "vhsdecode_gb300_session_destroy", "vhsdecode_gb300_session_set_stream",
    "vhsdecode_gb300_session_decode", "vhsdecode_gb300_session_get_field",
    "vhsdecode_gb300_session_copy_tbc", "vhsdecode_gb300_session_copy_lines",
    "vhsdecode_gb300_session_copy_dropouts", "vhsdecode_gb300_session_copy_stream",
    "vhsdecode_gb300_session_tbc_device", "vhsdecode_gb300_design_filters",
    "vhsdecode_gb300_session_copy_chroma", "vhsdecode_gb300_design_chroma",
    "vhsdecode_gb300_session_copy_chroma_stage",
    "vhsdecode_gb300_field_sync", "vhsdecode_gb300_tbc_resample_lines",
    "vhsdecode_gb300_find_pulses", "vhsdecode_gb300_vhs_angles",
    "vhsdecode_gb300_pulse_events_noalloc", "vhsdecode_gb300_vhs_demod",
    "vhsdecode_gb300_server_create", "vhsdecode_gb300_server_submit", "vhsdecode_gb300_server_wait",
    "vhsdecode_gb300_server_destroy", "vhsdecode_gb300_replace_spikes",
    "vhsdecode_gb300_decimate_half_rate",
]


class NativeError(RuntimeError):
    def __init__(self, status, message):
        super().__init__("%s (status %d)" % (message, status))
        self.status = status


class OperationCanceled(NativeError):
    pass


class BackendUnavailable(NativeError):
    pass


READ_CB = ctypes.CFUNCTYPE(ctypes.c_size_t, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint64,
                           ctypes.c_size_t)
CANCEL_CB = ctypes.CFUNCTYPE(ctypes.c_int32, ctypes.c_void_p)


class FlacInfo(ctypes.Structure):
    _fields_ = [("struct_size", ctypes.c_uint32), ("sample_rate", ctypes.c_uint32),
                ("channels", ctypes.c_uint32), ("bits_per_sample", ctypes.c_uint32),
                ("min_block", ctypes.c_uint32), ("max_block", ctypes.c_uint32),
                ("total_samples", ctypes.c_uint64), ("first_frame_offset", ctypes.c_uint64)]


class RuntimeInfo(ctypes.Structure):
    _fields_ = [("struct_size", ctypes.c_uint32), ("abi_version", ctypes.c_uint32),
                ("device_id", ctypes.c_int32), ("compute_major", ctypes.c_int32),
                ("compute_minor", ctypes.c_int32), ("multiprocessor_count", ctypes.c_int32),
                ("total_vram_bytes", ctypes.c_uint64), ("free_vram_bytes", ctypes.c_uint64),
                ("device_name", ctypes.c_char * 128)]


class RunConfig(ctypes.Structure):
    _fields_ = [("struct_size", ctypes.c_uint32), ("profile", ctypes.c_uint32),
                ("tape_speed", ctypes.c_uint32), ("device_id", ctypes.c_int32),
                ("sample_rate_mhz", ctypes.c_double), ("total_samples", ctypes.c_uint64),
                ("output_base_utf8", ctypes.c_char_p), ("overwrite", ctypes.c_int32),
                ("input_sample_format", ctypes.c_uint32), ("maximum_output_fields", ctypes.c_uint32),
                ("device_decimation_factor", ctypes.c_uint32), ("read_callback", READ_CB),
                ("cancel_callback", CANCEL_CB), ("user_data", ctypes.c_void_p)]


class RunConfigV2(ctypes.Structure):
    """config_v1 followed by the tape format and decode flags (vhsdecode_gb300_config_v2)."""
    _fields_ = RunConfig._fields_ + [("tape_format", ctypes.c_uint32), ("decode_flags", ctypes.c_uint32)]


class RunResult(ctypes.Structure):
    _fields_ = [("struct_size", ctypes.c_uint32), ("fields_written", ctypes.c_uint32),
                ("output_line_length", ctypes.c_uint32), ("output_field_lines", ctypes.c_uint32),
                ("elapsed_seconds", ctypes.c_double)]


class SessionConfig(ctypes.Structure):
    _fields_ = [("struct_size", ctypes.c_uint32), ("profile", ctypes.c_uint32),
                ("tape_speed", ctypes.c_uint32), ("device_id", ctypes.c_int32),
                ("sample_rate_mhz", ctypes.c_double), ("max_samples", ctypes.c_uint64),
                ("precision", ctypes.c_uint32), ("max_fields", ctypes.c_uint32),
                ("tape_format", ctypes.c_uint32), ("decimation", ctypes.c_uint32)]


class DecodeResult(ctypes.Structure):
    _fields_ = [("struct_size", ctypes.c_uint32), ("fields", ctypes.c_uint32),
                ("output_line_length", ctypes.c_uint32), ("output_field_lines", ctypes.c_uint32),
                ("blocks", ctypes.c_uint64), ("stream_samples", ctypes.c_uint64),
                ("repaired_blocks", ctypes.c_uint32), ("stop_reason", ctypes.c_uint32),
                ("device_ms", ctypes.c_double), ("demod_ms", ctypes.c_double),
                ("field_ms", ctypes.c_double), ("host_ms", ctypes.c_double),
                ("kernel_launches", ctypes.c_uint32), ("segments", ctypes.c_uint32),
                ("fft_plan", ctypes.c_uint32), ("reserved", ctypes.c_uint32)]


class FieldInfo(ctypes.Structure):
    _fields_ = [("struct_size", ctypes.c_uint32), ("is_first_field", ctypes.c_int32),
                ("span_start", ctypes.c_int64), ("file_loc", ctypes.c_int64),
                ("line0", ctypes.c_double), ("first_hsync", ctypes.c_double),
                ("mean_line_length", ctypes.c_double), ("next_field_offset", ctypes.c_double),
                ("line_count", ctypes.c_uint32), ("dropout_count", ctypes.c_uint32)]


class ServerConfig(ctypes.Structure):
    _fields_ = [("struct_size", ctypes.c_uint32), ("device_id", ctypes.c_int32),
                ("workers", ctypes.c_uint32), ("max_batch", ctypes.c_uint32),
                ("max_window_samples", ctypes.c_uint64), ("memory_budget_bytes", ctypes.c_uint64)]


class Window(ctypes.Structure):
    _fields_ = [("struct_size", ctypes.c_uint32), ("stream_id", ctypes.c_uint32),
                ("profile", ctypes.c_uint32), ("tape_speed", ctypes.c_uint32),
                ("sample_rate_mhz", ctypes.c_double), ("samples", ctypes.c_void_p),
                ("sample_count", ctypes.c_uint64), ("source_offset", ctypes.c_uint64),
                ("seek", ctypes.c_uint32), ("max_fields", ctypes.c_uint32),
                ("tbc_out", ctypes.c_void_p), ("tbc_capacity", ctypes.c_uint64),
                ("tape_format", ctypes.c_uint32), ("decimation", ctypes.c_uint32)]


class WindowResult(ctypes.Structure):
    _fields_ = [("struct_size", ctypes.c_uint32), ("status", ctypes.c_int32),
                ("stream_id", ctypes.c_uint32), ("fields", ctypes.c_uint32),
                ("first_field_is_first", ctypes.c_uint32), ("continued", ctypes.c_uint32),
                ("ticket", ctypes.c_uint64), ("sample_count", ctypes.c_uint64),
                ("next_source_offset", ctypes.c_uint64), ("queue_ms", ctypes.c_double),
                ("decode_ms", ctypes.c_double), ("latency_ms", ctypes.c_double),
                ("batched", ctypes.c_uint32), ("reserved", ctypes.c_uint32)]


_lib = None
_P = ctypes.POINTER
_vp = ctypes.c_void_p


def load(path: str = LIB_PATH):
    """Load the library (built by ``vhsd_gb300.build``); raises if it is missing."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise BackendUnavailable(STATUS_CUDA_UNAVAILABLE,
                                 "libvhsdecode_gb300.so is not built (%s)" % path)
    L = ctypes.CDLL(path)
    L.vhsdecode_gb300_get_abi_version.restype = ctypes.c_uint32
    L.vhsdecode_gb300_get_last_error.restype = ctypes.c_char_p
    L.vhsdecode_gb300_get_runtime_info.argtypes = [ctypes.c_int32, _P(RuntimeInfo)]
    # config_v1 or config_v2, told apart by struct_size
    L.vhsdecode_gb300_run.argtypes = [ctypes.c_void_p, _P(RunResult)]
    L.vhsdecode_gb300_session_create.argtypes = [_P(SessionConfig), _P(_vp)]
    L.vhsdecode_gb300_session_destroy.argtypes = [_vp]
    L.vhsdecode_gb300_session_destroy.restype = None
    L.vhsdecode_gb300_session_set_stream.argtypes = [_vp, _vp]
    L.vhsdecode_gb300_session_decode.argtypes = [_vp, _vp, ctypes.c_uint64, ctypes.c_uint32,
                                                 ctypes.c_uint32, _P(DecodeResult)]
    L.vhsdecode_gb300_session_get_field.argtypes = [_vp, ctypes.c_uint32, _P(FieldInfo)]
    L.vhsdecode_gb300_session_copy_tbc.argtypes = [_vp, ctypes.c_uint32, ctypes.c_uint32, _vp]
    L.vhsdecode_gb300_session_copy_chroma.argtypes = [_vp, ctypes.c_uint32, ctypes.c_uint32, _vp]
    L.vhsdecode_gb300_session_copy_chroma_stage.argtypes = [_vp, ctypes.c_uint32, ctypes.c_uint32, _vp,
                                                            ctypes.c_uint64, _P(ctypes.c_uint64)]
    L.vhsdecode_gb300_design_chroma.argtypes = [ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32,
                                                ctypes.c_double, _vp, _vp, _vp, _vp, _vp, _vp]
    L.vhsdecode_gb300_session_copy_lines.argtypes = [_vp, ctypes.c_uint32, _vp, ctypes.c_uint32]
    L.vhsdecode_gb300_session_copy_dropouts.argtypes = [_vp, ctypes.c_uint32, _vp, _vp, _vp,
                                                        ctypes.c_uint32, _P(ctypes.c_uint32)]
    L.vhsdecode_gb300_session_copy_stream.argtypes = [_vp, ctypes.c_uint32, ctypes.c_uint64,
                                                      ctypes.c_uint64, _vp]
    L.vhsdecode_gb300_session_tbc_device.argtypes = [_vp, _P(_vp), _P(ctypes.c_uint64)]
    L.vhsdecode_gb300_design_filters.argtypes = [ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32,
                                                 ctypes.c_double, _vp, _vp, _vp, _vp, _vp]
    L.vhsdecode_gb300_field_sync.argtypes = [ctypes.c_uint32, ctypes.c_double, _vp, _vp,
                                             ctypes.c_uint64, ctypes.c_int64, _vp, _vp, _vp, _vp,
                                             ctypes.c_uint32, _P(ctypes.c_uint32)]
    L.vhsdecode_gb300_tbc_resample_lines.argtypes = [_vp, ctypes.c_uint64, _vp, ctypes.c_uint32,
                                                     ctypes.c_uint32, ctypes.c_uint32,
                                                     ctypes.c_uint32, ctypes.c_double,
                                                     ctypes.c_double, _vp]
    L.vhsdecode_gb300_find_pulses.argtypes = [_vp, ctypes.c_uint64, ctypes.c_double, ctypes.c_int64,
                                              ctypes.c_int64, _vp, _vp, ctypes.c_uint64,
                                              _P(ctypes.c_uint64)]
    L.vhsdecode_gb300_vhs_angles.argtypes = [_vp, _vp, ctypes.c_uint64, _vp]
    L.vhsdecode_gb300_vhs_demod.argtypes = [_vp, _vp, ctypes.c_uint64, ctypes.c_double, _vp]
    L.vhsdecode_gb300_replace_spikes.argtypes = [_vp, _vp, ctypes.c_uint64, ctypes.c_float]
    L.vhsdecode_gb300_decimate_half_rate.argtypes = [_vp, ctypes.c_uint32, ctypes.c_uint64, _vp]
    L.vhsdecode_gb300_server_create.argtypes = [_P(ServerConfig), _P(_vp)]
    L.vhsdecode_gb300_server_submit.argtypes = [_vp, _P(Window), _P(ctypes.c_uint64)]
    L.vhsdecode_gb300_server_wait.argtypes = [_vp, ctypes.c_uint64, _P(WindowResult)]
    L.vhsdecode_gb300_server_destroy.argtypes = [_vp]
    L.vhsdecode_gb300_server_destroy.restype = None
    L.vhsdecode_gb300_pulse_events_noalloc.argtypes = [_vp, ctypes.c_int64, ctypes.c_double, _vp,
                                                       ctypes.c_int64, _vp, _vp]
    L.vhsdecode_gb300_flac_info.argtypes = [_vp, ctypes.c_uint64, _P(FlacInfo)]
    L.vhsdecode_gb300_flac_decode.argtypes = [_vp, ctypes.c_uint64, _vp, ctypes.c_uint64,
                                              _P(ctypes.c_uint64), ctypes.c_int32]
    for name in EXPORTS:
        if not hasattr(L, name):
            raise NativeError(STATUS_INTERNAL_ERROR, "missing export " + name)
    if L.vhsdecode_gb300_get_abi_version() != ABI_VERSION:
        raise NativeError(STATUS_INTERNAL_ERROR, "ABI version mismatch")
    _lib = L
    return L


def check(status):
    if status == STATUS_OK:
        return
    msg = (load().vhsdecode_gb300_get_last_error() or b"").decode("utf-8", "replace")
    if status == STATUS_CANCELLED:
        raise OperationCanceled(status, msg)
    if status == STATUS_CUDA_UNAVAILABLE:
        raise BackendUnavailable(status, msg)
    raise NativeError(status, msg)


def _ptr(a):
    return ctypes.c_void_p(a.ctypes.data)


def flac_info(data):
    """STREAMINFO of a FLAC stream (bytes), through the C ABI (no GPU needed)."""
    info = FlacInfo()
    info.struct_size = ctypes.sizeof(FlacInfo)
    buf = np.frombuffer(bytes(data), np.uint8)
    check(load().vhsdecode_gb300_flac_info(_ptr(buf), len(buf), ctypes.byref(info)))
    return info


def flac_decode(data, device=0):
    """int16 samples of a 16-bit mono FLAC stream, decoded on the GPU (one call
    when STREAMINFO states the length; a second, larger one when it is short)."""
    buf = np.frombuffer(bytes(data), np.uint8)
    n = ctypes.c_uint64(0)
    L = load()
    out = np.empty(max(1, flac_info(data).total_samples), np.int16)
    check(L.vhsdecode_gb300_flac_decode(_ptr(buf), len(buf), _ptr(out), len(out), ctypes.byref(n),
                                        device))
    if n.value > len(out):
        out = np.empty(n.value, np.int16)
        check(L.vhsdecode_gb300_flac_decode(_ptr(buf), len(buf), _ptr(out), len(out),
                                            ctypes.byref(n), device))
    return out[:n.value]


def runtime_info(device=0):
    info = RuntimeInfo()
    info.struct_size = ctypes.sizeof(RuntimeInfo)
    check(load().vhsdecode_gb300_get_runtime_info(device, ctypes.byref(info)))
    return info


def design_filters(profile, sample_rate_mhz=40.0, tape_speed=TAPE_SP, tape_format=FORMAT_VHS,
                   sub=False):
    """(rf_video, video, sync, env b0/b1/a1); with ``sub`` also (sub_high, sub b0/b1/a1)."""
    n = 16385
    rv = np.zeros(n)
    v = np.zeros(2 * n)
    s = np.zeros(2 * n)
    h = np.zeros(2 * n)
    env = np.zeros(6)
    check(load().vhsdecode_gb300_design_filters(profile, tape_speed, tape_format, sample_rate_mhz,
                                                _ptr(rv), _ptr(v), _ptr(s), _ptr(h), _ptr(env)))
    out = (rv, v[0::2] + 1j * v[1::2], s[0::2] + 1j * s[1::2], env[:3])
    if sub:
        out = out + (h[0::2] + 1j * h[1::2], env[3:])
    return out


def design_chroma(profile, sample_rate_mhz=40.0, tape_speed=TAPE_SP, tape_format=FORMAT_VHS, tables=False):
    """Chroma design of the library: dict with rf_sos and final_sos (4 x 6),
    burst_start, burst_end, move, rf_edge, final_edge, rotation, field_samples
    and, with ``tables``, the heterodyne (4 x field) and burst sin/cos tables."""
    rf = np.zeros(24)
    fin = np.zeros(24)
    g = np.zeros(8, np.int32)
    check(load().vhsdecode_gb300_design_chroma(profile, tape_speed, tape_format, sample_rate_mhz, _ptr(rf),
                                               _ptr(fin), _ptr(g), None, None, None))
    out = {"rf_sos": rf.reshape(4, 6), "final_sos": fin.reshape(4, 6), "burst_start": int(g[0]),
           "burst_end": int(g[1]), "move": int(g[2]), "rf_edge": int(g[3]), "final_edge": int(g[4]),
           "rotation": [int(g[5]), int(g[6])], "field_samples": int(g[7])}
    if tables:
        n = out["field_samples"]
        het = np.zeros(4 * n, np.float32)
        bs = np.zeros(n, np.float32)
        bc = np.zeros(n, np.float32)
        check(load().vhsdecode_gb300_design_chroma(profile, tape_speed, tape_format, sample_rate_mhz, _ptr(rf),
                                                   _ptr(fin), _ptr(g), _ptr(het), _ptr(bs), _ptr(bc)))
        out.update(heterodyne=het.reshape(4, n), burst_sin=bs, burst_cos=bc)
    return out


def field_sync(profile, pulses, span_len, state, ref=None, sample_rate_mhz=40.0):
    """Host control plane on raw pulses; ``state`` is a 2-element int32 array updated in place."""
    starts = np.ascontiguousarray([p[0] for p in pulses], np.int64)
    lens = np.ascontiguousarray([p[1] for p in pulses], np.int64)
    out = np.zeros(5)
    locs = np.zeros(2048)
    cnt = ctypes.c_uint32(0)
    refp = None
    if ref is not None:
        ref = np.ascontiguousarray(ref, np.float64)
        refp = _ptr(ref)
    check(load().vhsdecode_gb300_field_sync(profile, sample_rate_mhz, _ptr(starts), _ptr(lens),
                                            len(starts), int(span_len), refp, _ptr(state), _ptr(out),
                                            _ptr(locs), len(locs), ctypes.byref(cnt)))
    return {"first_field": bool(out[0]), "line0": out[1], "first_hsync": out[2],
            "mean_line": out[3], "next_offset": out[4], "locs": locs[:cnt.value].copy()}


def tbc_resample_lines(source, locations, first_line, line_count, outlen, nominal=0.0,
                       smoothing=0.0):
    src = np.ascontiguousarray(source, np.float64)
    loc = np.ascontiguousarray(locations, np.float64)
    out = np.zeros(line_count * outlen)
    check(load().vhsdecode_gb300_tbc_resample_lines(_ptr(src), len(src), _ptr(loc), len(loc),
                                                    first_line, line_count, outlen, nominal,
                                                    smoothing, _ptr(out)))
    return out


def find_pulses(ref, high, min_len, max_len):
    r = np.ascontiguousarray(ref, np.float64)
    cap = max(16, len(r) // 2 + 1)
    st = np.zeros(cap, np.int64)
    ln = np.zeros(cap, np.int64)
    cnt = ctypes.c_uint64(0)
    check(load().vhsdecode_gb300_find_pulses(_ptr(r), len(r), float(high), int(min_len),
                                             int(max_len), _ptr(st), _ptr(ln), cap,
                                             ctypes.byref(cnt)))
    n = cnt.value
    return list(zip(st[:n].tolist(), ln[:n].tolist()))


def vhs_angles(re, im):
    re = np.ascontiguousarray(re, np.float32)
    im = np.ascontiguousarray(im, np.float32)
    out = np.zeros(len(re), np.float32)
    check(load().vhsdecode_gb300_vhs_angles(_ptr(re), _ptr(im), len(re), _ptr(out)))
    return out


def vhs_demod(re, im, fs):
    re = np.ascontiguousarray(re, np.float32)
    im = np.ascontiguousarray(im, np.float32)
    out = np.zeros(len(re), np.float32)
    check(load().vhsdecode_gb300_vhs_demod(_ptr(re), _ptr(im), len(re), float(fs), _ptr(out)))
    return out


def decimate_half_rate(source):
    """Device 2:1 half-band decimation of an int16 or float32 capture
    (len // 2 float32 samples)."""
    src = np.ascontiguousarray(source)
    if src.dtype == np.int16:
        fmt = INPUT_INT16
    elif src.dtype == np.float32:
        fmt = INPUT_FLOAT32
    else:
        raise TypeError("int16 or float32 capture expected")
    out = np.zeros(len(src) // 2, np.float32)
    check(load().vhsdecode_gb300_decimate_half_rate(_ptr(src), fmt, len(src), _ptr(out)))
    return out


def replace_spikes(demod, diffed, max_value):
    d = np.ascontiguousarray(demod, np.float32).copy()
    f = np.ascontiguousarray(diffed, np.float32)
    check(load().vhsdecode_gb300_replace_spikes(_ptr(d), _ptr(f), len(d), float(max_value)))
    return d


class Session:
    """Device-resident decode context (session API of include/vhsdecode_gb300.h)."""

    def __init__(self, profile, max_samples, precision=PRECISION_FP32_FUSED, device=0,
                 sample_rate_mhz=40.0, max_fields=0, tape_format=FORMAT_VHS, decimation=1,
                 tape_speed=TAPE_SP):
        L = load()
        cfg = SessionConfig()
        cfg.struct_size = ctypes.sizeof(SessionConfig)
        cfg.profile = profile
        cfg.tape_speed = tape_speed
        cfg.tape_format = tape_format
        cfg.device_id = device
        cfg.sample_rate_mhz = sample_rate_mhz
        cfg.max_samples = int(max_samples)
        cfg.precision = precision
        cfg.max_fields = max_fields
        cfg.decimation = decimation
        h = ctypes.c_void_p()
        check(L.vhsdecode_gb300_session_create(ctypes.byref(cfg), ctypes.byref(h)))
        self._h = h
        self.profile = profile
        self.last = None

    def close(self):
        if getattr(self, "_h", None):
            load().vhsdecode_gb300_session_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def set_stream(self, stream_handle):
        check(load().vhsdecode_gb300_session_set_stream(self._h, ctypes.c_void_p(stream_handle)))

    def decode(self, rf, max_fields=0, demod_only=False, device_ptr=None, count=None, float_input=None,
               chroma=False):
        """Decode int16 samples (or float32 ones: a float32 array, or
        ``float_input=True`` with ``device_ptr``); ``chroma`` renders the
        colour-under chroma (and refines the lines from the burst) as the
        reference's default decode does."""
        r = DecodeResult()
        r.struct_size = ctypes.sizeof(DecodeResult)
        flags = DECODE_DEMOD_ONLY if demod_only else 0
        if chroma:
            flags |= DECODE_CHROMA
        if device_ptr is not None:
            flags |= DECODE_DEVICE_INPUT
            ptr, n = ctypes.c_void_p(device_ptr), int(count)
            if float_input:
                flags |= DECODE_FLOAT_INPUT
        else:
            if float_input or (float_input is None and np.asarray(rf).dtype == np.float32):
                rf = np.ascontiguousarray(rf, np.float32)
                flags |= DECODE_FLOAT_INPUT
            else:
                rf = np.ascontiguousarray(rf, np.int16)
            ptr, n = _ptr(rf), len(rf)
        check(load().vhsdecode_gb300_session_decode(self._h, ptr, n, max_fields, flags,
                                                    ctypes.byref(r)))
        self.last = r
        return r

    def field(self, i):
        fi = FieldInfo()
        fi.struct_size = ctypes.sizeof(FieldInfo)
        check(load().vhsdecode_gb300_session_get_field(self._h, i, ctypes.byref(fi)))
        return fi

    def tbc(self, first=0, count=None, out=None):
        if count is None:
            count = self.last.fields - first
        n = count * self.last.output_field_lines * self.last.output_line_length
        if out is None:
            out = np.zeros(n, np.uint16)
        check(load().vhsdecode_gb300_session_copy_tbc(self._h, first, count, _ptr(out)))
        return out.reshape(count, self.last.output_field_lines, self.last.output_line_length)

    def chroma(self, first=0, count=None, out=None):
        if count is None:
            count = self.last.fields - first
        n = count * self.last.output_field_lines * self.last.output_line_length
        if out is None:
            out = np.zeros(n, np.uint16)
        check(load().vhsdecode_gb300_session_copy_chroma(self._h, first, count, _ptr(out)))
        return out.reshape(count, self.last.output_field_lines, self.last.output_line_length)

    def chroma_stage(self, field, stage):
        """Intermediate chroma of one field (0 TBC, 1 band-passed up-conversion,
        2 probe windows, 3 kept burst sequence + rotation index, 4 averages,
        5 hsync-refined lines before the burst refinement)."""
        n = max(self.last.output_field_lines * self.last.output_line_length,
                self.last.output_field_lines * 5 + 1, 1 << 20)
        out = np.zeros(n)
        cnt = ctypes.c_uint64(0)
        check(load().vhsdecode_gb300_session_copy_chroma_stage(self._h, field, stage, _ptr(out), n,
                                                               ctypes.byref(cnt)))
        return out[:cnt.value]

    def chroma_into(self, first, count, host_ptr):
        check(load().vhsdecode_gb300_session_copy_chroma(self._h, first, count, ctypes.c_void_p(host_ptr)))

    def tbc_into(self, first, count, host_ptr):
        check(load().vhsdecode_gb300_session_copy_tbc(self._h, first, count,
                                                      ctypes.c_void_p(host_ptr)))

    def lines(self, i):
        fi = self.field(i)
        out = np.zeros(fi.line_count)
        check(load().vhsdecode_gb300_session_copy_lines(self._h, i, _ptr(out), len(out)))
        return out

    def dropouts(self, i):
        fi = self.field(i)
        n = max(1, fi.dropout_count)
        a = np.zeros(n, np.int32)
        b = np.zeros(n, np.int32)
        c = np.zeros(n, np.int32)
        cnt = ctypes.c_uint32(0)
        check(load().vhsdecode_gb300_session_copy_dropouts(self._h, i, _ptr(a), _ptr(b), _ptr(c), n,
                                                           ctypes.byref(cnt)))
        k = cnt.value
        return list(zip(a[:k].tolist(), b[:k].tolist(), c[:k].tolist()))

    def stream(self, channel, start, count):
        out = np.zeros(count)
        check(load().vhsdecode_gb300_session_copy_stream(self._h, channel, start, count, _ptr(out)))
        return out

    def tbc_device(self):
        p = ctypes.c_void_p()
        b = ctypes.c_uint64()
        check(load().vhsdecode_gb300_session_tbc_device(self._h, ctypes.byref(p), ctypes.byref(b)))
        return p.value, b.value


class Server:
    """Window server (serving API of include/vhsdecode_gb300.h): windows of many
    client streams decoded concurrently on one GPU, in order per stream."""

    def __init__(self, max_window_samples, workers=4, memory_budget=0, device=0, max_batch=1):
        L = load()
        cfg = ServerConfig(ctypes.sizeof(ServerConfig), device, workers, max_batch,
                           int(max_window_samples), int(memory_budget))
        h = _vp()
        check(L.vhsdecode_gb300_server_create(ctypes.byref(cfg), ctypes.byref(h)))
        self._h = h
        self._keep = {}

    def submit(self, stream_id, profile, rf, source_offset=0, seek=False, max_fields=0, tbc_out=None,
               sample_rate_mhz=40.0, tape_speed=TAPE_SP, tape_format=FORMAT_VHS, decimation=1):
        """Queue a window (``rf``: int16 host array, kept alive until ``wait``); returns a ticket.
        With ``decimation=2`` the samples run at twice ``sample_rate_mhz``."""
        rf = np.ascontiguousarray(rf, np.int16)
        w = Window(ctypes.sizeof(Window), stream_id, profile, tape_speed, float(sample_rate_mhz),
                   rf.ctypes.data, len(rf), int(source_offset), 1 if seek else 0, int(max_fields),
                   tbc_out.ctypes.data if tbc_out is not None else None,
                   tbc_out.size if tbc_out is not None else 0, int(tape_format), int(decimation))
        t = ctypes.c_uint64(0)
        check(load().vhsdecode_gb300_server_submit(self._h, ctypes.byref(w), ctypes.byref(t)))
        self._keep[t.value] = (rf, tbc_out)
        return t.value

    def wait(self, ticket):
        """Block until the window is done; returns its WindowResult (raises on a failed window)."""
        r = WindowResult()
        r.struct_size = ctypes.sizeof(WindowResult)
        st = load().vhsdecode_gb300_server_wait(self._h, ticket, ctypes.byref(r))
        self._keep.pop(ticket, None)
        check(st)
        return r

    def close(self):
        if self._h:
            load().vhsdecode_gb300_server_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
