"""ctypes loader for oracle/oracle_c.c (test infrastructure).

The shared object is built by ``oracle/build_oracle.py`` (called from
``__graft_entry__.build()``) into ``oracle/_build/``.
"""
import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_SO = os.path.join(_HERE, "_build", "liboracle.so")
_lib = None

_dp = ctypes.POINTER(ctypes.c_double)
_fp = ctypes.POINTER(ctypes.c_float)
_i64p = ctypes.POINTER(ctypes.c_int64)
_u16p = ctypes.POINTER(ctypes.c_uint16)


def build(force: bool = False) -> str:
    os.makedirs(os.path.dirname(_SO), exist_ok=True)
    src = os.path.join(_HERE, "oracle_c.c")
    if force or not os.path.exists(_SO) or os.path.getmtime(_SO) < os.path.getmtime(src):
        subprocess.check_call(["gcc", "-O2", "-fPIC", "-shared", "-ffp-contract=off",
                               "-fno-fast-math", "-o", _SO, src, "-lm"])
    return _SO


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(_SO)
        L.oracle_vhs_rust_demod.argtypes = [_dp, _dp, ctypes.c_int64, ctypes.c_double, _dp]
        L.oracle_vhs_rust_angles.argtypes = [_fp, _fp, ctypes.c_int64, _fp]
        L.oracle_vhs_envelope.argtypes = [_dp, ctypes.c_int64, ctypes.c_double, ctypes.c_double,
                                          ctypes.c_double, _dp, _fp]
        L.oracle_vhs_raw_envelope.argtypes = [_dp, ctypes.c_int64, _fp]
        L.oracle_filtfilt1_f64.argtypes = [_dp, ctypes.c_int64, ctypes.c_double, ctypes.c_double,
                                           ctypes.c_double, _dp, _dp]
        L.oracle_find_pulses.argtypes = [_dp, ctypes.c_int64, ctypes.c_double, ctypes.c_int64,
                                         ctypes.c_int64, _i64p, _i64p, ctypes.c_int64]
        L.oracle_find_pulses.restype = ctypes.c_int64
        L.oracle_sinc_resample.argtypes = [_dp, ctypes.c_int64, _dp, _dp, ctypes.c_int64, _fp, _dp]
        L.oracle_hz_to_u16.argtypes = [_dp, ctypes.c_int64, ctypes.c_double, ctypes.c_double,
                                       ctypes.c_double, ctypes.c_double, ctypes.c_double, _u16p]
        L.oracle_build_sinc_lut.argtypes = [_fp]
        L.oracle_smooth_levels.argtypes = [_dp, ctypes.c_int64, ctypes.c_double]
        L.oracle_find_dropouts.argtypes = [_dp, ctypes.c_int64, ctypes.c_int64, ctypes.c_double,
                                           ctypes.c_double, ctypes.c_int64, ctypes.c_int64, _i64p,
                                           _i64p, ctypes.c_int64]
        L.oracle_find_dropouts.restype = ctypes.c_int64
        L.oracle_decimate_half_s16.argtypes = [ctypes.POINTER(ctypes.c_int16), ctypes.c_int64, _fp]
        L.oracle_decimate_half_f32.argtypes = [_fp, ctypes.c_int64, _fp]
        L.oracle_sosfiltfilt_f32.argtypes = [_dp, ctypes.c_int64, _dp, ctypes.c_int, ctypes.c_int64, _fp, _fp]
        L.oracle_sosfiltfilt_f64.argtypes = [_dp, ctypes.c_int64, _dp, ctypes.c_int, ctypes.c_int64, _dp, _dp]
        L.oracle_mean_f32_fast.argtypes = [_fp, ctypes.c_int64]
        L.oracle_mean_f32_fast.restype = ctypes.c_float
        L.oracle_chroma_heterodyne.argtypes = [ctypes.c_int64, ctypes.c_double, ctypes.c_double, _dp]
        L.oracle_chroma_carrier.argtypes = [ctypes.c_int64, ctypes.c_double, _dp, _dp]
        L.oracle_chroma_burst_value.argtypes = [_dp, ctypes.c_int64, _dp, _dp, ctypes.c_int, ctypes.c_double,
                                                ctypes.c_int64, _dp]
        L.oracle_chroma_upconvert_ntsc.argtypes = [_dp, ctypes.c_int64, ctypes.c_int64, ctypes.c_int64, _i64p,
                                                   _i64p, _dp, ctypes.c_int64, ctypes.c_double, ctypes.c_double,
                                                   ctypes.c_double, ctypes.c_double, _dp]
        L.oracle_chroma_agc_comb_u16.argtypes = [_dp, ctypes.c_int64, ctypes.c_int64, ctypes.c_int64,
                                                 ctypes.c_int64, ctypes.c_int64, ctypes.c_double, ctypes.c_int64,
                                                 ctypes.c_int64, ctypes.c_int, ctypes.c_int, _u16p, _dp]
        L.oracle_chroma_rms.argtypes = [_dp, ctypes.c_int64, ctypes.c_int]
        L.oracle_chroma_rms.restype = ctypes.c_double
        _lib = L
    return _lib


def ptr(a, t):
    return a.ctypes.data_as(t)


def vhs_rust_demod(re, im, fs):
    re = np.ascontiguousarray(re, np.float64)
    im = np.ascontiguousarray(im, np.float64)
    out = np.empty(len(re), np.float64)
    lib().oracle_vhs_rust_demod(ptr(re, _dp), ptr(im, _dp), len(re), fs, ptr(out, _dp))
    return out


def vhs_rust_angles(re, im):
    re = np.ascontiguousarray(re, np.float32)
    im = np.ascontiguousarray(im, np.float32)
    out = np.empty(len(re), np.float32)
    lib().oracle_vhs_rust_angles(ptr(re, _fp), ptr(im, _fp), len(re), ptr(out, _fp))
    return out


def vhs_envelope(filtered, b0, b1, a1):
    filtered = np.ascontiguousarray(filtered, np.float64)
    out = np.empty(len(filtered), np.float64)
    work = np.empty(len(filtered) + 12, np.float32)
    lib().oracle_vhs_envelope(ptr(filtered, _dp), len(filtered), b0, b1, a1, ptr(out, _dp),
                              ptr(work, _fp))
    return out


def vhs_raw_envelope(filtered):
    filtered = np.ascontiguousarray(filtered, np.float64)
    out = np.empty(len(filtered), np.float32)
    lib().oracle_vhs_raw_envelope(ptr(filtered, _dp), len(filtered), ptr(out, _fp))
    return out


def filtfilt1_f64(x, b0, b1, a1):
    x = np.ascontiguousarray(x, np.float64)
    out = np.empty_like(x)
    work = np.empty(len(x) + 12)
    lib().oracle_filtfilt1_f64(ptr(x, _dp), len(x), b0, b1, a1, ptr(out, _dp), ptr(work, _dp))
    return out


def find_pulses(ref, high, min_len, max_len):
    ref = np.ascontiguousarray(ref, np.float64)
    cap = max(16, len(ref) // 2 + 1)
    starts = np.empty(cap, np.int64)
    lens = np.empty(cap, np.int64)
    n = lib().oracle_find_pulses(ptr(ref, _dp), len(ref), float(high), int(min_len), int(max_len),
                                 ptr(starts, _i64p), ptr(lens, _i64p), cap)
    return list(zip(starts[:n].tolist(), lens[:n].tolist()))


def sinc_resample(src, positions, level, lut):
    src = np.ascontiguousarray(src, np.float64)
    positions = np.ascontiguousarray(positions, np.float64)
    level = np.ascontiguousarray(level, np.float64)
    out = np.empty(len(positions), np.float64)
    lib().oracle_sinc_resample(ptr(src, _dp), len(src), ptr(positions, _dp), ptr(level, _dp),
                               len(positions), ptr(lut, _fp), ptr(out, _dp))
    return out


def hz_to_u16(x, ire0, output_scale, hz_ire, output_zero, vsync_ire):
    x = np.ascontiguousarray(x, np.float64)
    out = np.empty(len(x), np.uint16)
    lib().oracle_hz_to_u16(ptr(x, _dp), len(x), ire0, output_scale, hz_ire, float(output_zero),
                           vsync_ire, ptr(out, _u16p))
    return out


def smooth_levels(la, alpha):
    la = np.ascontiguousarray(la, np.float64).copy()
    lib().oracle_smooth_levels(ptr(la, _dp), len(la), alpha)
    return la


def find_dropouts(env, start, end, thr, hyst, merge=30, min_len=10):
    env = np.ascontiguousarray(env, np.float64)
    cap = max(16, (end - start) // 2 + 2)
    s = np.empty(cap, np.int64)
    e = np.empty(cap, np.int64)
    k = lib().oracle_find_dropouts(ptr(env, _dp), int(start), int(end), float(thr), float(hyst),
                                   merge, min_len, ptr(s, _i64p), ptr(e, _i64p), cap)
    assert k >= 0
    return list(zip(s[:k].tolist(), e[:k].tolist()))


_LUT = None


def sinc_lut():
    global _LUT
    if _LUT is None:
        lut = np.empty((65537, 16), np.float32)
        lib().oracle_build_sinc_lut(ptr(lut, _fp))
        _LUT = lut
    return _LUT


def decimate_half(src):
    """2:1 half-band decimation (cuda-fast 20-MSPS reader mode) of an int16 or
    float32 capture: len(src) // 2 float32 samples."""
    src = np.ascontiguousarray(src)
    out = np.zeros(len(src) // 2, np.float32)
    if src.dtype == np.int16:
        lib().oracle_decimate_half_s16(ptr(src, ctypes.POINTER(ctypes.c_int16)), len(src), ptr(out, _fp))
    elif src.dtype == np.float32:
        lib().oracle_decimate_half_f32(ptr(src, _fp), len(src), ptr(out, _fp))
    else:
        raise TypeError("int16 or float32 capture expected")
    return out


def sosfiltfilt_f32(x, sos, edge):
    """Float32 forward-backward SOS cascade (``SosFilter.ApplyForwardBackwardFloat32``)."""
    x = np.ascontiguousarray(x, np.float64)
    sos = np.ascontiguousarray(sos, np.float64)
    n = len(x)
    if n <= edge:
        raise ValueError("input length must be greater than the pad length")
    out = np.empty(n, np.float32)
    work = np.empty(n + 2 * edge, np.float32)
    lib().oracle_sosfiltfilt_f32(ptr(x, _dp), n, ptr(sos, _dp), len(sos), edge, ptr(out, _fp), ptr(work, _fp))
    return out


def sosfiltfilt_f64(x, sos, edge):
    """Binary64 forward-backward SOS cascade (``SosFilter.ApplyForwardBackward``)."""
    x = np.ascontiguousarray(x, np.float64)
    sos = np.ascontiguousarray(sos, np.float64)
    n = len(x)
    if edge != 0 and n <= edge:
        raise ValueError("input length must be greater than the pad length")
    out = np.empty(n)
    work = np.empty(n + 2 * edge)
    lib().oracle_sosfiltfilt_f64(ptr(x, _dp), n, ptr(sos, _dp), len(sos), edge, ptr(out, _dp), ptr(work, _dp))
    return out


def mean_f32_fast(v):
    v = np.ascontiguousarray(v, np.float32)
    return float(lib().oracle_mean_f32_fast(ptr(v, _fp), len(v)))


def chroma_heterodyne(n, scale, offset):
    out = np.empty(n)
    lib().oracle_chroma_heterodyne(n, scale, offset, ptr(out, _dp))
    return out


def chroma_carrier(n, wave_scale):
    s = np.empty(n)
    c = np.empty(n)
    lib().oracle_chroma_carrier(n, wave_scale, ptr(s, _dp), ptr(c, _dp))
    return s, c


def chroma_burst_value(burst, bsin, bcos, f32, line_scale, start_minus_line):
    out = np.empty(5)
    lib().oracle_chroma_burst_value(ptr(burst, _dp), len(burst), ptr(bsin, _dp), ptr(bcos, _dp), int(bool(f32)),
                                    float(line_scale), int(start_minus_line), ptr(out, _dp))
    return out


def chroma_upconvert_ntsc(chroma, line_offset, line_length, lines, rots, phases, cu_hz, fsc_mhz,
                          target_even, target_odd):
    chroma = np.ascontiguousarray(chroma, np.float64)
    lines = np.ascontiguousarray(lines, np.int64)
    rots = np.ascontiguousarray(rots, np.int64)
    phases = np.ascontiguousarray(phases, np.float64)
    out = np.empty(len(chroma))
    lib().oracle_chroma_upconvert_ntsc(ptr(chroma, _dp), len(chroma), line_offset, line_length, ptr(lines, _i64p),
                                       ptr(rots, _i64p), ptr(phases, _dp), len(lines), cu_hz, fsc_mhz,
                                       target_even, target_odd, ptr(out, _dp))
    return out


def chroma_agc_comb_u16(chroma, lines, line_length, burst_start, burst_end, burst_abs_ref, burst_line, dist,
                        retain_f32, f32_rms):
    chroma = np.ascontiguousarray(chroma, np.float64)
    out = np.empty(len(chroma), np.uint16)
    work = np.empty(line_length)
    lib().oracle_chroma_agc_comb_u16(ptr(chroma, _dp), len(chroma), lines, line_length, burst_start, burst_end,
                                     burst_abs_ref, burst_line, dist, int(bool(retain_f32)), int(bool(f32_rms)),
                                     ptr(out, _u16p), ptr(work, _dp))
    return out


def chroma_rms(v, f32):
    v = np.ascontiguousarray(v, np.float64)
    return float(lib().oracle_chroma_rms(ptr(v, _dp), len(v), int(bool(f32))))
