"""C-ABI library checks that need no GPU: load, exports, struct layouts, host stages."""
import ctypes
import os
import re

import numpy as np
import pytest

from conftest import HAVE_GPU, ROOT


def _declared_functions():
    text = open(os.path.join(ROOT, "include", "vhsdecode_gb300.h")).read()
    return sorted(set(re.findall(r"VHSDECODE_GB300_CALL\s+(vhsdecode_gb300_\w+)\s*\(", text)))


def test_library_exports_every_declared_symbol(lib):
    names = _declared_functions()
    assert len(names) >= 19
    for n in names:
        assert hasattr(lib, n), n
    from vhsd_gb300 import native
    assert sorted(native.EXPORTS) == names


def test_abi_version(lib):
    from vhsd_gb300 import native
    assert lib.vhsdecode_gb300_get_abi_version() == native.ABI_VERSION


def test_struct_sizes_match_c_layout(lib, tmp_path):
    # the C compiler's layout of include/vhsdecode_gb300.h against the ctypes mirrors
    import subprocess
    from vhsd_gb300 import native
    structs = {"runtime_info_v1": native.RuntimeInfo, "config_v1": native.RunConfig,
               "config_v2": native.RunConfigV2,
               "result_v1": native.RunResult, "session_config_v1": native.SessionConfig,
               "decode_result_v1": native.DecodeResult, "field_info_v1": native.FieldInfo,
               "server_config_v1": native.ServerConfig, "window_v1": native.Window,
               "window_result_v1": native.WindowResult}
    src = tmp_path / "sizes.c"
    src.write_text('#include <stdio.h>\n#include "vhsdecode_gb300.h"\nint main(void){\n' + "".join(
        'printf("%%zu\\n", sizeof(vhsdecode_gb300_%s));\n' % k for k in structs) + "return 0;}\n")
    exe = tmp_path / "sizes"
    subprocess.check_call(["gcc", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)])
    sizes = [int(x) for x in subprocess.check_output([str(exe)]).split()]
    for (name, cls), size in zip(structs.items(), sizes):
        assert ctypes.sizeof(cls) == size, name


def test_runtime_info_rejects_bad_struct_size(lib):
    from vhsd_gb300 import native
    info = native.RuntimeInfo()
    info.struct_size = 12
    st = lib.vhsdecode_gb300_get_runtime_info(0, ctypes.byref(info))
    assert st in (native.STATUS_INVALID_ARGUMENT, native.STATUS_CUDA_UNAVAILABLE)
    assert st == native.STATUS_INVALID_ARGUMENT


@pytest.mark.skipif(HAVE_GPU, reason="checks the no-GPU status")
def test_no_gpu_reports_cuda_unavailable(lib):
    from vhsd_gb300 import native
    with pytest.raises(native.BackendUnavailable):
        native.runtime_info(0)
    with pytest.raises(native.BackendUnavailable):
        native.Session(native.PROFILE_PAL, 1 << 20)


def test_null_pointer_status(lib):
    from vhsd_gb300 import native
    assert lib.vhsdecode_gb300_run(None, None) == native.STATUS_NULL_POINTER
    assert b"null" in lib.vhsdecode_gb300_get_last_error()


def test_last_error_is_per_thread(lib):
    # vhsdecode_cuda_fast.cpp:23-28: the message of a failed call is thread-local,
    # so a caller reads its own failure even when another thread fails in between
    import threading
    from vhsd_gb300 import native
    both_failed = threading.Barrier(2)
    seen = {}

    def null_run():
        st = lib.vhsdecode_gb300_run(None, None)
        both_failed.wait()
        seen["run"] = (st, lib.vhsdecode_gb300_get_last_error())

    def bad_info():
        info = native.RuntimeInfo()
        info.struct_size = 12
        st = lib.vhsdecode_gb300_get_runtime_info(0, ctypes.byref(info))
        both_failed.wait()
        seen["info"] = (st, lib.vhsdecode_gb300_get_last_error())

    threads = [threading.Thread(target=null_run), threading.Thread(target=bad_info)]
    for t in threads:
        t.start()
    for t in threads:
        t.join(timeout=30)
    assert seen["run"][0] == native.STATUS_NULL_POINTER
    assert b"null" in seen["run"][1] and b"struct_size" not in seen["run"][1]
    assert seen["info"][0] == native.STATUS_INVALID_ARGUMENT
    assert b"struct_size" in seen["info"][1]


def test_run_rejects_unsupported_options(lib):
    # vhsdecode_cuda_fast.cpp:255-275: input format FLOAT32 or INT16 (or FLAC here),
    # decimation factor 1 or 2 (2 with a decode rate the source halves to)
    from vhsd_gb300 import native
    cfg = native.RunConfig()
    cfg.struct_size = ctypes.sizeof(cfg)
    cfg.profile = native.PROFILE_PAL
    cfg.sample_rate_mhz = 40.0
    cfg.output_base_utf8 = b"/tmp/x"
    cfg.input_sample_format = 3   # FLOAT32, INT16 and FLAC are defined
    cfg.device_decimation_factor = 1
    cfg.read_callback = native.READ_CB(lambda u, d, o, c: 0)
    res = native.RunResult()
    res.struct_size = ctypes.sizeof(res)

    def run():
        return lib.vhsdecode_gb300_run(ctypes.byref(cfg), ctypes.byref(res))
    assert run() == native.STATUS_INVALID_ARGUMENT
    cfg.input_sample_format = native.INPUT_INT16
    cfg.device_decimation_factor = 3
    assert run() == native.STATUS_INVALID_ARGUMENT
    cfg.device_decimation_factor = 2
    cfg.sample_rate_mhz = 60.0
    assert run() == native.STATUS_INVALID_ARGUMENT
    # accepted options reach the read: an empty capture is an input error
    for fmt, factor, mhz in [(native.INPUT_FLOAT32, 1, 40.0), (native.INPUT_INT16, 2, 20.0),
                             (native.INPUT_FLOAT32, 2, 20.0)]:
        cfg.input_sample_format, cfg.device_decimation_factor, cfg.sample_rate_mhz = fmt, factor, mhz
        assert run() == native.STATUS_INPUT_ERROR
    cfg.struct_size = 8
    assert run() == native.STATUS_INVALID_ARGUMENT


def test_run_v2_decode_flags(lib):
    # config_v2.decode_flags: 0 or DECODE_CHROMA; any other bit is refused
    from vhsd_gb300 import native
    cfg = native.RunConfigV2()
    cfg.struct_size = ctypes.sizeof(cfg)
    cfg.profile = native.PROFILE_NTSC
    cfg.sample_rate_mhz = 40.0
    cfg.output_base_utf8 = b"/tmp/x"
    cfg.input_sample_format = native.INPUT_INT16
    cfg.device_decimation_factor = 1
    cfg.read_callback = native.READ_CB(lambda u, d, o, c: 0)
    res = native.RunResult()
    res.struct_size = ctypes.sizeof(res)

    def run():
        return lib.vhsdecode_gb300_run(ctypes.byref(cfg), ctypes.byref(res))
    for bad in (native.DECODE_FLOAT_INPUT, 0x100, native.DECODE_CHROMA | 0x2):
        cfg.decode_flags = bad
        assert run() == native.STATUS_INVALID_ARGUMENT
    for ok in (0, native.DECODE_CHROMA):   # accepted: the empty capture is an input error
        cfg.decode_flags = ok
        assert run() == native.STATUS_INPUT_ERROR


def test_session_rejects_bad_decimation(lib):
    from vhsd_gb300 import native
    with pytest.raises(native.NativeError) as e:
        native.Session(native.PROFILE_NTSC, 1 << 20, sample_rate_mhz=20.0, decimation=3)
    assert e.value.status in (native.STATUS_INVALID_ARGUMENT, native.STATUS_CUDA_UNAVAILABLE)


@pytest.mark.parametrize("system,tape,speed", [
    ("PAL", "VHS", "sp"), ("NTSC", "VHS", "sp"), ("PAL", "SVHS", "sp"), ("NTSC", "SVHS", "sp"),
    ("PAL", "VHS", "lp"), ("PAL", "VHS", "ep"), ("NTSC", "VHS", "lp"), ("NTSC", "VHS", "ep"),
    ("NTSC", "SVHS", "ep")])
def test_filter_design_matches_oracle(lib, system, tape, speed):
    from vhsd_gb300 import native
    from oracle import filters, formats
    prof = native.PROFILE_PAL if system == "PAL" else native.PROFILE_NTSC
    fmt_id = native.FORMAT_SVHS if tape == "SVHS" else native.FORMAT_VHS
    spd = {"sp": native.TAPE_SP, "lp": native.TAPE_LP, "ep": native.TAPE_EP}[speed]
    rv, v, s, env, sub_high, sub_env = native.design_filters(prof, tape_format=fmt_id, sub=True,
                                                             tape_speed=spd)
    fl = filters.FilterSet(formats.get(system, tape, speed), 40e6)

    def rel(a, b):
        return np.max(np.abs(a - b)) / np.max(np.abs(b))

    # the NTSC band-pass is evaluated from its 16th-order polynomial, as the reference does
    assert rel(rv, fl.half("rf_video")) < 1e-6
    assert rel(v, fl.half("video")) < 1e-10
    assert rel(s, fl.half("video_lp05")) < 1e-10
    np.testing.assert_allclose(env, [fl.env_b[0], fl.env_b[1], fl.env_a1], rtol=1e-15)
    if tape == "SVHS" or speed != "sp":
        # S-VHS: Video carries the measured S-VHS luma table and the 2 MHz high shelf;
        # VHS LP/EP: the plain VHS Video filter with the 820 kHz sub-deemphasis high-pass
        assert rel(sub_high, (fl.video * fl.sub_highpass)[:16385]) < 1e-10
        np.testing.assert_allclose(sub_env, [fl.sub_amp_b[0], fl.sub_amp_b[1], fl.sub_amp_a1],
                                   rtol=1e-15)
    else:
        assert not np.any(sub_high) and not np.any(sub_env)


def test_svhs_custom_luma_table_only_at_tabulated_rates(lib):
    # the reference skips the file filter at rates without a resource table
    from vhsd_gb300 import native
    from oracle import filters, formats
    fl = filters.FilterSet(formats.get("PAL", "SVHS"), 28e6)
    _, v, _, _ = native.design_filters(native.PROFILE_PAL, 28.0, tape_format=native.FORMAT_SVHS)
    assert np.max(np.abs(v - fl.half("video"))) / np.max(np.abs(fl.half("video"))) < 1e-10
    assert filters.custom_luma_table("svhs-sp-linear-subdeemphasis", 28e6, 32768) is None


@pytest.mark.parametrize("system", ["PAL", "NTSC"])
def test_host_control_plane_matches_oracle(lib, system, request):
    from vhsd_gb300 import native
    from oracle import field, formats, sync
    fields, ch = request.getfixturevalue("pal_oracle" if system == "PAL" else "ntsc_oracle")
    prof = native.PROFILE_PAL if system == "PAL" else native.PROFILE_NTSC
    sp = sync.SyncParams(formats.get(system), 40e6)
    _, vlp, _, _ = ch
    state = np.array([-1, 0], np.int32)
    good = [f for f in fields if "error" not in f]
    assert len(good) >= 3
    for f in good:
        s0 = f["span_start"]
        _, slen = field.resolve_span(s0, field.read_length(sp))
        r = native.field_sync(prof, f["pulses"], slen, state, ref=vlp[s0:s0 + slen])
        assert r["first_field"] == f["first_field"]
        assert r["line0"] == f["line0"]
        assert r["first_hsync"] == f["first_hsync"]
        assert r["mean_line"] == f["mean_line"]
        assert r["next_offset"] == f["next_offset"]
        assert len(r["locs"]) == sp.output_lines + 10


def test_field_sync_rejects_empty_pulses(lib):
    from vhsd_gb300 import native
    state = np.array([-1, 0], np.int32)
    with pytest.raises(native.NativeError):
        native.field_sync(native.PROFILE_PAL, [], 1000000, state)


@pytest.mark.skipif(HAVE_GPU, reason="checks the no-GPU status")
def test_server_create_without_gpu_reports_unavailable(lib):
    from vhsd_gb300 import native
    cfg = native.ServerConfig(ctypes.sizeof(native.ServerConfig), 0, 2, 0, 1 << 22, 0)
    h = ctypes.c_void_p()
    st = lib.vhsdecode_gb300_server_create(ctypes.byref(cfg), ctypes.byref(h))
    assert st == native.STATUS_CUDA_UNAVAILABLE
    bad = native.ServerConfig(8, 0, 2, 0, 1 << 22, 0)
    assert lib.vhsdecode_gb300_server_create(ctypes.byref(bad), ctypes.byref(h)) == native.STATUS_INVALID_ARGUMENT


def test_unsupported_formats_are_rejected(lib):
    # format validation precedes any device work, so this holds with or without a GPU
    from vhsd_gb300 import native
    for prof, tape in ((native.PROFILE_PAL_M, native.FORMAT_VHS), (native.PROFILE_PAL, 7)):
        with pytest.raises(native.NativeError) as ei:
            native.Session(prof, 1 << 20, tape_format=tape)
        assert ei.value.status == native.STATUS_INVALID_ARGUMENT


def _host_run(lib, read, cancel=None, total=0, base="/tmp/vhsd_host_run"):
    from vhsd_gb300 import native
    cfg = native.RunConfig()
    cfg.struct_size = ctypes.sizeof(cfg)
    cfg.profile = native.PROFILE_PAL
    cfg.sample_rate_mhz = 40.0
    cfg.total_samples = total
    cfg.output_base_utf8 = base.encode()
    cfg.overwrite = 1
    cfg.input_sample_format = native.INPUT_INT16
    cfg.device_decimation_factor = 1
    keep = [native.READ_CB(read)]
    cfg.read_callback = keep[0]
    if cancel is not None:
        keep.append(native.CANCEL_CB(cancel))
        cfg.cancel_callback = keep[1]
    res = native.RunResult()
    res.struct_size = ctypes.sizeof(res)
    return lib.vhsdecode_gb300_run(ctypes.byref(cfg), ctypes.byref(res))


def _no_outputs(base):
    import glob
    return not glob.glob(base + "*")


def test_run_cancel_before_startup_writes_nothing(lib, tmp_path):
    # cancellation is polled before any device work (vhsdecode_cuda_fast.cpp:280-284)
    from vhsd_gb300 import native
    base = str(tmp_path / "c0")
    calls = []
    st = _host_run(lib, lambda u, d, o, c: calls.append(c) or 0, cancel=lambda u: 1, base=base)
    assert st == native.STATUS_CANCELLED
    assert not calls and _no_outputs(base)


def test_run_cancel_during_prefetch(lib, tmp_path, monkeypatch):
    # a cancel callback that flips after two reads: the prefetch thread polls it
    # before each read and stops; the run reports CANCELLED and leaves no files
    from vhsd_gb300 import native
    monkeypatch.setenv("VHSD_RUN_WINDOW_GRIDS", "40")   # the first window needs 10 reads
    base = str(tmp_path / "c2")
    reads = []

    def read(u, d, off, count):
        reads.append((off, count))
        ctypes.memset(d, 0, count * 2)
        return count

    st = _host_run(lib, read, cancel=lambda u: 1 if len(reads) >= 2 else 0, base=base)
    assert st == native.STATUS_CANCELLED
    assert len(reads) == 2 and reads[1][0] == reads[0][1]   # in order, contiguous
    assert _no_outputs(base)


def test_run_read_overrun_is_an_input_error(lib, tmp_path):
    from vhsd_gb300 import native
    base = str(tmp_path / "ov")
    st = _host_run(lib, lambda u, d, o, c: c + 1, base=base)
    assert st == native.STATUS_INPUT_ERROR
    assert b"overran" in lib.vhsdecode_gb300_get_last_error()
    assert _no_outputs(base)


def test_flac_stream_info_matches_reference_header_cases(lib):
    # LibsndfilePcm16SampleLoaderTests.cs:1038-1075: STREAMINFO packing, and the
    # headers the reference's loader refuses
    import struct
    from vhsd_gb300 import native

    def header(rate, channels, bits, total):
        b = bytearray(4 + 4 + 34)
        b[:4] = b"fLaC"
        b[4] = 0x80
        b[7] = 34
        packed = (rate << 44) | ((channels - 1) << 41) | ((bits - 1) << 36) | total
        b[18:26] = struct.pack(">Q", packed)
        return bytes(b)

    info = native.flac_info(header(40_000, 1, 16, 123_456_789))
    assert (info.sample_rate, info.channels, info.bits_per_sample, info.total_samples) == \
        (40_000, 1, 16, 123_456_789)
    assert info.first_frame_offset == 42

    def invalid(block_type, block_len, payload):
        b = bytearray(8 + payload)
        b[:4] = b"fLaC"
        b[4] = block_type
        b[7] = block_len
        return bytes(b)

    for bad in (b"OggS" + bytes(40), b"fLaC", invalid(0x81, 0x22, 34), invalid(0x80, 0x22, 33),
                invalid(0x80, 0x21, 33)):
        with pytest.raises(native.NativeError) as e:
            native.flac_info(bad)
        assert e.value.status == native.STATUS_INPUT_ERROR


def test_flac_writer_and_reader_round_trip():
    # the test-side writer covers every subframe and residual form; its
    # stream decodes (by the bit-level reader) to the samples it was given
    from oracle import flac
    from vhsd_gb300 import ldf
    rng = np.random.default_rng(3)
    t = np.arange(70_000)
    x = (6000 * np.sin(2 * np.pi * 0.11 * t) + rng.normal(0, 300, len(t))).astype(np.int16)
    x[4096 * 3:4096 * 4] &= ~1          # a frame with a wasted bit
    x[4096 * 6:4096 * 7] = -1234         # a constant frame
    for bs in (4096, 1152, 4608):
        data = ldf.write(x, blocksize=bs, seed=bs, wasted_frames=(3,))
        assert flac.stream_info(data)["total_samples"] == len(x)
        assert np.array_equal(flac.decode(data), x)


@pytest.mark.parametrize("system,fs", [("PAL", 40.0), ("NTSC", 40.0), ("PAL", 20.0), ("NTSC", 28.0)])
def test_chroma_design_matches_oracle(lib, system, fs):
    # the library's chroma filters, burst window and tables equal the oracle's bit for bit
    from oracle import chroma, formats
    from vhsd_gb300 import native
    prof = native.PROFILE_PAL if system == "PAL" else native.PROFILE_NTSC
    d = native.design_chroma(prof, fs, tables=(fs == 40.0))
    cp = chroma.ChromaParams(formats.get(system), fs * 1e6)
    assert np.array_equal(d["rf_sos"], cp.rf_sos)
    assert np.array_equal(d["final_sos"], cp.final_sos)
    assert (d["burst_start"], d["burst_end"], d["move"]) == (cp.burst_start, cp.burst_end, cp.offset)
    assert d["rf_edge"] == chroma.default_pad_length(cp.rf_sos) == 27
    assert d["final_edge"] == chroma.default_pad_length(cp.final_sos) == 27
    assert d["rotation"] == cp.rotation and d["field_samples"] == cp.field_samples
    if fs == 40.0:
        het, bsin, bcos = cp.tables()
        for p in range(4):
            assert np.array_equal(d["heterodyne"][p].astype(np.float64), het[p])
        assert np.array_equal(d["burst_sin"].astype(np.float64), bsin)
        assert np.array_equal(d["burst_cos"].astype(np.float64), bcos)


@pytest.mark.parametrize("system", ["PAL", "NTSC"])
@pytest.mark.parametrize("tape,speed", [("VHS", "lp"), ("VHS", "ep"), ("SVHS", "sp"), ("SVHS", "ep")])
def test_chroma_design_matches_oracle_per_format(lib, system, tape, speed):
    # the chroma filters, burst window, offset and rotation follow the format's
    # RF parameters (band-pass edges, colour-under carrier, rotation, offset),
    # which differ between tape formats and speeds
    from oracle import chroma, formats
    from vhsd_gb300 import native
    prof = native.PROFILE_PAL if system == "PAL" else native.PROFILE_NTSC
    sp = {"sp": native.TAPE_SP, "lp": native.TAPE_LP, "ep": native.TAPE_EP}[speed]
    tf = native.FORMAT_SVHS if tape == "SVHS" else native.FORMAT_VHS
    d = native.design_chroma(prof, 40.0, tape_speed=sp, tape_format=tf)
    cp = chroma.ChromaParams(formats.get(system, tape, speed), 40e6)
    assert np.array_equal(d["rf_sos"], cp.rf_sos)
    assert np.array_equal(d["final_sos"], cp.final_sos)
    assert (d["burst_start"], d["burst_end"], d["move"]) == (cp.burst_start, cp.burst_end, cp.offset)
    assert d["rotation"] == cp.rotation and d["field_samples"] == cp.field_samples
