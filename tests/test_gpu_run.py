"""vhsdecode_gb300_run: the whole-run handoff, streamed in bounded windows.

The capture comes through the read callback in order; it is decoded in
windows that start on the 983,040-sample grid and carry the field sequence
across window joins.  Small windows (VHSD_RUN_WINDOW_GRIDS=3) put several joins
into a 12-field capture.  Checked here:
* the files equal one whole-capture session decode (TBC bytes, field order,
  fileLoc, dropouts) and the oracle's field list (fileLoc, isFirstField,
  dropOuts identical; TBC within 1 LSB on >= 99.9 % of samples);
* a short read mid-stream ends the input cleanly;
* a cancellation during the decode returns CANCELLED and leaves no files;
* a field limit across windows;
* with DECODE_CHROMA, the windowed luma and _chroma.tbc equal one whole
  chroma decode (PAL and NTSC);
* a chroma workspace allocation forced to fail fails the run and the session
  decode (no files, an error status) instead of reporting unwritten chroma.
Faults are made on the host (callbacks), never on the device.
"""
import ctypes
import glob
import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

LSB_FRACTION = 0.999


@pytest.fixture(scope="module")
def pal12():
    from oracle import field, formats
    from vhsd_gb300 import synth
    rf, _ = synth.generate(synth.config("pal_small", fields=12, seed=12))
    fields, _ = field.decode_capture(rf, formats.get("PAL"))
    return rf, [f for f in fields if "error" not in f]


def _run(rf, base, read=None, cancel=None, max_fields=0, total=None, chroma=False, profile=None):
    from vhsd_gb300 import native
    L = native.load()
    data = np.ascontiguousarray(rf, np.int16)

    def default_read(u, dst, off, count):
        k = max(0, min(count, len(data) - off))
        if k:
            ctypes.memmove(dst, data[off:].ctypes.data, k * 2)
        return k

    cfg = native.RunConfigV2() if chroma else native.RunConfig()
    cfg.struct_size = ctypes.sizeof(cfg)
    if chroma:
        cfg.tape_format = native.FORMAT_VHS
        cfg.decode_flags = native.DECODE_CHROMA
    cfg.profile = native.PROFILE_PAL if profile is None else profile
    cfg.tape_speed = native.TAPE_SP
    cfg.sample_rate_mhz = 40.0
    cfg.total_samples = len(data) if total is None else total
    cfg.output_base_utf8 = base.encode()
    cfg.overwrite = 1
    cfg.input_sample_format = native.INPUT_INT16
    cfg.maximum_output_fields = max_fields
    cfg.device_decimation_factor = 1
    keep = [native.READ_CB(read or default_read)]
    cfg.read_callback = keep[0]
    if cancel is not None:
        keep.append(native.CANCEL_CB(cancel))
        cfg.cancel_callback = keep[1]
    res = native.RunResult()
    res.struct_size = ctypes.sizeof(res)
    st = L.vhsdecode_gb300_run(ctypes.byref(cfg), ctypes.byref(res))
    return st, res


def _outputs(base):
    tbc = np.fromfile(base + ".tbc", np.uint16)
    meta = json.loads(open(base + ".tbc.json").read())
    return tbc, meta


def _session_fields(rf, max_fields=0):
    from vhsd_gb300 import native
    with native.Session(native.PROFILE_PAL, len(rf)) as s:
        r = s.decode(rf, max_fields=max_fields)
        tb = s.tbc().copy()
        info = [(s.field(i).is_first_field, s.field(i).file_loc, s.dropouts(i)) for i in range(r.fields)]
    return tb, info


def test_windowed_run_equals_whole_decode_and_oracle(gpu, pal12, tmp_path, monkeypatch):
    rf, good = pal12
    monkeypatch.setenv("VHSD_RUN_WINDOW_GRIDS", "3")
    base = str(tmp_path / "w3")
    st, res = _run(rf, base)
    assert st == 0
    tbc, meta = _outputs(base)
    whole, info = _session_fields(rf)
    assert res.fields_written == len(info) == len(good) >= 10
    assert tbc.tobytes() == whole.tobytes()
    per = res.output_line_length * res.output_field_lines
    for i, (f, fld) in enumerate(zip(good, meta["fields"])):
        first, loc, drops = info[i]
        assert fld["isFirstField"] == bool(first) == f["first_field"], i
        assert fld["fileLoc"] == loc == int(np.floor(f["span_start"] + f["line0"] + 1024)), i
        d = fld["dropOuts"]
        got = list(zip(d["fieldLine"], d["startx"], d["endx"]))
        assert got == [tuple(x) for x in drops] == [tuple(x) for x in f["dropouts"]], i
        diff = np.abs(tbc[i * per:(i + 1) * per].astype(np.int64) - f["tbc"].astype(np.int64))
        assert np.mean(diff <= 1) >= LSB_FRACTION, i
    # one default-size window gives the same files
    monkeypatch.delenv("VHSD_RUN_WINDOW_GRIDS")
    st, _ = _run(rf, str(tmp_path / "w40"))
    assert st == 0
    for ext in (".tbc", ".tbc.json", "_chroma.tbc"):
        assert open(base + ext, "rb").read() == open(str(tmp_path / "w40") + ext, "rb").read()


@pytest.mark.parametrize("system", ["PAL", "NTSC"])
def test_windowed_run_with_chroma_equals_whole_decode(gpu, system, tmp_path, monkeypatch):
    # chroma through run(): the rotation index and the VHS field number (NTSC's
    # burst phase target) carry across window joins, so the windowed files
    # equal one whole-capture decode byte for byte
    from vhsd_gb300 import native, synth
    rf, _ = synth.generate(synth.config("pal_small" if system == "PAL" else "ntsc_small", fields=12, seed=21))
    prof = native.PROFILE_PAL if system == "PAL" else native.PROFILE_NTSC
    monkeypatch.setenv("VHSD_RUN_WINDOW_GRIDS", "3")
    base = str(tmp_path / "c3")
    st, res = _run(rf, base, chroma=True, profile=prof)
    assert st == 0
    tbc, meta = _outputs(base)
    chroma = np.fromfile(base + "_chroma.tbc", np.uint16)
    with native.Session(prof, len(rf)) as s:
        r = s.decode(rf, chroma=True)
        assert res.fields_written == r.fields >= 10
        assert tbc.tobytes() == s.tbc().tobytes()
        assert chroma.tobytes() == s.chroma().tobytes()
        locs = [s.field(i).file_loc for i in range(r.fields)]
    assert [f["fileLoc"] for f in meta["fields"]] == locs
    assert chroma.size == tbc.size and np.count_nonzero(chroma != 32767) > chroma.size // 4


def test_short_read_mid_stream_ends_input(gpu, pal12, tmp_path, monkeypatch):
    rf, _ = pal12
    monkeypatch.setenv("VHSD_RUN_WINDOW_GRIDS", "3")
    cut = 7_500_001
    data = np.ascontiguousarray(rf, np.int16)

    def short_read(u, dst, off, count):
        k = max(0, min(count, cut - off))   # the source ends early: a short count
        if k:
            ctypes.memmove(dst, data[off:].ctypes.data, k * 2)
        return k

    base = str(tmp_path / "short")
    st, res = _run(rf, base, read=short_read, total=len(rf))
    assert st == 0 and res.fields_written > 0
    tbc, meta = _outputs(base)
    whole, info = _session_fields(np.ascontiguousarray(rf[:cut]))
    assert res.fields_written == len(info)
    assert tbc.tobytes() == whole.tobytes()
    assert [f["fileLoc"] for f in meta["fields"]] == [x[1] for x in info]


def test_cancel_during_decode_leaves_no_files(gpu, pal12, tmp_path, monkeypatch):
    rf, _ = pal12
    monkeypatch.setenv("VHSD_RUN_WINDOW_GRIDS", "3")
    polls = []

    def cancel(u):
        polls.append(1)
        return 1 if len(polls) >= 5 else 0

    base = str(tmp_path / "cx")
    st, _ = _run(rf, base, cancel=cancel)
    from vhsd_gb300 import native
    assert st == native.STATUS_CANCELLED
    assert not glob.glob(base + "*")


def test_field_limit_across_windows(gpu, pal12, tmp_path, monkeypatch):
    rf, _ = pal12
    monkeypatch.setenv("VHSD_RUN_WINDOW_GRIDS", "3")
    base = str(tmp_path / "lim")
    st, res = _run(rf, base, max_fields=7)
    assert st == 0 and res.fields_written == 7
    tbc, meta = _outputs(base)
    whole, info = _session_fields(rf, max_fields=7)
    assert tbc.tobytes() == whole.tobytes()
    assert len(meta["fields"]) == 7
    assert os.path.getsize(base + "_chroma.tbc") == tbc.size * 2


def test_forced_chroma_workspace_failure_fails_closed(gpu, tmp_path, monkeypatch):
    # tools/build-cuda-fast-native.ps1:290-305: with the chroma workspace
    # allocation forced to fail, a chroma run must fail instead of reporting
    # chroma it never wrote.  The session path fails the same way and its
    # session decodes once the allocation succeeds, with the chroma of a fresh
    # session.  The fault is made on the host.
    from vhsd_gb300 import native, synth
    rf, _ = synth.generate(synth.config("pal_small", fields=4))
    monkeypatch.setenv("VHSD_FORCE_CHROMA_WORKSPACE_FAILURE", "1")
    base = str(tmp_path / "fx")
    st, _ = _run(rf, base, chroma=True)
    assert st == native.STATUS_INTERNAL_ERROR
    assert b"chroma workspace" in native.load().vhsdecode_gb300_get_last_error()
    assert not glob.glob(base + "*")
    with native.Session(native.PROFILE_PAL, len(rf)) as s:
        with pytest.raises(native.NativeError, match="chroma workspace"):
            s.decode(rf, chroma=True)
        monkeypatch.delenv("VHSD_FORCE_CHROMA_WORKSPACE_FAILURE")
        r = s.decode(rf, chroma=True)
        assert r.fields > 0
        got = s.chroma().copy()
    with native.Session(native.PROFILE_PAL, len(rf)) as s:
        s.decode(rf, chroma=True)
        assert np.array_equal(s.chroma(), got)
