"""Float32 input and 2:1 device decimation through the C ABI, against the oracle.

Mirrors the reference's own checks of these options
(src/VHSDecode.CudaFast.Native/tests/synthetic_ntsc_test.cpp:272-465): a float32
capture of the same samples decodes identically to the int16 one, and an NTSC
decode with device_decimation_factor 2 at 20 MSPS gives whole 910 x 263
fields.  Beyond that the decimator is bit-exact to the oracle, and the
decimated decode meets the decode tolerances against the oracle decoding the
oracle's decimated capture.
"""
import ctypes
import os

import numpy as np
import pytest

from test_gpu_parity import FREQ_TOL_HZ, LINE_TOL, LSB_FRACTION

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n", [1, 2, 3, 31, 4095, 4096 + 13, 4096 + 30, 100003, (1 << 20) + 7])
def test_device_decimator_bit_exact(gpu, n):
    from oracle import native as onative
    from vhsd_gb300 import native
    rng = np.random.default_rng(n)
    x16 = rng.integers(-32768, 32768, n).astype(np.int16)
    x32 = (rng.standard_normal(n) * 5000.0).astype(np.float32)
    for x in (x16, x32):
        got = native.decimate_half_rate(x)
        want = onative.decimate_half(x)
        assert got.shape == want.shape == (n // 2,)
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32))


def test_float_input_decodes_like_int16(gpu, ntsc_capture):
    from vhsd_gb300 import native
    rf, _ = ntsc_capture
    with native.Session(native.PROFILE_NTSC, len(rf)) as s:
        r16 = s.decode(rf)
        tb16 = s.tbc().copy()
        lines16 = [s.lines(i).copy() for i in range(r16.fields)]
        drops16 = [s.dropouts(i) for i in range(r16.fields)]
        r32 = s.decode(rf.astype(np.float32))
        assert r32.fields == r16.fields > 0
        assert s.tbc().tobytes() == tb16.tobytes()
        for i in range(r32.fields):
            assert np.array_equal(s.lines(i), lines16[i])
            assert s.dropouts(i) == drops16[i]


@pytest.mark.parametrize("precision", [0, 1], ids=["fp32_fused", "fp64_plain"])
def test_float_device_input_plain_and_fused(gpu, precision, pal_capture):
    import torch
    from vhsd_gb300 import native
    rf, _ = pal_capture
    d = torch.from_numpy(rf.astype(np.float32)).cuda()
    with native.Session(native.PROFILE_PAL, len(rf), precision=precision) as s:
        s.decode(rf)
        want = s.tbc().copy()
        s.decode(None, device_ptr=d.data_ptr(), count=len(rf), float_input=True)
        assert s.tbc().tobytes() == want.tobytes()


@pytest.fixture(scope="module")
def decimated_oracle(ntsc_capture):
    from oracle import field, formats
    from oracle import native as onative
    rf, _ = ntsc_capture
    plane = onative.decimate_half(rf)
    fields, ch = field.decode_capture(plane, formats.get("NTSC"), fs=20e6)
    return fields, ch


@pytest.mark.parametrize("precision", [0, 1], ids=["fp32_fused", "fp64_plain"])
def test_decimated_decode_matches_oracle(gpu, precision, ntsc_capture, decimated_oracle):
    # a 40-MSPS NTSC capture decoded at 20 MSPS through the device decimator
    from vhsd_gb300 import native
    rf, _ = ntsc_capture
    fields, (video, _, _, _) = decimated_oracle
    good = [f for f in fields if "error" not in f]
    assert good
    with native.Session(native.PROFILE_NTSC, len(rf), precision=precision, sample_rate_mhz=20.0,
                        decimation=2) as s:
        r = s.decode(rf, demod_only=True)
        assert r.stream_samples == len(video)
        v = s.stream(0, 0, len(video))
        assert np.max(np.abs(v - video)) < FREQ_TOL_HZ
        assert np.median(np.abs(v - video)) < 2.0
        r = s.decode(rf)
        assert r.fields == len(good)
        tb = s.tbc()
        for i, f in enumerate(good):
            info = s.field(i)
            assert bool(info.is_first_field) == f["first_field"]
            assert info.span_start == f["span_start"]
            assert np.max(np.abs(s.lines(i) - f["locs"])) < LINE_TOL
            d = np.abs(tb[i].astype(np.int64).ravel() - f["tbc"].astype(np.int64))
            assert np.mean(d <= 1) >= LSB_FRACTION
            assert s.dropouts(i) == [tuple(x) for x in f["dropouts"]]
        # float source samples through the float decimator: same result
        r32 = s.decode(rf.astype(np.float32))
        assert r32.fields == r.fields
        assert s.tbc().tobytes() == tb.tobytes()


def _run(rf, base, fmt, factor, mhz, max_fields=0):
    from vhsd_gb300 import native
    L = native.load()
    data = rf if fmt == native.INPUT_INT16 else rf.astype(np.float32)
    esz = data.dtype.itemsize

    def read(user, dst, offset, count):
        k = max(0, min(count, len(data) - offset))
        if k:
            ctypes.memmove(dst, data[offset:].ctypes.data, k * esz)
        return k
    cb = native.READ_CB(read)
    cfg = native.RunConfig()
    cfg.struct_size = ctypes.sizeof(cfg)
    cfg.profile = native.PROFILE_NTSC
    cfg.tape_speed = native.TAPE_SP
    cfg.sample_rate_mhz = mhz
    cfg.total_samples = len(data)
    cfg.output_base_utf8 = base.encode()
    cfg.overwrite = 1
    cfg.input_sample_format = fmt
    cfg.maximum_output_fields = max_fields
    cfg.device_decimation_factor = factor
    cfg.read_callback = cb
    res = native.RunResult()
    res.struct_size = ctypes.sizeof(res)
    native.check(L.vhsdecode_gb300_run(ctypes.byref(cfg), ctypes.byref(res)))
    return res


def test_run_input_formats_and_half_rate(gpu, ntsc_capture, tmp_path):
    # synthetic_ntsc_test.cpp:337-465: float32 and int16 runs write identical
    # files; the half-rate run writes whole 910 x 263 fields
    from vhsd_gb300 import native
    rf, _ = ntsc_capture
    a = _run(rf, str(tmp_path / "f32"), native.INPUT_FLOAT32, 1, 40.0)
    b = _run(rf, str(tmp_path / "s16"), native.INPUT_INT16, 1, 40.0)
    assert a.fields_written == b.fields_written > 0
    for ext in (".tbc", ".tbc.json"):
        assert (tmp_path / ("f32" + ext)).read_bytes() == (tmp_path / ("s16" + ext)).read_bytes()
    h = _run(rf, str(tmp_path / "half"), native.INPUT_INT16, 2, 20.0, max_fields=2)
    assert h.fields_written == 2
    assert (h.output_line_length, h.output_field_lines) == (910, 263)
    assert os.path.getsize(tmp_path / "half.tbc") == 2 * 910 * 263 * 2
    # the metadata keys of the cuda-fast writer (tbc_writer.cpp:209-310)
    import json
    for base, res in (("s16", b), ("half", h)):
        meta = json.loads((tmp_path / (base + ".tbc.json")).read_text())
        vp = meta["videoParameters"]
        assert vp["system"] == "NTSC" and vp["isSourcePal"] is False and vp["tapeFormat"] == "VHS"
        assert vp["numberOfSequentialFields"] == res.fields_written == len(meta["fields"])
        assert (vp["fieldWidth"], vp["fieldHeight"]) == (910, 263)
        assert (vp["colourBurstStart"], vp["colourBurstEnd"]) == (76, 112)
        assert (vp["activeVideoStart"], vp["activeVideoEnd"]) == (134, 894)
        assert vp["sampleRate"] == 14318182 and vp["black16bIre"] < vp["white16bIre"]
        for k, fld in enumerate(meta["fields"]):
            assert fld["seqNo"] == k + 1 and isinstance(fld["isFirstField"], bool)
            d = fld["dropOuts"]
            assert len(d["fieldLine"]) == len(d["startx"]) == len(d["endx"])
        locs = [fld["fileLoc"] for fld in meta["fields"]]
        assert locs == sorted(locs)
        assert [f["isFirstField"] for f in meta["fields"][:2]] != [True, True]
    assert not (tmp_path / "s16.tbc.json.tmp").exists()
    # neutral chroma in the luma geometry (the managed finalisation truncates both files)
    chroma = np.fromfile(tmp_path / "half_chroma.tbc", np.uint16)
    assert chroma.size == 2 * 910 * 263 and np.all(chroma == 32767)
