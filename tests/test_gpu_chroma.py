"""Colour-under chroma on the device against the oracle, through the C ABI.

Tolerances:
* the chroma channel of the stitched stream (the float32 block band-pass, roll
  and mean removal) is bit-exact;
* line locations after the burst refinement: within 0.01 sample;
* uint16 luma TBC and uint16 chroma: |diff| <= 1 LSB on >= 99.9 % of samples
  (the chroma TBC sums its taps in float pairs, the final band-pass runs on
  overlapping chunks, and the NTSC carrier cosine is evaluated in float after
  an exact turn reduction: each agrees with the reference to float rounding);
* field count, field order and dropout decisions identical.

The uint16 chroma bar holds end to end for the FP64 plain path (PAL and NTSC
VHS SP, PAL and NTSC S-VHS, NTSC EP, NTSC at 20 MSPS directly and through the
device decimator); float32 input gives the int16 decode's bits.  The FP32
fused path's line locations differ from the FP64 oracle's by about 1e-4
sample (its demodulated sync is within 1 kHz, not exact), and the reference
TBC rounds each source position to float32, a 1/32-sample grid at the
positions of a field span: where the two locations fall on either side of a
grid point the 627 kHz chroma moves by up to a few percent of its amplitude,
and the final band-pass spreads that over its impulse response.  So the FP32
path is checked stage by stage, each stage fed the device's own inputs: the
probe windows, the burst sequence and averages, the refined lines, and the
field decode to uint16 (1 LSB on >= 99.9 %).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

LINE_TOL = 0.01
LSB_FRACTION = 0.999


def _oracle(rf, system, fs=40e6, tape_format="VHS"):
    from oracle import chroma, demod, field, formats
    fmt = formats.get(system, tape_format)
    fields, ch = field.decode_capture(rf, fmt, fs=fs, with_chroma=True)
    return fields, ch


def _decode(rf, profile, chroma=True, fs_mhz=40.0, tape_format=None, precision=None, tape_speed=None):
    from vhsd_gb300 import native
    kw = {}
    if tape_format is not None:
        kw["tape_format"] = tape_format
    if precision is not None:
        kw["precision"] = precision
    if tape_speed is not None:
        kw["tape_speed"] = tape_speed
    s = native.Session(profile, len(rf), sample_rate_mhz=fs_mhz, **kw)
    r = s.decode(rf, chroma=chroma)
    out = {"fields": r.fields, "tbc": s.tbc().copy(), "first": [], "locs": [], "drops": []}
    if chroma:
        out["chroma"] = s.chroma().copy()
    for i in range(r.fields):
        out["first"].append(bool(s.field(i).is_first_field))
        out["locs"].append(s.lines(i))
        out["drops"].append(s.dropouts(i))
    out["session"] = s
    return out


def _check_fields(dev, good, lines):
    assert dev["fields"] == len(good) >= 2
    for i, f in enumerate(good):
        assert dev["first"][i] == f["first_field"], i
        n = min(lines, len(f["locs"]), len(dev["locs"][i]))
        assert np.max(np.abs(dev["locs"][i][:n] - f["locs"][:n])) < LINE_TOL, i
        lum = np.abs(dev["tbc"][i].astype(np.int64).ravel() - f["tbc"].astype(np.int64))
        assert np.mean(lum <= 1) >= LSB_FRACTION, (i, np.mean(lum <= 1))
        chd = np.abs(dev["chroma"][i].astype(np.int64).ravel() - f["chroma"].astype(np.int64))
        assert np.mean(chd <= 1) >= LSB_FRACTION, (i, np.mean(chd <= 1), chd.max())
        assert [tuple(d) for d in dev["drops"][i]] == [tuple(d) for d in f["dropouts"]], i


def test_chroma_stream_bit_exact(gpu, pal_capture):
    from oracle import chroma, formats
    from vhsd_gb300 import native
    rf, _ = pal_capture
    cp = chroma.ChromaParams(formats.get("PAL"))
    want = chroma.chroma_stream(rf, cp)
    with native.Session(native.PROFILE_PAL, len(rf)) as s:
        s.decode(rf, demod_only=True, chroma=True)
        got = s.stream(3, 0, len(want))
    assert np.array_equal(got, want)


@pytest.mark.parametrize("system", ["PAL", "NTSC"])
def test_fp64_chroma_fields_match_oracle(gpu, pal_capture, ntsc_capture, system):
    from vhsd_gb300 import native
    rf, _ = pal_capture if system == "PAL" else ntsc_capture
    fields, _ = _oracle(rf, system)
    good = [f for f in fields if "error" not in f]
    prof = native.PROFILE_PAL if system == "PAL" else native.PROFILE_NTSC
    dev = _decode(rf, prof, precision=native.PRECISION_FP64_PLAIN)
    _check_fields(dev, good, 320 if system == "PAL" else 270)
    dev["session"].close()


@pytest.mark.parametrize("case", ["pal_svhs", "ntsc_svhs", "ntsc_ep"])
def test_fp64_chroma_other_formats_match_oracle(gpu, case, request):
    # the same colour-under chroma behind S-VHS's own luma path (sub-deemphasis,
    # custom luma filters) and behind NTSC EP's narrower RF filters and
    # long-play burst level: the FP64 path end to end against the oracle
    from oracle import field, formats
    from vhsd_gb300 import native
    fixture, system, tape, speed = {
        "pal_svhs": ("svhs_capture", "PAL", "SVHS", "sp"),
        "ntsc_svhs": ("svhs_ntsc_capture", "NTSC", "SVHS", "sp"),
        "ntsc_ep": ("ntsc_capture", "NTSC", "VHS", "ep"),
    }[case]
    rf, _ = request.getfixturevalue(fixture)
    fields, _ = field.decode_capture(rf, formats.get(system, tape, speed), with_chroma=True)
    good = [f for f in fields if "error" not in f]
    prof = native.PROFILE_PAL if system == "PAL" else native.PROFILE_NTSC
    dev = _decode(rf, prof, precision=native.PRECISION_FP64_PLAIN,
                  tape_format=native.FORMAT_SVHS if tape == "SVHS" else native.FORMAT_VHS,
                  tape_speed=native.TAPE_EP if speed == "ep" else native.TAPE_SP)
    _check_fields(dev, good, 320 if system == "PAL" else 270)
    dev["session"].close()


def test_fp64_chroma_at_20_msps_matches_oracle(gpu, ntsc20_capture):
    # the chroma filters and burst geometry designed for a 20 MSPS decode
    # (the chroma offset, the band-pass edges and pad length at that rate)
    from oracle import field, formats
    from vhsd_gb300 import native
    rf, _ = ntsc20_capture
    fields, _ = field.decode_capture(rf, formats.get("NTSC"), fs=20e6, with_chroma=True)
    good = [f for f in fields if "error" not in f]
    dev = _decode(rf, native.PROFILE_NTSC, fs_mhz=20.0, precision=native.PRECISION_FP64_PLAIN)
    _check_fields(dev, good, 270)
    dev["session"].close()


@pytest.mark.parametrize("system", ["PAL", "NTSC"])
def test_fp32_chroma_stages_match_oracle(gpu, pal_capture, ntsc_capture, system):
    from oracle import chroma, field, formats, sync, tbc
    from vhsd_gb300 import native
    rf, _ = pal_capture if system == "PAL" else ntsc_capture
    fmt = formats.get(system)
    cp = chroma.ChromaParams(fmt)
    sp = sync.SyncParams(fmt, 40e6)
    fields, _ = _oracle(rf, system)
    good = [f for f in fields if "error" not in f]
    prof = native.PROFILE_PAL if system == "PAL" else native.PROFILE_NTSC
    dev = _decode(rf, prof)
    s = dev["session"]
    cstream = s.stream(3, 0, s.last.stream_samples)
    het, bsin, bcos = cp.tables()
    nominal = float(round(fmt["sys"]["line_period"] * sp.mhz))
    smoothing = fmt["sys"]["frame_lines"] / 2.0
    win0, win = 2 * cp.burst_start - cp.burst_end, 2 * cp.burst_end - cp.burst_start
    filt = lambda v: chroma.native.sosfiltfilt_f32(v, cp.final_sos, 27).astype(np.float64)
    assert dev["fields"] == len(good)
    for i, f in enumerate(good):
        span = cstream[f["span_start"]:f["span_start"] + f["span_len"]]
        pre = s.chroma_stage(i, 5)
        final = dev["locs"][i]
        # the line-1 chroma TBC at the probe windows, from the device's hsync lines
        ana = tbc.resample_field(span, pre, 1, cp.out_lines, cp.outlen, nominal, smoothing)
        windows = s.chroma_stage(i, 2).reshape(cp.out_lines, win)
        full = ana.reshape(cp.out_lines, cp.outlen)[:, win0:win0 + win]
        assert np.max(np.abs(windows - full)) <= 1e-6 * max(1.0, np.max(np.abs(full)))
        # burst probes of the kept sequence from the device's windows
        st3 = s.chroma_stage(i, 3)
        rows, chosen = st3[:-1].reshape(cp.out_lines, 5), int(st3[-1])
        field_ana = np.zeros(cp.field_samples)
        field_ana.reshape(cp.out_lines, cp.outlen)[:, win0:win0 + win] = windows
        seq = []
        for pl in range(cp.out_lines):
            rot = (cp.rotation[chosen] * (pl + 1)) % 4
            scale = (pre[pl + 2] - pre[pl + 1]) / max(1, int(round(sp.nominal))) if pl < cp.out_lines - 1 else 1.0
            r = chroma.probe_burst(field_ana, het, rot, cp.burst_start, cp.burst_end, bsin, bcos, scale, pl + 1, 1,
                                   cp.outlen, filt, True)
            seq.append(r)
            assert abs(r["phase"] - rows[pl, 0]) < 1e-9 or abs(abs(r["phase"] - rows[pl, 0]) - 360.0) < 1e-9, pl
            assert abs(r["offset"] - rows[pl, 1]) < 1e-9
            assert np.allclose([r["mag"], r["i"], r["q"]], rows[pl, 2:], rtol=1e-12, atol=1e-9)
        # the kept rotation sequence is the oracle's own choice for this field
        assert [p["rot"] for p in seq] == [p["rot"] for p in f["phase"]["seq"]], i
        # phase averages and the burst refinement of the device's lines
        summ = chroma.summarize(0, seq, cp.out_lines + 1)
        st4 = s.chroma_stage(i, 4)
        assert np.allclose(st4, [summ["avg"], summ["even"], summ["odd"], summ["mag_avg"]], rtol=0, atol=1e-9)
        refined = chroma.refine_from_burst(pre, cp.outlen, cp.fsc_ratio, summ, cp.ntsc)
        if cp.ntsc:
            refined = refined - ((117.25 / 360.0) / sp.fsc_mhz) * sp.mhz
        n = min(len(refined), len(final))
        assert np.max(np.abs(refined[:n] - final[:n])) < 1e-9
        # the field decode from the device's final lines and burst sequence
        ofl = field.output_first_line(sp, f["first_field"])
        c = tbc.resample_field(span, final, ofl, cp.out_lines, cp.outlen, nominal, smoothing)
        # the float-pair tap sums round like the binary64 ones except within
        # about 2^-46 of a float rounding boundary: at most one float ulp, rarely
        tb = s.chroma_stage(i, 0)
        cf = c.astype(np.float32).astype(np.float64)
        off = tb != cf
        assert np.mean(off) < 1e-4
        assert np.all(np.abs(tb[off] - cf[off]) <= np.spacing(np.abs(cf[off]).astype(np.float32)).astype(np.float64))
        want = chroma.decode_field_chroma(c, cp, dict(summ, seq=seq), f["first_field"], f["field_number"], ofl)
        chd = np.abs(dev["chroma"][i].astype(np.int64).ravel() - want.astype(np.int64))
        assert np.mean(chd <= 1) >= LSB_FRACTION, (i, np.mean(chd <= 1), chd.max())
        # end to end against the oracle's own lines: within 0.01 sample, luma as the luma tests
        m = min(len(f["locs"]), len(final))
        assert np.max(np.abs(final[:m] - f["locs"][:m])) < LINE_TOL
        lum = np.abs(dev["tbc"][i].astype(np.int64).ravel() - f["tbc"].astype(np.int64))
        assert np.mean(lum <= 1) >= LSB_FRACTION
    s.close()


def test_chroma_off_is_the_skip_chroma_decode(gpu, pal_capture, pal_oracle):
    # without the flag: no burst refinement, the luma of the --skip_chroma decode
    from vhsd_gb300 import native
    rf, _ = pal_capture
    fields, _ = pal_oracle
    good = [f for f in fields if "error" not in f]
    dev = _decode(rf, native.PROFILE_PAL, chroma=False)
    for i, f in enumerate(good):
        n = min(320, len(f["locs"]), len(dev["locs"][i]))
        assert np.max(np.abs(dev["locs"][i][:n] - f["locs"][:n])) < LINE_TOL, i
    with pytest.raises(native.NativeError):
        dev["session"].chroma()
    dev["session"].close()


def test_float_input_chroma_equals_int16(gpu, ntsc_capture):
    # the block stage's float-source pass: a float32 capture of the int16
    # values decodes to the same luma and chroma bits, host and device input
    import torch
    from vhsd_gb300 import native
    rf, _ = ntsc_capture
    with native.Session(native.PROFILE_NTSC, len(rf)) as s:
        s.decode(rf, chroma=True)
        tb, ch = s.tbc().copy(), s.chroma().copy()
        s.decode(rf.astype(np.float32), chroma=True)
        assert s.tbc().tobytes() == tb.tobytes()
        assert s.chroma().tobytes() == ch.tobytes()
        d = torch.from_numpy(rf.astype(np.float32)).cuda()
        s.decode(None, device_ptr=d.data_ptr(), count=len(rf), float_input=True, chroma=True)
        assert s.chroma().tobytes() == ch.tobytes()


def test_fp64_decimated_chroma_matches_oracle(gpu, ntsc_capture):
    # 40 MSPS through the device 2:1 decimator, chroma decoded at 20 MSPS from
    # the float capture: against the oracle's chroma decode of the oracle's
    # decimated capture
    from oracle import field, formats
    from oracle import native as onative
    from vhsd_gb300 import native
    rf, _ = ntsc_capture
    plane = onative.decimate_half(rf)
    fields, _ = field.decode_capture(plane, formats.get("NTSC"), fs=20e6, with_chroma=True)
    good = [f for f in fields if "error" not in f]
    with native.Session(native.PROFILE_NTSC, len(rf), precision=native.PRECISION_FP64_PLAIN,
                        sample_rate_mhz=20.0, decimation=2) as s:
        r = s.decode(rf, chroma=True)
        dev = {"fields": r.fields, "tbc": s.tbc().copy(), "chroma": s.chroma().copy(),
               "first": [bool(s.field(i).is_first_field) for i in range(r.fields)],
               "locs": [s.lines(i) for i in range(r.fields)],
               "drops": [s.dropouts(i) for i in range(r.fields)]}
    _check_fields(dev, good, 270)
