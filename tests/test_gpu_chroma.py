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


def _decode(rf, profile, chroma=True, fs_mhz=40.0, tape_format=None, precision=None):
    from vhsd_gb300 import native
    kw = {}
    if tape_format is not None:
        kw["tape_format"] = tape_format
    if precision is not None:
        kw["precision"] = precision
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


def test_pal_chroma_fields_match_oracle(gpu, pal_capture):
    from vhsd_gb300 import native
    rf, _ = pal_capture
    fields, _ = _oracle(rf, "PAL")
    good = [f for f in fields if "error" not in f]
    dev = _decode(rf, native.PROFILE_PAL)
    _check_fields(dev, good, 320)
    dev["session"].close()


def test_ntsc_chroma_fields_match_oracle(gpu, ntsc_capture):
    from vhsd_gb300 import native
    rf, _ = ntsc_capture
    fields, _ = _oracle(rf, "NTSC")
    good = [f for f in fields if "error" not in f]
    dev = _decode(rf, native.PROFILE_NTSC)
    _check_fields(dev, good, 270)
    dev["session"].close()


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
