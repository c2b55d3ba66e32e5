"""Edge cases of the session decode and parity at the configured full sizes.

Edge cases follow what the reference's decode loop has to survive: empty and
sub-block inputs, exactly one block, a field limit, inputs beyond the session
capacity and misaligned device pointers (rejected, not decoded).  The full-size
case decodes the 60-field NTSC VHS workload the headline throughput is quoted
on and compares every field with the oracle.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FREQ_TOL_HZ = 1000.0
LINE_TOL = 0.01
LSB_FRACTION = 0.999


def test_empty_and_short_inputs(gpu):
    from vhsd_gb300 import native
    with native.Session(native.PROFILE_PAL, 1 << 20) as s:
        r = s.decode(np.zeros(0, np.int16))
        assert r.blocks == 0 and r.fields == 0 and r.stream_samples == 0
        r = s.decode(np.zeros(32767, np.int16))
        assert r.blocks == 0 and r.fields == 0
        # the same with colour-under chroma: no blocks, no chroma stages
        for n in (0, 32767):
            r = s.decode(np.zeros(n, np.int16), chroma=True)
            assert r.blocks == 0 and r.fields == 0


def test_exactly_one_block_matches_oracle(gpu, pal_capture):
    from vhsd_gb300 import native
    from oracle import demod, filters, formats
    rf, _ = pal_capture
    x = rf[5 * 30720:5 * 30720 + 32768].copy()
    fmt = formats.get("PAL")
    fl = filters.FilterSet(fmt, 40e6)
    dmax = (fmt["sys"]["ire0"] + fmt["sys"]["hz_ire"] * 100.0) * 2.0
    video, vlp, env, _ = demod.demod_stream(x, fl, 40e6, dmax)
    with native.Session(native.PROFILE_PAL, len(x)) as s:
        r = s.decode(x, demod_only=True)
        assert r.blocks == 1 and r.stream_samples == 30720
        v = s.stream(0, 0, 30720)
        y = s.stream(1, 0, 30720)
    assert np.max(np.abs(v - video)) < FREQ_TOL_HZ
    assert np.max(np.abs(y - vlp)) < FREQ_TOL_HZ


def test_field_limit_stops_early(gpu, pal_capture, pal_oracle):
    from vhsd_gb300 import native
    rf, _ = pal_capture
    fields, _ = pal_oracle
    good = [f for f in fields if "error" not in f]
    with native.Session(native.PROFILE_PAL, len(rf)) as s:
        r = s.decode(rf, max_fields=1)
        assert r.fields == 1 and r.stop_reason == 1
        tb = s.tbc()
        d = np.abs(tb[0].astype(np.int64).ravel() - good[0]["tbc"].astype(np.int64))
        assert np.mean(d <= 1) >= LSB_FRACTION


def test_rejects_oversized_and_misaligned_inputs(gpu):
    import torch
    from vhsd_gb300 import native
    with native.Session(native.PROFILE_NTSC, 100000) as s:
        with pytest.raises(native.NativeError) as ei:
            s.decode(np.zeros(100001, np.int16))
        assert ei.value.status == native.STATUS_INVALID_ARGUMENT
        d = torch.zeros(70000, dtype=torch.int16, device="cuda")
        with pytest.raises(native.NativeError) as ei:
            s.decode(None, device_ptr=d.data_ptr() + 2, count=65536)
        assert ei.value.status == native.STATUS_INVALID_ARGUMENT
        # the session stays usable after a rejected call
        r = s.decode(None, device_ptr=d.data_ptr(), count=65536, demod_only=True)
        assert r.blocks == 2


@pytest.fixture(scope="module")
def ntsc60():
    import sys
    import os
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    from oracle import field, formats
    rf = bench.workload("ntsc60")
    fields, ch = field.decode_capture(rf, formats.get("NTSC"))
    return rf, fields, ch


def test_full_size_ntsc60_matches_oracle(gpu, ntsc60):
    # the 60-field NTSC VHS workload (41 M samples, 200 dropouts): every field
    from vhsd_gb300 import native
    rf, fields, (video, _, _, _) = ntsc60
    good = [f for f in fields if "error" not in f]
    assert len(good) >= 60
    with native.Session(native.PROFILE_NTSC, len(rf)) as s:
        r = s.decode(rf)
        assert r.fields == len(good)
        v = s.stream(0, 0, len(video))
        assert np.max(np.abs(v - video)) < FREQ_TOL_HZ
        tb = s.tbc()
        drops = 0
        for i, f in enumerate(good):
            info = s.field(i)
            assert bool(info.is_first_field) == f["first_field"], i
            assert info.span_start == f["span_start"], i
            assert np.max(np.abs(s.lines(i) - f["locs"])) < LINE_TOL, i
            d = np.abs(tb[i].astype(np.int64).ravel() - f["tbc"].astype(np.int64))
            assert np.mean(d <= 1) >= LSB_FRACTION, (i, np.mean(d <= 1))
            got = s.dropouts(i)
            assert got == [tuple(x) for x in f["dropouts"]], i
            drops += len(got)
        assert drops > 0


def _full_size_parity(rf, fields, video, vlp, prof, tape_format, min_fields):
    from vhsd_gb300 import native
    good = [f for f in fields if "error" not in f]
    assert len(good) >= min_fields
    with native.Session(prof, len(rf), tape_format=tape_format) as s:
        r = s.decode(rf, demod_only=True)
        v = s.stream(0, 0, len(video))
        y = s.stream(1, 0, len(vlp))
        assert np.max(np.abs(v - video)) < FREQ_TOL_HZ
        assert np.max(np.abs(y - vlp)) < FREQ_TOL_HZ
        r = s.decode(rf)
        assert r.fields == len(good)
        tb = s.tbc()
        pulse_steps = 0
        for i, f in enumerate(good):
            info = s.field(i)
            assert bool(info.is_first_field) == f["first_field"], i
            assert info.span_start == f["span_start"], i
            got = s.lines(i)
            diff = np.abs(got - f["locs"])
            # Lines without a refinable hsync (the vertical interval) sit on
            # the integer start of their sync pulse.  The FP32 sync stream is
            # within 1 kHz of the oracle's, so a sample on the threshold can
            # open a pulse one sample apart: such a line may differ by exactly
            # one sample (seen on one line of 100 S-VHS fields).  Every other
            # line is within the 0.01-sample bar.
            step = (diff == 1.0) & (got == np.round(got)) & (f["locs"] == np.round(f["locs"]))
            pulse_steps += int(np.sum(step))
            assert np.max(diff[~step]) < LINE_TOL, i
            # the output lines rendered from such a line location (o = L - first
            # line - 1 and o = L - first line) are left out of the 1-LSB count
            d = np.abs(tb[i].astype(np.int64) - f["tbc"].astype(np.int64).reshape(tb[i].shape))
            ofl = (3 if f["first_field"] else 4) if prof == native.PROFILE_PAL else 1
            keep = np.ones(d.shape[0], bool)
            for L in np.nonzero(step)[0]:
                for o in (L - ofl - 1, L - ofl):
                    if 0 <= o < d.shape[0]:
                        keep[o] = False
            assert np.mean(d[keep] <= 1) >= LSB_FRACTION, (i, np.mean(d[keep] <= 1))
            assert s.dropouts(i) == [tuple(x) for x in f["dropouts"]], i
        assert pulse_steps <= max(1, len(good) // 50)


def test_full_size_svhs100_matches_oracle(gpu):
    # PAL S-VHS, 100 fields (81 M samples): sub-deemphasis on every block, +/-0.5 % timebase
    # wobble at 15 Hz and +/-2-sample head-switch jumps every field
    import bench
    from oracle import field, formats
    from vhsd_gb300 import native
    rf = bench.workload("svhs100")
    fields, (video, vlp, _, _) = field.decode_capture(rf, formats.get("PAL", "SVHS"))
    _full_size_parity(rf, fields, video, vlp, native.PROFILE_PAL, native.FORMAT_SVHS, 100)


def test_full_size_pal4_matches_oracle(gpu):
    # PAL VHS, 4 fields (3.2 M samples): bars, ramp and noise fields, 40 dB SNR
    import bench
    from oracle import field, formats
    from vhsd_gb300 import native
    rf = bench.workload("pal4")
    fields, (video, vlp, _, _) = field.decode_capture(rf, formats.get("PAL"))
    _full_size_parity(rf, fields, video, vlp, native.PROFILE_PAL, native.FORMAT_VHS, 3)
