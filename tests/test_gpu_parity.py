"""Device parity against the CPU oracle, through the C ABI.

Tolerances (stated once, used below):
* demodulated / filtered video frequency: within 1 kHz;
* line locations: within 0.01 sample;
* uint16 TBC: |diff| <= 1 LSB on >= 99.9% of samples (FP32 fused path);
  the FP64 plain path is held to the same bar;
* field count, field order and dropout decisions identical.
Integer / index work (pulses, angles, TBC arithmetic on identical inputs) is bit-exact.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FREQ_TOL_HZ = 1000.0
LINE_TOL = 0.01
LSB_FRACTION = 0.999


def test_device_atan2_bit_exact(gpu):
    from vhsd_gb300 import native
    from oracle import native as onative
    rng = np.random.default_rng(7)
    n = 1 << 16
    re = (rng.standard_normal(n) * 10 ** rng.uniform(-3, 4, n)).astype(np.float32)
    im = (rng.standard_normal(n) * 10 ** rng.uniform(-3, 4, n)).astype(np.float32)
    special = np.array([0.0, -0.0, 1.0, -1.0, np.inf, -np.inf, np.nan, 1e-45, -1e-45, 3e38],
                       np.float32)
    re[:100] = np.resize(special, 100)
    im[:100] = np.resize(special[::-1], 100)
    a = native.vhs_angles(re, im)
    b = onative.vhs_rust_angles(re, im)
    # NaN results agree as NaN (the payload bits of a generated NaN are the
    # hardware's canonical pattern); every other result is bit-identical.
    nan = np.isnan(b)
    assert np.array_equal(np.isnan(a), nan)
    assert a[~nan].view(np.uint32).tolist() == b[~nan].view(np.uint32).tolist()


def test_device_fm_demod_bit_exact(gpu):
    from vhsd_gb300 import native
    from oracle import native as onative
    rng = np.random.default_rng(11)
    n = 1 << 16
    # phases stepping by up to +-pi with equal, opposite and near-boundary angles
    ph = np.cumsum(rng.uniform(-np.pi, np.pi, n))
    ph[1000:1010] = ph[999]
    ph[2000:2010] = np.pi * np.array([1, -1] * 5)
    amp = 10 ** rng.uniform(-40, 4, n)
    re = (amp * np.cos(ph)).astype(np.float32)
    im = (amp * np.sin(ph)).astype(np.float32)
    im[3000:3010] = np.array([0.0, -0.0] * 5, np.float32)
    re[3000:3010] = np.array([1.0, 1.0, -1.0, -1.0, 1e-45, -1e-45, 2.0, 3.0, -2.0, -3.0], np.float32)
    re[4000:4010] = np.float32(np.nan)
    a = native.vhs_demod(re, im, 40e6)
    b = onative.vhs_rust_demod(re.astype(np.float64), im.astype(np.float64), 40e6).astype(np.float32)
    nan = np.isnan(b)
    assert np.array_equal(np.isnan(a), nan)
    assert a[~nan].view(np.uint32).tolist() == b[~nan].view(np.uint32).tolist()


def test_parallel_replace_spikes_matches_sequential(gpu):
    # dense, overlapping spike windows where the order of replacements matters
    from vhsd_gb300 import native
    from oracle import demod as odemod
    rng = np.random.default_rng(99)
    for it in range(40):
        n = 32 * int(rng.integers(1, 300))
        d = rng.normal(0.0, 1.0, n).astype(np.float32)
        f = rng.normal(0.0, 1.0, n).astype(np.float32)
        dens = rng.choice([0.002, 0.02, 0.1, 0.5])
        hit = rng.random(n) < dens
        d[hit] = rng.uniform(3.0, 9.0, hit.sum()).astype(np.float32)
        f[rng.random(n) < dens] += np.float32(rng.uniform(0, 8))
        want = odemod.replace_spikes(d.astype(np.float64), f.astype(np.float64), 2.5).astype(np.float32)
        got = native.replace_spikes(d, f, 2.5)
        assert got.tobytes() == want.tobytes(), (it, n, dens)


def test_device_pulses_match_state_machine(gpu):
    from vhsd_gb300 import native
    from oracle import native as onative
    rng = np.random.default_rng(0x50414C)
    specials = [np.nan, -np.inf, -1.0, 0.0, 1.0, np.inf]
    for it in range(60):
        n = int(rng.integers(1, 20000))
        d = rng.random(n) * 20.0 - 10.0
        mask = rng.integers(0, 20, n) == 0
        d[mask] = np.array(specials)[rng.integers(0, len(specials), mask.sum())]
        high = rng.random() * 12 - 6
        mn = int(rng.integers(0, 12))
        mx = int(rng.integers(mn, 64))
        assert native.find_pulses(d, high, mn, mx) == onative.find_pulses(d, high, mn, mx)


def test_device_tbc_bit_exact_against_oracle(gpu):
    from vhsd_gb300 import native
    from oracle import tbc
    import json
    import os
    g = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "sinc_lut_rows.json")))
    for c in g["cases"]:
        src = np.arange(c["source_length"], dtype=np.float64)
        locs = c["locations"]
        nominal = max(1.0, float(np.median(np.diff(locs))))
        want = tbc.resample_field(src, locs, c["first_line"], c["line_count"], c["outlen"], nominal, 0.0)
        got = native.tbc_resample_lines(src, locs, c["first_line"], c["line_count"], c["outlen"])
        assert got.tobytes() == want.tobytes(), c["name"]
    # larger plan with wow smoothing and outlier factors
    idx = np.arange(220000)
    src = np.sin(idx * 0.0031) + np.cos(idx * 0.0007)
    locs = 1000.25 + np.arange(101) * 2000.125 + 0.01 * np.arange(101) ** 2
    locs[40] += 700.0
    want = tbc.resample_field(src, locs, 3, 90, 1024, 2000.125, 1.5)
    got = native.tbc_resample_lines(src, locs, 3, 90, 1024, 2000.125, 1.5)
    # smoothing is evaluated in closed form on the device: equal to float rounding
    assert np.max(np.abs(got - want)) <= 2 * np.max(np.abs(want)) * 2 ** -24


def _session_decode(system, rf, precision):
    from vhsd_gb300 import native
    prof = native.PROFILE_PAL if system == "PAL" else native.PROFILE_NTSC
    s = native.Session(prof, len(rf), precision=precision)
    r = s.decode(rf)
    return s, r


@pytest.mark.parametrize("precision", [0, 1], ids=["fp32_fused", "fp64_plain"])
@pytest.mark.parametrize("system", ["PAL", "NTSC"])
def test_stream_channels_match_oracle(gpu, system, precision, request):
    rf, _ = request.getfixturevalue("pal_capture" if system == "PAL" else "ntsc_capture")
    _, (video, vlp, env, _) = request.getfixturevalue("pal_oracle" if system == "PAL" else "ntsc_oracle")
    from vhsd_gb300 import native
    prof = native.PROFILE_PAL if system == "PAL" else native.PROFILE_NTSC
    with native.Session(prof, len(rf), precision=precision) as s:
        r = s.decode(rf, demod_only=True)
        n = len(video)
        assert r.stream_samples == n
        v = s.stream(0, 0, n)
        y = s.stream(1, 0, n)
        e = s.stream(2, 0, n)
    dv = np.abs(v - video)
    dy = np.abs(y - vlp)
    assert np.max(dv) < FREQ_TOL_HZ, np.max(dv)
    assert np.max(dy) < FREQ_TOL_HZ, np.max(dy)
    assert np.median(dv) < 2.0 and np.median(dy) < 2.0, (np.median(dv), np.median(dy))
    de = np.abs(e - env) / np.maximum(np.abs(env), 1.0)
    assert np.quantile(de, 0.999) < 1e-3
    if precision == 1:
        assert np.max(dv) < 1.0 and np.max(dy) < 1.0


@pytest.mark.parametrize("precision", [0, 1], ids=["fp32_fused", "fp64_plain"])
@pytest.mark.parametrize("system", ["PAL", "NTSC"])
def test_fields_and_tbc_match_oracle(gpu, system, precision, request):
    rf, _ = request.getfixturevalue("pal_capture" if system == "PAL" else "ntsc_capture")
    fields, _ = request.getfixturevalue("pal_oracle" if system == "PAL" else "ntsc_oracle")
    good = [f for f in fields if "error" not in f]
    from vhsd_gb300 import native
    prof = native.PROFILE_PAL if system == "PAL" else native.PROFILE_NTSC
    with native.Session(prof, len(rf), precision=precision) as s:
        r = s.decode(rf)
        assert r.fields == len(good)
        tb = s.tbc()
        for i, f in enumerate(good):
            info = s.field(i)
            assert bool(info.is_first_field) == f["first_field"]
            assert info.span_start == f["span_start"]
            locs = s.lines(i)
            assert np.max(np.abs(locs - f["locs"])) < LINE_TOL
            d = np.abs(tb[i].astype(np.int64).ravel() - f["tbc"].astype(np.int64))
            assert np.mean(d <= 1) >= LSB_FRACTION, (i, np.mean(d <= 1), d.max())
            assert s.dropouts(i) == [tuple(x) for x in f["dropouts"]]


def test_decode_is_deterministic(gpu, pal_capture):
    from vhsd_gb300 import native
    rf, _ = pal_capture
    with native.Session(native.PROFILE_PAL, len(rf)) as s:
        s.decode(rf)
        a = s.tbc().copy()
        s.decode(rf)
        b = s.tbc()
    assert a.tobytes() == b.tobytes()


def test_chroma_decode_is_deterministic(gpu, pal_capture):
    # the reference's release gates require identical output bytes run to run;
    # the default decode (luma and colour-under chroma) twice on one session
    from vhsd_gb300 import native
    rf, _ = pal_capture
    with native.Session(native.PROFILE_PAL, len(rf)) as s:
        s.decode(rf, chroma=True)
        a, ca = s.tbc().copy(), s.chroma().copy()
        s.decode(rf, chroma=True)
        b, cb = s.tbc(), s.chroma()
    assert a.tobytes() == b.tobytes()
    assert ca.tobytes() == cb.tobytes()


def test_device_input_pointer_path(gpu, pal_capture):
    import torch
    from vhsd_gb300 import native
    rf, _ = pal_capture
    d = torch.from_numpy(rf.copy()).cuda()
    with native.Session(native.PROFILE_PAL, len(rf)) as s:
        s.decode(rf)
        host = s.tbc().copy()
        s.decode(None, device_ptr=d.data_ptr(), count=len(rf))
        dev = s.tbc()
    assert host.tobytes() == dev.tobytes()


def test_pinned_input_graph_replay_matches(gpu, ntsc_capture):
    # pinned host input and device input take the captured-graph pipeline;
    # pageable input queues the same work directly: all give identical output
    import torch
    from vhsd_gb300 import native
    rf, _ = ntsc_capture
    pinned = torch.from_numpy(rf.copy()).pin_memory()
    with native.Session(native.PROFILE_NTSC, len(rf)) as s:
        s.decode(rf)
        want = s.tbc().copy()
        locs = [s.lines(i).copy() for i in range(s.decode(rf).fields)]
        for _ in range(2):  # capture, then replay
            r = s.decode(pinned.numpy())
            assert s.tbc().tobytes() == want.tobytes()
            assert all(np.array_equal(s.lines(i), locs[i]) for i in range(r.fields))
        assert r.segments >= 1 and r.kernel_launches > 0


def test_field_recovery_matches_oracle(gpu, pal_capture):
    # a capture that starts mid-field: the first attempt fails and the engine
    # moves on by the reference's recovery step, then decodes the next fields
    from oracle import field, formats
    from vhsd_gb300 import native
    rf, _ = pal_capture
    x = np.ascontiguousarray(rf[1115360:])
    fields, _ = field.decode_capture(x, formats.get("PAL"))
    assert any("error" in f for f in fields)
    good = [f for f in fields if "error" not in f]
    assert good
    with native.Session(native.PROFILE_PAL, len(x)) as s:
        r = s.decode(x)
        assert r.fields == len(good)
        tb = s.tbc()
        for i, f in enumerate(good):
            info = s.field(i)
            assert info.span_start == f["span_start"]
            assert bool(info.is_first_field) == f["first_field"]
            assert np.max(np.abs(s.lines(i) - f["locs"])) < LINE_TOL
            d = np.abs(tb[i].astype(np.int64).ravel() - f["tbc"].astype(np.int64))
            assert np.mean(d <= 1) >= LSB_FRACTION
            assert s.dropouts(i) == [tuple(y) for y in f["dropouts"]]


@pytest.mark.parametrize("precision", [0, 1], ids=["fp32_fused", "fp64_plain"])
def test_20msps_fields_match_oracle(gpu, precision, ntsc20_capture, ntsc20_oracle):
    # NTSC VHS sampled at 20 MSPS (the serving mix's 20 MSPS streams)
    from vhsd_gb300 import native
    rf, _ = ntsc20_capture
    fields, (video, _, _, _) = ntsc20_oracle
    good = [f for f in fields if "error" not in f]
    with native.Session(native.PROFILE_NTSC, len(rf), precision=precision, sample_rate_mhz=20.0) as s:
        r = s.decode(rf, demod_only=True)
        v = s.stream(0, 0, len(video))
        assert np.max(np.abs(v - video)) < FREQ_TOL_HZ
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


@pytest.mark.parametrize("precision", [0, 1], ids=["fp32_fused", "fp64_plain"])
@pytest.mark.parametrize("system", ["PAL", "NTSC"])
def test_svhs_matches_oracle(gpu, system, precision, request):
    # S-VHS: custom luma filters and the nonlinear sub-deemphasis on the video,
    # +/-0.5 % timebase wobble and +/-2-sample head-switch jumps in the capture
    from vhsd_gb300 import native
    cap, orc = ("svhs_capture", "svhs_oracle") if system == "PAL" else ("svhs_ntsc_capture",
                                                                         "svhs_ntsc_oracle")
    rf, _ = request.getfixturevalue(cap)
    fields, (video, vlp, env, _) = request.getfixturevalue(orc)
    good = [f for f in fields if "error" not in f]
    assert len(good) >= 3
    prof = native.PROFILE_PAL if system == "PAL" else native.PROFILE_NTSC
    with native.Session(prof, len(rf), precision=precision, tape_format=native.FORMAT_SVHS) as s:
        r = s.decode(rf, demod_only=True)
        n = len(video)
        assert r.stream_samples == n
        v = s.stream(0, 0, n)
        y = s.stream(1, 0, n)
        e = s.stream(2, 0, n)
        dv = np.abs(v - video)
        dy = np.abs(y - vlp)
        assert np.max(dv) < FREQ_TOL_HZ, np.max(dv)
        assert np.max(dy) < FREQ_TOL_HZ, np.max(dy)
        # no systematic offset (FP32 rounding alone is well under 2 Hz)
        assert np.median(dv) < 2.0 and np.median(dy) < 2.0, (np.median(dv), np.median(dy))
        de = np.abs(e - env) / np.maximum(np.abs(env), 1.0)
        assert np.quantile(de, 0.999) < 1e-3
        if precision == 1:
            assert np.max(dv) < 1.0 and np.max(dy) < 1.0
        r = s.decode(rf)
        assert r.fields == len(good)
        tb = s.tbc()
        for i, f in enumerate(good):
            info = s.field(i)
            assert bool(info.is_first_field) == f["first_field"]
            assert info.span_start == f["span_start"]
            assert np.max(np.abs(s.lines(i) - f["locs"])) < LINE_TOL
            d = np.abs(tb[i].astype(np.int64).ravel() - f["tbc"].astype(np.int64))
            assert np.mean(d <= 1) >= LSB_FRACTION, (i, np.mean(d <= 1), d.max())
            assert s.dropouts(i) == [tuple(x) for x in f["dropouts"]]


def test_svhs_sub_deemphasis_changes_the_video(gpu, svhs_capture):
    # the same capture decoded as VHS-filtered S-VHS levels without the
    # sub-deemphasis branch differs: the correction is really applied
    from vhsd_gb300 import native
    from oracle import demod, filters, formats
    rf, _ = svhs_capture
    fmt = formats.get("PAL", "SVHS")
    fl = filters.FilterSet(fmt, 40e6)
    x = rf[10 * 30720:10 * 30720 + 32768].astype(np.float64)
    v_sub, _, _, _, _ = demod.demod_block(x, fl, 40e6, None)
    fl.sub = None
    v_lin, _, _, _, _ = demod.demod_block(x, fl, 40e6, None)
    with native.Session(native.PROFILE_PAL, len(rf), tape_format=native.FORMAT_SVHS) as s:
        s.decode(rf, demod_only=True)
        got = s.stream(0, 10 * 30720, 30720)
    keep = slice(1024, 1024 + 30720)
    assert np.max(np.abs(got - v_sub[keep])) < FREQ_TOL_HZ
    assert np.quantile(np.abs(v_sub[keep] - v_lin[keep]), 0.9) > 10 * FREQ_TOL_HZ


@pytest.mark.parametrize("plan", [0, 1, 4, 5])
def test_every_fft_radix_plan_matches_oracle(gpu, plan, pal_capture, pal_oracle, monkeypatch):
    # the autotuner may pick any radix plan: each must meet the stage tolerances
    from vhsd_gb300 import native
    rf, _ = pal_capture
    _, (video, vlp, env, _) = pal_oracle
    monkeypatch.setenv("VHSD_FFT_PLAN", str(plan))
    with native.Session(native.PROFILE_PAL, len(rf)) as s:
        r = s.decode(rf, demod_only=True)
        assert r.fft_plan == plan
        n = len(video)
        v = s.stream(0, 0, n)
        y = s.stream(1, 0, n)
        e = s.stream(2, 0, n)
    assert np.max(np.abs(v - video)) < FREQ_TOL_HZ
    assert np.max(np.abs(y - vlp)) < FREQ_TOL_HZ
    assert np.quantile(np.abs(e - env) / np.maximum(np.abs(env), 1.0), 0.999) < 1e-3


@pytest.mark.parametrize("precision", [0, 1], ids=["fp32_fused", "fp64_plain"])
@pytest.mark.parametrize("system,speed", [("PAL", "lp"), ("NTSC", "ep")])
def test_long_play_matches_oracle(gpu, system, speed, precision, request):
    # VHS LP/EP: the format's sub-deemphasis on every block (820 kHz high-pass,
    # exponent 0.12, first scale 0.1) and, for NTSC EP, the narrower RF filters
    from oracle import field, formats
    from vhsd_gb300 import native
    rf, _ = request.getfixturevalue("pal_capture" if system == "PAL" else "ntsc_capture")
    fields, (video, vlp, env, _) = field.decode_capture(rf, formats.get(system, "VHS", speed))
    good = [f for f in fields if "error" not in f]
    assert len(good) >= 2
    prof = native.PROFILE_PAL if system == "PAL" else native.PROFILE_NTSC
    spd = native.TAPE_LP if speed == "lp" else native.TAPE_EP
    with native.Session(prof, len(rf), precision=precision, tape_speed=spd) as s:
        r = s.decode(rf, demod_only=True)
        n = len(video)
        v = s.stream(0, 0, n)
        y = s.stream(1, 0, n)
        assert np.max(np.abs(v - video)) < FREQ_TOL_HZ
        assert np.max(np.abs(y - vlp)) < FREQ_TOL_HZ
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
            assert np.mean(d <= 1) >= LSB_FRACTION, (i, np.mean(d <= 1), d.max())
            assert s.dropouts(i) == [tuple(x) for x in f["dropouts"]]
    # the long-play decode differs from the SP decode of the same capture
    with native.Session(prof, len(rf), precision=precision) as s:
        s.decode(rf, demod_only=True)
        v_sp = s.stream(0, 0, n)
    assert np.quantile(np.abs(v - v_sp), 0.9) > 10.0 * 1000.0 / 100.0
