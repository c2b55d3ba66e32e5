"""Pins the CPU oracle against the reference's own known answers (no GPU)."""
import hashlib
import json
import math
from fractions import Fraction
import os

import numpy as np

from oracle import demod, field, filters, formats, native, sync, tbc

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _golden_lut():
    g = json.load(open(os.path.join(GOLDEN, "sinc_lut_rows.json")))
    lut = native.sinc_lut().copy()
    for r, h in zip(g["rows"], g["values_hex"]):
        lut[r] = np.frombuffer(bytes.fromhex(h), "<f4")
    return g, lut


def test_tbc_sinc_sha256_golden_vectors():
    # TbcParallelResamplerTests.cs:76-89, 141-152, 154-167 (platform-independent hashes)
    g, lut = _golden_lut()
    for c in g["cases"]:
        src = np.arange(c["source_length"], dtype=np.float64)
        locs = c["locations"]
        nominal = max(1.0, float(np.median(np.diff(locs))))
        out = tbc.resample_field(src, locs, c["first_line"], c["line_count"], c["outlen"], nominal,
                                 0.0, lut=lut)
        digest = hashlib.sha256(out.astype("<f8").tobytes()).hexdigest().upper()
        assert digest == c["sha256"], c["name"]


def test_linear_positions_bit_exact():
    # TbcParallelResamplerTests.cs:11-56: positions equal the scaled-coordinate formula bitwise
    rng = np.random.default_rng(0x51C02026)
    for _ in range(64):
        outlen = int(rng.integers(1, 258))
        n = int(rng.integers(4, 40))
        locs = np.empty(n)
        locs[0] = (rng.random() - 0.5) * 1e6
        for i in range(1, n):
            locs[i] = locs[i - 1] + 0.001 + rng.random() * 10000.0
        first = int(rng.integers(0, n - 1))
        count = int(rng.integers(0, n - first))
        pos = tbc.linear_positions(locs, first, count, outlen, 2000.125)
        for i in range(len(pos)):
            si = first * outlen + i
            left = si // outlen
            scaled = si * (2000.125 / outlen)
            frac = min(max((scaled - left * 2000.125) / 2000.125, 0.0), 1.0)
            exp = locs[left] + (locs[left + 1] - locs[left]) * frac
            assert np.float64(exp).tobytes() == np.float64(pos[i]).tobytes()


def test_linear_positions_non_monotonic():
    # TbcParallelResamplerTests.cs:58-74
    pos = tbc.linear_positions([20.0, 30.0, 25.0, 40.0], 1, 1, 4, 10.0)
    assert list(pos) == [30.0, 28.75, 27.5, 26.25]


def test_pulse_state_machine_known_answer():
    # PulseDetectionReuseTests.cs:306-318: [(1,2),(4,3)] before the x3 position scale
    p = native.find_pulses(np.array([5.0, 1.0, 1.0, 5.0, 1.0, 1.0, 1.0, 5.0]), 2.0, 2, 3)
    assert p == [(1, 2), (4, 3)]
    assert native.find_pulses(np.array([]), 2.0, 0, 10) == []


def test_pulse_state_machine_special_values_match_reference_loop():
    # PulseDetectionReuseTests.cs:232-298: NaN / inf inputs follow the scalar loop
    rng = np.random.default_rng(0x50414C)
    specials = [np.nan, -np.inf, -1.0, 0.0, 1.0, np.inf]
    for it in range(200):
        n = int(rng.integers(0, 4097))
        d = rng.random(n) * 20.0 - 10.0
        mask = rng.integers(0, 20, n) == 0
        d[mask] = np.array(specials)[rng.integers(0, len(specials), mask.sum())]
        high = specials[it % 6] if it % 17 == 0 else rng.random() * 12 - 6
        mn = int(rng.integers(0, 12))
        mx = int(rng.integers(mn, 32))
        assert native.find_pulses(d, high, mn, mx) == _scalar_pulses(d, high, mn, mx)


def _scalar_pulses(d, high, mn, mx):
    out = []
    if len(d) == 0:
        return out
    inp = d[0] <= high
    cur = 0
    for p, v in enumerate(d):
        if inp:
            if v > high:
                ln = p - cur
                if mn <= ln <= mx and cur != 0:
                    out.append((cur, ln))
                inp = False
        elif v <= high:
            cur = p
            inp = True
    return out


def test_replace_spikes_known_answers():
    # CompatibilityTests.cs:2600-2635
    d = np.full(50, 10.0)
    dd = np.full(50, 1.0)
    d[20] = 100.0
    demod.replace_spikes(d, dd, 50.0)
    assert np.all(d[12:49] == 1.0) and d[11] == 10.0 and d[49] == 10.0
    d = np.full(50, 10.0)
    d[20] = 100.0
    demod.replace_spikes(d, np.full(50, 200.0), 50.0)
    assert d[20] == 100.0
    d = np.full(80, 10.0)
    d[20] = 100.0
    d[40] = 100.0
    demod.replace_spikes(d, np.full(80, 1.0), 50.0)
    assert np.all(d[12:70] == 1.0) and d[11] == 10.0 and d[70] == 10.0


def test_format_table_matches_snapshot():
    g = json.load(open(os.path.join(GOLDEN, "format_params.json")))
    keys = [k for k in g if k.count("/") == 2]
    assert len(keys) == 12   # PAL/NTSC x VHS/SVHS x sp/lp/ep
    for key in keys:
        fmt = formats.get(*key.split("/"))
        sub = bool(g[key]["rf"].get("use_sub_deemphasis"))
        for k, v in g[key]["sys"].items():
            assert fmt["sys"].get(k) == v, (key, k)
        for k, v in g[key]["rf"].items():
            if k.startswith("nonlinear_") and not sub:
                continue   # read only by the sub-deemphasis (and the off-by-default nldeemp)
            mine = fmt["rf"].get(k)
            assert (mine or None) == (v or None) or mine == v, (key, k, mine, v)
        assert (formats.sub_deemphasis(fmt) is not None) == sub


def test_custom_luma_tables_match_reference_resources():
    # the shipped binary tables are the reference's text resources value for value
    import hashlib
    g = json.load(open(os.path.join(GOLDEN, "format_params.json")))["custom_luma_tables_sha256"]
    data = os.path.join(os.path.dirname(GOLDEN), "..", "vhs-decode-dotnet_gb300", "data")
    for name, digest in g.items():
        blob = open(os.path.join(data, name + ".f64"), "rb").read()
        assert len(blob) == 16385 * 16
        assert hashlib.sha256(blob).hexdigest() == digest, name


def test_vhs_demod_recovers_constant_frequency():
    # analytic-signal FM known answer (CompatibilityTests.cs:2403-2426), VHS angle form
    n, fs, f0 = 4096, 40e6, 4.1e6
    t = np.arange(n)
    z = np.exp(2j * np.pi * f0 * t / fs)
    d = native.vhs_rust_demod(z.real, z.imag, fs)
    assert d[0] == 0.0
    assert np.max(np.abs(d[1:] - f0)) < 150.0  # float polynomial atan2, << 1 kHz


def test_envelope_of_constant_carrier_is_flat():
    n = 32768
    x = np.full(n, 1000.0)
    fl = filters.FilterSet(formats.get("PAL"), 40e6)
    env = native.vhs_envelope(x, fl.env_b[0], fl.env_b[1], fl.env_a1)
    assert np.max(np.abs(env - 1000.0)) < 1e-2


def test_sync_params_nominal_line():
    sp = sync.SyncParams(formats.get("NTSC"), 40e6)
    assert sp.nominal == 2542.0
    sp = sync.SyncParams(formats.get("PAL"), 40e6)
    assert sp.nominal == 2560.0


# ---------------------------------------------------------------------------
# Known answers of the reference's sync, hsync, dropout, TBC, demod and
# stitching tests, reproduced on the oracle with the tests' own inputs.

def _sync_params(fs, line_us, hsync_us, eq_us, vsync_us, hsync_tol=0.5, eq_tol=0.5,
                 ire0=0.0, hz_ire=1.0, vsync_ire=-40.0, system="NTSC", num_pulses=6):
    """A ``SyncAnalyzer`` + ``VideoOutputConverter`` pair built from explicit values, as the
    reference tests construct them (SyncAnalysis.cs:34-66; defaults 0.5 µs tolerances)."""
    sp = object.__new__(sync.SyncParams)
    sp.system, sp.fs, sp.mhz = system, fs, fs / 1e6
    sp.nominal = line_us * sp.mhz       # UsecToSamples(linePeriodUs)
    sp.line_period_us = line_us
    sp.hsync_us, sp.eq_us, sp.vsync_us = hsync_us, eq_us, vsync_us
    sp.num_pulses = num_pulses
    sp.hsync_tol, sp.eq_tol = hsync_tol, eq_tol
    sp.ire0, sp.hz_ire, sp.vsync_ire = ire0, hz_ire, vsync_ire
    return sp


def _paint(a, start, length, value):
    a[start:start + length] = value


def test_vhs_right_hsync_preserves_initial_crossing():
    # CompatibilityTests.cs:8049-8101: right-edge validation against the -10 midpoint crossing
    # (150.5), recovered line from the initial -20 crossing (150 1/3)
    sp = _sync_params(10e6, 10.0, 5.0, 2.5, 8.0)
    lp = np.full(900, 20.0)
    for line in range(8):
        _paint(lp, 101 + line * 100, 50, -40.0)
    locs = np.array([101.0 + line * 100.0 for line in range(8)])
    refined, _ = sync.refine_hsync(sp, lp, locs, np.zeros(8, bool), -20.0)
    assert abs(refined[0] - 100.89583333333333) <= 1e-12


def test_vhs_right_hsync_uses_failed_provisional_left_crossing():
    # CompatibilityTests.cs:8103-8160
    sp = _sync_params(10e6, 10.0, 5.0, 2.5, 8.0)
    lp = np.full(900, 20.0)
    for line in range(8):
        o = line * 100
        lp[91 + o:125 + o] = -40.0
        lp[125 + o:131 + o] = -10.0
        lp[131 + o:134 + o] = -40.0
        lp[134 + o:150 + o] = 40.0
    locs = np.array([101.0 + line * 100.0 for line in range(8)])
    refined, filled = sync.refine_hsync(sp, lp, locs, np.zeros(8, bool), -20.0)
    assert abs(refined[0] - locs[0]) <= 1e-12
    assert filled[0]


def test_sync_analyzer_classifies_pulses_and_builds_line_locations():
    # CompatibilityTests.cs:8164-8283 (BuildLineLocations, which no decode path calls, is left out)
    sp = _sync_params(10e6, 10.0, 4.0, 2.0, 8.0)
    assert sp.nominal == 100.0
    ref = np.full(800, 10.0)
    for s, ln in ((100, 40), (200, 40), (300, 20), (350, 80), (500, 40), (600, 40), (700, 40)):
        _paint(ref, s, ln, -10.0)
    # FindRawPulses(threshold 0, 1 µs .. 10 µs): lengths round(usec)
    raw = native.find_pulses(ref, 0.0, int(round(sp.usec(1.0))), int(round(sp.usec(10.0))))
    assert len(raw) == 7 and raw[0] == (100, 40) and raw[3] == (350, 80)
    timing = sync.estimate_timing(sp, raw, vhs_empty_median_units=False)
    med = sync.np_median([ln for _, ln in raw if sync.in_range(ln, sp.usec(4.0 - 1.75),
                                                               sp.usec(4.0 + 2.0))])
    assert abs(med - 40.0) <= 1e-12
    assert sync.in_range(40, *timing["hsync"])
    assert sync.in_range(20, *timing["eq"])
    assert sync.in_range(80, *timing["vsync"])
    tape = _sync_params(10e6, 10.0, 4.0, 2.0, 8.0, hsync_tol=0.7, eq_tol=0.9)
    tape_timing = sync.estimate_timing(tape, raw, vhs_empty_median_units=False)
    assert not sync.in_range(34, *timing["hsync"]) and sync.in_range(34, *tape_timing["hsync"])
    assert not sync.in_range(12, *timing["eq"]) and sync.in_range(12, *tape_timing["eq"])
    classified = sync.classify_pulses(sp, raw, timing)
    assert len(classified) == 7
    assert classified[0][0] == sync.HSYNC
    assert classified[2][0] == sync.EQ
    assert classified[3][0] == sync.VSYNC
    assert abs(sync.mean_line_length(sp, classified) - 100.0) <= 1e-12
    nearest = [(sync.HSYNC, 100, 40, False), (sync.HSYNC, 190, 40, True),
               (sync.HSYNC, 310, 40, True), (sync.HSYNC, 410, 40, True)]
    locs, filled = sync.build_upstream_line_locations(nearest, 100.0, 0, 100.0, 4)
    assert list(locs) == [100, 190, 310, 400] and not filled.any()
    equal = [(sync.HSYNC, 90, 40, True), (sync.HSYNC, 110, 40, True), (sync.HSYNC, 300, 40, True)]
    locs, _ = sync.build_upstream_line_locations(equal, 100.0, 0, 100.0, 1, prefer_earlier=True)
    assert list(locs) == [90]
    # FromParameters on the format table (SyncAnalysis.cs:89-111)
    pal = sync.SyncParams(formats.get("PAL"), 40e6)
    assert pal.nominal == 2560.0 and pal.num_pulses == 5


def test_vhs_timing_preserves_empty_hsync_median_units():
    # CompatibilityTests.cs:8284-8312
    sp = _sync_params(40e6, 63.55, 4.7, 2.3, 27.1, hsync_tol=0.7, eq_tol=0.9)
    noise = [(100, 17), (200, 23), (300, 294), (700, 50), (900, 12)]
    standard = sync.estimate_timing(sp, noise, vhs_empty_median_units=False)
    v040 = sync.estimate_timing(sp, noise)
    assert abs(sum(standard["hsync"]) / 2 - 188.0) <= 1e-12
    assert abs(sum(v040["hsync"]) / 2 - 4.7) <= 1e-12
    assert not sync.in_range(17, *standard["hsync"])
    for ln in (17, 23, 12):
        assert sync.in_range(ln, *v040["hsync"])
    assert not sync.in_range(50, *v040["hsync"])


def test_dropout_threshold_uses_float32_envelope_mean():
    # TapeDropoutNumericsCompatibilityTests.cs:10-69: numpy float32 mean, threshold = mean*0.18f
    high = np.frombuffer(np.uint32(0x411FFC18).tobytes(), np.float32)[0]
    low = np.frombuffer(np.uint32(0x3FDCD8C5).tobytes(), np.float32)[0]
    env = np.full(320, float(high))
    env[125:141] = float(low)
    mean32 = np.mean(env.astype(np.float32), dtype=np.float32)
    assert np.float32(mean32).view(np.uint32) == 0x41195DA5
    assert np.float32(mean32 * np.float32(0.18)).view(np.uint32) == 0x3FDCD8C5
    # the field's hsync pulses at 10, 110, 210 give line starts every 100 samples
    sp = _sync_params(1e6, 100.0, 10.0, 5.0, 20.0)
    sp.output_lines = 2
    sp.outlinelen = 4
    locs = np.array([10.0, 110.0, 210.0, 310.0])
    # DetectTapeDropouts over lines 1..3 with the test's hysteresis of 2.0
    thr = float(np.float32(mean32 * np.float32(0.18)))
    ranges = native.find_dropouts(env, int(np.floor(locs[1])), int(np.ceil(locs[3])), thr, 2.0)
    drops = field.map_rf_to_tbc(ranges, locs, 4, 1, 3, 0)
    assert drops == [(1, 0, 2)]


def _legacy_level_adjusts(locs, outlen, line_count, nominal, smoothing):
    # TbcDirectConversionTests.cs:284-333 (the test's allocation-based reference)
    inv = 1.0 / nominal
    factors = np.array([(locs[i + 1] * inv) - (locs[i] * inv) for i in range(line_count)])
    med = float(np.median(factors))
    mad = float(np.median(np.abs(factors - med)))
    thr = 15.0 * mad if mad > 0.0 else 0.001
    la = np.repeat(np.where(np.abs(factors - med) > thr, med, factors), outlen)
    if smoothing > 0.0:
        alpha = 1.0 / (smoothing * outlen)
        for i in range(1, len(la)):
            prev = la[i - 1]
            la[i] = _fma(la[i] - prev, alpha, prev)
    return la


def _fma(a, b, c):
    """a*b + c rounded once (exact rational arithmetic; int/int division rounds correctly)."""
    r = Fraction(float(a)) * Fraction(float(b)) + Fraction(float(c))
    return r.numerator / r.denominator


def test_tbc_direct_conversion_inputs():
    # TbcDirectConversionTests.cs:11-84: level adjusts bit-equal to the legacy reference; the
    # uint16 output equals FastMathConversion applied to the float resampler output
    outlen, lines, nominal = 1024, 100, 2000.125
    i = np.arange(220_000, dtype=np.float64)
    src = 4_000_000.0 + 1_500_000.0 * np.sin(i * 0.0031) + 250_000.0 * np.cos(i * 0.0007)
    li = np.arange(lines + 1, dtype=np.float64)
    locs = 1000.25 + li * nominal + 0.01 * li * li
    locs[50] += 50.0
    la = tbc.level_adjusts(locs, 0, lines, outlen, nominal, 1.5)
    legacy = _legacy_level_adjusts(locs, outlen, lines, nominal, 1.5)
    assert la[:len(legacy)].tobytes() == legacy.tobytes()
    hz = tbc.resample_field(src, locs, 0, lines, outlen, nominal, 1.5)
    u16 = native.hz_to_u16(hz, 4_000_000.25, 512.25, 100_000.125, 256.0, -40.0)
    inv = 1.0 / 100_000.125
    off = (256 + 0.5) - (-40.0 * 512.25)
    v = np.array([_fma(512.25 * (h - 4_000_000.25), inv, off) for h in hz[:4096]])
    exp = np.where(v <= 0.0, 0, np.where(v >= 65535.0, 65535, np.floor(np.maximum(v, 0))))
    assert np.array_equal(u16[:4096], exp.astype(np.uint16))


def _vhs_atan2_f32(y, x):
    # PortedMath.VhsRustAtan2Approximation (PortedMath.cs:519-544) in numpy float32
    f = np.float32
    x = (x + np.copysign(f(1.17549435e-38), x)).astype(f)
    swap = np.abs(x) < np.abs(y)
    with np.errstate(all="ignore"):
        inp = np.where(swap, x / y, y / x).astype(f)
        sq = (inp * inp).astype(f)
        r = f(-0.01172120)
        r = (f(0.05265332) + sq * r).astype(f)
        r = (f(-0.11643287) + sq * r).astype(f)
        r = (f(0.19354346) + sq * r).astype(f)
        r = (f(-0.33262347) + sq * r).astype(f)
        r = (f(0.99997726) + sq * r).astype(f)
        r = (inp * r).astype(f)
        half = np.where(inp >= 0.0, f(np.pi / 2), f(-np.pi / 2)).astype(f)
        r = np.where(swap, half - r, r).astype(f)
        pi = f(np.pi)
        xs, ys = x >= 0.0, y >= 0.0
        r = np.where(~xs & ys, pi + r, np.where(~xs & ~ys, -pi + r, r)).astype(f)
    return r


def _vhs_unwrap_scalar(re, im, fs):
    # UnwrapHilbertVhsRustApproximationScalar (PortedMath.cs:70-88, 546-551)
    f = np.float32
    with np.errstate(over="ignore"):
        re32, im32 = re.astype(f), im.astype(f)
    ang = _vhs_atan2_f32(im32, re32)
    tau = f(2 * np.pi)
    with np.errstate(all="ignore"):
        d = (ang[1:] - ang[:-1]).astype(f)
        d = (d - (np.floor((d / tau).astype(f)) * tau).astype(f)).astype(f)
        out = ((d * f(fs)).astype(f) / tau).astype(f)
    return np.concatenate([[0.0], out.astype(np.float64)])


def _unwrap_input(n):
    # VhsRustUnwrapSimdTests.cs:92-128
    nan1 = np.frombuffer(np.uint64(0xFFF8000000001234).tobytes(), np.float64)[0]
    nan2 = np.frombuffer(np.uint64(0x7FF8000000005678).tobytes(), np.float64)[0]
    tiny = np.finfo(np.float64).smallest_subnormal
    big = np.finfo(np.float64).max
    edge = [(0.0, 0.0), (-0.0, 0.0), (1.0, -1.0), (tiny, -tiny), (-big, big), (np.inf, 1.0),
            (1.0, -np.inf), (nan1, 2.0), (-3.0, nan2)]
    re = np.empty(n)
    im = np.empty(n)
    for i in range(n):
        if i < len(edge):
            re[i], im[i] = edge[i]
        elif i == 25:
            re[i], im[i] = np.inf, -2.0
        else:
            a = 1.0 + (i % 17)
            re[i], im[i] = math.cos(i * 0.0137) * a, math.sin(i * 0.0179) * (a + 0.25)
    return re, im


def _same_bits_or_nan(a, b):
    na, nb = np.isnan(a), np.isnan(b)
    return np.array_equal(na, nb) and a[~na].tobytes() == b[~nb].tobytes()


def test_vhs_unwrap_edge_vectors():
    # VhsRustUnwrapSimdTests.cs:9-57: the C restatement against the scalar loop, bit for bit
    # (NaN payloads are platform-defined; NaN positions must agree)
    for n in (1, 2, 3, 4, 5, 7, 8, 9, 12, 16, 17, 32768):
        re, im = _unwrap_input(n)
        got = native.vhs_rust_demod(re, im, 40e6)
        assert _same_bits_or_nan(got, _vhs_unwrap_scalar(re, im, 40e6)), n


def test_vhs_raw_envelope_edge_vectors():
    # RfEnvelopeSimdTests.cs:8-74: raw envelope == the test's scalar reference, bit for bit
    edge = [0.0, -0.0, 1.0, -1.0, np.finfo(np.float64).smallest_subnormal,
            -np.finfo(np.float64).smallest_subnormal, np.inf, -np.inf,
            np.frombuffer(np.uint64(0xFFF8000000001234).tobytes(), np.float64)[0],
            12345.6789012345, -98765.4321098765]
    for n in (1, 2, 3, 4, 5, 7, 8, 9, 32768):
        x = np.array([edge[i] if i < len(edge) else math.sin(i * 0.0031) * (1.0 + (i % 17))
                      for i in range(n)])
        exp = np.empty(n, np.float32)
        shift = 4 % n
        split = n - shift
        exp[shift:shift + split] = np.abs(x[:split].astype(np.float32))
        exp[:n - split] = np.abs(x[split:].astype(np.float32))
        got = native.vhs_raw_envelope(x)
        assert _same_bits_or_nan(got.astype(np.float64), exp.astype(np.float64)), n


def test_analytic_fm_demod_recovers_generated_frequency():
    # CompatibilityTests.cs:2403-2426 (the binary64 conjugate-product form)
    n, fs, f0 = 32, 32.0, 4.0
    z = np.exp(2j * np.pi * f0 * np.arange(n) / fs)
    d = demod.unwrap_conjugate_product(z, fs)
    assert d[0] == 0.0
    assert np.max(np.abs(d[1:] - f0)) <= 1e-12


def test_fm_block_through_frequency_filters():
    # CompatibilityTests.cs:2428-2520: identity filters recover the carrier; zero filters mute;
    # the sync-reference offset is a roll; the clip to 1.5 MHz .. 0.75 fs
    n, fs, carrier = 32, 32.0, 4.0
    raw = np.cos(2 * np.pi * carrier * np.arange(n) / fs)
    ident = np.ones(n, complex)
    video, dr, _, env, vlp = demod.demod_block_complex(raw, ident, ident, ident, fs)
    assert np.max(np.abs(env - 1.0)) <= 1e-12
    for arr in (dr, video, vlp):
        assert np.max(np.abs(arr[2:n - 2] - carrier)) <= 1e-10
    muted = demod.demod_block_complex(raw, ident, np.zeros(n, complex), np.zeros(n, complex), fs)
    assert not muted[0].any() and not muted[4].any()
    ph = np.cumsum(2 * np.pi * (3.0 + 0.75 * np.sin(2 * np.pi * np.arange(n) / n)) / fs)
    varied = np.cos(ph)
    a = demod.demod_block_complex(varied, ident, ident, ident, fs, video_lp_offset=0)[4]
    b = demod.demod_block_complex(varied, ident, ident, ident, fs, video_lp_offset=5)[4]
    assert np.array_equal(np.roll(a, -5), b)
    ldn, ldfs, low = 128, 8e6, 1e6
    low_fm = np.cos(2 * np.pi * low * np.arange(ldn) / ldfs)
    li = np.ones(ldn, complex)
    video, dr, _, _, vlp = demod.demod_block_complex(low_fm, li, li, li, ldfs, clip_for_video=True)
    assert np.max(np.abs(dr[4:ldn - 4] - low)) <= 1e-3
    assert np.max(np.abs(video[4:ldn - 4] - 1.5e6)) <= 1e-3
    assert np.max(np.abs(vlp[4:ldn - 4] - 1.5e6)) <= 1e-3


def test_overlap_save_stitching_geometry():
    # CompatibilityTests.cs:6883-6912: N=16, cut 2/2, stride 12; Read(begin 5, length 15)
    # returns input samples 7..21 (stream s <-> RF s + cut)
    rf = np.arange(64, dtype=np.float64)
    (inp,) = demod.stitch_span(rf, lambda b: (b,), 16, 2, 2, 5, 15)
    assert list(inp) == list(range(7, 22))
    # the production geometry (N=32768, cut 1024/1024) is the same formula
    rf = np.arange(5 * demod.STRIDE + demod.BLOCK, dtype=np.float64)
    (inp,) = demod.stitch_span(rf, lambda b: (b,), demod.BLOCK, demod.CUT, demod.CUT_END,
                               12345, 3 * demod.STRIDE)
    assert np.array_equal(inp, rf[12345 + demod.CUT:12345 + demod.CUT + 3 * demod.STRIDE])
