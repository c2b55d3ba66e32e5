"""Pins the CPU oracle against the reference's own known answers (no GPU)."""
import hashlib
import json
import os

import numpy as np

from oracle import demod, filters, formats, native, sync, tbc

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
    for key, fmt in (("PAL/VHS/sp", formats.PAL_VHS_SP), ("NTSC/VHS/sp", formats.NTSC_VHS_SP),
                     ("PAL/SVHS/sp", formats.PAL_SVHS_SP), ("NTSC/SVHS/sp", formats.NTSC_SVHS_SP)):
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
