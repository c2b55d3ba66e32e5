"""Regenerate the golden fixtures in this folder from the reference checkout.

Run with the reference checkout given as the first argument or in the
REFERENCE_ROOT environment variable; the outputs are committed so nothing
reads the reference at test time.

* format_params.json: the keys of the frozen upstream parameter snapshot
  (src/VHSDecode.Core/Formats/format-params.snapshot.json) that the RF -> TBC
  luma and chroma paths read, for PAL and NTSC, VHS and SVHS, at sp, lp and ep, and the
  SHA-256 of the S-VHS custom luma tables (src/VHSDecode.Core/Formats/custom/*.txt) converted as
  vhs-decode-dotnet_gb300/data/make_tables.py converts them.
* sinc_lut_rows.json: the rows of the reference's 65537 x 16 sinc LUT
  (src/VHSDecode.Core/Tbc/Resources/sinc_lut.npz) that the three
  platform-independent SHA-256 tests of tests/VHSDecode.Tests/
  TbcParallelResamplerTests.cs touch, with the test inputs and the expected
  hashes transcribed from that file (lines 76-89, 141-152, 154-167).
"""
import json
import os
import sys

import numpy as np

REF = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("REFERENCE_ROOT")
if not REF or not os.path.isdir(REF):
    sys.exit("usage: %s REFERENCE_ROOT (or set REFERENCE_ROOT)" % os.path.basename(__file__))
HERE = os.path.dirname(os.path.abspath(__file__))

SYS_KEYS = ["FPS", "ire0", "hz_ire", "vsync_ire", "line_period", "hsyncPulseUS", "eqPulseUS",
            "vsyncPulseUS", "numPulses", "outlinelen", "outfreq", "frame_lines", "field_lines",
            "outputZero", "fsc_mhz", "colorBurstUS", "burst_abs_ref"]
RF_KEYS = ["video_bpf_low", "video_bpf_high", "video_bpf_order", "video_bpf_supergauss",
           "video_lpf_extra", "video_lpf_extra_order", "video_hpf_extra", "video_hpf_extra_order",
           "video_rf_peak_freq", "video_rf_peak_gain", "video_rf_peak_bandwidth",
           "boost_rf_linear_0", "boost_rf_linear_20", "start_rf_linear", "boost_rf_linear_double",
           "video_lpf_freq", "video_lpf_order", "video_lpf_supergauss", "deemph_gain",
           "deemph_mid", "deemph_q", "color_under_carrier", "video_custom_luma_filters",
           "use_sub_deemphasis", "nonlinear_highpass_freq", "nonlinear_bandpass_upper",
           "nonlinear_bandpass_order", "nonlinear_amp_lpf_freq", "nonlinear_exp_scaling",
           "nonlinear_scaling_1", "nonlinear_scaling_2", "nonlinear_logistic_mid",
           "nonlinear_logistic_rate", "nonlinear_static_factor", "chroma_bpf_upper",
           "chroma_bpf_lower", "chroma_bpf_order", "chroma_rotation", "chroma_offset",
           "chroma_audio_notch_freq"]
SYS_KEYS_SUB = ["nonlinear_deviation"]

# (name, source length, locations, first line, line count, outlen, expected SHA-256)
HASH_CASES = [
    ("interior_and_bounded_edges", 64, [-4.25, 28.5, 67.75], 0, 2, 16,
     "7E3B3F5DCF0E5C38FB7C46E6E5CF362D596F9DECD7416445247F0A4C4878F33C"),
    ("negative_coordinates", 64, [-4.25, 28.5], 0, 1, 16,
     "426959AEB3440862EF1B3148CF09D4AF143D5F4F21944E04C6AAA62214F4C0BC"),
    ("source_shorter_than_taps", 8, [0.0, 7.0], 0, 1, 16,
     "5E5BED2929B57864FE4E2514C4D3754CF7168A6200A7C57FF45BDE2F97B1BD1F"),
]


def lut_rows_for(positions):
    rows = set()
    for p in positions:
        coord = np.float32(p)
        ci = int(coord)  # truncation toward zero
        frac = np.float32(coord - np.float32(ci))
        pp = np.float32(frac * np.float32(65536))
        ps = int(pp)
        for r in (ps, ps + 1):
            if r < 0:
                r += 65537
            rows.add(min(max(r, 0), 65536))
    return rows


def main():
    snap = json.load(open(os.path.join(REF, "src/VHSDecode.Core/Formats/format-params.snapshot.json")))
    out = {}
    for c in snap["cases"]:
        key = (c["system"], c["tape_format"], c["tape_speed"])
        if (key[0] in ("PAL", "NTSC") and key[1] in ("VHS", "SVHS")
                and key[2] in ("sp", "lp", "ep")):
            out["/".join(key)] = {"sys": {k: c["sysparams"].get(k) for k in SYS_KEYS + SYS_KEYS_SUB},
                                  "rf": {k: c["rfparams"].get(k) for k in RF_KEYS}}
    import hashlib
    import struct
    tables = {}
    for rate in (40000000, 17734475):
        txt = open(os.path.join(REF, "src/VHSDecode.Core/Formats/custom",
                                "svhs-sp-linear-subdeemphasis-%d.txt" % rate)).read()
        vals = [complex(x.strip()) for x in txt.splitlines() if x.strip()]
        blob = b"".join(struct.pack("<dd", v.real, v.imag) for v in vals)
        tables["svhs-sp-linear-subdeemphasis-%d" % rate] = hashlib.sha256(blob).hexdigest()
    out["custom_luma_tables_sha256"] = tables
    with open(os.path.join(HERE, "format_params.json"), "w") as f:
        json.dump(out, f, indent=1, sort_keys=True)

    sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
    from oracle import tbc  # noqa: E402  (positions only; pure numpy)
    lut = np.load(os.path.join(REF, "src/VHSDecode.Core/Tbc/Resources/sinc_lut.npz"))
    lut = lut["downscale_sinc_lut"]
    rows = set()
    cases = []
    for name, n, locs, fl, lc, outlen, digest in HASH_CASES:
        nominal = max(1.0, float(np.median(np.diff(locs))))
        pos = tbc.linear_positions(locs, fl, lc, outlen, nominal)
        rows |= lut_rows_for(pos)
        cases.append({"name": name, "source_length": n, "locations": locs, "first_line": fl,
                      "line_count": lc, "outlen": outlen, "sha256": digest})
    rows = sorted(rows)
    with open(os.path.join(HERE, "sinc_lut_rows.json"), "w") as f:
        json.dump({"rows": rows,
                   "values_hex": [lut[r].astype("<f4").tobytes().hex() for r in rows],
                   "cases": cases}, f, indent=1)


if __name__ == "__main__":
    main()
