"""Regenerate the binary filter tables in this folder from the reference checkout.

The S-VHS formats multiply the video filter by a measured luma response
(``video_custom_luma_filters`` entry ``{"type": "file", "filename":
"svhs-sp-linear-subdeemphasis"}`` of the PAL/NTSC SVHS cases of
src/VHSDecode.Core/Formats/format-params.snapshot.json).  The reference embeds
it as text resources ``Formats/custom/svhs-sp-linear-subdeemphasis-<rate>.txt``
(one Python complex literal per line, bins 0..16384 of a 32768-point block) and
loads them in ``DecodeFilterSetBuilder.TryLoadCustomFilter``
(src/VHSDecode.Core/Dsp/DecodeFilterSet.cs:1560-1609, 1658-1714).  The table is data with
no generator, so it is carried over value for value: each line is parsed to the
nearest binary64 (as .NET's double.Parse does) and written as little-endian
float64 (re, im) pairs.  The decoder library reads these files at session
creation; nothing reads the reference at run time.

Run with the reference checkout given as the first argument or in the
REFERENCE_ROOT environment variable.
"""
import hashlib
import os
import struct
import sys

REF = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("REFERENCE_ROOT")
if not REF or not os.path.isdir(REF):
    sys.exit("usage: %s REFERENCE_ROOT (or set REFERENCE_ROOT)" % os.path.basename(__file__))
HERE = os.path.dirname(os.path.abspath(__file__))
RATES = (40000000, 17734475)
BINS = 16385


def convert(rate):
    src = os.path.join(REF, "src/VHSDecode.Core/Formats/custom",
                       f"svhs-sp-linear-subdeemphasis-{rate}.txt")
    text = open(src, "rb").read()
    vals = [complex(line.strip()) for line in text.decode("ascii").splitlines() if line.strip()]
    if len(vals) != BINS:
        sys.exit(f"{src}: {len(vals)} bins, expected {BINS}")
    out = os.path.join(HERE, f"svhs-sp-linear-subdeemphasis-{rate}.f64")
    with open(out, "wb") as f:
        for v in vals:
            f.write(struct.pack("<dd", v.real, v.imag))
    print(os.path.basename(out), "source sha256", hashlib.sha256(text).hexdigest(),
          "table sha256", hashlib.sha256(open(out, "rb").read()).hexdigest())


if __name__ == "__main__":
    for r in RATES:
        convert(r)
