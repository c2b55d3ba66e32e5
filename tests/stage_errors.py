"""Per-stage error of the GPU decode paths against the CPU oracle (FP64).

Run on a GPU machine:  python tests/stage_errors.py [workload ...]
(workloads: pal4, ntsc60, svhs20; default all three).  Prints one markdown
table row per workload and path: the stream channels' absolute errors (video
and sync reference in Hz, envelope relative), the largest line-location
difference, the share of TBC samples identical / within 1 LSB and the largest
difference, and whether field count, first-field flags and dropouts match.
Not collected by pytest (the parity tests assert the tolerances; this reports
the measured errors).
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "vhs-decode-dotnet_gb300")):
    if p not in sys.path:
        sys.path.insert(0, p)

WORKLOADS = {
    "pal4": ("PAL", "VHS", "pal4"),
    "ntsc60": ("NTSC", "VHS", "ntsc60"),
    "svhs20": ("PAL", "SVHS", "svhs_small"),
}


def capture(name):
    from vhsd_gb300 import synth
    _, _, cfg = WORKLOADS[name]
    if name == "svhs20":
        rf, _ = synth.generate(synth.config(cfg, fields=20))
    else:
        import bench
        rf = bench.workload(cfg)
    return rf


def report(name):
    from vhsd_gb300 import native
    from oracle import field, formats
    system, tape, _ = WORKLOADS[name]
    rf = capture(name)
    fields, (video, vlp, env, _) = field.decode_capture(rf, formats.get(system, tape))
    good = [f for f in fields if "error" not in f]
    prof = native.PROFILE_PAL if system == "PAL" else native.PROFILE_NTSC
    tfmt = native.FORMAT_SVHS if tape == "SVHS" else native.FORMAT_VHS
    rows = []
    for prec, label in ((native.PRECISION_FP32_FUSED, "FP32 fused"), (native.PRECISION_FP64_PLAIN, "FP64 plain")):
        with native.Session(prof, len(rf), precision=prec, tape_format=tfmt) as s:
            s.decode(rf, demod_only=True)
            n = len(video)
            dv = np.abs(s.stream(0, 0, n) - video)
            dy = np.abs(s.stream(1, 0, n) - vlp)
            de = np.abs(s.stream(2, 0, n) - env) / np.maximum(np.abs(env), 1.0)
            r = s.decode(rf)
            tb = s.tbc()
            dl, same, within, dmax, parity, drops = 0.0, 0, 0, 0, True, True
            total = 0
            for i, f in enumerate(good[: r.fields]):
                dl = max(dl, float(np.max(np.abs(s.lines(i) - f["locs"]))))
                d = np.abs(tb[i].astype(np.int64).ravel() - f["tbc"].astype(np.int64))
                same += int(np.sum(d == 0))
                within += int(np.sum(d <= 1))
                dmax = max(dmax, int(d.max()))
                total += d.size
                parity &= bool(s.field(i).is_first_field) == f["first_field"]
                drops &= s.dropouts(i) == [tuple(x) for x in f["dropouts"]]
        rows.append("| %s | %s | %d / %d | %.2f / %.1f | %.2f / %.1f | %.1e | %.1e | %.5f %% | %.5f %% | %d | %s |" % (
            name, label, r.fields, len(good),
            float(np.quantile(dv, 0.999)), float(dv.max()),
            float(np.quantile(dy, 0.999)), float(dy.max()),
            float(np.quantile(de, 0.999)), dl,
            100.0 * same / max(total, 1), 100.0 * within / max(total, 1), dmax,
            "yes" if (parity and drops and r.fields == len(good)) else "NO"))
    return rows


def main():
    names = sys.argv[1:] or list(WORKLOADS)
    print("| workload | path | fields (GPU / oracle) | video err Hz p99.9 / max | sync err Hz p99.9 / max "
          "| envelope rel. err p99.9 | line loc. max diff (samples) | TBC identical | TBC within 1 LSB "
          "| TBC max diff (LSB) | parity, dropouts, counts identical |")
    print("|---|---|---|---|---|---|---|---|---|---|---|")
    for n in names:
        for row in report(n):
            print(row, flush=True)


if __name__ == "__main__":
    main()
