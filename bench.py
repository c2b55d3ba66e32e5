"""Benchmark: RF MSPS of the VHS demod + TBC path on one GB300.

Workload (default): synthetic NTSC VHS SP RF, 60 fields (~41M int16 samples
at 40 MSPS, 200 seeded 2-40 us carrier dropouts at 5 %, 38 dB SNR) -- the
configuration the headline metric is quoted on.  A step decodes the whole
capture as the reference's default decode does: block demodulation, sync
pulses, host field control plane, hsync refinement, sinc TBC to 4fSC uint16,
dropout detection, and colour-under chroma (block band-pass, burst probes and
burst refinement of the lines, chroma TBC, up-conversion, comb and gain to
uint16).  --luma-only times the --skip_chroma decode instead.

value  = RF samples / s with the capture already in HBM (device-resident);
e2e    = the same through the C ABI with host buffers: pinned host int16 in,
         uint16 luma (and chroma) of every field back to pinned host memory,
         per step;
roofline = the fused block demodulator against the measured HBM copy peak;
cpu_baseline = the CPU oracle restatement on the host cores.
Inputs and intermediate streams (>400 MB) are larger than L2, so no flush
is needed between steps.
"""
import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "vhs-decode-dotnet_gb300")
for _p in (ROOT, PKG):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "RF MSPS demod+TBC on 1 GB300"
WORKLOADS = {
    "ntsc60": ("NTSC VHS SP, 60 fields, 40 MSPS int16, 200 dropouts, 38 dB SNR", "NTSC", "VHS"),
    "pal4": ("PAL VHS SP, 4 fields, 40 MSPS int16, 40 dB SNR", "PAL", "VHS"),
    "svhs100": ("PAL S-VHS SP, 100 fields, 40 MSPS int16, 42 dB SNR, +/-0.5 % wobble at 15 Hz, "
                "+/-2-sample head-switch jumps per field (sub-deemphasis on)", "PAL", "SVHS"),
}
BLOCK, STRIDE = 32768, 30720
# every workload is captured at 40 MSPS
CAPTURE_RATE = 40e6
# seconds of timed CPU work in `--impl reference` (its steps decode a leading
# sample of the capture sized to fit)
REFERENCE_BUDGET_S = 100.0
# algorithmic bytes of the fused demodulator per 32768-sample block:
# int16 block in (65536 B) + video, sync, envelope float32 kept samples out (3 x 30720 x 4 B)
DEMOD_BYTES_PER_BLOCK = BLOCK * 2 + 3 * STRIDE * 4


def workload(name):
    from vhsd_gb300 import synth
    cache = os.path.join("/tmp", "vhsd_workload_%s.npy" % name)
    if os.path.exists(cache):
        return np.load(cache)
    rf, _ = synth.generate(synth.config(name))
    try:
        np.save(cache, rf)
    except OSError:
        pass
    return rf


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return d.get("hbm_gbs", 6800.0), "measured"
    return 6800.0, "fallback"


def profile_traffic_per_block(workload="ntsc60"):
    """DRAM bytes per block of the fused demodulator from the committed ncu summary."""
    p = os.path.join(ROOT, "profiles", "demod_fp32_%s.md" % workload)
    if not os.path.exists(p):
        return None
    for line in open(p):
        if line.strip().startswith("dram_bytes_per_block:"):
            try:
                return float(line.split(":", 1)[1].split()[0])
            except ValueError:
                return None
    return None


class ClockSampler:
    """nvidia-smi in loop mode (every 20 ms) from start() to stop(); the
    samples that arrive inside the windows between mark() pairs are the ones
    reported (the timed regions)."""

    FIELDS = ("clocks.sm,clocks.max.sm,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, device=0):
        self.samples = []          # (arrival time, fields)
        self.windows = []
        self._proc = None
        self._t = None
        self._open = None
        self.gpu_id = self.device_pci_id(device)

    @staticmethod
    def device_pci_id(device):
        """The PCI bus id of the bench's CUDA device (nvidia-smi numbers GPUs physically and
        ignores CUDA_VISIBLE_DEVICES, so a plain index could name another user's GPU)."""
        try:
            import torch
            p = torch.cuda.get_device_properties(device)
            return "%08X:%02X:%02X.0" % (p.pci_domain_id, p.pci_bus_id, p.pci_device_id)
        except Exception:
            vis = os.environ.get("CUDA_VISIBLE_DEVICES", "").split(",")
            return vis[device].strip() if device < len(vis) and vis[device].strip() else str(device)

    def start(self):
        try:
            self._proc = subprocess.Popen(
                ["nvidia-smi", "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                 "-i", self.gpu_id, "-lms", "20"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True, bufsize=1)
        except Exception:
            self._proc = None
            return

        def run():
            for line in self._proc.stdout:
                self.samples.append((time.monotonic(), [x.strip() for x in line.split(",")]))
        self._t = threading.Thread(target=run, daemon=True)
        self._t.start()

    def wait_first(self, timeout=3.0):
        """Blocks until the sampler has produced a line (or timeout)."""
        t0 = time.monotonic()
        while self._proc is not None and not self.samples and time.monotonic() - t0 < timeout:
            time.sleep(0.01)

    def mark(self):
        """Opens, then closes, a timed window."""
        now = time.monotonic()
        if self._open is None:
            self._open = now
        else:
            self.windows.append((self._open, now))
            self._open = None

    def stop(self):
        if self._proc is not None:
            time.sleep(0.05)
            self._proc.terminate()
            try:
                self._proc.wait(timeout=5)
            except Exception:
                self._proc.kill()
        if self._t:
            self._t.join(timeout=5)
        inside = [f for (t, f) in self.samples if any(a <= t <= b for a, b in self.windows)]
        if not inside and self.windows:   # windows shorter than the sampling period: the next sample
            after = [f for (t, f) in self.samples if t >= self.windows[0][0]]
            inside = after[:1]
        sm = [float(s[0]) for s in inside if s and s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in inside if len(s) > 1 and s[1].replace(".", "").isdigit()]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for s in inside:
            for name, v in zip(names, s[2:6]):
                if v.strip().lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": sorted(reasons),
                "samples": len(inside), "period_ms": 20, "gpu": self.gpu_id}


def dist_init(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if args.impl == "ours" else "gloo")
    return world, rank, local


def max_over_ranks(x, world, device=None):
    if world <= 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def make_pool(procs):
    import multiprocessing as mp
    return mp.get_context("spawn").Pool(procs)


def cpu_oracle_msps(rf, system, procs, pool=None, tape="VHS", chroma=True):
    """Oracle decode of the capture: block demod (and the chroma block band-pass)
    over a spawn pool, field path (with the chroma field decode) sequential."""
    from oracle import demod, field, formats
    fmt = formats.get(system, tape)
    nblocks = demod.block_count(len(rf))
    own = pool is None
    if own:
        pool = make_pool(procs)
    t0 = time.perf_counter()
    chunks = np.array_split(np.arange(nblocks), procs * 4)
    try:
        parts = pool.map(_oracle_demod_part,
                         [(rf[int(c[0]) * STRIDE: (int(c[-1]) * STRIDE + BLOCK)], system, tape, len(c), chroma)
                          for c in chunks if len(c)])
    finally:
        if own:
            pool.close()
    video = np.concatenate([p[0] for p in parts])
    vlp = np.concatenate([p[1] for p in parts])
    env = np.concatenate([p[2] for p in parts])
    cch = np.concatenate([p[3] for p in parts]) if chroma else None
    fields, _ = field.decode_capture(rf, fmt, channels=(video, vlp, env, False), with_chroma=chroma,
                                     chroma_channel=cch)
    dt = time.perf_counter() - t0
    return len(rf) / dt / 1e6, dt, len([f for f in fields if "error" not in f])


_FILTERS = {}


def _oracle_demod_part(args):
    rf, system, tape, nb, chroma = args
    from oracle import chroma as ochroma, demod, formats
    from oracle.filters import FilterSet
    fmt = formats.get(system, tape)
    if (system, tape) not in _FILTERS:
        _FILTERS[(system, tape)] = (FilterSet(fmt, 40e6), ochroma.ChromaParams(fmt, 40e6))
    filt, cp = _FILTERS[(system, tape)]
    dmax = (fmt["sys"]["ire0"] + fmt["sys"]["hz_ire"] * 100.0) * 2.0
    v, l, e, _ = demod.demod_stream(rf, filt, 40e6, dmax, 0, nb)
    c = ochroma.chroma_stream(rf, cp, 0, nb) if chroma else None
    return v, l, e, c


def run_reference(args, world, rank):
    if rank != 0:
        return
    rf = workload(args.workload)
    desc, system, tape = WORKLOADS[args.workload]
    procs = os.cpu_count() or 1
    pool = make_pool(procs)
    chroma = not args.luma_only
    head = rf[: 4 * 1048576]
    rates = []
    for _ in range(max(1, args.warmup)):
        rates.append(cpu_oracle_msps(head, system, procs, pool, tape, chroma)[0])
    # each step decodes a leading sample of the capture sized so the timed
    # steps take about REFERENCE_BUDGET_S in all (the whole capture when it fits)
    per_step = REFERENCE_BUDGET_S / max(1, args.steps)
    n_step = int(min(len(rf), max(len(head), max(rates) * 1e6 * per_step)))
    sample = rf[:n_step]
    times = []
    for _ in range(args.steps):
        msps, dt, nf = cpu_oracle_msps(sample, system, procs, pool, tape, chroma)
        times.append(dt)
    pool.close()
    avg = sum(times) / len(times)
    value = len(sample) / avg / 1e6
    line = {"metric": METRIC, "value": round(value, 3), "unit": "MSPS", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(avg * 1e3, 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "impl": "reference",
            "config": {"workload": args.workload, "description": desc, "samples": int(len(rf))},
            "cpu_baseline": {"value": round(value, 3), "unit": "MSPS", "cores": procs, "kind": "port",
                             "sample": "the first %d samples (%.1f s) of the workload capture per step "
                                       "(oracle restatement: numpy FFT block demod%s over a spawn pool + "
                                       "sequential field path)"
                                       % (len(sample), len(sample) / CAPTURE_RATE,
                                          " and chroma band-pass" if chroma else "")},
            "e2e": {"value": round(value, 3), "unit": "MSPS", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def run_ours(args, world, rank, local):
    import torch
    from vhsd_gb300 import native
    torch.cuda.set_device(local)
    desc, system, tape = WORKLOADS[args.workload]
    prof = native.PROFILE_PAL if system == "PAL" else native.PROFILE_NTSC
    tfmt = native.FORMAT_SVHS if tape == "SVHS" else native.FORMAT_VHS
    rf = workload(args.workload)
    n = len(rf)
    sess = native.Session(prof, n, precision=native.PRECISION_FP32_FUSED, device=local, tape_format=tfmt)
    stream = torch.cuda.current_stream()
    sess.set_stream(stream.cuda_stream)
    d_rf = torch.from_numpy(rf).to("cuda")
    clocks = ClockSampler(local)
    clocks.start()
    # device-resident value: the reference's default decode (luma and
    # colour-under chroma) unless --luma-only
    chroma = not args.luma_only
    for _ in range(max(3, args.warmup)):
        sess.decode(None, device_ptr=d_rf.data_ptr(), count=n, chroma=chroma)
    torch.cuda.synchronize()
    clocks.wait_first()
    barrier(world)
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    demod_ms = []
    fields = 0
    launches = 0
    clocks.mark()
    e0.record(stream)
    for _ in range(args.steps):
        r = sess.decode(None, device_ptr=d_rf.data_ptr(), count=n, chroma=chroma)
        demod_ms.append(r.demod_ms)
        fields = r.fields
        launches += r.kernel_launches
    e1.record(stream)
    torch.cuda.synchronize()
    clocks.mark()
    barrier(world)
    ms = e0.elapsed_time(e1) / args.steps
    ms = max_over_ranks(ms, world, "cuda")
    nblocks = int(r.blocks)
    value = world * n / (ms / 1e3) / 1e6
    stage = r
    # the same decode without chroma (the reference's --skip_chroma decode)
    other = None
    if chroma:
        for _ in range(2):
            sess.decode(None, device_ptr=d_rf.data_ptr(), count=n)
        torch.cuda.synchronize()
        g0 = torch.cuda.Event(enable_timing=True)
        g1 = torch.cuda.Event(enable_timing=True)
        g0.record(stream)
        for _ in range(args.steps):
            sess.decode(None, device_ptr=d_rf.data_ptr(), count=n)
        g1.record(stream)
        torch.cuda.synchronize()
        lms = max_over_ranks(g0.elapsed_time(g1) / args.steps, world, "cuda")
        other = {"value": round(world * n / (lms / 1e3) / 1e6, 3), "unit": "MSPS", "ms_per_step": round(lms, 3),
                 "decode": "luma only (the reference's --skip_chroma decode: no chroma, no burst refinement)"}
    # e2e through the C ABI: pinned host in, TBC out
    h_rf = torch.from_numpy(rf).pin_memory()
    tbc_elems = fields * r.output_field_lines * r.output_line_length
    h_tbc = torch.empty(max(1, tbc_elems), dtype=torch.int16).pin_memory()
    h_chroma = torch.empty(max(1, tbc_elems), dtype=torch.int16).pin_memory()

    def e2e_step():
        sess.decode(h_rf.numpy(), chroma=chroma)
        sess.tbc_into(0, fields, h_tbc.data_ptr())
        if chroma:
            sess.chroma_into(0, fields, h_chroma.data_ptr())

    for _ in range(2):
        e2e_step()
    torch.cuda.synchronize()
    barrier(world)
    f0 = torch.cuda.Event(enable_timing=True)
    f1 = torch.cuda.Event(enable_timing=True)
    clocks.mark()
    f0.record(stream)
    for _ in range(args.steps):
        e2e_step()
    f1.record(stream)
    torch.cuda.synchronize()
    clocks.mark()
    clk = clocks.stop()
    e2e_ms = max_over_ranks(f0.elapsed_time(f1) / args.steps, world, "cuda")
    e2e_value = world * n / (e2e_ms / 1e3) / 1e6
    peak, peak_kind = peaks()
    avg_demod = sum(demod_ms) / len(demod_ms)
    # the same blocks as one fused-demod launch (a demod-only decode): the
    # kernel's own rate, beside the pipelined segments' average above
    single = []
    for _ in range(5):
        rs = sess.decode(None, device_ptr=d_rf.data_ptr(), count=n, demod_only=True)
        single.append(rs.demod_ms)
    single_ms = statistics.median(single[1:])
    single_achieved = DEMOD_BYTES_PER_BLOCK * nblocks / (single_ms / 1e3) / 1e9
    achieved = DEMOD_BYTES_PER_BLOCK * nblocks / (avg_demod / 1e3) / 1e9
    tpb = profile_traffic_per_block(args.workload)
    # plain FP64 baseline (one block at a time) on the same capture, one step
    plain = None
    if not args.skip_plain:
        ps = native.Session(prof, n, precision=native.PRECISION_FP64_PLAIN, device=local, tape_format=tfmt)
        ps.set_stream(stream.cuda_stream)
        ps.decode(None, device_ptr=d_rf.data_ptr(), count=n, chroma=chroma)
        torch.cuda.synchronize()
        p0 = torch.cuda.Event(enable_timing=True)
        p1 = torch.cuda.Event(enable_timing=True)
        p0.record(stream)
        ps.decode(None, device_ptr=d_rf.data_ptr(), count=n, chroma=chroma)
        p1.record(stream)
        torch.cuda.synchronize()
        pms = p0.elapsed_time(p1)
        plain = {"value": round(n / (pms / 1e3) / 1e6, 3), "unit": "MSPS",
                 "ms_per_step": round(pms, 3), "ratio_fp32_over_plain": round(value / world / (n / (pms / 1e3) / 1e6), 2)}
        ps.close()
    decimated = None
    if rank == 0 and world == 1 and not args.skip_decimated:
        decimated = run_decimated(args, local, rf, prof, tfmt, stream)
    cpu = None
    if rank == 0 and world == 1 and not args.skip_cpu:
        procs = os.cpu_count() or 1
        pool = make_pool(procs)
        cpu_oracle_msps(rf[: 4 * 1048576], system, procs, pool, tape, chroma)
        msps, dt, nf = cpu_oracle_msps(rf, system, procs, pool, tape, chroma)
        pool.close()
        cpu = {"value": round(msps, 3), "unit": "MSPS", "cores": procs, "kind": "port",
               "sample": "whole workload capture (%d samples, %.1f s): oracle restatement, block "
                         "demod%s over %d spawn processes + sequential field path"
                         % (n, dt, " and chroma band-pass" if chroma else "", procs)}
    serving = None
    if rank == 0 and world == 1 and not args.skip_serve:
        serving = run_serving(args, local)
    flac_leg = None
    if rank == 0 and world == 1 and not args.skip_flac:
        flac_leg = run_flac(rf)
    if rank == 0:
        decode = ("luma and colour-under chroma (the reference's default decode: burst-refined lines, "
                  "uint16 luma and chroma fields)" if chroma else "luma only (--skip_chroma)")
        line = {"metric": METRIC, "value": round(value, 3), "unit": "MSPS", "n_gpus": world,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms, 3),
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
                "data": "synthetic",
                "config": {"workload": args.workload, "description": desc, "samples": int(n),
                           "blocks": nblocks, "fields": int(fields),
                           "precision": "fp32 fused demod, fp64 sync/TBC",
                           "decode": decode,
                           "fft_plan": int(r.fft_plan),
                           "l2": "inputs and streams larger than L2 (no flush)",
                           "parallelism": "replicas" if world > 1 else "single"},
                "e2e": {"value": round(e2e_value, 3), "unit": "MSPS",
                        "h2d_bytes_per_step": int(n * 2),
                        "d2h_bytes_per_step": int(tbc_elems * 2 * (2 if chroma else 1))},
                "roofline": {"bound": "hbm", "achieved": round(single_achieved, 1), "peak": peak,
                             "unit": "GB/s", "frac": round(single_achieved / peak, 4),
                             "traffic": (round(tpb * nblocks) if tpb else None),
                             "kernel": "vhsd_demod_fp32_kernel", "peak_kind": peak_kind,
                             "kernel_ms": round(single_ms, 4),
                             "algorithmic_bytes": int(DEMOD_BYTES_PER_BLOCK * nblocks),
                             "launch": "all blocks of the workload in one persistent launch "
                                       "(CUDA events on the launching stream, median of 4)",
                             "pipelined_segments": {
                                 "kernel_ms_sum": round(avg_demod, 4),
                                 "achieved": round(achieved, 1),
                                 "note": "the decode's segment launches overlap on two streams; "
                                         "their summed durations exceed the step's wall time, so "
                                         "this is not a per-launch rate"}},
                "cpu_baseline": cpu,
                "luma_only": other,
                "plain_fp64": plain,
                "decimated": decimated,
                "serving": serving,
                "flac_decode": flac_leg,
                "gpu_launches": int(launches),
                "clocks": clk,
                "stage_ms": {"demod": round(avg_demod, 4), "field_kernels_and_host": round(stage.field_ms, 4),
                             "host_control": round(stage.host_ms, 4)}}
        print(json.dumps(line))
    sess.close()


# Serving mix of 2-s windows (share, profile, tape format, MSPS, label).  The
# NTSC LaserDisc share is decoded as NTSC VHS windows of the same sample rate
# and length (the LaserDisc demod branch is not built), so the offered sample
# load is the mix's own: 200 windows/s x 68 M samples = 13.6 GSPS.
SERVE_MIX = [(0.40, "PAL", "VHS", 40.0, "pal_vhs_40"), (0.30, "NTSC", "VHS", 20.0, "ntsc_vhs_20"),
             (0.15, "PAL", "SVHS", 40.0, "pal_svhs_40"),
             (0.15, "NTSC", "VHS", 40.0, "ntsc_ld_40 as ntsc_vhs_40")]
SERVE_TILE_FIELDS = 8


def serve_source(system, tape, mhz, seconds):
    """Seeded synthetic capture of `seconds`, built by repeating an 8-field
    synthetic recording (the joins are FM phase jumps, decoded like head
    switches).  Cached in /tmp."""
    from vhsd_gb300 import synth
    cache = os.path.join("/tmp", "vhsd_serve_%s_%s_%d_%d.npy" % (system, tape, int(mhz), SERVE_TILE_FIELDS))
    if os.path.exists(cache):
        tile = np.load(cache)
    else:
        name = "svhs_small" if tape == "SVHS" else ("pal4" if system == "PAL" else "ntsc_small")
        cfg = synth.config(name, fields=SERVE_TILE_FIELDS, fs=mhz * 1e6,
                           seed=(33 if tape == "SVHS" else 31) if system == "PAL" else 32)
        tile, _ = synth.generate(cfg)
        try:
            np.save(cache, tile)
        except OSError:
            pass
    n = int(seconds * mhz * 1e6)
    return np.resize(tile, n)


def run_serving(args, local):
    """Poisson arrivals of 2-s windows over 32 client streams into the window
    server; returns latency percentiles and aggregate RF MSPS."""
    import torch
    from vhsd_gb300 import native
    rng = np.random.default_rng(2024)
    win_s, rate, nstreams, dur = 2.0, float(args.serve_rate), 32, float(args.serve_seconds)
    src_s = 6.0
    sources = {}
    for share, system, tape, mhz, label in SERVE_MIX:
        key = (system, tape, mhz)
        if key not in sources:
            host = serve_source(system, tape, mhz, src_s)
            sources[key] = torch.from_numpy(host).pin_memory().numpy()
    # streams: formats by the mix shares
    counts = [int(round(m[0] * nstreams)) for m in SERVE_MIX]
    counts[0] += nstreams - sum(counts)
    streams = []
    for (share, system, tape, mhz, label), c in zip(SERVE_MIX, counts):
        for _ in range(c):
            streams.append({"system": system, "tape": tape, "mhz": mhz, "label": label, "offset": None,
                            "left": 0})
    max_win = int(win_s * 40e6)
    prof = {"PAL": native.PROFILE_PAL, "NTSC": native.PROFILE_NTSC}
    tfmt = {"VHS": native.FORMAT_VHS, "SVHS": native.FORMAT_SVHS}
    per_field = {"PAL": 313 * 1135, "NTSC": 263 * 910}
    outs = {sysn: [torch.empty(130 * per_field[sysn], dtype=torch.int16).pin_memory().numpy().view(np.uint16)
                   for _ in range(8)] for sysn in ("PAL", "NTSC")}
    sv = native.Server(max_win, workers=args.serve_workers, device=local, max_batch=args.serve_batch)

    def window(st):
        src = sources[(st["system"], st["tape"], st["mhz"])]
        n = int(win_s * st["mhz"] * 1e6)
        seek = st["offset"] is None or st["left"] <= 0 or st["offset"] + 2 * n > len(src)
        if seek:
            st["offset"] = int(rng.integers(0, len(src) - n))
            st["left"] = int(rng.integers(1, 11))   # windows until the next seek
        else:
            st["offset"] += n - int(0.12 * st["mhz"] * 1e6)   # 0.12 s preroll overlap
        st["left"] -= 1
        return src[st["offset"]:st["offset"] + n], st["offset"], seek

    # warm-up: `workers` windows of every format at once, so each worker has a
    # slot of each format before the timed arrivals start
    warm = []
    for key in sources:
        st0 = next(x for x in streams if (x["system"], x["tape"], x["mhz"]) == key)
        for i in range(args.serve_workers):
            x, off, seek = window(dict(st0))
            warm.append(sv.submit(1000 + len(warm), prof[st0["system"]], x, off, seek=True,
                                  sample_rate_mhz=st0["mhz"], tbc_out=outs[st0["system"]][i % 8],
                                  tape_format=tfmt[st0["tape"]]))
    for t in warm:
        sv.wait(t)
    # arrivals
    arrivals = np.cumsum(rng.exponential(1.0 / rate, size=int(rate * dur * 1.5) + 10))
    arrivals = arrivals[arrivals < dur]
    tickets = []
    t0 = time.perf_counter()
    samples = 0
    for k, ta in enumerate(arrivals):
        now = time.perf_counter() - t0
        if ta > now:
            time.sleep(ta - now)
        si = int(rng.integers(0, nstreams))
        st = streams[si]
        x, off, seek = window(st)
        samples += len(x)
        tickets.append(sv.submit(si, prof[st["system"]], x, off, seek=seek, sample_rate_mhz=st["mhz"],
                                 tbc_out=outs[st["system"]][k % 8], tape_format=tfmt[st["tape"]]))
    res = [sv.wait(t) for t in tickets]
    t_end = time.perf_counter() - t0
    # capacity: the same mix closed-loop, two windows per worker always in
    # flight, for a few seconds; headroom = capacity / offered load - 1
    inflight = []
    cap_samples = 0
    t1 = time.perf_counter()
    k = 0
    while time.perf_counter() - t1 < args.serve_capacity_seconds or inflight:
        while len(inflight) < 2 * args.serve_workers and time.perf_counter() - t1 < args.serve_capacity_seconds:
            si = int(rng.integers(0, nstreams))
            st = streams[si]
            x, off, seek = window(st)
            cap_samples += len(x)
            inflight.append(sv.submit(si, prof[st["system"]], x, off, seek=seek, sample_rate_mhz=st["mhz"],
                                      tbc_out=outs[st["system"]][k % 8], tape_format=tfmt[st["tape"]]))
            k += 1
        sv.wait(inflight.pop(0))
    cap_s = time.perf_counter() - t1
    sv.close()
    capacity = cap_samples / cap_s / 1e6
    offered = samples / dur / 1e6
    lat = np.array([r.latency_ms for r in res])
    ok = sum(1 for r in res if r.status == 0)
    return {"windows": len(res), "ok": ok, "offered_windows_per_s": rate, "streams": nstreams,
            "window_s": win_s, "workers": args.serve_workers, "max_batch": args.serve_batch,
            "mean_batch": round(float(np.mean([r.batched for r in res])), 2), "seconds": round(t_end, 3),
            "capacity_msps": round(capacity, 1), "headroom": round(capacity / offered - 1.0, 3),
            "p50_ms": round(float(np.percentile(lat, 50)), 2), "p99_ms": round(float(np.percentile(lat, 99)), 2),
            "mean_queue_ms": round(float(np.mean([r.queue_ms for r in res])), 2),
            "msps": round(samples / t_end / 1e6, 1),
            "offered_msps": round(offered, 1),
            "fields": int(sum(r.fields for r in res)),
            "mix": [m[4] for m in SERVE_MIX],
            "data": "synthetic, 8-field recordings repeated to 6 s per format; TBC copied to pinned host"}


def run_flac(rf):
    """Device FLAC decoding of the workload written as a 16-bit mono FLAC stream
    (vhsd_gb300.ldf writer, 4096-sample frames; cached in /tmp): samples per
    second through vhsdecode_gb300_flac_decode, host bytes in, host samples
    out (the copies inside the timed calls)."""
    from vhsd_gb300 import native
    cache = os.path.join("/tmp", "vhsd_workload_flac_%d.bin" % len(rf))
    if os.path.exists(cache):
        data = open(cache, "rb").read()
    else:
        from vhsd_gb300 import ldf   # the writer makes the input; it is not timed
        data = ldf.write(rf, seed=60)
        try:
            open(cache, "wb").write(data)
        except OSError:
            pass
    got = native.flac_decode(data)   # warm-up, and a check that it is lossless
    if not np.array_equal(got, rf):
        raise RuntimeError("FLAC decode differs from the capture")
    times = []
    for _ in range(3):
        t0 = time.perf_counter()
        native.flac_decode(data)
        times.append(time.perf_counter() - t0)
    t = min(times)
    return {"value": round(len(rf) / t / 1e6, 1), "unit": "MSPS", "ms": round(t * 1e3, 2),
            "compressed_bytes": len(data), "frames": (len(rf) + 4095) // 4096,
            "note": "host FLAC bytes in, host int16 out, best of 3; bit-exact to the capture"}


def run_decimated(args, local, rf, prof, tfmt, stream):
    """The same capture decoded at half its rate through the device 2:1
    decimator (the reference's --decode-at-20msps / preview mode): whole
    decodes from device-resident int16, source samples per second."""
    import torch
    from vhsd_gb300 import native
    n = len(rf)
    ds = native.Session(prof, n, device=local, tape_format=tfmt, sample_rate_mhz=20.0, decimation=2)
    ds.set_stream(stream.cuda_stream)
    d_rf = torch.from_numpy(rf).to("cuda")
    for _ in range(3):
        ds.decode(None, device_ptr=d_rf.data_ptr(), count=n)
    torch.cuda.synchronize()
    q0 = torch.cuda.Event(enable_timing=True)
    q1 = torch.cuda.Event(enable_timing=True)
    steps = max(1, args.steps)
    q0.record(stream)
    for _ in range(steps):
        r = ds.decode(None, device_ptr=d_rf.data_ptr(), count=n)
    q1.record(stream)
    torch.cuda.synchronize()
    ms = q0.elapsed_time(q1) / steps
    ds.close()
    return {"value": round(n / (ms / 1e3) / 1e6, 3), "unit": "MSPS (source samples)",
            "ms_per_step": round(ms, 3), "decode_rate_mhz": 20.0, "fields": int(r.fields),
            "kernel_launches": int(r.kernel_launches)}


def run_profile_demod(args, local):
    """Demod-only decodes of the workload (one fused demodulator launch each),
    for kernel captures: warm-up, then --steps decodes; prints the kernel times.
    With --decimate the workload is tiled 3x (larger than L2) and decoded at half
    its rate through the device decimator."""
    import torch
    from vhsd_gb300 import native
    desc, system, tape = WORKLOADS[args.workload]
    prof = native.PROFILE_PAL if system == "PAL" else native.PROFILE_NTSC
    rf = workload(args.workload)
    extra = {}
    if args.decimate:
        rf = np.tile(rf, 3)
        extra = {"sample_rate_mhz": 20.0, "decimation": 2}
    sess = native.Session(prof, len(rf), device=local,
                          tape_format=native.FORMAT_SVHS if tape == "SVHS" else native.FORMAT_VHS, **extra)
    d_rf = torch.from_numpy(rf).to("cuda")
    for _ in range(args.warmup):
        sess.decode(None, device_ptr=d_rf.data_ptr(), count=len(rf), demod_only=True)
    ms = []
    for _ in range(args.steps):
        r = sess.decode(None, device_ptr=d_rf.data_ptr(), count=len(rf), demod_only=True)
        ms.append(r.demod_ms)
    torch.cuda.synchronize()
    print(json.dumps({"workload": args.workload, "blocks": int(r.blocks), "demod_ms": ms}))
    sess.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="ntsc60", choices=sorted(WORKLOADS))
    ap.add_argument("--skip-cpu", action="store_true")
    ap.add_argument("--skip-plain", action="store_true")
    ap.add_argument("--skip-serve", action="store_true")
    ap.add_argument("--serve-rate", type=float, default=200.0, help="window arrivals per second")
    ap.add_argument("--serve-seconds", type=float, default=20.0)
    ap.add_argument("--serve-capacity-seconds", type=float, default=4.0)
    ap.add_argument("--serve-batch", type=int, default=1,
                    help="windows a free worker demodulates in one launch (1: no batching)")
    ap.add_argument("--skip-flac", action="store_true")
    ap.add_argument("--luma-only", action="store_true",
                    help="decode without chroma (the reference's --skip_chroma); default: luma and chroma")
    ap.add_argument("--serve-workers", type=int, default=4)
    ap.add_argument("--skip-decimated", action="store_true")
    ap.add_argument("--profile-demod", action="store_true",
                    help="only demod-only decodes of the workload (for kernel captures)")
    ap.add_argument("--decimate", action="store_true",
                    help="with --profile-demod: the workload tiled 3x through the 2:1 decimator")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    world, rank, local = dist_init(args)
    if args.profile_demod:
        run_profile_demod(args, local)
    elif args.impl == "reference":
        run_reference(args, world, rank)
    else:
        run_ours(args, world, rank, local)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
