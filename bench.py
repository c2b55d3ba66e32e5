"""Benchmark: RF MSPS of the VHS demod + TBC path on one GB300.

Workload (default): synthetic NTSC VHS SP RF, 60 fields (~41M int16 samples
at 40 MSPS, 200 seeded 2-40 us carrier dropouts at 5 %, 38 dB SNR) -- the
configuration the headline metric is quoted on.  A step decodes the whole
capture: block demodulation, sync pulses, host field control plane, hsync
refinement, sinc TBC to 4fSC uint16 and dropout detection.

value  = RF samples / s with the capture already in HBM (device-resident);
e2e    = the same through the C ABI with host buffers: pinned host int16 in,
         uint16 TBC of every field back to pinned host memory, per step;
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
    "ntsc60": ("NTSC VHS SP, 60 fields, 40 MSPS int16, 200 dropouts, 38 dB SNR", "NTSC"),
    "pal4": ("PAL VHS SP, 4 fields, 40 MSPS int16, 40 dB SNR", "PAL"),
}
BLOCK, STRIDE = 32768, 30720
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


def profile_traffic_per_block():
    """DRAM bytes per block of the fused demodulator from the committed ncu summary."""
    p = os.path.join(ROOT, "profiles", "demod_fp32_pal4.md")
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
    def __init__(self):
        self.samples = []
        self._stop = threading.Event()
        self._t = None

    def start(self):
        def run():
            q = ("nvidia-smi --query-gpu=clocks.sm,clocks.max.sm,clocks_event_reasons.hw_slowdown,"
                 "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
                 "clocks_event_reasons.sw_power_cap --format=csv,noheader,nounits -i 0")
            while not self._stop.is_set():
                try:
                    out = subprocess.run(q, shell=True, capture_output=True, text=True, timeout=5).stdout
                    line = out.strip().splitlines()[0]
                    self.samples.append([x.strip() for x in line.split(",")])
                except Exception:
                    pass
                self._stop.wait(0.2)
        self._t = threading.Thread(target=run, daemon=True)
        self._t.start()

    def stop(self):
        self._stop.set()
        if self._t:
            self._t.join(timeout=10)
        sm = [float(s[0]) for s in self.samples if s and s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if len(s) > 1 and s[1].replace(".", "").isdigit()]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for s in self.samples:
            for name, v in zip(names, s[2:6]):
                if v.strip().lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": sorted(reasons),
                "samples": len(self.samples)}


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


def cpu_oracle_msps(rf, system, procs, pool=None):
    """Oracle decode of the capture: block demod over a spawn pool, field path sequential."""
    from oracle import demod, field, formats
    fmt = formats.get(system)
    nblocks = demod.block_count(len(rf))
    own = pool is None
    if own:
        pool = make_pool(procs)
    t0 = time.perf_counter()
    chunks = np.array_split(np.arange(nblocks), procs * 4)
    try:
        parts = pool.map(_oracle_demod_part,
                         [(rf[int(c[0]) * STRIDE: (int(c[-1]) * STRIDE + BLOCK)], system, len(c))
                          for c in chunks if len(c)])
    finally:
        if own:
            pool.close()
    video = np.concatenate([p[0] for p in parts])
    vlp = np.concatenate([p[1] for p in parts])
    env = np.concatenate([p[2] for p in parts])
    fields, _ = field.decode_capture(rf, fmt, channels=(video, vlp, env, False))
    dt = time.perf_counter() - t0
    return len(rf) / dt / 1e6, dt, len([f for f in fields if "error" not in f])


_FILTERS = {}


def _oracle_demod_part(args):
    rf, system, nb = args
    from oracle import demod, formats
    from oracle.filters import FilterSet
    fmt = formats.get(system)
    if system not in _FILTERS:
        _FILTERS[system] = FilterSet(fmt, 40e6)
    dmax = (fmt["sys"]["ire0"] + fmt["sys"]["hz_ire"] * 100.0) * 2.0
    v, l, e, _ = demod.demod_stream(rf, _FILTERS[system], 40e6, dmax, 0, nb)
    return v, l, e


def run_reference(args, world, rank):
    if rank != 0:
        return
    rf = workload(args.workload)
    desc, system = WORKLOADS[args.workload]
    procs = os.cpu_count() or 1
    pool = make_pool(procs)
    for _ in range(args.warmup):
        cpu_oracle_msps(rf[: 4 * 1048576], system, procs, pool)
    times = []
    for _ in range(args.steps):
        msps, dt, nf = cpu_oracle_msps(rf, system, procs, pool)
        times.append(dt)
    pool.close()
    avg = sum(times) / len(times)
    value = len(rf) / avg / 1e6
    line = {"metric": METRIC, "value": round(value, 3), "unit": "MSPS", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(avg * 1e3, 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "impl": "reference",
            "config": {"workload": args.workload, "description": desc, "samples": int(len(rf))},
            "cpu_baseline": {"value": round(value, 3), "unit": "MSPS", "cores": procs, "kind": "port",
                             "sample": "whole workload capture per step (oracle restatement: "
                                       "numpy FFT block demod over a spawn pool + sequential field path)"},
            "e2e": {"value": round(value, 3), "unit": "MSPS", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def run_ours(args, world, rank, local):
    import torch
    from vhsd_gb300 import native
    torch.cuda.set_device(local)
    desc, system = WORKLOADS[args.workload]
    prof = native.PROFILE_PAL if system == "PAL" else native.PROFILE_NTSC
    rf = workload(args.workload)
    n = len(rf)
    sess = native.Session(prof, n, precision=native.PRECISION_FP32_FUSED, device=local)
    stream = torch.cuda.current_stream()
    sess.set_stream(stream.cuda_stream)
    d_rf = torch.from_numpy(rf).to("cuda")
    # device-resident value
    for _ in range(max(3, args.warmup)):
        sess.decode(None, device_ptr=d_rf.data_ptr(), count=n)
    torch.cuda.synchronize()
    clocks = ClockSampler()
    clocks.start()
    barrier(world)
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    demod_ms = []
    fields = 0
    launches = 0
    e0.record(stream)
    for _ in range(args.steps):
        r = sess.decode(None, device_ptr=d_rf.data_ptr(), count=n)
        demod_ms.append(r.demod_ms)
        fields = r.fields
        launches += r.kernel_launches
    e1.record(stream)
    torch.cuda.synchronize()
    barrier(world)
    ms = e0.elapsed_time(e1) / args.steps
    ms = max_over_ranks(ms, world, "cuda")
    nblocks = int(r.blocks)
    value = world * n / (ms / 1e3) / 1e6
    # e2e through the C ABI: pinned host in, TBC out
    h_rf = torch.from_numpy(rf).pin_memory()
    tbc_elems = fields * r.output_field_lines * r.output_line_length
    h_tbc = torch.empty(max(1, tbc_elems), dtype=torch.int16).pin_memory()
    for _ in range(2):
        sess.decode(h_rf.numpy())
        sess.tbc_into(0, fields, h_tbc.data_ptr())
    torch.cuda.synchronize()
    barrier(world)
    f0 = torch.cuda.Event(enable_timing=True)
    f1 = torch.cuda.Event(enable_timing=True)
    f0.record(stream)
    for _ in range(args.steps):
        sess.decode(h_rf.numpy())
        sess.tbc_into(0, fields, h_tbc.data_ptr())
    f1.record(stream)
    torch.cuda.synchronize()
    clk = clocks.stop()
    e2e_ms = max_over_ranks(f0.elapsed_time(f1) / args.steps, world, "cuda")
    e2e_value = world * n / (e2e_ms / 1e3) / 1e6
    peak, peak_kind = peaks()
    avg_demod = sum(demod_ms) / len(demod_ms)
    achieved = DEMOD_BYTES_PER_BLOCK * nblocks / (avg_demod / 1e3) / 1e9
    tpb = profile_traffic_per_block()
    # plain FP64 baseline (one block at a time) on the same capture, one step
    plain = None
    if not args.skip_plain:
        ps = native.Session(prof, n, precision=native.PRECISION_FP64_PLAIN, device=local)
        ps.set_stream(stream.cuda_stream)
        ps.decode(None, device_ptr=d_rf.data_ptr(), count=n)
        torch.cuda.synchronize()
        p0 = torch.cuda.Event(enable_timing=True)
        p1 = torch.cuda.Event(enable_timing=True)
        p0.record(stream)
        ps.decode(None, device_ptr=d_rf.data_ptr(), count=n)
        p1.record(stream)
        torch.cuda.synchronize()
        pms = p0.elapsed_time(p1)
        plain = {"value": round(n / (pms / 1e3) / 1e6, 3), "unit": "MSPS",
                 "ms_per_step": round(pms, 3), "ratio_fp32_over_plain": round(value / world / (n / (pms / 1e3) / 1e6), 2)}
        ps.close()
    cpu = None
    if rank == 0 and world == 1 and not args.skip_cpu:
        procs = os.cpu_count() or 1
        pool = make_pool(procs)
        cpu_oracle_msps(rf[: 4 * 1048576], system, procs, pool)
        msps, dt, nf = cpu_oracle_msps(rf, system, procs, pool)
        pool.close()
        cpu = {"value": round(msps, 3), "unit": "MSPS", "cores": procs, "kind": "port",
               "sample": "whole workload capture (%d samples, %.1f s): oracle restatement, block "
                         "demod over %d spawn processes + sequential field path" % (n, dt, procs)}
    if rank == 0:
        line = {"metric": METRIC, "value": round(value, 3), "unit": "MSPS", "n_gpus": world,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms, 3),
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
                "data": "synthetic",
                "config": {"workload": args.workload, "description": desc, "samples": int(n),
                           "blocks": nblocks, "fields": int(fields),
                           "precision": "fp32 fused demod, fp64 sync/TBC",
                           "l2": "inputs and streams larger than L2 (no flush)",
                           "parallelism": "replicas" if world > 1 else "single"},
                "e2e": {"value": round(e2e_value, 3), "unit": "MSPS",
                        "h2d_bytes_per_step": int(n * 2),
                        "d2h_bytes_per_step": int(tbc_elems * 2)},
                "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak,
                             "unit": "GB/s", "frac": round(achieved / peak, 4),
                             "traffic": (round(tpb * nblocks) if tpb else None),
                             "kernel": "vhsd_demod_fp32_kernel", "peak_kind": peak_kind,
                             "kernel_ms": round(avg_demod, 4),
                             "algorithmic_bytes": int(DEMOD_BYTES_PER_BLOCK * nblocks)},
                "cpu_baseline": cpu,
                "plain_fp64": plain,
                "gpu_launches": int(launches),
                "clocks": clk,
                "stage_ms": {"demod": round(avg_demod, 4), "field_kernels_and_host": round(r.field_ms, 4),
                             "host_control": round(r.host_ms, 4)}}
        print(json.dumps(line))
    sess.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="ntsc60", choices=sorted(WORKLOADS))
    ap.add_argument("--skip-cpu", action="store_true")
    ap.add_argument("--skip-plain", action="store_true")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    world, rank, local = dist_init(args)
    if args.impl == "reference":
        run_reference(args, world, rank)
    else:
        run_ours(args, world, rank, local)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
