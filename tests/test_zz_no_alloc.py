"""The no-allocation pulse edge scan against the allocating device entry point.

Collected last on purpose (file name), so it also runs after every other test
has used the device.  Each case calls the no-allocation entry twice in a row
on fresh inputs and compares the pulses built from its events with
``vhsdecode_gb300_find_pulses`` on the same samples: integer work, so the
pulse lists must be identical.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _pulses_from_events(events, mn, mx):
    # pairing of start/end events into (start, length), as the host control
    # plane does for a span that starts at stream index 0
    out, cur = [], -1
    for e in events:
        pos = int(e) >> 1
        if (int(e) & 1) == 0:
            cur = pos
        else:
            if cur > 0 and mn <= pos - cur <= mx:
                out.append((cur, pos - cur))
            cur = -1
    return out


def _noalloc_events(lib, x, high, capacity):
    import torch
    d = torch.from_numpy(x).cuda()
    ev = torch.empty(max(capacity, 1), dtype=torch.int64, device="cuda")
    tot = torch.empty(1, dtype=torch.int64, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    st = lib.vhsdecode_gb300_pulse_events_noalloc(
        ctypes.c_void_p(d.data_ptr()), len(x), high, ctypes.c_void_p(ev.data_ptr()), capacity,
        ctypes.c_void_p(tot.data_ptr()), ctypes.c_void_p(stream))
    assert st == 0, lib.vhsdecode_gb300_get_last_error()
    torch.cuda.synchronize()
    n = int(tot.cpu()[0])
    return n, ev.cpu().numpy()[:min(n, capacity)]


def _case(rng, n):
    specials = np.array([np.nan, -np.inf, -1.0, 0.0, 1.0, np.inf])
    x = (rng.random(n) * 20.0 - 10.0).astype(np.float32)
    mask = rng.integers(0, 25, n) == 0
    x[mask] = specials[rng.integers(0, len(specials), mask.sum())]
    return x, float(rng.random() * 12 - 6)


def test_no_alloc_pulses_match_allocating_entry(gpu):
    from vhsd_gb300 import native
    lib = native.load()
    rng = np.random.default_rng(0x4E41)
    for n in (0, 1, 1023, 1025, 40961, 300007):
        for _ in range(2):  # two calls in a row share the fixed scratch
            x, high = _case(rng, n)
            total, ev = _noalloc_events(lib, x, high, 2 * n + 16)
            assert total == len(ev)
            assert np.all(np.diff(ev) > 0)
            mn, mx = 2, 40
            want = native.find_pulses(x.astype(np.float64), high, mn, mx) if n else []
            assert _pulses_from_events(ev, mn, mx) == [tuple(p) for p in want]


def test_no_alloc_counts_past_capacity(gpu):
    from vhsd_gb300 import native
    lib = native.load()
    rng = np.random.default_rng(5)
    x, high = _case(rng, 50000)
    full_n, full = _noalloc_events(lib, x, high, 2 * len(x))
    part_n, part = _noalloc_events(lib, x, high, 7)
    assert part_n == full_n and part.tolist() == full[:7].tolist()


def test_no_alloc_rejects_length_above_limit(gpu):
    import torch
    from vhsd_gb300 import native
    lib = native.load()
    d = torch.zeros(16, dtype=torch.float32, device="cuda")
    tot = torch.zeros(1, dtype=torch.int64, device="cuda")
    st = lib.vhsdecode_gb300_pulse_events_noalloc(
        ctypes.c_void_p(d.data_ptr()), (1 << 24) + 1, 0.0, None, 0,
        ctypes.c_void_p(tot.data_ptr()), None)
    assert st == native.STATUS_INVALID_ARGUMENT
    assert b"limit" in lib.vhsdecode_gb300_get_last_error()
