"""Window server (continuous batching of decode windows) through the C ABI.

The bar: every window's result is the same decoded alone and decoded in a mix
with other streams' windows (bit-identical TBC, same field counts and
parities); a stream's consecutive windows continue its field sequence; the
server admits slots inside a device-memory budget that holds only one.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

LSB_FRACTION = 0.999


def _windows(rf, n, length):
    step = (len(rf) - length) // max(1, n - 1)
    return [(i * step, rf[i * step:i * step + length]) for i in range(n)]


def _run(server, jobs, per_field):
    """jobs: (stream, profile, offset, samples, max_fields[, tape format]); all submitted
    before any wait."""
    outs, tickets = [], []
    for job in jobs:
        stream, prof, off, x, mf = job[:5]
        tape = job[5] if len(job) > 5 else 0
        out = np.zeros(mf * per_field[prof], np.uint16)
        tickets.append(server.submit(stream, prof, x, source_offset=off, seek=True, max_fields=mf,
                                     tbc_out=out, tape_format=tape))
        outs.append(out)
    res = [server.wait(t) for t in tickets]
    return res, outs


def test_window_alone_equals_in_mix(gpu, pal_capture, ntsc_capture, svhs_capture):
    from vhsd_gb300 import native
    pal, _ = pal_capture
    ntsc, _ = ntsc_capture
    svhs, _ = svhs_capture
    per_field = {native.PROFILE_PAL: 313 * 1135, native.PROFILE_NTSC: 263 * 910}
    length = 1_400_000
    jobs = []
    for k, (off, x) in enumerate(_windows(pal, 3, length)):
        jobs.append((k, native.PROFILE_PAL, off, x, 2))
    for k, (off, x) in enumerate(_windows(ntsc, 3, length)):
        jobs.append((10 + k, native.PROFILE_NTSC, off, x, 2))
    for k, (off, x) in enumerate(_windows(svhs, 2, length)):
        jobs.append((20 + k, native.PROFILE_PAL, off, x, 2, native.FORMAT_SVHS))
    with native.Server(length, workers=1) as sv:
        alone = []
        for j in jobs:
            r, o = _run(sv, [j], per_field)
            alone.append((r[0], o[0]))
    with native.Server(length, workers=4) as sv:
        mix_r, mix_o = _run(sv, jobs, per_field)
    assert sum(ra.fields for ra, _ in alone) > 0
    for (ra, oa), rb, ob in zip(alone, mix_r, mix_o):
        assert ra.status == 0 and rb.status == 0
        assert ra.fields == rb.fields
        assert ra.first_field_is_first == rb.first_field_is_first
        assert oa.tobytes() == ob.tobytes()


def test_stream_windows_continue_the_field_sequence(gpu, ntsc_capture):
    from vhsd_gb300 import native
    rf, _ = ntsc_capture
    per = 263 * 910
    with native.Session(native.PROFILE_NTSC, len(rf)) as s:
        r = s.decode(rf)
        whole = s.tbc().reshape(r.fields, -1).copy()
        parity = [bool(s.field(i).is_first_field) for i in range(r.fields)]
    with native.Server(len(rf), workers=2) as sv:
        first_len = len(rf) // 2
        out_a = np.zeros(r.fields * per, np.uint16)
        ta = sv.submit(7, native.PROFILE_NTSC, rf[:first_len], 0, seek=True, tbc_out=out_a)
        ra = sv.wait(ta)
        off = ra.next_source_offset
        out_b = np.zeros(r.fields * per, np.uint16)
        tb = sv.submit(7, native.PROFILE_NTSC, rf[off:], off, seek=False, tbc_out=out_b)
        rb = sv.wait(tb)
    assert ra.status == 0 and rb.status == 0 and rb.continued == 1
    assert ra.fields + rb.fields == r.fields
    got = np.concatenate([out_a[:ra.fields * per], out_b[:rb.fields * per]]).reshape(r.fields, -1)
    assert bool(ra.first_field_is_first) == parity[0]
    assert bool(rb.first_field_is_first) == parity[ra.fields]
    # the continuation window starts on the stream's block/span grid: bit-identical
    assert off % 983040 == 0
    assert got.tobytes() == whole.tobytes()


def test_admission_within_a_one_slot_budget(gpu, pal_capture, ntsc_capture):
    from vhsd_gb300 import native
    pal, _ = pal_capture
    ntsc, _ = ntsc_capture
    length = 1_400_000
    per_field = {native.PROFILE_PAL: 313 * 1135, native.PROFILE_NTSC: 263 * 910}
    jobs = [(0, native.PROFILE_PAL, 0, pal[:length], 2), (1, native.PROFILE_NTSC, 0, ntsc[:length], 2),
            (2, native.PROFILE_PAL, 0, pal[:length], 2), (3, native.PROFILE_NTSC, 0, ntsc[:length], 2)]
    with native.Server(length, workers=3) as sv:
        ref_r, ref_o = _run(sv, jobs, per_field)
    # a budget for one slot: formats take turns on it, windows wait for memory
    import torch
    torch.cuda.synchronize()
    f0, _ = torch.cuda.mem_get_info()
    probe = native.Session(native.PROFILE_PAL, length)
    f1, _ = torch.cuda.mem_get_info()
    probe.close()
    footprint = f0 - f1
    assert footprint > 0
    with native.Server(length, workers=3, memory_budget=int(1.5 * footprint)) as sv:
        r, o = _run(sv, jobs, per_field)
    for a, b, oa, ob in zip(ref_r, r, ref_o, o):
        assert a.status == 0 and b.status == 0 and a.fields == b.fields
        assert oa.tobytes() == ob.tobytes()


def test_unsupported_window_is_rejected(gpu, pal_capture):
    from vhsd_gb300 import native
    pal, _ = pal_capture
    with native.Server(1 << 21, workers=1) as sv:
        with pytest.raises(native.NativeError) as e:
            sv.submit(0, native.PROFILE_PAL, pal[:1 << 20], tape_speed=3)   # no VP parameters
        assert e.value.status == native.STATUS_INVALID_ARGUMENT
        with pytest.raises(native.NativeError) as e:
            sv.submit(0, native.PROFILE_PAL_M, pal[:1 << 20])
        assert e.value.status == native.STATUS_INVALID_ARGUMENT
        with pytest.raises(native.NativeError):
            sv.submit(0, native.PROFILE_PAL, pal[:1 << 22])   # longer than the slots


def test_decimated_windows_match_the_session(gpu, ntsc_capture, pal_capture):
    # preview mode of the reference (40-MSPS windows decoded at 20 MSPS through
    # the device decimator) beside full-rate windows in one server: each
    # window's fields equal a decimating session's decode of the same samples
    from vhsd_gb300 import native
    ntsc, _ = ntsc_capture
    pal, _ = pal_capture
    length = 1_400_000
    per = 263 * 910
    wins = _windows(ntsc, 2, length)
    with native.Server(length, workers=3) as sv:
        tickets, outs = [], []
        for k, (off, x) in enumerate(wins):
            out = np.zeros(2 * per, np.uint16)
            tickets.append(sv.submit(k, native.PROFILE_NTSC, x, source_offset=off, seek=True, max_fields=2,
                                     tbc_out=out, sample_rate_mhz=20.0, decimation=2))
            outs.append(out)
        pal_out = np.zeros(2 * 313 * 1135, np.uint16)
        tp = sv.submit(9, native.PROFILE_PAL, pal[:length], seek=True, max_fields=2, tbc_out=pal_out)
        res = [sv.wait(t) for t in tickets]
        assert sv.wait(tp).fields > 0
    with native.Session(native.PROFILE_NTSC, length, sample_rate_mhz=20.0, decimation=2) as s:
        for (off, x), r, out in zip(wins, res, outs):
            d = s.decode(x, max_fields=2)
            assert r.status == 0 and r.fields == d.fields > 0
            assert out[:d.fields * per].tobytes() == s.tbc()[:d.fields].tobytes()
            # continuation offsets are source samples: twice the decode-rate grid
            assert (r.next_source_offset - off) % (2 * 983040) == 0


def test_batched_windows_equal_alone(gpu, pal_capture, ntsc_capture, ntsc20_capture, svhs_capture):
    # cross-stream batching: windows of different streams and formats (PAL VHS,
    # NTSC VHS at 40 and 20 MSPS, PAL S-VHS with sub-deemphasis, NTSC VHS LP)
    # queued behind one worker are demodulated in one persistent launch; each
    # window's result equals its decode alone, bit for bit
    from vhsd_gb300 import native
    pal, _ = pal_capture
    ntsc, _ = ntsc_capture
    ntsc20, _ = ntsc20_capture
    svhs, _ = svhs_capture
    per_field = {native.PROFILE_PAL: 313 * 1135, native.PROFILE_NTSC: 263 * 910}
    length = 1_400_000
    jobs = []   # (stream, profile, offset, samples, max fields, tape format, MSPS, speed)
    for k, (off, x) in enumerate(_windows(pal, 2, length)):
        jobs.append((k, native.PROFILE_PAL, off, x, 2, native.FORMAT_VHS, 40.0, native.TAPE_SP))
    for k, (off, x) in enumerate(_windows(ntsc, 2, length)):
        jobs.append((10 + k, native.PROFILE_NTSC, off, x, 2, native.FORMAT_VHS, 40.0, native.TAPE_SP))
    for k, (off, x) in enumerate(_windows(ntsc20, 1, 900_000)):
        jobs.append((20 + k, native.PROFILE_NTSC, off, x, 2, native.FORMAT_VHS, 20.0, native.TAPE_SP))
    for k, (off, x) in enumerate(_windows(svhs, 2, length)):
        jobs.append((30 + k, native.PROFILE_PAL, off, x, 2, native.FORMAT_SVHS, 40.0, native.TAPE_SP))
    off, x = _windows(ntsc, 1, length)[0]
    jobs.append((40, native.PROFILE_NTSC, off, x, 2, native.FORMAT_VHS, 40.0, native.TAPE_LP))

    def run(server):
        outs, tickets = [], []
        for stream, prof, off, x, mf, tape, mhz, speed in jobs:
            out = np.zeros(mf * per_field[prof], np.uint16)
            tickets.append(server.submit(stream, prof, x, source_offset=off, seek=True, max_fields=mf,
                                         tbc_out=out, tape_format=tape, sample_rate_mhz=mhz,
                                         tape_speed=speed))
            outs.append(out)
        return [server.wait(t) for t in tickets], outs

    with native.Server(length, workers=1) as sv:
        alone = []
        for j in range(len(jobs)):
            saved = list(jobs)
            jobs[:] = [saved[j]]
            r, o = run(sv)
            jobs[:] = saved
            alone.append((r[0], o[0]))
    with native.Server(length, workers=1, max_batch=8) as sv:
        res, outs = run(sv)
    assert max(r.batched for r in res) >= 4   # the queued windows went into one launch
    for (ra, oa), rb, ob in zip(alone, res, outs):
        assert ra.status == 0 and rb.status == 0
        assert ra.fields == rb.fields > 0
        assert ra.first_field_is_first == rb.first_field_is_first
        assert oa.tobytes() == ob.tobytes()
