"""Device FLAC decoding of .ldf RF captures, through the C ABI.

FLAC is lossless: the device decoder must return exactly the int16 samples the
.ldf writer (vhsd_gb300/ldf.py, RFC 9639) was given, for every subframe and
residual form the writer produces, at several block sizes and at the full size
of the 60-field NTSC workload (the bit-level reader oracle/flac.py reads the
writer's streams back the same way, tests/test_abi_cpu.py).  A damaged stream is an input error, and run()
fed FLAC bytes writes the same files as run() fed the int16 samples.
"""
import ctypes
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def rf_small():
    from vhsd_gb300 import synth
    rf, _ = synth.generate(synth.config("pal_small"))
    x = rf.copy()
    x[4096 * 3:4096 * 4] &= ~1        # a frame with a wasted bit
    x[4096 * 6:4096 * 7] = 77         # a constant frame
    return x


@pytest.mark.parametrize("blocksize", [4096, 1152, 4608])
def test_flac_round_trip_is_bit_exact(gpu, rf_small, blocksize):
    from vhsd_gb300 import ldf, native
    data = ldf.write(rf_small, blocksize=blocksize, seed=blocksize, wasted_frames=(3,))
    info = native.flac_info(data)
    assert info.total_samples == len(rf_small) and info.channels == 1
    got = native.flac_decode(data)
    assert got.dtype == np.int16 and np.array_equal(got, rf_small)


def test_flac_full_size_round_trip(gpu):
    # the 41 M-sample NTSC workload: lossless at full size
    import bench
    from vhsd_gb300 import ldf, native
    rf = bench.workload("ntsc60")
    data = ldf.write(rf, seed=60)
    got = native.flac_decode(data)
    assert np.array_equal(got, rf)


def test_damaged_flac_is_an_input_error(gpu, rf_small):
    from vhsd_gb300 import ldf, native
    data = bytearray(ldf.write(rf_small[:200_000], seed=1))
    # a flipped bit in the middle of the stream: the frame's CRC-16 (or its
    # structure) no longer matches
    data[len(data) // 2] ^= 0x10
    with pytest.raises(native.NativeError) as e:
        native.flac_decode(bytes(data))
    assert e.value.status == native.STATUS_INPUT_ERROR
    # a stream cut inside its last frame
    good = ldf.write(rf_small[:200_000], seed=1)
    with pytest.raises(native.NativeError):
        native.flac_decode(good[:-100])


def _run(data, base, fmt, monkeypatch, grids="3"):
    from vhsd_gb300 import native
    monkeypatch.setenv("VHSD_RUN_WINDOW_GRIDS", grids)
    L = native.load()
    if fmt == native.INPUT_FLAC:
        src = np.frombuffer(data, np.uint8)
        esz = 1
    else:
        src = np.ascontiguousarray(data, np.int16)
        esz = 2

    def read(u, dst, off, count):
        k = max(0, min(count, len(src) - off))
        if k:
            ctypes.memmove(dst, src[off:].ctypes.data, k * esz)
        return k

    cb = native.READ_CB(read)
    cfg = native.RunConfig()
    cfg.struct_size = ctypes.sizeof(cfg)
    cfg.profile = native.PROFILE_PAL
    cfg.sample_rate_mhz = 40.0
    cfg.total_samples = len(src)
    cfg.output_base_utf8 = base.encode()
    cfg.overwrite = 1
    cfg.input_sample_format = fmt
    cfg.device_decimation_factor = 1
    cfg.read_callback = cb
    res = native.RunResult()
    res.struct_size = ctypes.sizeof(res)
    native.check(L.vhsdecode_gb300_run(ctypes.byref(cfg), ctypes.byref(res)))
    return res


def test_run_from_flac_bytes_equals_int16(gpu, tmp_path, monkeypatch):
    # a 12-field capture: its FLAC stream spans several read chunks and the
    # decode several windows
    from vhsd_gb300 import ldf, native, synth
    rf, _ = synth.generate(synth.config("pal_small", fields=12, seed=12))
    data = ldf.write(rf, seed=12)
    monkeypatch.setenv("VHSD_RUN_FLAC_CHUNK", str(1 << 20))   # frames straddle the chunk joins
    assert len(data) > (1 << 22)
    a = _run(data, str(tmp_path / "flac"), native.INPUT_FLAC, monkeypatch)
    b = _run(rf, str(tmp_path / "s16"), native.INPUT_INT16, monkeypatch)
    assert a.fields_written == b.fields_written > 8
    for ext in (".tbc", ".tbc.json", "_chroma.tbc"):
        assert (tmp_path / ("flac" + ext)).read_bytes() == (tmp_path / ("s16" + ext)).read_bytes()
    assert not [p for p in os.listdir(tmp_path) if p.endswith(".tmp")]
