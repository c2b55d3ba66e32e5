import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "vhs-decode-dotnet_gb300")
for p in (ROOT, PKG):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a)")


def _have_gpu():
    try:
        import torch  # noqa: F401
        return torch.cuda.is_available()
    except Exception:
        return os.path.exists("/dev/nvidia0")


HAVE_GPU = _have_gpu()


@pytest.fixture(scope="session")
def lib():
    from vhsd_gb300 import build, native
    if not os.path.exists(native.LIB_PATH):
        build.build()
    return native.load()


@pytest.fixture(scope="session")
def gpu(lib):
    if not HAVE_GPU:
        pytest.skip("no GPU")
    return lib


@pytest.fixture(scope="session")
def pal_capture():
    from vhsd_gb300 import synth
    rf, info = synth.generate(synth.config("pal_small"))
    return rf, info


@pytest.fixture(scope="session")
def ntsc_capture():
    from vhsd_gb300 import synth
    rf, info = synth.generate(synth.config("ntsc_small"))
    return rf, info


@pytest.fixture(scope="session")
def pal_oracle(pal_capture):
    from oracle import field, formats
    rf, _ = pal_capture
    fields, ch = field.decode_capture(rf, formats.get("PAL"))
    return fields, ch


@pytest.fixture(scope="session")
def ntsc_oracle(ntsc_capture):
    from oracle import field, formats
    rf, _ = ntsc_capture
    fields, ch = field.decode_capture(rf, formats.get("NTSC"))
    return fields, ch


@pytest.fixture(scope="session")
def ntsc20_capture():
    from vhsd_gb300 import synth
    rf, info = synth.generate(synth.config("ntsc_small", fs=20e6))
    return rf, info


@pytest.fixture(scope="session")
def ntsc20_oracle(ntsc20_capture):
    from oracle import field, formats
    rf, _ = ntsc20_capture
    fields, ch = field.decode_capture(rf, formats.get("NTSC"), fs=20e6)
    return fields, ch


@pytest.fixture(scope="session")
def svhs_capture():
    from vhsd_gb300 import synth
    rf, info = synth.generate(synth.config("svhs_small"))
    return rf, info


@pytest.fixture(scope="session")
def svhs_oracle(svhs_capture):
    from oracle import field, formats
    rf, _ = svhs_capture
    fields, ch = field.decode_capture(rf, formats.get("PAL", "SVHS"))
    return fields, ch


@pytest.fixture(scope="session")
def svhs_ntsc_capture():
    from vhsd_gb300 import synth
    rf, info = synth.generate(synth.config("svhs_ntsc_small"))
    return rf, info


@pytest.fixture(scope="session")
def svhs_ntsc_oracle(svhs_ntsc_capture):
    from oracle import field, formats
    rf, _ = svhs_ntsc_capture
    fields, ch = field.decode_capture(rf, formats.get("NTSC", "SVHS"))
    return fields, ch
