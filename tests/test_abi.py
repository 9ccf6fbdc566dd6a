"""CPU-side checks of the C-ABI library: it loads, exports every symbol the
header declares, and the ctypes binding covers exactly that set."""
import re
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def header_symbols():
    text = (ROOT / "include" / "mczi_gpu.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return set(re.findall(r"\b(mczi_[a-z0-9_]+)\s*\(", text))


@pytest.fixture(scope="module")
def lib():
    from mczi_gb300 import build
    build.build_gpu_lib()
    from mczi_gb300 import _native
    return _native.load()


def test_exports_every_declared_symbol(lib):
    syms = header_symbols()
    assert len(syms) >= 15
    for s in sorted(syms):
        assert hasattr(lib, s), s
    out = subprocess.run(["nm", "-D", "--defined-only", str(ROOT / "mczi_gb300" / "lib" / "libmczi_gpu.so")],
                         capture_output=True, text=True, check=True).stdout
    exported = set(re.findall(r"\b(mczi_[a-z0-9_]+)\b", out))
    assert syms <= exported


def test_binding_matches_header(lib):
    from mczi_gb300 import _native
    assert {n for n, _, _ in _native.SIGNATURES} == header_symbols()


def test_no_device_fails_loudly(lib):
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    import ctypes as C
    from mczi_gb300 import _native
    h = C.c_void_p()
    assert lib.mczi_open(0, C.byref(h)) == _native.MCZI_ERR_DEVICE
    from mczi_gb300.mc import Context
    with pytest.raises(_native.MCZIError):
        Context(0)
    # the native serving loop opens its worker contexts the same way
    srv = C.c_void_p()
    idx = b">i\nACGTACGTACGTACGT\n"
    assert lib.mczi_serve_open(0, idx, len(idx), 5, 3, 1, 4, 0, C.byref(srv)) == _native.MCZI_ERR_DEVICE
    assert not srv.value
    assert lib.mczi_serve_error(None, 0) == b"no usable CUDA device"
    from mczi_gb300.serve import ZIServer
    with pytest.raises(_native.MCZIError):
        ZIServer(idx, 5, 3, workers=1)


def test_serve_open_validates_before_device_work(lib):
    import ctypes as C
    from mczi_gb300 import _native
    srv = C.c_void_p()
    idx = b">i\nACGTACGT\n"
    assert lib.mczi_serve_open(0, idx, len(idx), 5, 3, 0, 4, 0, C.byref(srv)) == _native.MCZI_ERR_INVALID_CONFIG
    assert lib.mczi_serve_error(None, 0) == b"workers must be in [1, 64]"
    assert lib.mczi_serve_open(0, idx, len(idx), 5, 3, 1, 0, 0, C.byref(srv)) == _native.MCZI_ERR_INVALID_CONFIG
    assert lib.mczi_serve_error(None, 0) == b"max_batch must be in [1, 4096]"
    assert lib.mczi_serve_submit(None, idx, len(idx), C.byref(C.c_uint64())) == _native.MCZI_ERR_STATE
    assert lib.mczi_serve_close(None) == _native.MCZI_ERR_STATE


def test_oracle_not_imported_by_product():
    for p in (ROOT / "mczi_gb300").rglob("*.py"):
        text = p.read_text()
        assert "oracle_ref" not in text and "libmczi_oracle" not in text, p
