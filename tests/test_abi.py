"""
The C-ABI library without a GPU: it builds for sm_103a, loads, exports every
function include/fsgpu.h declares, and fails loudly (an error code, a Python
exception) when no CUDA device is present.  No compute call is made here.
"""
import ctypes as ct
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "fsgpu.h")


def declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(fsg_\w+)\s*\(", src)))


@pytest.fixture(scope="module")
def lib():
    from fractalshades_gb300.csrc import build as nb
    path = nb.build()
    return ct.CDLL(path)


def test_header_declares_the_boundary():
    names = declared_functions()
    for required in ["fsg_ctx_create", "fsg_ref_create", "fsg_std_tiles",
                     "fsg_perturb_tiles", "fsg_cancel", "fsg_last_error"]:
        assert required in names


def test_library_exports_every_declared_symbol(lib):
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, f"not exported: {missing}"


def test_binding_covers_the_header():
    from fractalshades_gb300 import _native as nat
    assert sorted(nat.SYMBOLS) == declared_functions()


def test_version(lib):
    lib.fsg_version.restype = ct.c_char_p
    assert b"sm_103a" in lib.fsg_version()


def _has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.mark.skipif(_has_gpu(), reason="checks the no-device path")
def test_no_device_is_an_error_not_a_fallback(lib):
    from fractalshades_gb300 import _native as nat
    h = ct.c_void_p()
    lib.fsg_ctx_create.argtypes = [ct.c_int, ct.POINTER(ct.c_void_p)]
    rc = lib.fsg_ctx_create(0, ct.byref(h))
    assert rc == nat.FSG_ERR_NODEV
    with pytest.raises(nat.GPUError):
        nat.Context(0)


def test_null_arguments_are_rejected(lib):
    lib.fsg_ref_create.argtypes = [ct.c_void_p, ct.c_void_p, ct.c_void_p]
    assert lib.fsg_ref_create(None, None, None) < 0
    lib.fsg_perturb_tiles.argtypes = [ct.c_void_p, ct.c_void_p, ct.c_void_p, ct.c_int32, ct.c_int32]
    assert lib.fsg_perturb_tiles(None, None, None, 0, 0) < 0
    lib.fsg_last_error.restype = ct.c_char_p
    assert lib.fsg_last_error(None) == b"no context"


# ---------------------------------------------------------------------------
# the arbitrary-precision host library (include/fsghost.h)
# ---------------------------------------------------------------------------
HOST_HEADER = os.path.join(ROOT, "include", "fsghost.h")


def host_declared_functions():
    src = open(HOST_HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(fsh_\w+)\s*\(", src)))


def test_host_library_exports_and_binding_cover_the_header():
    from fractalshades_gb300.csrc import build as nb
    from fractalshades_gb300 import _host
    hl = ct.CDLL(nb.build_host())
    names = host_declared_functions()
    assert "fsh_orbit_mn" in names and "fsh_nucleus_m2" in names
    assert not [n for n in names if not hasattr(hl, n)]
    assert sorted(_host.SYMBOLS) == names
