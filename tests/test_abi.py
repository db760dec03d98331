"""The C-ABI library loads on a CPU-only machine and exports every function that
include/ctdm.h declares (no compute calls)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_functions():
    text = open(os.path.join(ROOT, "include", "ctdm.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"^\s*(?:CTDM_API\s+)?(?:const\s+)?[A-Za-z_][A-Za-z0-9_]*\s*\*?\s*([A-Za-z_][A-Za-z0-9_]*)\s*\(",
                       text, re.M)
    return sorted(set(n for n in names if n not in ("if", "while")))


@pytest.fixture(scope="module")
def lib():
    from ctdm_gb300 import build
    path = build.build()
    return ctypes.CDLL(path)


def test_header_parsed():
    names = header_functions()
    for n in ("ctdm_reconstruct_device", "DCT_UWLS_Unwrapped", "BatchRecon", "cuFFT3D", "EdwardSphere"):
        assert n in names


def test_every_declared_symbol_exported(lib):
    missing = [n for n in header_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binding_covers_header():
    from ctdm_gb300 import _lib
    assert set(header_functions()) <= set(_lib.EXPORTED)


def test_params_struct_layout(lib):
    from ctdm_gb300 import _lib
    _lib.load()
    p = _lib.Params()
    _lib.load().ctdm_params_default(ctypes.byref(p))
    assert p.n_holo == 1024 and p.r_vol == 256 and p.iterations == 101
    assert p.carrier_r == -1 and abs(p.n_med - 1.333) < 1e-12
    assert p.qpi_method == 1   # Algorithm A by default (CTDM_QPI_A)
    assert ctypes.sizeof(_lib.Params) == 12 * 4 + 3 * 8 + 8   # trailing int padded to 8


def test_version_and_error_without_gpu(lib):
    from ctdm_gb300 import _lib
    L = _lib.load()
    assert b"sm_103a" in L.ctdm_version()
    # invalid arguments are rejected on the host before any CUDA call
    p = _lib.Params()
    L.ctdm_params_default(ctypes.byref(p))
    p.n_holo = 100
    rc = L.ctdm_reconstruct_device(ctypes.c_void_p(1), ctypes.byref(p), 4, 1, 1, 1, 1, 1, None)
    assert rc == 1 and b"unsupported" in L.ctdm_last_error()


def test_plan_table_without_gpu(lib):
    """Plan counts and the pinning checks need no GPU."""
    from ctdm_gb300 import _lib
    import ctdm_gb300 as C
    _lib.load()
    assert C.plan_count(256) == 3 and C.plan_count(64) == 1 and C.plan_count(100) == 0
    C.set_plans(512, (1, 2, 0), device=3)
    assert C.plans(512, device=3) == ((1, 2, 0), False)
    with pytest.raises(C.CtdmError):
        C.set_plans(512, (0, 3, 0), device=3)


def test_workspace_bound_without_gpu(lib):
    """ctdm_workspace_bytes is host arithmetic: it grows with the volume, the angles,
    Goldstein and the accelerated loop, and refuses what the pipeline refuses."""
    import ctdm_gb300 as C
    base = C.default_params(n_holo=1024, m_crop=256, r_vol=256, iterations=10, dx=0.1e-6)
    w = C.workspace_bytes(base, 121)
    r3 = 256 ** 3
    assert 25 * r3 * 1 < w < 60 * r3
    bigger = C.default_params(n_holo=1024, m_crop=256, r_vol=512, iterations=10, dx=0.1e-6)
    assert C.workspace_bytes(bigger, 121) > 4 * w
    assert C.workspace_bytes(base, 181) > w
    gold = C.default_params(n_holo=1024, m_crop=256, r_vol=256, iterations=10, dx=0.1e-6, run_goldstein=1)
    assert C.workspace_bytes(gold, 121) > w + 121 * 256 * 256 * 20
    acc = C.default_params(n_holo=1024, m_crop=256, r_vol=256, iterations=10, dx=0.1e-6, accelerated=1)
    assert C.workspace_bytes(acc, 121) == w + 8 * r3
    bad = C.default_params(n_holo=1024, m_crop=256, r_vol=100, iterations=10, dx=0.1e-6)
    with pytest.raises(C.CtdmError):
        C.workspace_bytes(bad, 121)
