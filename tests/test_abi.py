"""The C-ABI library: it loads, exports every symbol declared in
include/ctm_gb300.h, answers workspace-size queries and validates arguments.
No kernel is launched (CPU only)."""

import ctypes
import os
import re

import pytest

import acetn_gb300 as gb
from acetn_gb300 import _abi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "ctm_gb300.h")


def declared():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(ctm_[a-z0-9_]+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    gb.build()
    return _abi.load()


def test_every_declared_symbol_is_exported(lib):
    names = declared()
    assert len(names) >= 10
    for name in names:
        assert hasattr(lib, name), name
    assert sorted(names) == _abi.exported_symbols()


def test_version(lib):
    assert b"sm_103a" in lib.ctm_version()


def fake_site(D, chi, d=2, base=0x10000):
    s = _abi.CtmSite()
    s.A = base
    for k in range(4):
        s.C[k] = base + 0x1000 * (k + 1)
        s.E[k] = base + 0x100000 * (k + 1)
        s.c_rows[k] = s.c_cols[k] = chi
        s.e_rows[k] = s.e_cols[k] = chi
    return s


def opts(chi, proj="half-system", svd="rsvd", os_=2, prec="fp64"):
    class C:
        pass
    c = C()
    c.projectors, c.svd_type, c.rsvd_oversampling = proj, svd, os_
    c.svd_cutoff, c.rsvd_niter = 1e-12, 2
    return _abi.opts_struct(c, chi, prec)


def test_projector_dims_host_only(lib):
    D, chi = 6, 144
    sites = [fake_site(D, chi, base=0x10000 * (i + 1)) for i in range(4)]
    arr = (_abi.SITE_P * 4)(*[ctypes.pointer(s) for s in sites])
    out = [_abi.c_i64() for _ in range(5)]
    o = opts(chi, os_=16)
    st = lib.ctm_projector_dims(arr, D, 0, ctypes.byref(o), *[ctypes.byref(x) for x in out])
    assert st == 0
    p1, p2, n, q, cap = (x.value for x in out)
    assert (p1, p2, n, q, cap) == (chi * 36, chi * 36, chi * 36, 160, 144)
    o = opts(chi, svd="full-rank")
    assert lib.ctm_projector_dims(arr, D, 0, ctypes.byref(o), *[ctypes.byref(x) for x in out]) == 0
    assert out[3].value == 0 and out[4].value == 144


def test_projector_dims_rejects_bad_options(lib):
    sites = [fake_site(2, 4, base=0x10000 * (i + 1)) for i in range(4)]
    arr = (_abi.SITE_P * 4)(*[ctypes.pointer(s) for s in sites])
    o = opts(4)
    o.projectors = 7
    out = [_abi.c_i64() for _ in range(5)]
    st = lib.ctm_projector_dims(arr, 2, 0, ctypes.byref(o), *[ctypes.byref(x) for x in out])
    assert st == _abi.CTM_ERR_INVALID
    assert b"projector" in lib.ctm_last_error()


def test_mismatched_chain_is_rejected(lib):
    sites = [fake_site(2, 4, base=0x10000 * (i + 1)) for i in range(4)]
    sites[0].c_rows[0] = 5  # C[0] rows no longer match E[3] columns
    arr = (_abi.SITE_P * 4)(*[ctypes.pointer(s) for s in sites])
    out = [_abi.c_i64() for _ in range(5)]
    o = opts(4)
    st = lib.ctm_projector_dims(arr, 2, 0, ctypes.byref(o), *[ctypes.byref(x) for x in out])
    assert st == _abi.CTM_ERR_INVALID


def test_workspace_queries_launch_nothing(lib):
    sz = ctypes.c_size_t(0)
    st = lib.ctm_matmul(ctypes.c_void_p(0x1000), ctypes.c_void_p(0x2000), ctypes.c_void_p(0x3000),
                        512, 512, 512, 0, None, ctypes.byref(sz), None)
    assert st == 0 and sz.value > 0
    s = fake_site(6, 144)
    sz = ctypes.c_size_t(0)
    sh = (_abi.c_i64 * 6)()
    st = lib.ctm_quarter_tensor(ctypes.pointer(s), 6, 2, 0, ctypes.c_void_p(0x1000), sh, 0, None,
                                ctypes.byref(sz), None)
    assert st == 0
    n = 144 * 36
    # the quarter tensor needs its two N^2-sized intermediates (one of them 2 N^2)
    assert sz.value >= 3 * n * n * 8
    assert list(sh) == [144, 6, 6, 144, 6, 6]
    sites = [fake_site(6, 144, base=0x10000 * (i + 1)) for i in range(4)]
    arr = (_abi.SITE_P * 4)(*[ctypes.pointer(x) for x in sites])
    o = opts(144, os_=16)
    sz = ctypes.c_size_t(0)
    st = lib.ctm_calculate_projectors(arr, 6, 2, 0, ctypes.byref(o), ctypes.c_void_p(0x1000),
                                      ctypes.c_void_p(0x2000), ctypes.c_void_p(0x3000),
                                      ctypes.c_void_p(0x4000), None, ctypes.byref(sz), None)
    assert st == 0 and sz.value > 2 * n * n * 8


def test_null_ws_bytes_is_invalid(lib):
    st = lib.ctm_matmul(None, None, None, 4, 4, 4, 0, None, None, None)
    assert st == _abi.CTM_ERR_INVALID


def test_bad_sizes_are_invalid(lib):
    sz = ctypes.c_size_t(0)
    st = lib.ctm_matmul(None, None, None, 0, 4, 4, 0, None, ctypes.byref(sz), None)
    assert st == _abi.CTM_ERR_INVALID
    st = lib.ctm_svd_f64(None, 5000, 10, None, None, None, None, ctypes.byref(sz), None)
    assert st == _abi.CTM_ERR_UNSUPPORTED
    st = lib.ctm_qr(None, 10, 11, None, 0, None, ctypes.byref(sz), None)
    assert st == _abi.CTM_ERR_INVALID
    st = lib.ctm_qr(None, 100, 10, None, 7, None, ctypes.byref(sz), None)
    assert st == _abi.CTM_ERR_INVALID


def test_svd_f32_validation_and_workspace_query(lib):
    sz = ctypes.c_size_t(0)
    # q > n and q > 1024 are rejected before any launch
    st = lib.ctm_svd_f32(None, 10, 11, None, None, None, None, ctypes.byref(sz), None)
    assert st == _abi.CTM_ERR_UNSUPPORTED
    st = lib.ctm_svd_f32(None, 5000, 1025, None, None, None, None, ctypes.byref(sz), None)
    assert st == _abi.CTM_ERR_UNSUPPORTED
    # the D=6, chi=144 Rayleigh-Ritz size: B^T (5184 x 160) copy, the QR's
    # buffers and the Jacobi scratch
    n, q = 144 * 36, 160
    st = lib.ctm_svd_f32(ctypes.c_void_p(0x1000), n, q, ctypes.c_void_p(0x2000),
                         ctypes.c_void_p(0x3000), ctypes.c_void_p(0x4000), None,
                         ctypes.byref(sz), None)
    assert st == 0 and sz.value >= 3 * n * q * 4


def test_linalg_wrappers_reject_cpu_tensors():
    import torch
    with pytest.raises(ValueError):
        gb.linalg.qr(torch.zeros(8, 4, dtype=torch.float64))
    with pytest.raises(ValueError):
        gb.linalg.svd_f32(torch.zeros(8, 4, dtype=torch.float32))


def test_qr_workspace_query(lib):
    # FP32 Cholesky-QR at the D=6, chi=144 range-finder size: the input copy,
    # the second buffer and one q x q Gram per row slab
    n, q = 144 * 36, 160
    for dtype, es in ((0, 8), (1, 4)):
        sz = ctypes.c_size_t(0)
        st = lib.ctm_qr(ctypes.c_void_p(0x1000), n, q, None, dtype, None, ctypes.byref(sz), None)
        assert st == 0 and sz.value >= 2 * n * q * es


def test_no_cpu_fallback():
    import torch
    with pytest.raises(ValueError):
        gb.linalg.matmul(torch.zeros(2, 2, dtype=torch.float64), torch.zeros(2, 2, dtype=torch.float64))
