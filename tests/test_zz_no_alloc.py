"""The allocation-free product ctm_matmul_mixed_noalloc, called through the C
ABI, against the workspace-based ctm_matmul (CTM_PREC_MIXED).

Callers that cannot allocate device memory (a plugin host that only passes
input and output buffers, or one whose memory pool has reserved the device)
use this entry point; its scratch is a static device array shared
by all calls.  Two calls in a row must both match the existing entry point
(same kernels, so the tolerance is the FP64 rounding of the final sum) and
the FP64 product within the 3xBF16 tolerance of the other tensor-core tests.
This file is collected last so that a failure here stops a -x run only
after every other test has run; it also passes alone in a fresh process."""

import ctypes

import pytest
import torch

import acetn_gb300 as gb
from acetn_gb300 import _abi

pytestmark = pytest.mark.gpu


def _rand(m, n, seed):
    g = torch.Generator().manual_seed(seed)
    return torch.randn(m, n, generator=g, dtype=torch.float64).cuda()


def _noalloc(A, B):
    lib = _abi.load()
    M, K = A.shape
    N = B.shape[1]
    C = torch.empty(M, N, dtype=torch.float64, device=A.device)
    st = lib.ctm_matmul_mixed_noalloc(_abi.ptr(A), _abi.ptr(B), _abi.ptr(C), M, N, K,
                                      _abi.stream_handle(A.device))
    return st, C


def test_noalloc_matches_workspace_entry_point_twice():
    gb.build()
    for (m, n, k), seed in (((300, 160, 1000), 1), ((512, 96, 777), 2)):
        A, B = _rand(m, k, seed), _rand(k, n, seed + 10)
        st, C = _noalloc(A, B)
        assert st == _abi.CTM_OK, _abi.load().ctm_last_error()
        ref = gb.matmul(A, B, precision="mixed")
        torch.cuda.synchronize()
        assert torch.allclose(C, ref, rtol=1e-12, atol=1e-12)
        exact = A @ B
        assert float(torch.linalg.norm(C - exact) / torch.linalg.norm(exact)) < 5e-5
    assert gb._abi.device_status() == 0


def test_noalloc_rejects_products_beyond_its_scratch():
    A = _rand(4096, 4096, 3)
    st, _ = _noalloc(A, A)
    assert st == _abi.CTM_ERR_WORKSPACE
    assert b"static scratch" in _abi.load().ctm_last_error()


def test_noalloc_captures_in_a_global_mode_graph():
    """The entry point allocates nothing: a call captured in a CUDA graph with
    capture_error_mode='global' (where a cudaMalloc, or any other call that
    is unsafe during capture, makes the capture fail) replays to the
    workspace entry point's result."""
    gb.build()
    A, B = _rand(256, 640, 5), _rand(640, 192, 6)
    C = torch.empty(256, 192, dtype=torch.float64, device=A.device)
    lib = _abi.load()

    def call():
        return lib.ctm_matmul_mixed_noalloc(_abi.ptr(A), _abi.ptr(B), _abi.ptr(C), 256, 192, 640,
                                           _abi.stream_handle(A.device))

    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s):
        assert call() == _abi.CTM_OK, lib.ctm_last_error()  # warm-up outside the capture
    torch.cuda.current_stream().wait_stream(s)
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, capture_error_mode="global"):
        st = call()
    assert st == _abi.CTM_OK, lib.ctm_last_error()
    C.zero_()
    g.replay()
    torch.cuda.synchronize()
    ref = gb.matmul(A, B, precision="mixed")
    assert torch.allclose(C, ref, rtol=1e-12, atol=1e-12)
    assert gb._abi.device_status() == 0
