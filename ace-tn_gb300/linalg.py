"""Randomized SVDs of ``acetn.linalg`` on the GB300 library.

Same signatures and return conventions as the reference (U, S, V with
A ~= U diag(S) V^T; q clamped to min(q, m, n)), plus an optional ``omega``
argument: the (n x q) N(0,1) test matrix.  When it is None it is drawn with
``torch.randn`` on the device, as the reference does
(acetn/linalg/fused_matmul_svd_lowrank.py:32).
"""

import torch

from . import _abi


def _omega(omega, n, q, device):
    if omega is None:
        return torch.randn(n, q, dtype=torch.float64, device=device)
    if omega.shape != (n, q):
        raise ValueError(f"omega must have shape {(n, q)}, got {tuple(omega.shape)}")
    return omega.to(device=device, dtype=torch.float64).contiguous()


def svd_lowrank(A, q=6, niter=2, omega=None):
    """acetn/linalg/svd_lowrank.py:4-44."""
    _abi.require_cuda(A, "A")
    A = A.contiguous()
    m, n = A.shape
    q = min(q, m, n)
    om = _omega(omega, n, q, A.device)
    U = torch.empty(m, q, dtype=torch.float64, device=A.device)
    S = torch.empty(q, dtype=torch.float64, device=A.device)
    V = torch.empty(n, q, dtype=torch.float64, device=A.device)
    _abi.call("ctm_svd_lowrank", [_abi.ptr(A), m, n, q, niter, _abi.ptr(om), _abi.ptr(U),
                                  _abi.ptr(S), _abi.ptr(V)], A.device)
    return U, S, V


def fused_matmul_svd_lowrank(A, B, q=6, niter=2, omega=None, precision="fp64"):
    """acetn/linalg/fused_matmul_svd_lowrank.py:4-52."""
    _abi.require_cuda(A, "A")
    _abi.require_cuda(B, "B")
    A = A.contiguous()
    B = B.contiguous()
    m, k = A.shape
    k2, n = B.shape
    if k != k2:
        raise ValueError("A and B do not chain")
    q = min(q, m, n)
    om = _omega(omega, n, q, A.device)
    U = torch.empty(m, q, dtype=torch.float64, device=A.device)
    S = torch.empty(q, dtype=torch.float64, device=A.device)
    V = torch.empty(n, q, dtype=torch.float64, device=A.device)
    _abi.call("ctm_fused_matmul_svd_lowrank",
              [_abi.ptr(A), _abi.ptr(B), m, k, n, q, niter, _abi.ptr(om), _abi.ptr(U),
               _abi.ptr(S), _abi.ptr(V), _abi.PREC[precision]], A.device)
    return U, S, V


def fused_3matmul_svd_lowrank(A, B, C, D, q=6, niter=2, omega=None):
    """acetn/linalg/fused_3matmul_svd_lowrank.py:4-56."""
    for t, nm in ((A, "A"), (B, "B"), (C, "C"), (D, "D")):
        _abi.require_cuda(t, nm)
    A, B, C, D = (t.contiguous() for t in (A, B, C, D))
    m, k1 = A.shape
    if B.shape[0] != k1 or C.shape[0] != B.shape[1] or D.shape[0] != C.shape[1]:
        raise ValueError("factors do not chain")
    k2, k3, n = B.shape[1], C.shape[1], D.shape[1]
    q = min(q, m, n)
    om = _omega(omega, n, q, A.device)
    U = torch.empty(m, q, dtype=torch.float64, device=A.device)
    S = torch.empty(q, dtype=torch.float64, device=A.device)
    V = torch.empty(n, q, dtype=torch.float64, device=A.device)
    _abi.call("ctm_fused_3matmul_svd_lowrank",
              [_abi.ptr(A), _abi.ptr(B), _abi.ptr(C), _abi.ptr(D), m, k1, k2, k3, n, q, niter,
               _abi.ptr(om), _abi.ptr(U), _abi.ptr(S), _abi.ptr(V)], A.device)
    return U, S, V


def qr(A):
    """Thin QR (Q, R) of a tall float64 or float32 CUDA matrix, in the
    matrix's own precision: the ``torch.linalg.qr`` step of the range finders
    (acetn/linalg/svd_lowrank.py:36,39).  float32 is the arithmetic of the
    mixed path's range finder.  Columns of Q may differ in sign from LAPACK's."""
    if not isinstance(A, torch.Tensor) or not A.is_cuda:
        raise ValueError("A must be a CUDA tensor (the gb300 backend has no CPU path)")
    if A.dtype not in (torch.float64, torch.float32):
        raise ValueError(f"A must be float64 or float32, got {A.dtype}")
    n, q = A.shape
    if not n >= q >= 1:
        raise ValueError(f"qr needs rows >= columns >= 1, got {tuple(A.shape)}")
    Q = A.contiguous().clone()
    R = torch.empty(q, q, dtype=A.dtype, device=A.device)
    _abi.call("ctm_qr", [_abi.ptr(Q), n, q, _abi.ptr(R), 0 if A.dtype == torch.float64 else 1],
              A.device)
    return Q, R


def svd(A):
    """Thin SVD (U, S, V) of an FP64 matrix with at most 4096 rows and columns."""
    _abi.require_cuda(A, "A")
    A = A.contiguous()
    m, n = A.shape
    r = min(m, n)
    U = torch.empty(m, r, dtype=torch.float64, device=A.device)
    S = torch.empty(r, dtype=torch.float64, device=A.device)
    V = torch.empty(n, r, dtype=torch.float64, device=A.device)
    _abi.call("ctm_svd_f64", [_abi.ptr(A), m, n, _abi.ptr(U), _abi.ptr(S), _abi.ptr(V)], A.device)
    return U, S, V


def svd_f32(Bt):
    """SVD (U, S, V) of B = Bt^T for a float32 CUDA matrix Bt (n x q, n >= q):
    the FP32 Rayleigh-Ritz SVD of the mixed path (Cholesky-QR3 of Bt, then
    one-sided Jacobi).  U (q x q) and S in float64, V (n x q) in float32,
    B ~= U diag(S) V^T, S descending."""
    if not isinstance(Bt, torch.Tensor) or not Bt.is_cuda or Bt.dtype != torch.float32:
        raise ValueError("Bt must be a float32 CUDA tensor")
    Bt = Bt.contiguous()
    n, q = Bt.shape
    if not n >= q >= 1:
        raise ValueError(f"svd_f32 needs rows >= columns >= 1, got {tuple(Bt.shape)}")
    U = torch.empty(q, q, dtype=torch.float64, device=Bt.device)
    S = torch.empty(q, dtype=torch.float64, device=Bt.device)
    V = torch.empty(n, q, dtype=torch.float32, device=Bt.device)
    _abi.call("ctm_svd_f32", [_abi.ptr(Bt), n, q, _abi.ptr(U), _abi.ptr(S), _abi.ptr(V)],
              Bt.device)
    return U, S, V


def matmul(A, B, precision="fp64"):
    """A @ B with the library's FP64 or mixed-precision GEMM engine."""
    _abi.require_cuda(A, "A")
    _abi.require_cuda(B, "B")
    A = A.contiguous()
    B = B.contiguous()
    M, K = A.shape
    K2, N = B.shape
    if K != K2:
        raise ValueError("A and B do not chain")
    C = torch.empty(M, N, dtype=torch.float64, device=A.device)
    _abi.call("ctm_matmul", [_abi.ptr(A), _abi.ptr(B), _abi.ptr(C), M, N, K,
                             _abi.PREC[precision]], A.device)
    return C
