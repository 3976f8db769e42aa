"""Thin QR (``qr``, the torch.linalg.qr step of the range finders,
acetn/linalg/svd_lowrank.py:36,39) in FP64 and FP32 against numpy's QR in
float64: orthonormal Q, Y = Q R with R upper triangular, the same column
space, and no Householder fallback for inputs whose condition number the
shifted Cholesky-QR3 covers.  Shapes cover the single-CTA Householder branch,
the FP64 Cholesky-QR, and the FP32 slab kernels with q a multiple of 32, of 4
(16-byte copies) and odd (4-byte copies, scalar Gram reduction)."""

import numpy as np
import pytest
import torch

import acetn_gb300 as gb
from acetn_gb300 import _abi

pytestmark = pytest.mark.gpu


def conditioned(n, q, cond, seed):
    rng = np.random.default_rng(seed)
    u, _ = np.linalg.qr(rng.standard_normal((n, q)))
    v, _ = np.linalg.qr(rng.standard_normal((q, q)))
    s = np.logspace(0, -np.log10(cond), q)
    return (u * s) @ v.T


CASES = [
    # (n, q, dtype, cond, orthogonality tol, reconstruction tol)
    (300, 40, torch.float64, 1e6, 1e-12, 1e-12),     # Householder branch (n q^2 <= 4e6)
    (5184, 160, torch.float64, 1e6, 1e-12, 1e-12),   # FP64 Cholesky-QR3
    (5184, 160, torch.float32, 1e4, 1e-4, 5e-6),     # FP32 slabs, q % 32 == 0
    (5184, 148, torch.float32, 1e4, 1e-4, 5e-6),     # q % 4 == 0, partial column tile
    (3001, 147, torch.float32, 1e4, 1e-4, 5e-6),     # odd q, ragged last slab
    (12000, 192, torch.float32, 1e3, 1e-4, 5e-6),    # 64-row slabs, several waves
    (4000, 37, torch.float32, 1e3, 1e-4, 5e-6),      # two column tiles, 27-row slabs
]


@pytest.mark.parametrize("n,q,dtype,cond,otol,rtol", CASES)
def test_qr_orthonormal_and_reconstructs(n, q, dtype, cond, otol, rtol):
    y64 = conditioned(n, q, cond, n + q)
    Y = torch.from_numpy(y64).to("cuda", dtype)
    _abi.qr_fallbacks()  # reading clears the counter
    Q, R = gb.qr(Y)
    torch.cuda.synchronize()
    assert _abi.qr_fallbacks() == 0
    assert Q.dtype == dtype and Q.shape == (n, q) and R.shape == (q, q)
    q64, r64 = Q.double().cpu().numpy(), R.double().cpu().numpy()
    orth = np.abs(q64.T @ q64 - np.eye(q)).max()
    assert orth < otol, orth
    assert np.all(np.tril(r64, -1) == 0.0)
    yin = Y.double().cpu().numpy()
    rec = np.abs(q64 @ r64 - yin).max() / np.abs(yin).max()
    assert rec < rtol, rec
    # same column space as LAPACK's QR of the input
    qref, _ = np.linalg.qr(yin)
    proj = np.abs(qref @ (qref.T @ q64) - q64).max()
    assert proj < 10 * otol + cond * rtol, proj


def test_qr_rejects_bad_input():
    with pytest.raises(ValueError):
        gb.qr(torch.zeros(3, 5, dtype=torch.float64, device="cuda"))
    with pytest.raises(ValueError):
        gb.qr(torch.zeros(8, 4, dtype=torch.float16, device="cuda"))
    with pytest.raises(ValueError):
        gb.qr(torch.zeros(8, 4, dtype=torch.float64))
