"""The FP32 Rayleigh-Ritz SVD of the mixed path (``svd_f32``: Cholesky-QR3 of
B^T and one-sided Jacobi; an 8-CTA cluster Jacobi from q = 96) against
numpy's float64 SVD, on matrices with the graded spectrum of a converged
D=6, chi=144 environment (s/s0 from 1 down to ~2e-4) and on a flat one.
The bar: singular values to 2e-6 of s0 and U orthogonal to 5e-6 (FP32
rotations in Rutishauser's form: a numpy model of the kernel gives 5e-7 and
8e-7 at q = 100; the plain c x - s y form drifts the row norms by ~1e-4), the
reconstruction to 1e-5, the leading singular vectors to 1e-6, no
iteration-limit flag."""

import numpy as np
import pytest
import torch

import acetn_gb300 as gb
from acetn_gb300 import _abi

pytestmark = pytest.mark.gpu


def graded(q):
    x = np.arange(q)
    pts = [(0, 0.0), (0.225, -2.7), (0.45, -3.2), (0.9, -3.55), (1.0, -3.62)]
    xs = [p[0] * (q - 1) for p in pts]
    return 10 ** np.interp(x, xs, [p[1] for p in pts])


def make_bt(n, q, s, seed):
    rng = np.random.default_rng(seed)
    v, _ = np.linalg.qr(rng.standard_normal((n, q)))
    u, _ = np.linalg.qr(rng.standard_normal((q, q)))
    return (v * s) @ u.T  # B^T = V S U^T


@pytest.mark.parametrize("n,q,kind", [(1000, 36, "graded"), (1600, 100, "graded"),
                                      (5184, 160, "graded"), (5184, 160, "flat"),
                                      (3000, 224, "graded")])
def test_svd_f32_matches_float64(n, q, kind):
    s_true = graded(q) if kind == "graded" else np.linspace(1.0, 0.7, q)
    bt64 = make_bt(n, q, s_true, q + n)
    bt = torch.from_numpy(bt64).to("cuda", torch.float32)
    _abi.device_status()  # clears earlier flags
    U, S, V = gb.linalg.svd_f32(bt)
    torch.cuda.synchronize()
    assert _abi.device_status() == 0
    b32 = bt.double().cpu().numpy().T  # the rounded input, q x n
    s_ref = np.linalg.svd(b32, compute_uv=False)
    U, S, V = U.cpu().numpy(), S.cpu().numpy(), V.double().cpu().numpy()
    assert np.all(np.diff(S) <= 0)
    assert np.abs(S - s_ref).max() / s_ref[0] < 2e-6
    assert np.abs(U.T @ U - np.eye(q)).max() < 5e-6
    rec = np.abs((U * S) @ V.T - b32).max() / np.abs(b32).max()
    assert rec < 1e-5, rec
    # leading singular vectors (well separated in both spectra)
    u_ref = np.linalg.svd(b32, full_matrices=False)[0]
    top = 8 if kind == "graded" else 4
    align = np.abs(np.sum(U[:, :top] * u_ref[:, :top], axis=0))
    assert np.all(1.0 - align < 1e-6), align


def test_svd_f32_rejects_bad_input():
    with pytest.raises(ValueError):
        gb.linalg.svd_f32(torch.zeros(3, 5, dtype=torch.float32, device="cuda"))
    with pytest.raises(ValueError):
        gb.linalg.svd_f32(torch.zeros(8, 4, dtype=torch.float64, device="cuda"))
