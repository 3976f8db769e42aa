"""tcgen05 tensor-core GEMM engine against torch references.

BF16 mode is compared with the FP64 product of BF16-representable inputs
(tolerance 1e-5 relative: FP32 accumulation); 3xBF16 mode with the FP64
product of general inputs (tolerance 5e-5 normwise: about 16 significant
bits per operand)."""

import pytest
import torch

import acetn_gb300 as gb

pytestmark = pytest.mark.gpu

SHAPES = [(128, 16, 64), (256, 160, 512), (1000, 150, 777), (300, 272, 1000), (5184, 160, 5184)]
# long products with more output tiles than SMs: a direct (no split-K)
# epilogue in the persistent kernel (one CTA per SM walking the tiles, the
# accumulator double-buffered in tensor memory); 1300 rows leave a partial
# row tile
LONG_SHAPES = [(1024, 5120, 1000), (1300, 5120, 1000)]


def _rand(m, n, seed):
    g = torch.Generator().manual_seed(seed)
    return torch.randn(m, n, generator=g, dtype=torch.float64).cuda()


@pytest.mark.parametrize("m,n,k", SHAPES + LONG_SHAPES)
def test_bf16_single_pass(m, n, k):
    # inputs exactly representable in BF16: the only error left is the FP32
    # accumulation of exact products
    A = _rand(m, k, 1).to(torch.bfloat16).double()
    B = _rand(k, n, 2).to(torch.bfloat16).double()
    C = gb.matmul(A, B, precision="bf16")
    ref = A @ B
    err = (C - ref).abs().max() / ref.abs().max()
    assert err < 1e-5, float(err)


@pytest.mark.parametrize("m,n,k", SHAPES + LONG_SHAPES)
def test_split_bf16x3(m, n, k):
    A, B = _rand(m, k, 3), _rand(k, n, 4)
    C = gb.matmul(A, B, precision="mixed")
    ref = A @ B
    err = torch.linalg.norm(C - ref) / torch.linalg.norm(ref)
    assert err < 5e-5, float(err)
    one = gb.matmul(A, B, precision="bf16")
    err1 = torch.linalg.norm(one - ref) / torch.linalg.norm(ref)
    assert err < 0.05 * err1  # the split really adds the low-order products


def test_no_timeout_flags():
    A, B = _rand(512, 64, 5), _rand(64, 96, 6)
    gb.matmul(A, B, precision="mixed")
    assert gb._abi.device_status() == 0
