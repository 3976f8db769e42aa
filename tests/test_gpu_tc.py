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


@pytest.mark.parametrize("rows,cols,ld_src,ld_dst", [
    (64, 64, 64, 64),          # one cell
    (5184, 160, 192, 5184),    # a quarter-tensor-like tall operand
    (81, 81, 128, 128),        # odd sizes: ragged cells, the last word half padding
    (100, 37, 37, 101),        # odd leading dimensions: element-wise loads and stores
    (1, 70, 70, 2),            # a single row
    (130, 1, 1, 130),          # a single column
])
def test_transpose_bf16_exact(rows, cols, ld_src, ld_dst):
    """The BF16 transpose of the quarter-tensor operands (64 x 64 cells,
    2 x 2 blocks transposed from 32-bit words): dst == src^T bit for bit,
    for the hi and the lo array, and nothing written past the transposed
    block's rows."""
    import ctypes
    from acetn_gb300 import _abi
    lib = _abi.load()
    fn = lib.ctm_test_transpose_bf16
    fn.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64,
                   ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64,
                   ctypes.c_void_p]
    fn.restype = ctypes.c_int
    g = torch.Generator().manual_seed(rows * 1000 + cols)
    src = [torch.randn(rows, ld_src, generator=g).to(torch.bfloat16).cuda() for _ in range(2)]
    sentinel = torch.tensor(7.0, dtype=torch.bfloat16)
    dst = [torch.full((cols + 1, ld_dst), float(sentinel), dtype=torch.bfloat16, device="cuda")
           for _ in range(2)]
    st = fn(src[0].data_ptr(), src[1].data_ptr(), rows, cols, ld_src, dst[0].data_ptr(),
            dst[1].data_ptr(), ld_dst, ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert st == 0, lib.ctm_last_error()
    torch.cuda.synchronize()
    for s, d in zip(src, dst):
        assert torch.equal(d[:cols, :rows], s[:, :cols].t())
        assert torch.all(d[cols] == sentinel)  # the row after the last is untouched
