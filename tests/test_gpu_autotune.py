"""Tile-plan autotuner of the tensor-core GEMMs.

The tuner picks, per product shape, between 256- and 128-column N tiles and
between a K split that fills the SMs and none.  Every candidate computes the
same 3xBF16 product (only the FP32 summation order inside a K split
differs: ~sqrt(K) FP32 roundings), so a tuned product is checked against the
FP64 product at the engine's own 3xBF16 tolerance (5e-5 normwise) and
against the untuned plan at 2e-5 normwise; repeated calls with the tuned
plan are bitwise equal.
Calls under stream capture never tune."""

import pytest
import torch

import acetn_gb300 as gb

pytestmark = pytest.mark.gpu

# (M, N, K): a long-K product with few output tiles (the default plan splits
# K), a wide product (N tiles of 256 or 128 columns differ), a persistent one
SHAPES = [(512, 200, 20000), (1000, 512, 777), (2048, 5120, 1000)]


def _rand(m, n, seed):
    g = torch.Generator().manual_seed(seed)
    return torch.randn(m, n, generator=g, dtype=torch.float64).cuda()


@pytest.fixture
def tuner():
    gb.autotune(False, reset=True)
    yield
    gb.autotune(False, reset=True)


@pytest.mark.parametrize("m,n,k", SHAPES)
def test_tuned_product_matches(tuner, m, n, k):
    A, B = _rand(m, k, 11), _rand(k, n, 12)
    plain = gb.matmul(A, B, precision="mixed")
    assert gb.autotune(True) == 0
    tuned = gb.matmul(A, B, precision="mixed")
    table = gb.autotune_table()
    assert len(table) == 1
    row = table[0]
    assert (row["M"], row["N"], row["K"], row["passes"]) == (m, n, k, 3)
    assert 0 <= row["choice"] < 4
    assert 0 < row["best_ms"] <= row["default_ms"]
    again = gb.matmul(A, B, precision="mixed")
    assert torch.equal(tuned, again)
    ref = A @ B
    assert float(torch.linalg.norm(tuned - ref) / torch.linalg.norm(ref)) < 5e-5
    assert float(torch.linalg.norm(tuned - plain) / torch.linalg.norm(plain)) < 2e-5
    assert gb._abi.device_status() == 0


def test_capture_does_not_tune(tuner):
    A, B = _rand(768, 300, 13), _rand(300, 4000, 14)
    eager = gb.matmul(A, B, precision="mixed")  # sizes the workspace outside capture
    gb.autotune(True)
    C = torch.empty_like(eager)
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        C.copy_(gb.matmul(A, B, precision="mixed"))
    g.replay()
    torch.cuda.synchronize()
    assert gb.autotune_table() == []
    assert torch.equal(C, eager)


def _fixed_omega():
    g = torch.Generator(device="cuda")
    g.manual_seed(3)
    full = torch.randn(4096, 128, dtype=torch.float64, device="cuda", generator=g)
    return lambda n, q, dev: full[:n, :q].contiguous()


def test_tuned_mixed_moves(tuner):
    """One pair of mixed moves from a grown state with the tuner on (every
    product shape of the move is tuned on the spot) against the same pair
    untuned: the leading corner singular values agree to 1e-5 relative.  (The
    trailing ones are not compared: near the truncation a 1e-7 change of a
    product can rotate the kept subspace.)"""
    cfg = gb.CTMRGConfig(steps=4, precision="mixed", rsvd_oversampling=4,
                         disable_progressbar=True)
    st = gb.random_state(4, 48, 21, device="cuda")
    gb.ctmrg(st, cfg, omega_source=_fixed_omega())
    results = []
    for tune in (False, True):
        g = gb.IpepsState(st.nx, st.ny, st.dims, st.device)
        for s in st.site_list:
            v = st[s]
            g[s] = {"A": v["A"].clone(), "C": [c.clone() for c in v["C"]],
                    "E": [e.clone() for e in v["E"]]}
        gb.autotune(tune, reset=True)
        mover = gb.DirectionalMover(cfg, omega_source=_fixed_omega())
        mover.move_pair(g, *gb.pair_order(2, 2)[0])
        torch.cuda.synchronize()
        results.append([torch.linalg.svdvals(g[s]["C"][k])[:8] for s in g.site_list
                        for k in range(4)])
        if tune:
            assert len(gb.autotune_table()) > 0
    assert gb._abi.device_status() == 0
    for a, b in zip(*results):
        assert float(((a - b) / a[0]).abs().max()) < 1e-5
