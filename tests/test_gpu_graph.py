"""CUDA-graph capture of a CTMRG iteration (CTMRGGraph) against the eager
fixed-width path: with the same test matrices, replays must reproduce the
eager iterations exactly (same kernels, deterministic reductions).  The
left/right and up/down pairs of moves run at once must equal the reference's
sequential order bit for bit."""

import pytest
import torch

import acetn_gb300 as gb

pytestmark = pytest.mark.gpu


def clone(st):
    g = gb.IpepsState(st.nx, st.ny, st.dims, st.device)
    for s in st.site_list:
        v = st[s]
        g[s] = {"A": v["A"].clone(), "C": [c.clone() for c in v["C"]],
                "E": [e.clone() for e in v["E"]]}
    return g


def fixed_omega():
    g = torch.Generator(device="cuda")
    g.manual_seed(3)
    full = torch.randn(4096, 128, dtype=torch.float64, device="cuda", generator=g)
    return lambda n, q, dev: full[:n, :q].contiguous()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_graph_replay_matches_eager(precision):
    cfg = gb.CTMRGConfig(precision=precision, rsvd_oversampling=4, disable_progressbar=True)
    st = gb.random_state(3, 9, 5, device="cuda")
    gb.ctmrg(st, gb.CTMRGConfig(steps=3, rsvd_oversampling=4, disable_progressbar=True),
             omega_source=fixed_omega())
    eager = clone(st)
    mover = gb.DirectionalMover(cfg, omega_source=fixed_omega())
    mover.graph_mode = True
    for _ in range(2):
        for k, idx in gb.sweep_order(2, 2):
            mover.move(eager, k, idx)
    graphed = clone(st)
    g = gb.CTMRGGraph(graphed, cfg, omega_source=fixed_omega()).capture(warmup=0)
    g.replay(2)
    torch.cuda.synchronize()
    for s in st.site_list:
        for k in range(4):
            assert torch.equal(graphed[s]["C"][k], eager[s]["C"][k])
            assert torch.equal(graphed[s]["E"][k], eager[s]["E"][k])
    assert not g.truncated()
    e1 = float(gb.measure(graphed, gb.HeisenbergModel(1.0), verbose=False)["Energy"])
    e2 = float(gb.measure(eager, gb.HeisenbergModel(1.0), verbose=False)["Energy"])
    assert e1 == e2


def omega_stream(seed):
    g = torch.Generator(device="cuda")
    g.manual_seed(seed)
    return lambda n, q, dev: torch.randn(n, q, dtype=torch.float64, device=dev, generator=g)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_pairs_of_moves_equal_sequential_moves(precision):
    cfg = gb.CTMRGConfig(precision=precision, rsvd_oversampling=4, steps=3,
                         disable_progressbar=True)
    st = gb.random_state(3, 9, 5, device="cuda")
    a, b = clone(st), clone(st)
    gb.ctmrg(a, cfg, omega_source=omega_stream(11), pairs=True)
    gb.ctmrg(b, cfg, omega_source=omega_stream(11), pairs=False)
    torch.cuda.synchronize()
    for s in st.site_list:
        for k in range(4):
            assert torch.equal(a[s]["C"][k], b[s]["C"][k])
            assert torch.equal(a[s]["E"][k], b[s]["E"][k])


def test_graph_capture_requires_saturated_environment():
    st = gb.random_state(3, 16, 5, device="cuda")  # C starts at D^2 = 9 < chi
    with pytest.raises(ValueError):
        gb.CTMRGGraph(st, gb.CTMRGConfig()).capture()
