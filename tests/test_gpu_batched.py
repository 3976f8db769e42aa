"""BatchedCTMRG: independent iPEPS of uneven D and chi (float32 storage,
FP64 projectors) advanced together on one GPU -- each instance on its own
stream, one iteration of all instances captured as one CUDA graph -- must
give every instance exactly what it gets alone with the same test matrices."""

import pytest
import torch

import acetn_gb300 as gb

pytestmark = pytest.mark.gpu


def fixed_omega(seed):
    g = torch.Generator(device="cuda")
    g.manual_seed(seed)
    full = torch.randn(2048, 64, dtype=torch.float64, device="cuda", generator=g)
    return lambda n, q, dev: full[:n, :q].contiguous()


def to_f32(st):
    c = gb.IpepsState(st.nx, st.ny, st.dims, st.device)
    for s in st.site_list:
        v = st[s]
        c[s] = {"A": v["A"].float(), "C": [t.float() for t in v["C"]],
                "E": [t.float() for t in v["E"]]}
    return c


def clone(st):
    c = gb.IpepsState(st.nx, st.ny, st.dims, st.device)
    for s in st.site_list:
        v = st[s]
        c[s] = {"A": v["A"].clone(), "C": [t.clone() for t in v["C"]],
                "E": [t.clone() for t in v["E"]]}
    return c


def test_batched_graph_equals_instances_run_alone():
    gb.build()
    cfg = gb.CTMRGConfig(precision="fp64", rsvd_oversampling=2, disable_progressbar=True)
    specs = [(3, 9, 11), (2, 12, 12), (4, 16, 13)]
    states = []
    for D, chi, seed in specs:
        st = to_f32(gb.random_state(D, chi, seed, bias=1e-2, device="cuda"))
        gb.ctmrg(st, cfg, omega_source=fixed_omega(seed), steps=3)
        states.append(st)
    alone = [clone(st) for st in states]
    for st, (_, _, seed) in zip(alone, specs):
        mv = gb.DirectionalMover(cfg, omega_source=fixed_omega(seed))
        mv.graph_mode = True
        for _ in range(2):
            for kind, i1, i2 in gb.pair_order(2, 2):
                mv.move_pair(st, kind, i1, i2)
    together = [clone(st) for st in states]
    b = gb.BatchedCTMRG(together, cfg, omega_sources=[fixed_omega(s) for _, _, s in specs])
    assert b.saturated()
    b.capture(warmup=0)
    b.replay(2)
    torch.cuda.synchronize()
    assert not b.truncated()
    for x, y in zip(together, alone):
        for s in x.site_list:
            for k in range(4):
                assert x[s]["C"][k].dtype == torch.float32
                assert torch.equal(x[s]["C"][k], y[s]["C"][k])
                assert torch.equal(x[s]["E"][k], y[s]["E"][k])
    assert b.moves_per_iteration() == 3 * 8
    assert gb._abi.device_status() == 0


def test_batched_needs_saturated_environments():
    cfg = gb.CTMRGConfig(precision="fp64", disable_progressbar=True)
    b = gb.BatchedCTMRG([gb.random_state(3, 16, 5, device="cuda")], cfg)
    with pytest.raises(ValueError):
        b.capture()
