"""ctm_move_batched, the C entry point for a whole move (or a left/right,
up/down pair of moves) of the unit cell, called through the C ABI against
the Python DirectionalMover in its fixed-width form with the same test
matrices: the new corner and edge tensors must be identical (the same
kernels in the same order), for FP64 and the mixed form."""

import ctypes

import pytest
import torch

import acetn_gb300 as gb
from acetn_gb300 import _abi

pytestmark = pytest.mark.gpu


def clone(st):
    c = gb.IpepsState(st.nx, st.ny, st.dims, st.device)
    for s in st.site_list:
        v = st[s]
        c[s] = {"A": v["A"].clone(), "C": [t.clone() for t in v["C"]],
                "E": [t.clone() for t in v["E"]]}
    return c


def run_c(st, moves, cfg, omegas):
    """One call of ctm_move_batched; returns {(site, 'C'|'E', k): tensor}."""
    nx, ny, chi = st.nx, st.ny, st.dims["chi"]
    refs = [_abi.SiteRef(st[(x, y)]) for x in range(nx) for y in range(ny)]
    arr = (_abi.CtmSite * len(refs))(*[r.s for r in refs])
    D, d = refs[0].D, refs[0].d
    opts = _abi.opts_struct(cfg, chi, cfg.precision, fixed_width=True)
    mv = gb.DirectionalMover(cfg)
    specs = [mv._spec(st, k, idx) for k, idx in moves]
    outs, keep, targets = [], [], []
    om_ptrs = []
    t = 0
    for k, site_lists, jobs in specs:
        for sites, (s1, s2, i, j) in zip(site_lists, jobs):
            srefs = [_abi.SiteRef(st[s]) for s in sites]
            sarr = (_abi.SITE_P * 4)(*[r.pointer for r in srefs])
            p1r, p2r, nr, q, cap = (_abi.c_i64() for _ in range(5))
            _abi.check(_abi.load().ctm_projector_dims(sarr, D, k, ctypes.byref(opts),
                                                      ctypes.byref(p1r), ctypes.byref(p2r),
                                                      ctypes.byref(nr), ctypes.byref(q),
                                                      ctypes.byref(cap)), "dims")
            om = omegas[t].contiguous()
            keep.append(om)
            om_ptrs.append(om.data_ptr())
            cap = cap.value
            a = st[s1]["E"][(2 + k) % 4].shape[0]
            cc = st[s1]["E"][k % 4].shape[1]
            c1 = torch.empty(a, cap, dtype=torch.float64, device="cuda")
            c2 = torch.empty(cap, cc, dtype=torch.float64, device="cuda")
            e3 = torch.empty(cap, cap, D, D, dtype=torch.float64, device="cuda")
            outs += [c1, c2, e3]
            targets += [(s2, "C", (3 + k) % 4), (s2, "C", k), (s2, "E", (3 + k) % 4)]
            t += 1
    mv_arr = (ctypes.c_int32 * (2 * len(moves)))(*[v for m in moves for v in m])
    om_arr = (ctypes.c_void_p * len(om_ptrs))(*om_ptrs)
    out_arr = (ctypes.c_void_p * len(outs))(*[x.data_ptr() for x in outs])
    chi_new = torch.zeros(t, dtype=torch.int64, device="cuda")
    _abi.call("ctm_move_batched", [arr, nx, ny, D, d, mv_arr, len(moves), ctypes.byref(opts),
                                   om_arr, out_arr, ctypes.c_void_p(chi_new.data_ptr())],
              torch.device("cuda"))
    torch.cuda.synchronize()
    return dict(zip(targets, outs)), chi_new.cpu().tolist()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("moves", [[(0, 0)], [(0, 1), (2, 0)], [(1, 1), (3, 0)]])
def test_move_batched_equals_python_mover(precision, moves):
    gb.build()
    cfg = gb.CTMRGConfig(precision=precision, rsvd_oversampling=4, disable_progressbar=True)
    st = gb.random_state(3, 9, 21, device="cuda")
    gb.ctmrg(st, gb.CTMRGConfig(rsvd_oversampling=4, steps=2, disable_progressbar=True))
    g = torch.Generator(device="cuda")
    g.manual_seed(5)
    omegas = [torch.randn(9 * 9, 13, dtype=torch.float64, device="cuda", generator=g)
              for _ in range(4)]
    got, counts = run_c(st, moves, cfg, omegas)
    feed = iter(omegas)
    py = clone(st)
    mv = gb.DirectionalMover(cfg, omega_source=lambda n, q, dev: next(feed)[:n, :q].contiguous())
    mv.graph_mode = True
    if len(moves) == 1:
        mv.move(py, *moves[0])
    else:
        mv.moves_at_once(py, moves)
    torch.cuda.synchronize()
    assert counts == mv.last_counts.cpu().tolist()
    for (s, key, k), t in got.items():
        assert torch.equal(t, py[s][key][k]), (s, key, k)
    assert gb._abi.device_status() == 0


def test_move_batched_rejects_a_bad_pair():
    st = gb.random_state(2, 4, 1, device="cuda")
    cfg = gb.CTMRGConfig(disable_progressbar=True)
    with pytest.raises(ValueError):
        run_c(st, [(0, 0), (1, 0)], cfg, [torch.zeros(16, 6, dtype=torch.float64,
                                                      device="cuda")] * 4)
