"""The one-layer form of the mixed path's site-tensor steps (the reference's
two einsums, K = D^2 and D^2 d, as two tensor-core GEMMs) against the FP64
path and against the double-layer form: enlarged corners (max-normalised,
2e-5 as for the double-layer form) at D = 3, 4 and 6, and one move's energy
(1e-5) and edge-tensor spectra (1e-3, the truncated rSVD's amplification of
rounding) at D = 4, through the C ABI."""

import numpy as np
import pytest
import torch

import acetn_gb300 as gb
from _golden import bond_energies, gpu_state, load
from oracle import ctm_oracle as orc

pytestmark = pytest.mark.gpu


def omega_from(seed):
    s = orc.OmegaStream(seed)
    return lambda n, q, dev: torch.from_numpy(s(n, q)).to(dev)


def clone(st):
    g = gb.IpepsState(st.nx, st.ny, st.dims, st.device)
    for s in st.site_list:
        v = st[s]
        g[s] = {"A": v["A"].clone(), "C": [c.clone() for c in v["C"]],
                "E": [e.clone() for e in v["E"]]}
    return g


@pytest.fixture(autouse=True)
def restore_form():
    gb.build()
    prev = gb._abi.set_mixed_contraction("auto")
    yield
    gb._abi.set_mixed_contraction(prev)


def states():
    out = [gpu_state(load("move_d3_chi9.npz"), 9)]
    st = gb.random_state(4, 32, 1234, device="cuda")
    gb.ctmrg(st, gb.CTMRGConfig(rsvd_oversampling=4, steps=2, disable_progressbar=True),
             omega_source=omega_from(1))
    out.append(st)
    return out


def test_one_layer_quarter_tensor_matches_fp64_and_double_layer():
    for st in states():
        for k in range(4):
            q64, _ = gb.ProjectorCalculator.make_quarter_tensor(st[(0, 0)], k)
            gb._abi.set_mixed_contraction("one-layer")
            q1, _ = gb.ProjectorCalculator.make_quarter_tensor(st[(0, 0)], k, precision="mixed")
            gb._abi.set_mixed_contraction("double-layer")
            q2, _ = gb.ProjectorCalculator.make_quarter_tensor(st[(0, 0)], k, precision="mixed")
            m = q64.abs().max()
            assert float((q64 - q1).abs().max() / m) < 2e-5
            assert float((q1 - q2).abs().max() / m) < 2e-5
    assert gb._abi.device_status() == 0


@pytest.mark.parametrize("k", range(4))
def test_one_layer_move_matches_double_layer(k):
    st = states()[1]
    cfg = gb.CTMRGConfig(precision="mixed", rsvd_oversampling=4, disable_progressbar=True)
    out = {}
    for form in ("one-layer", "double-layer"):
        gb._abi.set_mixed_contraction(form)
        s1 = clone(st)
        gb.DirectionalMover(cfg, omega_source=omega_from(40 + k)).move(s1, k, 0)
        out[form] = (s1, bond_energies(s1))
    (a, ea), (b, eb) = out["one-layer"], out["double-layer"]
    # per bond, against the largest |bond energy|: each mixed form sits at
    # 1-2e-5 of it from the FP64 move on this state (measured 1.2e-5 apart)
    assert float(np.abs(ea - eb).max()) <= 5e-5 * float(np.abs(eb).max())
    for s in st.site_list:
        for kk in range(4):
            x = np.linalg.svd(a[s]["E"][kk].reshape(a[s]["E"][kk].shape[0], -1).cpu().numpy(),
                              compute_uv=False)
            y = np.linalg.svd(b[s]["E"][kk].reshape(b[s]["E"][kk].shape[0], -1).cpu().numpy(),
                              compute_uv=False)
            # the projectors of the two forms differ by their rounding, which
            # the truncated rSVD amplifies (measured 2e-4 of the largest value)
            assert np.abs(x - y).max() < 1e-3 * y.max()
    assert gb._abi.device_status() == 0


def test_one_layer_quarter_tensor_d6_chi144():
    ref = gb.random_state(6, 144, 99, device="cuda")
    st = gb.IpepsState(2, 2, {"phys": 2, "bond": 6, "chi": 144}, "cuda")
    g = torch.Generator().manual_seed(99)

    def rnd(*shape):
        t = torch.randn(*shape, generator=g, dtype=torch.float64)
        return (t / t.norm()).cuda()

    for s in ref.site_list:
        st[s] = {"A": ref[s]["A"], "C": [rnd(144, 144) for _ in range(4)],
                 "E": [rnd(144, 144, 6, 6) for _ in range(4)]}
    q64, _ = gb.ProjectorCalculator.make_quarter_tensor(st[(0, 0)], 1)
    gb._abi.set_mixed_contraction("one-layer")
    q1, _ = gb.ProjectorCalculator.make_quarter_tensor(st[(0, 0)], 1, precision="mixed")
    assert float((q64 - q1).abs().max() / q64.abs().max()) < 2e-5
    assert gb._abi.device_status() == 0


def test_contraction_form_is_validated():
    with pytest.raises(ValueError):
        gb._abi.set_mixed_contraction("three-layer")
