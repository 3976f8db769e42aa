"""The full update's two uses of the CTMRG path, through the C ABI.

* The norm tensor against golden vectors written by the reference's own
  build_norm_tensor and build_norm_tensor_core_blocked
  (tests/golden/make_norm_tensor.py), both bond directions, to 1e-12.
* absorb_bond (FastFullUpdater.absorb_bond) run as one pair of moves against
  the oracle's two sequential moves with the same rSVD test matrices, for
  all four bond directions: energy, corner spectra and bond RDMs to 1e-10.
"""

import numpy as np
import pytest
import torch

import acetn_gb300 as gb
from _golden import load, rel
from oracle import ctm_oracle as orc

pytestmark = pytest.mark.gpu

CFG = dict(projectors="half-system", svd_type="rsvd", rsvd_oversampling=2, rsvd_niter=2,
           svd_cutoff=1e-12)


def omega_from(stream):
    return lambda n, q, device: torch.from_numpy(stream(n, q)).to(device)


@pytest.fixture(scope="module", autouse=True)
def built():
    gb.build()
    assert torch.cuda.is_available()


@pytest.mark.parametrize("k,s1,s2", [(2, (0, 0), (1, 0)), (1, (0, 0), (0, 1))])
def test_norm_tensor_matches_reference_golden(k, s1, s2):
    z = load("norm_tensor_d2.npz")
    sites = {}
    for s in [(0, 0), (0, 1), (1, 0), (1, 1)]:
        key = f"{s[0]}_{s[1]}"
        sites[s] = {"A": z[f"{key}_A"], "C": [z[f"{key}_C{i}"] for i in range(4)],
                    "E": [z[f"{key}_E{i}"] for i in range(4)]}
    st = gb.IpepsState.from_arrays(sites, 2, 2, sites[(0, 0)]["C"][0].shape[0])
    a1q = torch.from_numpy(z[f"k{k}_a1q"]).cuda()
    a2q = torch.from_numpy(z[f"k{k}_a2q"]).cuda()
    n12 = gb.build_norm_tensor(st, (s1, s2, k), a1q, a2q).cpu().numpy()
    assert rel(n12, z[f"k{k}_n12"]) < 1e-12
    assert rel(n12, z[f"k{k}_n12_blocked"]) < 1e-12
    assert gb._abi.device_status() == 0


def test_norm_tensor_rejects_bad_shapes():
    st = gb.random_state(2, 4, 1, device="cuda")
    a = torch.zeros(2, 2, 3, 4, dtype=torch.float64, device="cuda")
    with pytest.raises(ValueError):
        gb.build_norm_tensor(st, ((0, 0), (1, 0), 2), a, a)


@pytest.mark.parametrize("k", [0, 1, 2, 3])
def test_absorb_bond_matches_two_sequential_oracle_moves(k):
    ost = orc.random_state(3, 9, seed=31)
    orc.ctmrg(ost, dict(CFG, svd_type="full-rank"), orc.OmegaStream(0), steps=2)
    gst = gb.IpepsState.from_arrays(ost.copy().sites, 2, 2, 9)
    s1, s2 = {0: ((1, 0), (0, 0)), 1: ((0, 1), (0, 0)), 2: ((0, 0), (1, 0)),
              3: ((0, 0), (0, 1))}[k]
    seq = {0: [(2, s1[0]), (0, s2[0])], 1: [(3, s1[1]), (1, s2[1])],
           2: [(0, s1[0]), (2, s2[0])], 3: [(1, s1[1]), (3, s2[1])]}[k]
    om = orc.OmegaStream(70 + k)
    mover = orc.Mover(CFG, om)
    for kk, idx in seq:
        mover.move(ost, kk, idx)
    gb.absorb_bond(gb.DirectionalMover(gb.CTMRGConfig(**CFG),
                                       omega_source=omega_from(orc.OmegaStream(70 + k))),
                   gst, (s1, s2, k))
    e = float(gb.measure(gst, gb.HeisenbergModel(1.0), verbose=False)["Energy"])
    e_ref = orc.measure(ost, orc.heisenberg_model(1.0))["Energy"]
    assert abs(e - e_ref) <= 1e-10 * abs(e_ref)
    for s in ost.sites:
        for kk in range(4):
            a = np.linalg.svd(gst[s]["C"][kk].cpu().numpy(), compute_uv=False)
            b = np.linalg.svd(ost[s]["C"][kk], compute_uv=False)
            assert rel(a / a[0], b / b[0]) < 1e-10
    rdm = gb.RDM(gst)
    for b in gst.bond_list:
        r = rdm[b].cpu().numpy()
        r_ref = orc.bond_rdm(ost, b.s1, b.s2, b.k)
        assert np.abs(r / np.einsum("pqpq->", r) - r_ref / np.einsum("pqpq->", r_ref)).max() < 1e-10
    assert gb._abi.device_status() == 0
