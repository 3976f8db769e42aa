"""The oracle (oracle/ctm_oracle.py) against the reference's own outputs
(tests/golden, generated by make_golden.py) and the reference's published
ground-state energies.  CPU only."""

import numpy as np
import pytest

from oracle import ctm_oracle as orc
from _golden import SITES_K, load, oracle_state, rel

CFG = dict(projectors="half-system", svd_type="rsvd", rsvd_oversampling=2, rsvd_niter=2,
           svd_cutoff=1e-12)


def test_quarter_tensors():
    z = load("move_d3_chi9.npz")
    st = oracle_state(z, 9)
    for k in range(4):
        q, _ = orc.make_quarter_tensor(st[(0, 0)], k)
        assert rel(q, z[f"quarter_00_k{k}"]) < 1e-13


@pytest.mark.parametrize("proj", ["half-system", "full-system"])
@pytest.mark.parametrize("svd", ["rsvd", "full-rank"])
def test_projector_pairs(proj, svd):
    z = load("move_d3_chi9.npz")
    st = oracle_state(z, 9)
    cfg = dict(CFG, projectors=proj, svd_type=svd)
    fn = orc.calculate_half_system if proj == "half-system" else orc.calculate_full_system
    for k in range(4):
        p1, p2 = fn(st, SITES_K[k], k, cfg, orc.OmegaStream(1000 + k))
        ob = p2.reshape(-1, p2.shape[-1]) @ p1.reshape(-1, p1.shape[-1]).T
        tag = f"proj_{proj[:4]}_{svd[:4]}_k{k}"
        assert p1.shape[-1] == int(z[tag + "_chi"])
        assert rel(ob, z[tag + "_oblique"]) < 1e-10


def test_rsvd_variants():
    z = load("move_d3_chi9.npz")
    st = oracle_state(z, 9)
    q1, _ = orc.make_quarter_tensor(st[(0, 0)], 0)
    q4, _ = orc.make_quarter_tensor(st[(0, 1)], 3)
    q2, _ = orc.make_quarter_tensor(st[(1, 0)], 1)
    q3, _ = orc.make_quarter_tensor(st[(1, 1)], 2)
    u, s, v = orc.fused_matmul_svd_lowrank(q1, q4, 11, 2, orc.OmegaStream(77))
    assert rel(s, z["rsvd_fused_s"]) < 1e-12
    assert rel(u @ np.diag(s) @ v.T, z["rsvd_fused_usv"]) < 1e-12
    u, s, v = orc.svd_lowrank(q1, 11, 2, orc.OmegaStream(78))
    assert rel(s, z["rsvd_plain_s"]) < 1e-12
    u, s, v = orc.fused_3matmul_svd_lowrank(q2, q1, q4, q3, 11, 2, orc.OmegaStream(79))
    assert rel(s, z["rsvd_fused3_s"]) < 1e-12


@pytest.mark.parametrize("k,name", list(enumerate(("left", "up", "right", "down"))))
def test_single_moves(k, name):
    z = load("move_d3_chi9.npz")
    st = oracle_state(z, 9)
    orc.Mover(CFG, orc.OmegaStream(2000 + k)).move(st, k, 0)
    m = orc.measure(st, orc.heisenberg_model(1.0))
    e_ref = float(z[f"move_{name}_meas_Energy"])
    assert abs(m["Energy"] - e_ref) <= 1e-10 * abs(e_ref)
    for s in st.sites:
        for kk in range(4):
            sv = np.linalg.svd(st[s]["C"][kk], compute_uv=False)
            assert rel(sv / sv[0], z[f"move_{name}_spec_{s[0]}{s[1]}_C{kk}"]) < 1e-11


@pytest.mark.parametrize("fname,chi,model,cfg", [
    ("ctmrg_d2_chi20_fullrank.npz", 20, orc.heisenberg_model(1.0),
     dict(CFG, svd_type="full-rank", steps=30)),
    ("ctmrg_ising_d3_chi12_full.npz", 12, orc.ising_model(1.0, 3.0),
     dict(CFG, projectors="full-system", svd_type="full-rank", steps=10)),
])
def test_ctmrg_full_rank_runs(fname, chi, model, cfg):
    z = load(fname)
    st = oracle_state(z, chi)
    orc.ctmrg(st, cfg, orc.OmegaStream(5))
    m = orc.measure(st, model)
    e_ref = float(z["out_meas_Energy"])
    assert abs(m["Energy"] - e_ref) <= 1e-10 * abs(e_ref)
    for (s1, s2, k) in orc.build_bond_list(2, 2):
        r = orc.bond_rdm(st, s1, s2, k)
        r = r / np.einsum("pqpq->", r)
        tag = f"out_bond_rdm_{s1[0]}{s1[1]}_{s2[0]}{s2[1]}_{k}"
        assert np.abs(r - z[tag]).max() < 1e-10


def test_ctmrg_rsvd_run_within_noise_floor():
    """rSVD trajectories amplify rounding differences: 30 iterations agree with
    the reference only to ~1e-4 relative in the energy, even in FP64."""
    z = load("ctmrg_d2_chi20_rsvd.npz")
    st = oracle_state(z, 20)
    orc.ctmrg(st, dict(CFG, steps=30), orc.OmegaStream(5))
    e = orc.measure(st, orc.heisenberg_model(1.0))["Energy"]
    e_ref = float(z["out_meas_Energy"])
    assert abs(e - e_ref) <= 1e-3 * abs(e_ref)


@pytest.mark.parametrize("case,model", [
    ("ising_dims_2_20_dtau_001_hx_295", orc.ising_model(1.0, 2.95)),
    ("heisenberg_dims_3_16_dtau_001", orc.heisenberg_model(1.0)),
])
def test_ground_state_fixtures(case, model):
    z = load(f"gs_{case}.npz")
    chi = z["in_00_C0"].shape[0]
    st = oracle_state(z, chi)
    e_pub = float(z["published_energy"])
    assert abs(orc.measure(st, model)["Energy"] - e_pub) <= 1e-10 * abs(e_pub)
    s2 = st.copy()
    orc.ctmrg(s2, dict(CFG, svd_type="full-rank", steps=5), orc.OmegaStream(31))
    e = orc.measure(s2, model)["Energy"]
    e_ref = float(z["after5_full_meas_Energy"])
    assert abs(e - e_ref) <= 1e-10 * abs(e_ref)


def test_random_state_seeding_is_deterministic():
    a = orc.random_state(3, 9, seed=5)
    b = orc.random_state(3, 9, seed=5)
    for s in a.sites:
        assert np.array_equal(a[s]["A"], b[s]["A"])
        assert abs(np.linalg.norm(a[s]["A"]) - 1.0) < 1e-14


def test_invalid_projector_type_raises():
    with pytest.raises(ValueError):
        orc.Mover(dict(CFG, projectors="quarter-system"), orc.OmegaStream(0))


def test_unknown_site_raises():
    st = orc.random_state(2, 4, seed=1)
    with pytest.raises(ValueError):
        st[(5, 5)]


def test_norm_tensor_matches_reference():
    """The full update's norm tensor (acetn/evolution/full_update.py:163-268),
    both bond directions, against the reference's build_norm_tensor and its
    blocked core (tests/golden/make_norm_tensor.py)."""
    z = load("norm_tensor_d2.npz")
    sites = {}
    for x in range(2):
        for y in range(2):
            key = f"{x}_{y}"
            sites[(x, y)] = {"A": z[f"{key}_A"], "C": [z[f"{key}_C{k}"] for k in range(4)],
                             "E": [z[f"{key}_E{k}"] for k in range(4)]}
    st = orc.OracleState(sites, 2, 2, 6)
    for k, s2 in ((2, (1, 0)), (1, (0, 1))):
        n12 = orc.norm_tensor(st, ((0, 0), s2, k), z[f"k{k}_a1q"], z[f"k{k}_a2q"])
        assert rel(n12, z[f"k{k}_n12"]) < 1e-13
        assert rel(n12, z[f"k{k}_n12_blocked"]) < 1e-13


def test_rsvd_known_answers():
    """The reference's known-answer tests of its randomized SVDs
    (tests/unit/test_linalg.py of the reference: exact recovery of low-rank
    matrices and products to 1e-10, orthonormal factors, ordered spectra),
    applied to the oracle's restatements."""
    rng = np.random.default_rng(3)
    omega = orc.OmegaStream(17)

    def rec(p, u, s, v):
        return np.linalg.norm(p - (u * s) @ v.T) / np.linalg.norm(p)

    low = rng.standard_normal((100, 10)) @ rng.standard_normal((10, 80))
    u, s, v = orc.svd_lowrank(low, 15, 3, omega)
    assert rec(low, u, s, v) < 1e-10
    assert np.allclose(u.T @ u, np.eye(15), atol=1e-10) and np.allclose(v.T @ v, np.eye(15), atol=1e-10)
    assert np.all(s[:-1] >= s[1:]) and np.all(s >= 0)
    a, b = rng.standard_normal((100, 10)), rng.standard_normal((10, 80))
    u, s, v = orc.fused_matmul_svd_lowrank(a, b, 12, 3, omega)
    assert rec(a @ b, u, s, v) < 1e-10
    a, b = rng.standard_normal((60, 10)), rng.standard_normal((10, 50))
    c, d = rng.standard_normal((50, 40)), rng.standard_normal((40, 70))
    u, s, v = orc.fused_3matmul_svd_lowrank(a, b, c, d, 10, 3, omega)
    assert rec(a @ b @ c @ d, u, s, v) < 1e-10
