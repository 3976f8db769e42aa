"""Parity at the benchmark configurations, through the C ABI.

* D=6, chi=144 (the metric's workload, oversampling 16): one FP64 move on a
  chi-saturated state against the oracle with the same rSVD test matrices;
  corner spectra, |entries| of the new corner and edge tensors (up to the
  sign of each projector column) and the trace-normalised site RDM to 1e-10.
* Transverse-field Ising, hx = 3, D=4, chi=64 (seeded N(0,1) site tensors
  plus 1e-2 on the up-spin entry A[0,0,0,0,0] before normalising): one move
  in FP64 against the oracle (energy and <sigma_x> to 1e-10) and the mixed
  form against the FP64 form with the same test matrices (energy and
  <sigma_x> to 1e-5 relative; the values are printed).
* Fixed-width projectors (the CUDA-graph form: zero columns past the
  truncation count) give the energies and corner spectra of the compact
  ones when the truncation keeps fewer than chi singular values.
"""

import numpy as np
import pytest
import torch

import acetn_gb300 as gb
from _golden import gpu_state, load, rel
from oracle import ctm_oracle as orc

pytestmark = pytest.mark.gpu


def omega_from(stream):
    return lambda n, q, device: torch.from_numpy(stream(n, q)).to(device)


def clone(st):
    c = gb.IpepsState(st.nx, st.ny, st.dims, st.device)
    for s in st.site_list:
        v = st[s]
        c[s] = {"A": v["A"].clone(), "C": [t.clone() for t in v["C"]],
                "E": [t.clone() for t in v["E"]]}
    return c


@pytest.fixture(scope="module", autouse=True)
def built():
    gb.build()
    assert torch.cuda.is_available()


def saturated_state(D, chi, seed):
    """Seeded site tensors with corner and edge tensors already at chi
    (N(0,1) entries, unit Frobenius norm): a chi-saturated input without the
    oracle's growth iterations."""
    ost = orc.random_state(D, chi, seed=seed)
    rng = np.random.default_rng(seed + 1)

    def rnd(*shape):
        t = rng.standard_normal(shape)
        return t / np.linalg.norm(t)

    for s in ost.sites:
        ost.sites[s]["C"] = [rnd(chi, chi) for _ in range(4)]
        ost.sites[s]["E"] = [rnd(chi, chi, D, D) for _ in range(4)]
    return ost


def test_fp64_move_d6_chi144_matches_oracle():
    cfg = dict(projectors="half-system", svd_type="rsvd", rsvd_oversampling=16, rsvd_niter=2,
               svd_cutoff=1e-12)
    ost = saturated_state(6, 144, seed=41)
    gst = gb.IpepsState.from_arrays(ost.copy().sites, 2, 2, 144)
    orc.Mover(cfg, orc.OmegaStream(17)).move(ost, 0, 0)
    gb.DirectionalMover(gb.CTMRGConfig(**cfg), omega_source=omega_from(orc.OmegaStream(17))
                        ).move(gst, 0, 0)
    for s in ost.sites:
        for kk in range(4):
            a = gst[s]["C"][kk].cpu().numpy()
            b = ost[s]["C"][kk]
            assert a.shape == b.shape
            sa = np.linalg.svd(a, compute_uv=False)
            sb = np.linalg.svd(b, compute_uv=False)
            assert rel(sa / sa[0], sb / sb[0]) < 1e-10
            assert rel(np.abs(a), np.abs(b)) < 1e-9
            assert rel(np.abs(gst[s]["E"][kk].cpu().numpy()), np.abs(ost[s]["E"][kk])) < 1e-9
    # the site RDM of a renormalised site (left move of column 0 writes column 1)
    r = gb.RDM(gst)[(1, 0)].cpu().numpy()
    r_ref = orc.site_rdm(ost[(1, 0)])
    assert np.abs(r / np.trace(r) - r_ref / np.trace(r_ref)).max() < 1e-10
    assert gb._abi.device_status() == 0


def test_tfim_d4_chi64_fp64_and_mixed():
    """TFIM h=3 D=4 chi=64 with the reference's rSVD defaults (2 power
    iterations, oversampling 2): the FP64 path matches the oracle to 1e-10;
    the mixed path's E and <sx> agree with FP64 (same test matrix) within
    1e-5 plus 3x the FP64 rSVD draw spread (FP64 with another test matrix).
    With two oversampling columns the truncation is sensitive to any
    perturbation: rounding-level changes elsewhere in the mixed path moved
    its error between 1e-6 and 1e-5 here."""
    cfg = dict(projectors="half-system", svd_type="rsvd", rsvd_oversampling=2, rsvd_niter=2,
               svd_cutoff=1e-12)
    ost = orc.random_state(4, 64, seed=2024, bias=1e-2)
    orc.ctmrg(ost, cfg, orc.OmegaStream(3), steps=3)
    start = ost.copy()
    orc.Mover(cfg, orc.OmegaStream(9)).move(ost, 0, 0)
    m_ref = orc.measure(ost, orc.ising_model(1.0, 3.0))
    out = {}
    for prec, seed in (("fp64", 9), ("mixed", 9), ("fp64-draw", 10)):
        gst = gb.IpepsState.from_arrays(start.copy().sites, 2, 2, 64)
        gb.DirectionalMover(gb.CTMRGConfig(**cfg, precision=prec.split("-")[0]),
                            omega_source=omega_from(orc.OmegaStream(seed))).move(gst, 0, 0)
        m = gb.measure(gst, gb.IsingModel(1.0, 3.0), verbose=False)
        out[prec] = (float(m["Energy"]), float(m["sx"]))
    e64, sx64 = out["fp64"]
    assert abs(e64 - m_ref["Energy"]) <= 1e-10 * abs(m_ref["Energy"])
    assert abs(sx64 - m_ref["sx"]) <= 1e-10 * abs(m_ref["sx"])
    emx, sxmx = out["mixed"]
    ed, sxd = out["fp64-draw"]
    # the state is a random one, not a ground state: E ~ -0.034 per site,
    # so relative errors are measured against a small number
    print(f"TFIM D=4 chi=64 mixed vs FP64: E {abs(emx - e64) / abs(e64):.2e}, "
          f"<sx> {abs(sxmx - sx64) / abs(sx64):.2e} relative; FP64 draw spread: "
          f"E {abs(ed - e64) / abs(e64):.2e}, <sx> {abs(sxd - sx64) / abs(sx64):.2e}")
    assert abs(emx - e64) <= 1e-5 * abs(e64) + 3.0 * abs(ed - e64)
    assert abs(sxmx - sx64) <= 1e-5 * abs(sx64) + 3.0 * abs(sxd - sx64)
    assert gb._abi.device_status() == 0


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_fixed_width_projectors_equal_compact_ones(precision):
    z = load("ctmrg_d2_chi20_rsvd.npz")
    st = gpu_state(z, 20)
    gb.ctmrg(st, gb.CTMRGConfig(steps=4, disable_progressbar=True),
             omega_source=omega_from(orc.OmegaStream(2)))
    # a cutoff that truncates below chi, so the fixed-width projectors carry
    # zero columns
    cfg = gb.CTMRGConfig(projectors="half-system", svd_type="rsvd", rsvd_oversampling=2,
                         rsvd_niter=2, svd_cutoff=1e-3, mixed_svd_floor=1e-3,
                         precision=precision)
    model = gb.HeisenbergModel(1.0)
    a = clone(st)
    gb.DirectionalMover(cfg, omega_source=omega_from(orc.OmegaStream(3))).move(a, 0, 0)
    b = clone(st)
    mv = gb.DirectionalMover(cfg, omega_source=omega_from(orc.OmegaStream(3)))
    mv.graph_mode = True
    mv.move(b, 0, 0)
    counts = mv.last_counts.cpu().tolist()
    assert min(counts) < 20, counts
    for s in st.site_list:
        for kk in range(4):
            ca, cb = a[s]["C"][kk], b[s]["C"][kk]
            assert cb.shape[1] >= ca.shape[1]
            sa = np.linalg.svd(ca.cpu().numpy(), compute_uv=False)
            sb = np.linalg.svd(cb.cpu().numpy(), compute_uv=False)[: sa.size]
            assert rel(sb, sa) < 1e-12
    ea = float(gb.measure(a, model, verbose=False)["Energy"])
    eb = float(gb.measure(b, model, verbose=False)["Energy"])
    assert abs(ea - eb) <= 1e-12 * abs(ea)
    assert gb._abi.device_status() == 0
