"""Reduced density matrices in mixed precision (bond RDMs on tensor cores in
3xBF16, site RDMs in FP32) against the FP64 path, through the C ABI,
trace-normalised: the golden D=3 chi=9 state written by the reference and a
D=6 chi=144 state grown by three CTMRG iterations (the metric's workload).
The worst differences are printed."""

import numpy as np
import pytest
import torch

import acetn_gb300 as gb
from _golden import gpu_state, load

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built():
    gb.build()
    assert torch.cuda.is_available()


def grown(D, chi, seed, iterations):
    """A seeded state whose environment has been grown by CTMRG iterations
    (random corner and edge tensors would make the RDM's trace a near
    cancellation and blow up every relative error)."""
    st = gb.random_state(D, chi, seed, device="cuda")
    g = torch.Generator(device="cuda")
    g.manual_seed(seed)
    gb.ctmrg(st, gb.CTMRGConfig(precision="mixed", rsvd_oversampling=16, steps=iterations,
                                disable_progressbar=True),
             omega_source=lambda n, q, dev: torch.randn(n, q, dtype=torch.float64, device=dev,
                                                        generator=g))
    return st


def _compare(st, tol_bond, tol_site):
    r64, rmx = gb.RDM(st, "fp64"), gb.RDM(st, "mixed")
    worst_b = worst_s = 0.0
    for b in st.bond_list:
        a = r64[b].cpu().numpy()
        m = rmx[b].cpu().numpy()
        a, m = a / np.einsum("pqpq->", a), m / np.einsum("pqpq->", m)
        worst_b = max(worst_b, float(np.abs(a - m).max()))
    for s in st.site_list:
        a = r64[s].cpu().numpy()
        m = rmx[s].cpu().numpy()
        worst_s = max(worst_s, float(np.abs(a / np.trace(a) - m / np.trace(m)).max()))
    print(f"mixed RDMs vs FP64 (trace-normalised, max |diff|): bond {worst_b:.2e}, "
          f"site {worst_s:.2e}")
    assert worst_b < tol_bond
    assert worst_s < tol_site


def test_mixed_rdms_golden_state():
    st = gpu_state(load("move_d3_chi9.npz"), 9)
    _compare(st, 1e-5, 1e-6)
    e64 = float(gb.measure(st, gb.HeisenbergModel(1.0), verbose=False)["Energy"])
    emx = float(gb.measure(st, gb.HeisenbergModel(1.0), verbose=False,
                           precision="mixed")["Energy"])
    # E ~ 6e-3 here: the bound is on the RDM-entry scale, not relative to E
    print(f"mixed measure vs FP64: |dE| = {abs(emx - e64):.2e}")
    assert abs(emx - e64) < 1e-6
    assert gb._abi.device_status() == 0


def test_mixed_rdms_d6_chi144():
    st = grown(6, 144, 77, 3)
    _compare(st, 1e-4, 1e-5)
    assert gb._abi.device_status() == 0


def test_rdm_rejects_bad_precision():
    st = gpu_state(load("move_d3_chi9.npz"), 9)
    with pytest.raises(ValueError):
        gb.RDM(st, "bf16")
