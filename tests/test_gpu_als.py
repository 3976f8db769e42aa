"""The GPU ALS solver (``ALSSolver`` / ``ctm_als_solve``) against vectors
written by the reference's own ALSSolver (``make_als.py``) and against the
oracle.  a1r and a2r are compared through their product a1r . a2r (the bond
index has a gauge: the initial SVD's signs), costs directly."""

import numpy as np
import pytest
import torch

import acetn_gb300 as gb
from _golden import load
from oracle import ctm_oracle as orc

pytestmark = pytest.mark.gpu

CASES = ["als_8_5_3", "als_12_6_2", "als_4_2_2"]


class Cfg:
    def __init__(self, niter, method):
        self.als_niter = niter
        self.als_tol = 1e-15
        self.als_method = method
        self.als_epsilon = 1e-12


def rel(a, b):
    return float(np.abs(a - b).max() / np.abs(b).max())


@pytest.mark.parametrize("case", CASES)
@pytest.mark.parametrize("method", ["cholesky", "pinv"])
@pytest.mark.parametrize("niter", [10, 100])
def test_gpu_als_matches_reference(case, method, niter):
    """Costs to 1e-11; products to 1e-9 with a fixed iteration count (the
    oracle ran all 10), else 1e-6 (the reference's stopping test is at the
    rounding level and may fire an iteration earlier or later)."""
    z = load(f"{case}.npz")
    shape = tuple(int(x) for x in z["shape"])
    n12 = torch.from_numpy(z["n12"]).cuda()
    a12g = torch.from_numpy(z["a12g"]).cuda()
    solver = gb.ALSSolver(n12, a12g, shape, Cfg(niter, method))
    a1r, a2r = solver.solve()
    assert a1r.shape == shape and a2r.shape == shape
    key = f"{method}_{niter}"
    prod = torch.einsum("yup,xuq->yxpq", a1r, a2r).cpu().numpy()
    cost = float(gb.ALSSolver.calculate_cost(a1r, a2r, a12g, n12))
    ref_cost = float(z[f"{key}_cost"])
    _, _, it_oracle = orc.als_solve(z["n12"], z["a12g"], shape, niter=niter, method=method)
    print(case, method, niter, "iters", solver.iterations, it_oracle,
          "a12", rel(prod, z[f"{key}_a12"]), "cost", abs(cost - ref_cost) / abs(ref_cost))
    assert abs(cost - ref_cost) <= 1e-11 * abs(ref_cost)
    bar = 1e-9 if (niter == 10 and it_oracle == 10 and solver.iterations == 10) else 1e-6
    assert rel(prod, z[f"{key}_a12"]) < bar
    assert gb._abi.device_status() == 0


def test_gpu_cost_matches_oracle():
    z = load("als_12_6_2.npz")
    shape = tuple(int(x) for x in z["shape"])
    g = np.random.default_rng(4)
    a1, a2 = g.standard_normal(shape), g.standard_normal(shape)
    cost = gb.ALSSolver.calculate_cost(*(torch.from_numpy(x).cuda()
                                         for x in (a1, a2, z["a12g"], z["n12"])))
    ref = orc.als_cost(a1, a2, z["a12g"], z["n12"])
    assert abs(float(cost) - ref) <= 1e-12 * abs(ref)


def test_gpu_als_converges_like_the_reference_test():
    """tests/unit/test_als.py:52-63 of the reference: the cost after 99 and
    after 100 iterations differs by less than tol (both runs stop at the
    same converged iteration)."""
    z = load("als_8_5_3.npz")
    shape = tuple(int(x) for x in z["shape"])
    n12 = torch.from_numpy(z["n12"]).cuda()
    a12g = torch.from_numpy(z["a12g"]).cuda()
    costs = []
    for n in (99, 100):
        a1r, a2r = gb.ALSSolver(n12, a12g, shape, Cfg(n, "cholesky")).solve()
        costs.append(float(gb.ALSSolver.calculate_cost(a1r, a2r, a12g, n12)))
    assert abs(costs[1] - costs[0]) < 1e-15 * abs(costs[0]) + 1e-9


def test_gpu_als_indefinite_norm_takes_the_lu_fallback():
    """Every shifted system of an indefinite norm tensor fails the Cholesky;
    the kernel's pivoted-LU fallback gives the reference's plain solve
    (als_solver.py:219-226): products and cost to 1e-9 after three
    iterations."""
    z = load("als_indefinite.npz")
    shape = tuple(int(x) for x in z["shape"])
    n12 = torch.from_numpy(z["n12"]).cuda()
    a12g = torch.from_numpy(z["a12g"]).cuda()
    solver = gb.ALSSolver(n12, a12g, shape, Cfg(3, "cholesky"))
    a1r, a2r = solver.solve()
    assert solver.iterations == 3
    prod = torch.einsum("yup,xuq->yxpq", a1r, a2r).cpu().numpy()
    assert rel(prod, z["cholesky_3_a12"]) < 1e-9
    ref = float(z["cholesky_3_cost"])
    cost = float(gb.ALSSolver.calculate_cost(a1r, a2r, a12g, n12))
    assert abs(cost - ref) <= 1e-9 * abs(ref)
    assert gb._abi.device_status() == 0
