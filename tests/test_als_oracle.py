"""The oracle's ALS solver (full update, acetn/evolution/als_solver.py)
against vectors written by the reference itself (``make_als.py``), and the
host-side checks of ``ALSSolver`` (no GPU needed)."""

import numpy as np
import pytest
import torch

import acetn_gb300 as gb
from _golden import load
from oracle import ctm_oracle as orc

CASES = ["als_8_5_3", "als_12_6_2", "als_4_2_2"]


def a12(a1r, a2r):
    return np.einsum("yup,xuq->yxpq", a1r, a2r)


def rel(a, b):
    return float(np.abs(a - b).max() / np.abs(b).max())


@pytest.mark.parametrize("case", CASES)
def test_initial_guess_matches_reference(case):
    z = load(f"{case}.npz")
    shape = tuple(int(x) for x in z["shape"])
    a1, a2 = orc.als_initialize(z["a12g"], shape)
    assert rel(a12(a1, a2), z["init_a12"]) < 1e-13


@pytest.mark.parametrize("case", CASES)
@pytest.mark.parametrize("method", ["cholesky", "pinv"])
@pytest.mark.parametrize("niter", [10, 100])
def test_als_solve_matches_reference(case, method, niter):
    """Costs to 1e-12; products to 1e-12 where the iteration count is fixed,
    to 1e-6 where the reference's stopping test (|d2 - d1| / |d1| < 1e-15, a
    rounding-level test) may fire one iteration earlier or later (measured
    5e-8 and 7e-9 apart)."""
    z = load(f"{case}.npz")
    shape = tuple(int(x) for x in z["shape"])
    a1, a2, it = orc.als_solve(z["n12"], z["a12g"], shape, niter=niter, method=method)
    key = f"{method}_{niter}"
    cost = orc.als_cost(a1, a2, z["a12g"], z["n12"])
    assert abs(cost - float(z[f"{key}_cost"])) <= 1e-12 * abs(float(z[f"{key}_cost"]))
    bar = 1e-12 if (niter == 10 and it == 10) else 1e-6
    assert rel(a12(a1, a2), z[f"{key}_a12"]) < bar


def test_als_converges_like_the_reference_test():
    """tests/unit/test_als.py:52-63 of the reference on the oracle: the cost
    after 99 and after 100 iterations differs by less than tol."""
    z = load("als_8_5_3.npz")
    shape = tuple(int(x) for x in z["shape"])
    c = []
    for n in (99, 100):
        a1, a2, _ = orc.als_solve(z["n12"], z["a12g"], shape, niter=n)
        c.append(orc.als_cost(a1, a2, z["a12g"], z["n12"]))
    assert abs(c[1] - c[0]) < 1e-15 * abs(c[0]) + 1e-9


def test_als_solver_host_checks():
    class Cfg:
        als_method = "lu"
    with pytest.raises(ValueError):
        gb.ALSSolver(None, None, (2, 2, 2), Cfg())
    s = gb.ALSSolver(torch.zeros(2, 2, 2, 2, dtype=torch.float64),
                     torch.zeros(2, 2, 2, 2, dtype=torch.float64), (2, 1, 2), object())
    assert (s.niter, s.tol, s.method, s.epsilon) == (100, 1e-15, "cholesky", 1e-12)
    with pytest.raises(ValueError):  # CPU tensors: no CPU path
        s.solve()


def test_als_indefinite_norm_falls_back_like_the_reference():
    """An indefinite (symmetric, not positive) norm tensor: every shifted
    system fails the Cholesky and the reference solves it directly
    (als_solver.py:219-226); three iterations, products and cost to 1e-10."""
    z = load("als_indefinite.npz")
    shape = tuple(int(x) for x in z["shape"])
    a1, a2, it = orc.als_solve(z["n12"], z["a12g"], shape, niter=3)
    assert it == 3
    assert rel(a12(a1, a2), z["cholesky_3_a12"]) < 1e-10
    ref = float(z["cholesky_3_cost"])
    assert abs(orc.als_cost(a1, a2, z["a12g"], z["n12"]) - ref) <= 1e-10 * abs(ref)
