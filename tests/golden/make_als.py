"""Generate ``als_*.npz``: the full update's ALS solver run by the Ace-TN
reference itself (``ALSSolver``, acetn/evolution/als_solver.py:6-270) on
seeded inputs, to pin the oracle's ``als_solve`` and the GPU solver.

Inputs follow the reference's own unit test (tests/unit/test_als.py:9-33):
random reduced tensors, a12g their product times a random gate near the
identity plus a small perturbation, a random norm tensor made positive and
gauge-fixed with the reference's
``positive_approx`` and ``gauge_fix`` (full_update.py:255-343).  Cases:
(nD, bD, pD) = (8, 5, 3) as in that test, (12, 6, 2) (a D=6, d=2 bond) and
(4, 2, 2); methods "cholesky" and "pinv"; 10 iterations (the convergence
test |d2 - d1| / |d1| < 1e-15 is not reached, so the iteration count is
fixed) and 100 iterations (the reference's default); and an indefinite norm
tensor (``als_indefinite.npz``) on which the Cholesky fails and the
reference falls back to a plain solve.

Run in a container where the reference source tree is available:

    python tests/golden/make_als.py /path/to/ace-tn
"""

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
from make_golden import _install_toml_stub  # noqa: E402

CASES = [(8, 5, 3, 21), (12, 6, 2, 22), (4, 2, 2, 23)]


def main(ref_root):
    _install_toml_stub()
    sys.path.insert(0, ref_root)
    import torch
    from torch import einsum
    from acetn.evolution.als_solver import ALSSolver
    from acetn.evolution.full_update import gauge_fix, positive_approx
    from acetn.ipeps.ipeps_config import EvolutionConfig

    for nD, bD, pD, seed in CASES:
        torch.manual_seed(seed)
        a1r = torch.rand(nD, bD, pD, dtype=torch.float64)
        a2r = torch.rand(nD, bD, pD, dtype=torch.float64)
        a12g = einsum("yup,xuq->yxpq", a1r, a2r)
        # a gate near the identity, as in FullUpdater.update_reduced_tensors
        # (full_update.py:87-88): the gated product has a larger bond than
        # bD, so the truncation is a genuine least-squares problem
        gate = (torch.eye(pD * pD, dtype=torch.float64)
                + 0.3 * torch.rand(pD * pD, pD * pD, dtype=torch.float64)).reshape(pD, pD, pD, pD)
        a12g = einsum("yxpq,pqrs->yxrs", a12g, gate)
        a12g += 1e-4 * torch.rand_like(a12g)
        n12 = torch.rand(nD, nD, nD, nD, dtype=torch.float64)
        nz = positive_approx(n12, nD)
        n12, a12g, *_ = gauge_fix(nz, a12g, nD)
        out = {"n12": n12.numpy(), "a12g": a12g.numpy(), "shape": np.array([nD, bD, pD])}
        i1, i2 = ALSSolver.initialize_reduced_tensors(a12g, (nD, bD, pD))
        out["init_a12"] = einsum("yup,xuq->yxpq", i1, i2).numpy()
        for method in ("cholesky", "pinv"):
            for niter in (10, 100):
                cfg = EvolutionConfig(als_niter=niter, als_tol=1e-15, als_method=method,
                                      backend="torch")
                solver = ALSSolver(n12.clone(), a12g.clone(), (nD, bD, pD), cfg)
                r1, r2 = solver.solve()
                key = f"{method}_{niter}"
                out[f"{key}_a12"] = einsum("yup,xuq->yxpq", r1, r2).numpy()
                out[f"{key}_cost"] = np.array(
                    float(ALSSolver.calculate_cost(r1, r2, a12g, n12)))
                out[f"{key}_a1r"] = r1.numpy()
                out[f"{key}_a2r"] = r2.numpy()
        name = f"als_{nD}_{bD}_{pD}.npz"
        np.savez(os.path.join(HERE, name), **out)
        print("wrote", name, {k: float(v) for k, v in out.items() if k.endswith("_cost")})

    # an indefinite norm tensor (symmetric, not made positive): the shifted
    # systems are indefinite, the Cholesky fails and solve_ar falls back to
    # torch.linalg.solve (als_solver.py:232-236); three iterations
    nD, bD, pD = 6, 3, 2
    torch.manual_seed(31)
    n = torch.randn(nD * nD, nD * nD, dtype=torch.float64)
    n12 = (0.5 * (n + n.T)).reshape(nD, nD, nD, nD).contiguous()
    a12g = torch.randn(nD, nD, pD, pD, dtype=torch.float64)
    cfg = EvolutionConfig(als_niter=3, als_tol=1e-15, als_method="cholesky", backend="torch")
    r1, r2 = ALSSolver(n12.clone(), a12g.clone(), (nD, bD, pD), cfg).solve()
    out = {"n12": n12.numpy(), "a12g": a12g.numpy(), "shape": np.array([nD, bD, pD]),
           "cholesky_3_a12": einsum("yup,xuq->yxpq", r1, r2).numpy(),
           "cholesky_3_cost": np.array(float(ALSSolver.calculate_cost(r1, r2, a12g, n12)))}
    np.savez(os.path.join(HERE, "als_indefinite.npz"), **out)
    print("wrote als_indefinite.npz", float(out["cholesky_3_cost"]))


if __name__ == "__main__":
    main(sys.argv[1])
