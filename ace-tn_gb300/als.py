"""``ALSSolver`` of the full update (acetn/evolution/als_solver.py:6-270) on
the GPU.

Same constructor and ``solve()`` as the reference: the norm tensor n12
(nD, nD, nD, nD), the gated product a12g (nD, nD, pD, pD), the reduced-tensor
shape (nD, bD, pD) and a config with ``als_niter``, ``als_tol``,
``als_method`` ("cholesky" or "pinv") and ``als_epsilon``.  The whole
iteration loop runs in libctm_gb300.so (``ctm_als_solve``): GETT contractions
for the systems, one single-CTA kernel per Cholesky solve, the FP64 Jacobi
SVD for the pseudo-inverse; float64 CUDA tensors only, no CPU fallback.  The
result is the reference's up to the gauge of the bond index (the SVD's
signs), i.e. a1r . a2r and the cost agree.
"""

import ctypes

import torch

from . import _abi

METHODS = {"cholesky": 0, "pinv": 1}


class ALSSolver:
    def __init__(self, n12, a12g, ar_shape, config):
        self.niter = int(getattr(config, "als_niter", 100))
        self.tol = float(getattr(config, "als_tol", 1e-15))
        self.method = getattr(config, "als_method", "cholesky")
        self.epsilon = float(getattr(config, "als_epsilon", 1e-12))
        if self.method not in METHODS:
            raise ValueError(f"Invalid ALS method: {self.method} provided.")
        self.n12 = n12
        self.a12g = a12g
        self.ar_shape = tuple(int(x) for x in ar_shape)
        self.iterations = None

    def _checked(self):
        nD, bD, pD = self.ar_shape
        for name, t, shape in (("n12", self.n12, (nD, nD, nD, nD)),
                               ("a12g", self.a12g, (nD, nD, pD, pD))):
            _abi.require_cuda(t, name)
            if tuple(t.shape) != shape:
                raise ValueError(f"{name} must have shape {shape}, got {tuple(t.shape)}")
        return self.n12.contiguous(), self.a12g.contiguous()

    def solve(self):
        """The updated reduced tensors (a1r, a2r), each (nD, bD, pD)."""
        n12, a12g = self._checked()
        nD, bD, pD = self.ar_shape
        a1r = torch.empty(nD, bD, pD, dtype=torch.float64, device=n12.device)
        a2r = torch.empty_like(a1r)
        it = ctypes.c_int32(0)
        _abi.call("ctm_als_solve", [_abi.ptr(n12), _abi.ptr(a12g), nD, bD, pD, self.niter,
                                    self.tol, METHODS[self.method], self.epsilon, _abi.ptr(a1r),
                                    _abi.ptr(a2r), ctypes.byref(it)], n12.device,
                  key=("als", nD, bD, pD, METHODS[self.method]))
        self.iterations = it.value
        return a1r, a2r

    @staticmethod
    def calculate_cost(a1r, a2r, a12g, n12):
        """<a12n|N|a12n> - 2 <a12n|N|a12g> (als_solver.py:253-262), a 0-d
        float64 tensor on the device."""
        for name, t in (("a1r", a1r), ("a2r", a2r), ("a12g", a12g), ("n12", n12)):
            _abi.require_cuda(t, name)
        nD, bD, pD = (int(x) for x in a1r.shape)
        if tuple(a2r.shape) != (nD, bD, pD) or tuple(a12g.shape) != (nD, nD, pD, pD) \
                or tuple(n12.shape) != (nD, nD, nD, nD):
            raise ValueError("calculate_cost: inconsistent shapes")
        out = torch.empty((), dtype=torch.float64, device=n12.device)
        a1r, a2r, a12g, n12 = (t.contiguous() for t in (a1r, a2r, a12g, n12))
        _abi.call("ctm_als_cost", [_abi.ptr(a1r), _abi.ptr(a2r), _abi.ptr(a12g), _abi.ptr(n12),
                                   nD, bD, pD, _abi.ptr(out)], n12.device,
                  key=("als_cost", nD, bD, pD))
        return out
