"""Reduced density matrices on the GB300 library.

Mirror of ``RDM`` (acetn/measurement/rdm.py:6-153): ``RDM(ipeps)[site]`` is
the (d, d) site RDM, ``RDM(ipeps)[bond]`` the (d, d, d, d) bond RDM of a
``Bond`` (or any (s1, s2, k) triple with attributes s1, s2, k).  Neither is
trace-normalised.
"""

import torch

from . import _abi
from .state import Bond


class RDM:
    """``precision``: "fp64" (the drop-in) or "mixed" (bond RDMs on tensor
    cores in 3xBF16, site RDMs in FP32; FP64 results)."""

    def __init__(self, ipeps, precision="fp64"):
        self.ipeps = ipeps
        if precision not in ("fp64", "mixed"):
            raise ValueError(f"Invalid precision: {precision} provided.")
        self.precision = precision

    def __getitem__(self, key):
        if isinstance(key, Bond) or hasattr(key, "k"):
            return self.build_bond_rdm(key)
        return self.build_site_rdm(key)

    def build_site_rdm(self, site):
        """rdm.py:35-67."""
        st = self.ipeps[site]
        if isinstance(st, dict) and not st:
            raise KeyError(site)
        ref = _abi.SiteRef(st)
        out = torch.empty(ref.d, ref.d, dtype=torch.float64, device=ref.device)
        _abi.call("ctm_site_rdm", [ref.pointer, ref.D, ref.d, _abi.PREC[self.precision],
                                   _abi.ptr(out)], ref.device,
                  key=("site_rdm", ref.shapes(), self.precision))
        return out

    def build_bond_rdm(self, bond):
        """rdm.py:69-99 with the contraction of rdm.py:102-153."""
        s1, s2, k = bond
        r1 = _abi.SiteRef(self.ipeps[s1])
        r2 = _abi.SiteRef(self.ipeps[s2])
        d = r1.d
        out = torch.empty(d, d, d, d, dtype=torch.float64, device=r1.device)
        _abi.call("ctm_bond_rdm", [r1.pointer, r2.pointer, r1.D, d, k, _abi.PREC[self.precision],
                                   _abi.ptr(out)], r1.device,
                  key=("bond_rdm", r1.shapes(), r2.shapes(), k, self.precision))
        return out
