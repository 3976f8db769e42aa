"""Projector construction on the GB300 library.

Mirror of ``ProjectorCalculator`` (acetn/renormalization/projectors.py:7-236):
same constructor argument (a CTMRG config), same ``calculate(ipeps, sites, k)``
returning ``(proj1, proj2)`` of shapes (chi, D, D, chi_new), same ValueError
for an invalid projector type or an undefined site.  ``omega_source(n, q,
device)`` supplies the rSVD test matrices (default: ``torch.randn`` on the
device, like the reference).
"""

import ctypes

import torch

from . import _abi
from .config import resolve


def default_omega(n, q, device):
    return torch.randn(n, q, dtype=torch.float64, device=device)


class PendingProjectors:
    """Projector pair whose truncated width is still on the device."""

    def __init__(self, p1buf, p2buf, p1_rows, p2_rows, qD1, qD4, chi_slot):
        self.p1buf, self.p2buf = p1buf, p2buf
        self.p1_rows, self.p2_rows = p1_rows, p2_rows
        self.qD1, self.qD4 = qD1, qD4
        self.chi_slot = chi_slot

    def finish(self, chi_new):
        chi_new = int(chi_new)
        p1 = self.p1buf[: self.p1_rows * chi_new].view(*self.qD1, chi_new)
        p2 = self.p2buf[: self.p2_rows * chi_new].view(*self.qD4, chi_new)
        return p1, p2


class ProjectorCalculator:
    """Computes projectors with half- or full-system contractions on the GPU."""

    def __init__(self, config, omega_source=None):
        self.config = resolve(config)
        self.projectors = self.config.projectors
        self.svd_type = self.config.svd_type
        self.svd_cutoff = self.config.svd_cutoff
        self.rsvd_niter = self.config.rsvd_niter
        self.rsvd_oversampling = self.config.rsvd_oversampling
        self.precision = self.config.precision
        self.mixed_svd_floor = self.config.mixed_svd_floor
        self.mixed_flags = self.config.mixed_flags
        self.omega_source = omega_source or default_omega
        self.set_calculate()

    def set_calculate(self):
        """acetn/renormalization/projectors.py:21-33."""
        if self.projectors is None or self.projectors == "full-system":
            self.calculate = self.calculate_full_system
        elif self.projectors == "half-system":
            self.calculate = self.calculate_half_system
        else:
            raise ValueError(f"Invalid ctmrg projector type: {self.projectors} provided.")

    @staticmethod
    def make_quarter_tensor(site_tensor, k, precision="fp64"):
        """acetn/renormalization/projectors.py:35-60: returns (qk matrix, 6-leg shape)."""
        ref = _abi.SiteRef(site_tensor)
        D, d = ref.D, ref.d
        c = site_tensor["C"][k % 4]
        e1 = site_tensor["E"][(3 + k) % 4]
        e2 = site_tensor["E"][k % 4]
        if c.shape[1] != e2.shape[0] or c.shape[0] != e1.shape[1]:
            raise ValueError("quarter tensor: corner and edge tensors do not chain")
        rows, cols = e2.shape[1] * D * D, e1.shape[0] * D * D
        Q = torch.empty(rows, cols, dtype=torch.float64, device=ref.device)
        sh = (_abi.c_i64 * 6)()
        _abi.call("ctm_quarter_tensor", [ref.pointer, D, d, k, _abi.ptr(Q), sh,
                                          _abi.PREC[precision]], ref.device,
                  key=("quarter", ref.shapes(), k, precision))
        return Q, tuple(sh)

    # ---------------------------------------------------------------- launches
    def _site_refs(self, ipeps, sites):
        return [_abi.SiteRef(ipeps[s]) for s in sites]

    def launch(self, ipeps, sites, k, chi_slot, precision=None, fixed_width=False):
        """Enqueues one projector pair; its width lands in ``chi_slot``.  With
        ``fixed_width`` the projectors keep chi_cap columns (zero beyond the
        truncation count) so that shapes do not depend on device data."""
        refs = self._site_refs(ipeps, sites)
        D, d = refs[0].D, refs[0].d
        device = refs[0].device
        chi = ipeps.dims["chi"]
        opts = _abi.opts_struct(self, chi, precision or self.precision, fixed_width)
        arr = (_abi.SITE_P * 4)(*[r.pointer for r in refs])
        p1r, p2r, nr, q, cap = (_abi.c_i64() for _ in range(5))
        _abi.check(_abi.load().ctm_projector_dims(arr, D, k, ctypes.byref(opts), ctypes.byref(p1r),
                                                  ctypes.byref(p2r), ctypes.byref(nr),
                                                  ctypes.byref(q), ctypes.byref(cap)),
                   "ctm_projector_dims")
        p1buf = torch.empty(p1r.value * cap.value, dtype=torch.float64, device=device)
        p2buf = torch.empty(p2r.value * cap.value, dtype=torch.float64, device=device)
        if self.svd_type == "rsvd":
            om = self.omega_source(nr.value, q.value, device)
            om = om.to(device=device, dtype=torch.float64).contiguous()
            om_ptr = _abi.ptr(om)
        else:
            om = None
            om_ptr = None
        key = ("proj", tuple(r.shapes() for r in refs), k, bytes(opts))
        _abi.call("ctm_calculate_projectors",
                  [arr, D, d, k, ctypes.byref(opts), om_ptr, _abi.ptr(p1buf), _abi.ptr(p2buf),
                   ctypes.c_void_p(chi_slot.data_ptr())], device, key=key)
        e1 = ipeps[sites[0]]["E"][(3 + k) % 4].shape[0]
        c4 = ipeps[sites[3]]["E"][(k + 3) % 4].shape[1]
        qD1 = (e1, D, D)
        qD4 = (c4, D, D)
        pend = PendingProjectors(p1buf, p2buf, p1r.value, p2r.value, qD1, qD4, chi_slot)
        pend.keep = (refs, om)
        pend.cap = cap.value
        return pend

    def _calculate(self, ipeps, sites, k):
        device = ipeps[sites[0]]["A"].device
        slot = torch.zeros(1, dtype=torch.int64, device=device)
        pend = self.launch(ipeps, sites, k, slot)
        return pend.finish(slot.item())

    def calculate_half_system(self, ipeps, sites, k):
        """acetn/renormalization/projectors.py:138-174."""
        return self._calculate(ipeps, sites, k)

    def calculate_full_system(self, ipeps, sites, k):
        """acetn/renormalization/projectors.py:176-217."""
        return self._calculate(ipeps, sites, k)
