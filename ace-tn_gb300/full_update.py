"""The two places where the full update of Ace-TN meets the CTMRG path.

* ``build_norm_tensor(ipeps, bond, a1q, a2q)`` -- the full update's norm
  tensor (acetn/evolution/full_update.py:163-236): the bond RDM's
  environment chain contracted with the reduced site tensors, on the GPU in
  FP64.
* ``absorb_bond(mover, ipeps, bond)`` -- ``FastFullUpdater.absorb_bond``
  (acetn/evolution/fast_full_update.py:71-101): the two directional moves
  that re-absorb an updated bond into the boundary.  They touch disjoint
  tensors, so they run as one pair (``DirectionalMover.moves_at_once``, the
  pairs of ``absorb_bond_dist``, :103-129) in the reference's order of the
  two moves; the result equals the sequential order bit for bit.
"""

import torch

from . import _abi


def build_norm_tensor(ipeps, bond, a1q, a2q):
    """n12[y, x, Y, X] for bond (s1, s2, k); a1q and a2q are (D, D, D, nD)
    float64 CUDA tensors (legs (r, d, u, y) and (d, l, u, x))."""
    s1, s2, k = bond
    r1 = _abi.SiteRef(ipeps[s1])
    r2 = _abi.SiteRef(ipeps[s2])
    D, d = r1.D, r1.d
    for name, t in (("a1q", a1q), ("a2q", a2q)):
        _abi.require_cuda(t, name)
        if t.dim() != 4 or tuple(t.shape[:3]) != (D, D, D):
            raise ValueError(f"{name} must have shape (D, D, D, nD) with D={D}, got {tuple(t.shape)}")
    if a1q.shape[3] != a2q.shape[3]:
        raise ValueError("a1q and a2q must have the same last dimension")
    nD = int(a1q.shape[3])
    a1q, a2q = a1q.contiguous(), a2q.contiguous()
    out = torch.empty(nD, nD, nD, nD, dtype=torch.float64, device=r1.device)
    _abi.call("ctm_norm_tensor", [r1.pointer, r2.pointer, D, d, k, _abi.ptr(a1q), _abi.ptr(a2q), nD,
                                  _abi.ptr(out)], r1.device,
              key=("norm_tensor", r1.shapes(), r2.shapes(), k, nD))
    return out


def absorb_bond(mover, ipeps, bond):
    """fast_full_update.py:71-101 with the moves of each case run as a pair."""
    s1, s2, k = bond
    if k == 0:    # right_move(s1[0]), then left_move(s2[0])
        moves = [(2, s1[0]), (0, s2[0])]
    elif k == 1:  # down_move(s1[1]), then up_move(s2[1])
        moves = [(3, s1[1]), (1, s2[1])]
    elif k == 2:  # left_move(s1[0]), then right_move(s2[0])
        moves = [(0, s1[0]), (2, s2[0])]
    elif k == 3:  # up_move(s1[1]), then down_move(s2[1])
        moves = [(1, s1[1]), (3, s2[1])]
    else:
        raise ValueError(f"bond direction must be 0..3, got {k}")
    mover.moves_at_once(ipeps, moves)
