"""CTMRG driver on the GB300 library.

Mirror of ``ctmrg(ipeps, config)`` (acetn/renormalization/ctmrg.py:4-31),
non-distributed branch: ``config.steps`` iterations of left/right moves for
every column followed by up/down moves for every row.
"""

from ._progress import tqdm

from .config import resolve
from .directional_mover import DirectionalMover


def sweep_order(nx, ny):
    """Move sequence of one iteration as (k, index) pairs (ctmrg.py:25-31)."""
    order = []
    for xi in range(nx):
        order.append((0, xi))
        order.append((2, (nx - xi + 1) % nx))
    for yi in range(ny):
        order.append((1, (ny - yi + 1) % ny))
        order.append((3, yi))
    return order


def pair_order(nx, ny):
    """The same iteration as (kind, i1, i2) pairs: kind 0 = left move of
    column i1 with the right move of column i2, kind 1 = up move of row i1
    with the down move of row i2 -- the consecutive moves of ctmrg.py:25-31,
    which touch disjoint tensors (the pairs of the reference's distributed
    branch, ctmrg.py:20-24)."""
    return ([(0, xi, (nx - xi + 1) % nx) for xi in range(nx)]
            + [(1, (ny - yi + 1) % ny, yi) for yi in range(ny)])


def ctmrg(ipeps, config, omega_source=None, steps=None, pairs=True):
    """``pairs`` runs each left/right (up/down) pair of moves at once
    (DirectionalMover.left_right_move); the result equals the sequential
    order of the reference bit for bit."""
    cfg = resolve(config)
    mover = DirectionalMover(cfg, omega_source)
    disable = cfg.disable_progressbar or getattr(ipeps, "rank", 0) != 0
    pbar = tqdm(desc="Renormalizing boundary tensors", unit=" sweeps", disable=disable)
    for _ in range(cfg.steps if steps is None else steps):
        pbar.update(1)
        if pairs:
            for kind, i1, i2 in pair_order(ipeps.nx, ipeps.ny):
                mover.move_pair(ipeps, kind, i1, i2)
        else:
            for k, idx in sweep_order(ipeps.nx, ipeps.ny):
                mover.move(ipeps, k, idx)
    pbar.close()
    return ipeps
