"""One CTMRG iteration captured as a CUDA graph.

Once the boundary dimension has saturated (every C/E at chi and every
truncation keeping chi_cap singular values), the moves of an iteration have
fixed shapes; ``CTMRGGraph`` captures the 2 (nx + ny) moves of one iteration
of ``ctmrg`` (acetn/renormalization/ctmrg.py:18-31), run as left/right and
up/down pairs on side streams, into one CUDA graph and
replays it, removing the host work and the per-move synchronisation of the
eager path.  The projectors are written with a fixed width (zero columns
beyond a truncation count smaller than chi), which leaves the physics
unchanged; ``truncated()`` reports whether any count fell below the width.

The state lives in static buffers owned by this object: ``ipeps`` points at
them after ``capture()`` and after every ``replay()``.
"""

import torch

from .config import resolve
from .ctmrg import pair_order
from .directional_mover import DirectionalMover


class CTMRGGraph:
    def __init__(self, ipeps, config, omega_source=None):
        self.ipeps = ipeps
        self.config = resolve(config)
        self.mover = DirectionalMover(self.config, omega_source)
        self.mover.graph_mode = True
        self.order = pair_order(ipeps.nx, ipeps.ny)
        self.graph = None
        self.static = None
        self.counts = []

    def _check_saturated(self):
        chi = self.ipeps.dims["chi"]
        for s in self.ipeps.site_list:
            for c in self.ipeps[s]["C"]:
                if tuple(c.shape) != (chi, chi):
                    raise ValueError("CTMRGGraph.capture needs every C at (chi, chi): run eager "
                                     "iterations until the environment has saturated")

    def _iteration(self):
        counts = []
        for kind, i1, i2 in self.order:
            self.mover.move_pair(self.ipeps, kind, i1, i2)
            counts.append(self.mover.last_counts)
        return counts

    def capture(self, warmup=1):
        """Runs ``warmup`` eager fixed-width iterations, then captures one."""
        self._check_saturated()
        for _ in range(warmup):
            self._iteration()
        ip = self.ipeps
        self.static = {s: {"C": [c.clone() for c in ip[s]["C"]],
                           "E": [e.clone() for e in ip[s]["E"]]} for s in ip.site_list}
        self._point_at_static()
        torch.cuda.synchronize()
        self.graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(self.graph):
            counts = self._iteration()
            self.counts = torch.cat(counts)
            for s in ip.site_list:
                for k in range(4):
                    self.static[s]["C"][k].copy_(ip[s]["C"][k])
                    self.static[s]["E"][k].copy_(ip[s]["E"][k])
        self._point_at_static()
        return self

    def _point_at_static(self):
        for s in self.ipeps.site_list:
            for k in range(4):
                self.ipeps[s]["C"][k] = self.static[s]["C"][k]
                self.ipeps[s]["E"][k] = self.static[s]["E"][k]

    def replay(self, iterations=1):
        if self.graph is None:
            raise RuntimeError("CTMRGGraph.replay before capture")
        for _ in range(iterations):
            self.graph.replay()
        self._point_at_static()

    def truncated(self):
        """True when a truncation of the last replay kept fewer than chi_cap
        singular values (synchronises)."""
        chi = self.ipeps.dims["chi"]
        return bool((self.counts < chi).any().item())
