"""Many independent iPEPS advanced together on one GPU.

A parameter sweep (say 32 transverse-field Ising states of uneven D and chi)
is a set of independent CTMRG runs.  One run at D = 3..5, chi = 48..100
leaves most of the GPU idle (its contractions are a few hundred tiles, its
QR and SVD run on a handful of SMs), and the reference cannot even hold two
runs in one process (its site tensors live in a class-level dictionary,
acetn/ipeps/tensor_network.py:12).  ``BatchedCTMRG`` owns one state and one
``DirectionalMover`` per instance and runs every instance's moves on its own
stream, so the kernels of all instances share the GPU at once; once every
environment has reached chi, one whole iteration of all instances is captured
as a single CUDA graph (fixed-width projectors, no host synchronisation) and
replayed.  Each instance computes exactly what ``ctmrg`` computes for it alone
with the same test matrices.
"""

import torch

from .config import resolve
from .ctmrg import pair_order
from .directional_mover import DirectionalMover


class BatchedCTMRG:
    def __init__(self, states, config, omega_sources=None):
        if not states:
            raise ValueError("BatchedCTMRG needs at least one state")
        self.states = list(states)
        self.config = resolve(config)
        sources = omega_sources or [None] * len(self.states)
        if len(sources) != len(self.states):
            raise ValueError("one omega source per state")
        self.movers = [DirectionalMover(self.config, src) for src in sources]
        for m in self.movers:
            m.graph_mode = True
        self.device = self.states[0][self.states[0].site_list[0]]["A"].device
        self.streams = [torch.cuda.Stream(self.device) for _ in self.states]
        self.graph = None
        self.static = None
        self.counts = None

    # ------------------------------------------------------------ helpers
    def saturated(self):
        for st in self.states:
            chi = st.dims["chi"]
            for s in st.site_list:
                if any(tuple(c.shape) != (chi, chi) for c in st[s]["C"]):
                    return False
        return True

    def grow(self, max_iterations=10):
        """Eager iterations, one instance after another, until every
        environment has reached chi (the widths still change, so these
        iterations synchronise once per pair of moves)."""
        for _ in range(max_iterations):
            if self.saturated():
                return
            for st, mv in zip(self.states, self.movers):
                mv.graph_mode = False
                for kind, i1, i2 in pair_order(st.nx, st.ny):
                    mv.move_pair(st, kind, i1, i2)
                mv.graph_mode = True
        if not self.saturated():
            raise RuntimeError("environments did not reach chi")

    def _iteration(self):
        """One iteration of every instance, each on its own stream forked
        from the current one; returns the truncation counts minus chi."""
        main = torch.cuda.current_stream(self.device)
        counts = []
        for st, mv, sm in zip(self.states, self.movers, self.streams):
            sm.wait_stream(main)
            with torch.cuda.stream(sm):
                for kind, i1, i2 in pair_order(st.nx, st.ny):
                    mv.move_pair(st, kind, i1, i2)
                    # truncation counts relative to this instance's chi
                    counts.append(mv.last_counts - st.dims["chi"])
        for st, sm in zip(self.states, self.streams):
            for s in st.site_list:
                for t in st[s]["C"] + st[s]["E"]:
                    t.record_stream(main)
            main.wait_stream(sm)
        return counts

    def iteration(self):
        """One eager (uncaptured) iteration of all instances at once."""
        if not self.saturated():
            raise ValueError("BatchedCTMRG.iteration needs saturated environments: call grow()")
        self.counts = torch.cat(self._iteration())

    # ------------------------------------------------------------ CUDA graph
    def capture(self, warmup=1):
        if not self.saturated():
            raise ValueError("BatchedCTMRG.capture needs saturated environments: call grow()")
        for _ in range(warmup):
            self._iteration()
        self.static = [{s: {"C": [c.clone() for c in st[s]["C"]],
                            "E": [e.clone() for e in st[s]["E"]]} for s in st.site_list}
                       for st in self.states]
        self._point_at_static()
        torch.cuda.synchronize(self.device)
        self.graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(self.graph):
            counts = self._iteration()
            self.counts = torch.cat(counts)
            for st, stat in zip(self.states, self.static):
                for s in st.site_list:
                    for k in range(4):
                        stat[s]["C"][k].copy_(st[s]["C"][k])
                        stat[s]["E"][k].copy_(st[s]["E"][k])
        self._point_at_static()
        return self

    def _point_at_static(self):
        for st, stat in zip(self.states, self.static):
            for s in st.site_list:
                for k in range(4):
                    st[s]["C"][k] = stat[s]["C"][k]
                    st[s]["E"][k] = stat[s]["E"][k]

    def replay(self, iterations=1):
        if self.graph is None:
            raise RuntimeError("BatchedCTMRG.replay before capture")
        for _ in range(iterations):
            self.graph.replay()
        self._point_at_static()

    def truncated(self):
        """True when a truncation of the last iteration kept fewer singular
        values than its instance's chi (synchronises)."""
        return bool((self.counts < 0).any().item())

    def moves_per_iteration(self):
        return sum(2 * (st.nx + st.ny) for st in self.states)
