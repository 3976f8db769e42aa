"""Directional moves on the GB300 library.

Mirror of ``DirectionalMover`` (acetn/renormalization/directional_mover.py:5-366)
for the non-distributed moves.  One move enqueues the projector pairs of all
rows (columns) of the move, reads their truncated widths with a single
device-to-host copy, then enqueues the boundary renormalization of every row
(column).  The rows of a move are independent (each renormalization reads
one site and writes another), so with ``concurrent`` (the default) they run
on side streams forked from and joined back into the caller's stream.  New tensors are written back by list-item assignment, as in
``renormalize_boundary`` of the reference.
"""

import torch

from . import _abi
from .config import resolve
from .projectors import ProjectorCalculator


class DirectionalMover:
    def __init__(self, config, omega_source=None):
        self.config = resolve(config)
        self.projector_calculator = ProjectorCalculator(self.config, omega_source)
        self.calculate_projectors = self.projector_calculator.calculate
        self.precision = self.config.precision
        # graph mode: no host synchronisation, projectors of fixed width chi_cap;
        # the truncation counts of the last move stay on the device
        self.graph_mode = False
        self.last_counts = None
        self.concurrent = True
        self._streams = {}

    # ---------------------------------------------------------------- streams
    def _fork(self, device, n):
        """Side streams for n concurrent rows, each ordered after the caller's
        stream; None when the rows run in order on the caller's stream."""
        if not self.concurrent or n < 2:
            return None
        key = torch.device(device).index
        pool = self._streams.setdefault(key, [])
        while len(pool) < n:
            pool.append(torch.cuda.Stream(device))
        main = torch.cuda.current_stream(device)
        for s in pool[:n]:
            s.wait_stream(main)
        return pool[:n]

    @staticmethod
    def _join(device, streams, tensors):
        if streams is None:
            return
        main = torch.cuda.current_stream(device)
        for t in tensors:
            t.record_stream(main)
        for s in streams:
            main.wait_stream(s)

    # ---------------------------------------------------------------- sites
    @staticmethod
    def left_sites(ipeps, xi, yi):
        """calculate_left_projectors (directional_mover.py:99-118)."""
        nx, ny = ipeps.nx, ipeps.ny
        xj, yj = (xi + 1) % nx, (yi - 1 + ny) % ny
        return [(xi, yi), (xj, yi), (xj, yj), (xi, yj)]

    @staticmethod
    def right_sites(ipeps, xi, yi):
        """calculate_right_projectors (directional_mover.py:120-139)."""
        nx, ny = ipeps.nx, ipeps.ny
        xj, yj = (xi - 1 + nx) % nx, (yi + 1) % ny
        return [(xi, yi), (xj, yi), (xj, yj), (xi, yj)]

    @staticmethod
    def up_sites(ipeps, xi, yi):
        """calculate_up_projectors (directional_mover.py:141-160)."""
        nx, ny = ipeps.nx, ipeps.ny
        xj, yj = (xi - 1 + nx) % nx, (yi - 1 + ny) % ny
        return [(xi, yi), (xi, yj), (xj, yj), (xj, yi)]

    @staticmethod
    def down_sites(ipeps, xi, yi):
        """calculate_down_projectors (directional_mover.py:162-181)."""
        nx, ny = ipeps.nx, ipeps.ny
        xj, yj = (xi + 1) % nx, (yi + 1) % ny
        return [(xi, yi), (xi, yj), (xj, yj), (xj, yi)]

    def calculate_left_projectors(self, ipeps, xi, yi):
        return self.calculate_projectors(ipeps, self.left_sites(ipeps, xi, yi), k=0)

    def calculate_right_projectors(self, ipeps, xi, yi):
        return self.calculate_projectors(ipeps, self.right_sites(ipeps, xi, yi), k=2)

    def calculate_up_projectors(self, ipeps, xi, yi):
        return self.calculate_projectors(ipeps, self.up_sites(ipeps, xi, yi), k=1)

    def calculate_down_projectors(self, ipeps, xi, yi):
        return self.calculate_projectors(ipeps, self.down_sites(ipeps, xi, yi), k=3)

    # ---------------------------------------------------------------- moves
    def _projectors_all(self, ipeps, site_lists, k):
        a = ipeps[site_lists[0][0]]["A"]
        _abi.require_cuda(a, "A", storage=True)  # before any stream is forked
        device = a.device
        slots = torch.zeros(len(site_lists), dtype=torch.int64, device=device)
        streams = self._fork(device, len(site_lists))
        pend = []
        for n, sites in enumerate(site_lists):
            if streams is None:
                pend.append(self.projector_calculator.launch(ipeps, sites, k, slots[n:n + 1],
                                                             fixed_width=self.graph_mode))
                continue
            with torch.cuda.stream(streams[n]):
                pend.append(self.projector_calculator.launch(ipeps, sites, k, slots[n:n + 1],
                                                             fixed_width=self.graph_mode))
        self._join(device, streams, [t for p in pend for t in (p.p1buf, p.p2buf)])
        if self.graph_mode:
            self.last_counts = slots
            proj1, proj2 = {}, {}
            for n, p in enumerate(pend):
                proj1[n], proj2[n] = p.finish(p.cap)
            return proj1, proj2
        chis = slots.tolist()  # the move's one device-to-host read
        proj1, proj2 = {}, {}
        for n, (p, c) in enumerate(zip(pend, chis)):
            if c < 1:
                raise RuntimeError("projector truncation left no singular value above the cutoff")
            proj1[n], proj2[n] = p.finish(c)
        return proj1, proj2

    def left_move(self, ipeps, xi):
        """directional_mover.py:23-40."""
        ny, nx = ipeps.ny, ipeps.nx
        proj1, proj2 = self._projectors_all(
            ipeps, [self.left_sites(ipeps, xi, yi) for yi in range(ny)], 0)
        self._renormalize_all(ipeps, proj1, proj2,
                              [((xi, yi), ((xi + 1) % nx, yi), yi, (yi + 1) % ny)
                               for yi in range(ny)], 0)

    def up_move(self, ipeps, yi):
        """directional_mover.py:42-59."""
        nx, ny = ipeps.nx, ipeps.ny
        proj1, proj2 = self._projectors_all(
            ipeps, [self.up_sites(ipeps, xi, yi) for xi in range(nx)], 1)
        self._renormalize_all(ipeps, proj1, proj2,
                              [((xi, yi), (xi, (yi - 1 + ny) % ny), xi, (xi + 1) % nx)
                               for xi in range(nx)], 1)

    def right_move(self, ipeps, xi):
        """directional_mover.py:61-78."""
        ny, nx = ipeps.ny, ipeps.nx
        proj1, proj2 = self._projectors_all(
            ipeps, [self.right_sites(ipeps, xi, yi) for yi in range(ny)], 2)
        self._renormalize_all(ipeps, proj1, proj2,
                              [((xi, yi), ((xi - 1 + nx) % nx, yi), yi, (yi - 1 + ny) % ny)
                               for yi in range(ny)], 2)

    def down_move(self, ipeps, yi):
        """directional_mover.py:80-97."""
        nx, ny = ipeps.nx, ipeps.ny
        proj1, proj2 = self._projectors_all(
            ipeps, [self.down_sites(ipeps, xi, yi) for xi in range(nx)], 3)
        self._renormalize_all(ipeps, proj1, proj2,
                              [((xi, yi), (xi, (yi + 1) % ny), xi, (xi - 1 + nx) % nx)
                               for xi in range(nx)], 3)

    def move(self, ipeps, k, idx):
        return (self.left_move, self.up_move, self.right_move, self.down_move)[k](ipeps, idx)

    # ---------------------------------------------------------------- renormalization
    def _renormalize_all(self, ipeps, proj1, proj2, jobs, k):
        """renormalize_boundary for every (s1, s2, i, j) of a move: each reads
        site s1 and writes site s2, and no s2 of a move is an s1 of it."""
        device = ipeps[jobs[0][0]]["A"].device
        streams = self._fork(device, len(jobs))
        outs = []
        for n, (s1, s2, i, j) in enumerate(jobs):
            if streams is None:
                self.renormalize_boundary(ipeps, proj1, proj2, s1, s2, i, j, k)
                continue
            with torch.cuda.stream(streams[n]):
                self.renormalize_boundary(ipeps, proj1, proj2, s1, s2, i, j, k)
            outs += [ipeps[s2]["C"][(3 + k) % 4], ipeps[s2]["C"][k], ipeps[s2]["E"][(3 + k) % 4]]
        self._join(device, streams, outs)

    def renormalize_boundary(self, ipeps, proj1, proj2, s1, s2, i, j, k):
        """directional_mover.py:273-303: writes C[(3+k)%4], C[k], E[(3+k)%4] of s2."""
        site = ipeps[s1]
        ref = _abi.SiteRef(site)
        D, d, device = ref.D, ref.d, ref.device
        p1i, p2j, p2i, p1j = (t.contiguous() for t in (proj1[i], proj2[j], proj2[i], proj1[j]))
        x1i, x2j, x2i, x1j = p1i.shape[-1], p2j.shape[-1], p2i.shape[-1], p1j.shape[-1]
        a = site["E"][(2 + k) % 4].shape[0]
        cc = site["E"][k % 4].shape[1]
        # the C ABI takes projector widths only: their leading legs must chain
        # with the site's tensors (the reference's einsums would fail otherwise)
        expect = ((p1i, site["C"][(3 + k) % 4].shape[1]), (p2j, site["C"][k % 4].shape[0]),
                  (p2i, site["E"][(3 + k) % 4].shape[0]), (p1j, site["E"][(3 + k) % 4].shape[1]))
        for p, rows in expect:
            if p.dim() != 4 or p.shape[0] != rows or p.shape[1] != D or p.shape[2] != D:
                raise ValueError(f"projector of shape {tuple(p.shape)} does not chain with "
                                 f"site {s1} in direction {k}")
            _abi.require_cuda(p, "projector")
        c1 = torch.empty(a, x1i, dtype=torch.float64, device=device)
        c2 = torch.empty(x2j, cc, dtype=torch.float64, device=device)
        e3 = torch.empty(x2i, x1j, D, D, dtype=torch.float64, device=device)
        key = ("renorm", ref.shapes(), k, x1i, x2j, x2i, x1j, self.precision)
        _abi.call("ctm_renormalize_boundary",
                  [ref.pointer, D, d, k, _abi.ptr(p1i), x1i, _abi.ptr(p2j), x2j, _abi.ptr(p2i),
                   x2i, _abi.ptr(p1j), x1j, _abi.ptr(c1), _abi.ptr(c2), _abi.ptr(e3),
                   _abi.PREC[self.precision]], device, key=key)
        dt = ipeps[s2]["A"].dtype  # float32 storage keeps its type
        ipeps[s2]["C"][(3 + k) % 4] = c1.to(dt)
        ipeps[s2]["C"][k] = c2.to(dt)
        ipeps[s2]["E"][(3 + k) % 4] = e3.to(dt)
