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
    def _spec(self, ipeps, k, idx):
        """Site quadruples of every row (column) of move (k, idx) and the
        (s1, s2, i, j) renormalization jobs (directional_mover.py:23-97)."""
        nx, ny = ipeps.nx, ipeps.ny
        if k == 0:
            return (k, [self.left_sites(ipeps, idx, yi) for yi in range(ny)],
                    [((idx, yi), ((idx + 1) % nx, yi), yi, (yi + 1) % ny) for yi in range(ny)])
        if k == 1:
            return (k, [self.up_sites(ipeps, xi, idx) for xi in range(nx)],
                    [((xi, idx), (xi, (idx - 1 + ny) % ny), xi, (xi + 1) % nx)
                     for xi in range(nx)])
        if k == 2:
            return (k, [self.right_sites(ipeps, idx, yi) for yi in range(ny)],
                    [((idx, yi), ((idx - 1 + nx) % nx, yi), yi, (yi - 1 + ny) % ny)
                     for yi in range(ny)])
        return (k, [self.down_sites(ipeps, xi, idx) for xi in range(nx)],
                [((xi, idx), (xi, (idx + 1) % ny), xi, (xi - 1 + nx) % nx) for xi in range(nx)])

    def _projectors_all(self, ipeps, specs):
        """Projector pairs of every row of every move in ``specs``, each on
        its own side stream; one device-to-host read of the truncated widths
        for all of them (none in graph mode)."""
        rows = [(m, k, sites) for m, (k, site_lists, _) in enumerate(specs) for sites in site_lists]
        a = ipeps[rows[0][2][0]]["A"]
        _abi.require_cuda(a, "A", storage=True)  # before any stream is forked
        device = a.device
        slots = torch.zeros(len(rows), dtype=torch.int64, device=device)
        streams = self._fork(device, len(rows))
        pend = []
        for n, (_, k, sites) in enumerate(rows):
            if streams is None:
                pend.append(self.projector_calculator.launch(ipeps, sites, k, slots[n:n + 1],
                                                             fixed_width=self.graph_mode))
                continue
            with torch.cuda.stream(streams[n]):
                pend.append(self.projector_calculator.launch(ipeps, sites, k, slots[n:n + 1],
                                                             fixed_width=self.graph_mode))
        self._join(device, streams, [t for p in pend for t in (p.p1buf, p.p2buf)])
        proj = [({}, {}) for _ in specs]
        row_in_move = [0] * len(specs)
        if self.graph_mode:
            self.last_counts = slots
            widths = [p.cap for p in pend]
        else:
            widths = slots.tolist()  # the one device-to-host read
        for (m, _, _), p, c in zip(rows, pend, widths):
            if c < 1:
                raise RuntimeError("projector truncation left no singular value above the cutoff")
            n = row_in_move[m]
            proj[m][0][n], proj[m][1][n] = p.finish(c)
            row_in_move[m] += 1
        return proj

    def _run(self, ipeps, specs):
        proj = self._projectors_all(ipeps, specs)
        self._renormalize_all(ipeps, [(proj[m][0], proj[m][1], job, k)
                                      for m, (k, _, jobs) in enumerate(specs) for job in jobs])

    def left_move(self, ipeps, xi):
        """directional_mover.py:23-40."""
        self._run(ipeps, [self._spec(ipeps, 0, xi)])

    def up_move(self, ipeps, yi):
        """directional_mover.py:42-59."""
        self._run(ipeps, [self._spec(ipeps, 1, yi)])

    def right_move(self, ipeps, xi):
        """directional_mover.py:61-78."""
        self._run(ipeps, [self._spec(ipeps, 2, xi)])

    def down_move(self, ipeps, yi):
        """directional_mover.py:80-97."""
        self._run(ipeps, [self._spec(ipeps, 3, yi)])

    def move(self, ipeps, k, idx):
        return (self.left_move, self.up_move, self.right_move, self.down_move)[k](ipeps, idx)

    def left_right_move(self, ipeps, x1, x2):
        """The left move of column x1 and the right move of column x2 at once.
        A left move reads C0, C3, E0, E2, E3 and writes C0, C3, E3; a right
        move reads C1, C2, E0, E1, E2 and writes C1, C2, E1 (directional_mover.py
        :273-366 with k = 0, 2): neither reads what the other writes, so the
        result equals left_move(x1) followed by right_move(x2) bit for bit.
        The reference runs the same pair on two groups of ranks
        (left_right_move_dist, directional_mover.py:183-226); here the rows
        of both moves run on side streams of one GPU."""
        self._run(ipeps, [self._spec(ipeps, 0, x1), self._spec(ipeps, 2, x2)])

    def up_down_move(self, ipeps, y1, y2):
        """The up move of row y1 and the down move of row y2 at once (they
        touch disjoint tensors as left and right do; the reference's
        up_down_move_dist, directional_mover.py:228-271)."""
        self._run(ipeps, [self._spec(ipeps, 1, y1), self._spec(ipeps, 3, y2)])

    def moves_at_once(self, ipeps, moves):
        """Runs data-independent moves [(k, idx), ...] together (all their
        rows on side streams), drawing the rSVD test matrices in the listed
        order: one left and one right move, or one up and one down move."""
        kinds = sorted(k % 2 for k, _ in moves)
        if len(moves) != 2 or kinds[0] != kinds[1] or moves[0][0] == moves[1][0]:
            raise ValueError("moves_at_once takes a left/right or an up/down pair of moves")
        self._run(ipeps, [self._spec(ipeps, k, idx) for k, idx in moves])

    def move_pair(self, ipeps, k, idx1, idx2):
        """left_right_move (k = 0) or up_down_move (k = 1)."""
        if k == 0:
            return self.left_right_move(ipeps, idx1, idx2)
        return self.up_down_move(ipeps, idx1, idx2)

    # ---------------------------------------------------------------- renormalization
    def _renormalize_all(self, ipeps, jobs):
        """renormalize_boundary for every (proj1, proj2, (s1, s2, i, j), k):
        each reads site s1 and writes site s2, no s2 of a move is an s1 of
        it, and the moves of a pair write tensors the other does not read."""
        device = ipeps[jobs[0][2][0]]["A"].device
        streams = self._fork(device, len(jobs))
        outs = []
        for n, (proj1, proj2, (s1, s2, i, j), k) in enumerate(jobs):
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
