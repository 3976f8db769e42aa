"""CTMRG moves/s of the GB300 library at D=6, chi=144 (Heisenberg J=1, 2x2 unit
cell, d=2, half-system rSVD projectors, oversampling 16, 2 power iterations).

A step is one directional move (projectors of both rows/columns of the move,
then the boundary renormalization of both).  The environment is first grown
to chi (two untimed CTMRG iterations), then W untimed moves, then K timed
moves, each bracketed by CUDA events on the launching stream with an L2
flush (a 256 MiB write) between moves outside the events.

Usage: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
       [--precision fp64|mixed]
Under torchrun every rank runs an independent replica (the path does not
shard: "scaling": "weak"); rank 0 prints one JSON line.
"""

import argparse
import importlib
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

D, CHI, PHYS, OVERSAMPLING, NITER, SEED = 6, 144, 2, 16, 2, 20250
N_Q = CHI * D * D
METRIC = "CTMRG moves/s at D=6, chi=144 (Heisenberg, 2x2, half-system rSVD os=16 niter=2)"
# DRAM bytes (read + write) of one launch of the double-layer contraction GEMM
# at this workload (M = D^4 = 1296, N = chi^2 = 20736, K = 1296, 3xBF16),
# from the ncu capture summarised in profiles/tc_gemm_double_layer_d6_chi144.md
DL_GEMM_TRAFFIC = 118.590208e6 + 56.284160e6


def move_flops(D, chi, q, d=2, ny=2, niter=2):
    """Algorithmic FLOPs of one move (GEMM-shaped work only; QR and the
    q x N SVD excluded), per row: two quarter tensors, the rSVD GEMM chain,
    the two projector products, and the boundary renormalization."""
    n = chi * D * D
    per_row = (2 * (2 * chi**3 * D**2 + 2 * chi**3 * D**4 + 4 * chi**2 * D**6 * d)
               + 2 * n * n * q * (4 + 4 * niter)
               + 4 * n * n * chi
               + 4 * chi**3 * D**4 + 4 * chi**2 * D**6 * d + 8 * chi**3 * D**2)
    return ny * per_row


class ClockSampler:
    """nvidia-smi clock / throttle-reason samples during the timed region:
    sampled every 50 ms from before the region starts (start() waits for the
    first sample), each sample stamped on arrival; stop() keeps the samples
    that arrived inside the window set by mark_start() / mark_end() (plus one
    sampling interval), or the nearest one when the region is shorter than
    the interval."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    INTERVAL_MS = 50

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []
        self.t0 = self.t1 = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.QUERY}", "--format=csv,noheader,nounits",
                 "-i", str(self.index), "-lms", str(self.INTERVAL_MS)],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            deadline = time.monotonic() + 5.0
            while not self.lines and time.monotonic() < deadline and self.proc.poll() is None:
                time.sleep(0.01)
        except (OSError, ValueError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append((time.monotonic(), line.strip()))

    def mark_start(self):
        self.t0 = time.monotonic()

    def mark_end(self):
        self.t1 = time.monotonic()

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, mx, reasons = [], None, set()
        names = ["active", "hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown",
                 "sw_power_cap"]
        lines = list(self.lines)
        in_window = True
        if self.t0 is not None and self.t1 is not None and lines:
            slack = self.INTERVAL_MS / 1e3
            keep = [x for x in lines if self.t0 <= x[0] <= self.t1 + slack]
            if not keep:
                in_window = False
                keep = [min(lines, key=lambda x: abs(x[0] - 0.5 * (self.t0 + self.t1)))]
            lines = keep
        for _, line in lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for name, val in zip(names[1:], parts[5:9]):
                if val.lower() in ("active", "1", "yes"):
                    reasons.add(name)
        out = {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx,
               "reasons": sorted(reasons), "samples": len(sm),
               "interval_ms": self.INTERVAL_MS}
        if self.t0 is not None and self.t1 is not None:
            out["window_ms"] = round(1e3 * (self.t1 - self.t0), 1)
            out["in_window"] = in_window
        return out


def package():
    mod = importlib.import_module("ace-tn_gb300")
    sys.modules.setdefault("acetn_gb300", mod)
    return mod


def cpu_cores():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def cpu_model():
    try:
        with open("/proc/cpuinfo") as fh:
            for line in fh:
                if line.lower().startswith(("model name", "cpu part")):
                    return line.split(":", 1)[1].strip()
    except OSError:
        pass
    return "unknown"


# --------------------------------------------------------------------- oracle legs
def oracle_moves(st_np, moves, seed=1):
    """Times ``moves`` directional moves of the oracle (numpy, all host
    threads) starting from a saturated state; returns seconds per move."""
    from oracle import ctm_oracle as orc
    cfg = dict(projectors="half-system", svd_type="rsvd", rsvd_oversampling=OVERSAMPLING,
               rsvd_niter=NITER, svd_cutoff=1e-12)
    mover = orc.Mover(cfg, orc.OmegaStream(seed))
    order = orc.sweep_order(2, 2)
    times = []
    for i in range(moves):
        k, idx = order[i % len(order)]
        t0 = time.perf_counter()
        mover.move(st_np, k, idx)
        times.append(time.perf_counter() - t0)
    return times


def run_reference(args, rank):
    """--impl reference: the reference's CPU path restated by the oracle
    (numpy/LAPACK on the host cores), same config, metric and unit."""
    if rank != 0:
        return None
    import numpy as np
    from oracle import ctm_oracle as orc
    st = orc.random_state(D, CHI, seed=SEED)
    cfg = dict(projectors="half-system", svd_type="rsvd", rsvd_oversampling=OVERSAMPLING,
               rsvd_niter=NITER, svd_cutoff=1e-12)
    t0 = time.perf_counter()
    orc.ctmrg(st, cfg, orc.OmegaStream(SEED), steps=2)  # grow the environment to chi
    grow_s = time.perf_counter() - t0
    oracle_moves(st, args.warmup, seed=SEED + 1)
    times = oracle_moves(st, args.steps, seed=SEED + 2)
    total = sum(times)
    value = args.steps / total
    q = CHI + OVERSAMPLING
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "moves/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * total / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"heisenberg_2x2_D{D}_chi{CHI}_rsvd_os{OVERSAMPLING}_niter{NITER}",
                   "D": D, "chi": CHI, "phys": PHYS, "projectors": "half-system",
                   "svd_type": "rsvd", "seed": SEED},
        "cpu_baseline": {"value": value, "unit": "moves/s", "cores": cpu_cores(), "kind": "port",
                         "sample": f"{args.steps} moves after 2 growth iterations "
                                   f"({grow_s:.1f} s) and {args.warmup} warm-up moves",
                         "cpu_model": cpu_model()},
        "e2e": {"value": value, "unit": "moves/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
        "tflops": move_flops(D, CHI, q) / (total / args.steps) / 1e12,
    }
    return line


# --------------------------------------------------------------------- gb300 arm
def state_bytes(st):
    n = 0
    for s in st.site_list:
        v = st[s]
        n += v["A"].numel() * 8 + sum(t.numel() * 8 for t in v["C"]) + sum(t.numel() * 8 for t in v["E"])
    return n


def run_gb300(args, rank, world, local_rank):
    import numpy as np
    import torch
    import torch.distributed as dist

    gb = package()
    gb.build()
    dev = torch.device("cuda", local_rank)
    torch.cuda.set_device(dev)
    stream = torch.cuda.current_stream(dev)
    cfg = gb.CTMRGConfig(projectors="half-system", svd_type="rsvd", rsvd_oversampling=OVERSAMPLING,
                         rsvd_niter=NITER, svd_cutoff=1e-12, precision=args.precision,
                         disable_progressbar=True)
    gen = torch.Generator(device=dev)
    gen.manual_seed(SEED + rank)

    def omega(n, q, device):
        return torch.randn(n, q, dtype=torch.float64, device=device, generator=gen)

    st = gb.random_state(D, CHI, SEED, d=PHYS, device=dev)
    mover = gb.DirectionalMover(cfg, omega_source=omega)
    order = gb.sweep_order(2, 2)
    for _ in range(2):  # grow the environment to chi
        for k, idx in order:
            mover.move(st, k, idx)
    pos = 0
    for _ in range(args.warmup):
        k, idx = order[pos % len(order)]
        mover.move(st, k, idx)
        pos += 1
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    torch.cuda.synchronize(dev)
    if world > 1:
        dist.barrier()
    clocks = ClockSampler(local_rank)
    clocks.start()
    launches0 = gb._abi.kernel_launches()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(args.steps)]
    torch.cuda.synchronize(dev)
    clocks.mark_start()
    for i in range(args.steps):
        flush.zero_()
        k, idx = order[pos % len(order)]
        ev[i][0].record(stream)
        mover.move(st, k, idx)
        ev[i][1].record(stream)
        pos += 1
    torch.cuda.synchronize(dev)
    clocks.mark_end()
    launches = gb._abi.kernel_launches() - launches0
    qr_fallbacks = gb._abi.qr_fallbacks(dev)
    clk = clocks.stop()
    # per-kernel-class timing (CUDA events inside the library) on a separate,
    # untimed pass with the rows of each move run one after the other, so
    # that no two kernels of the pass share the GPU
    prof_moves = max(1, min(args.steps, 4))
    mover.concurrent = False
    pev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
           for _ in range(prof_moves)]
    gb._abi.profile_begin()
    for i in range(prof_moves):
        flush.zero_()
        k, idx = order[pos % len(order)]
        pev[i][0].record(stream)
        mover.move(st, k, idx)
        pev[i][1].record(stream)
        pos += 1
    torch.cuda.synchronize(dev)
    prof = gb._abi.profile_end()
    prof_move_ms = sum(a.elapsed_time(b) for a, b in pev) / prof_moves
    mover.concurrent = True
    ms = [a.elapsed_time(b) for a, b in ev]
    total_s = sum(ms) / 1e3
    eager = None
    if args.graph:
        # one CTMRG iteration (8 moves) captured as a CUDA graph and replayed;
        # the rSVD test matrices come from torch's default CUDA generator
        eager_total, eager_value = aggregate(total_s, args.steps, world, dev)
        eager = {"value": eager_value, "ms_per_step": 1e3 * eager_total / args.steps}
        graph = gb.CTMRGGraph(st, cfg).capture(warmup=1)
        graph.replay(1)
        replays = max(1, -(-args.steps // len(order)))
        gev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
               for _ in range(replays)]
        clocks = ClockSampler(local_rank)
        clocks.start()
        torch.cuda.synchronize(dev)
        clocks.mark_start()
        for i in range(replays):
            flush.zero_()
            gev[i][0].record(stream)
            graph.replay(1)
            gev[i][1].record(stream)
        torch.cuda.synchronize(dev)
        clocks.mark_end()
        clk = clocks.stop()
        total_s = sum(a.elapsed_time(b) for a, b in gev) / 1e3
        graph_truncated = graph.truncated()
        args.steps_timed = replays * len(order)
    total_max, value = aggregate(total_s, getattr(args, "steps_timed", args.steps), world, dev)

    # ---- e2e: host buffers through the public API, copies inside the timed region
    host = {s: {"A": st[s]["A"].cpu().pin_memory(),
                "C": [c.cpu().pin_memory() for c in st[s]["C"]],
                "E": [e.cpu().pin_memory() for e in st[s]["E"]]} for s in st.site_list}
    e2e_steps = max(1, min(args.steps, 4))
    h2d = d2h = 0
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    for i in range(e2e_steps):
        k, idx = order[pos % len(order)]
        pos += 1
        dst = gb.IpepsState(2, 2, st.dims, dev)
        for s in st.site_list:
            hs = host[s]
            dst[s] = {"A": hs["A"].to(dev, non_blocking=True),
                      "C": [c.to(dev, non_blocking=True) for c in hs["C"]],
                      "E": [e.to(dev, non_blocking=True) for e in hs["E"]]}
        h2d = state_bytes(dst)
        before = {s: (list(dst[s]["C"]), list(dst[s]["E"])) for s in st.site_list}
        mover.move(dst, k, idx)
        # read back the step's result: the tensors the move replaced (two
        # corners and one edge of each renormalised site), found by identity
        moved = 0
        for s in st.site_list:
            for key, old_list in zip(("C", "E"), before[s]):
                for n, t in enumerate(dst[s][key]):
                    if t is not old_list[n]:
                        host[s][key][n] = t.to("cpu", non_blocking=True)
                        moved += t.numel() * t.element_size()
        torch.cuda.synchronize(dev)
        for s in st.site_list:
            host[s]["C"] = [c if c.is_pinned() else c.pin_memory() for c in host[s]["C"]]
            host[s]["E"] = [e if e.is_pinned() else e.pin_memory() for e in host[s]["E"]]
        d2h = moved
    e2e_s = time.perf_counter() - t0
    e2e_value = world * e2e_steps / e2e_s

    compare = None
    if rank == 0 and not args.no_compare:
        compare = compare_paths(gb, st, cfg, dev, args.precision)

    peaks = {}
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            peaks = json.load(fh)
    except OSError:
        pass
    if args.precision == "mixed":
        # the double-layer contraction GEMMs (enlarged corners and edge
        # renormalization, 3xBF16 on tcgen05) are the largest kernel class
        dom_ms, dom_work, dom_n = prof["tc_gemm_double_layer"]
        dom = "tc_gemm_persistent_kernel (double-layer contraction, 3xBF16)"
        peak = peaks.get("bf16_tflops_sustained") or 1700.0
        peak_src = ("MEASURED_PEAKS.json bf16_tflops_sustained" if peaks
                    else "fallback 1.7 PF/s")
        bound = "tensor"
        traffic = DL_GEMM_TRAFFIC
    else:
        dom_ms, dom_work, dom_n = prof["gett_f64"]
        dom = "gett_kernel<double>"
        peak = fp64_peak_tflops(dev)
        peak_src = ("cuBLAS DGEMM 8192^3 measured by bench.py on this GPU "
                    "(no FP64 entry in MEASURED_PEAKS.json)")
        bound = "fp64"
        traffic = None
    achieved = (dom_work / (dom_ms / 1e3)) / 1e12 if dom_ms > 0 else None
    q = CHI + OVERSAMPLING
    line = None
    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "moves/s", "n_gpus": world,
            "steps": getattr(args, "steps_timed", args.steps), "warmup": args.warmup,
            "ms_per_step": 1e3 * total_max / getattr(args, "steps_timed", args.steps),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64" if args.precision == "fp64" else "bf16/3xbf16+f64",
            "data": "synthetic",
            "config": {"workload": f"heisenberg_2x2_D{D}_chi{CHI}_rsvd_os{OVERSAMPLING}_niter{NITER}",
                       "D": D, "chi": CHI, "phys": PHYS, "projectors": "half-system",
                       "svd_type": "rsvd", "precision": args.precision, "seed": SEED,
                       "l2": "256 MiB flush between timed moves; quarter tensors 215 MB each",
                       "parallelism": f"replicas x{world}"},
            "tflops": move_flops(D, CHI, q) / (total_max / getattr(args, "steps_timed", args.steps))
                      / 1e12,
            "roofline": {"bound": bound, "kernel": dom, "achieved": achieved, "peak": peak,
                         "unit": "TFLOP/s", "frac": (achieved / peak) if achieved else None,
                         "traffic": traffic, "launches": dom_n, "peak_source": peak_src,
                         "traffic_source": ("ncu dram__bytes_read.sum + dram__bytes_write.sum, "
                                            "one launch, profiles/tc_gemm_double_layer_d6_chi144.md "
                                            "(captured before the operand swap of this GEMM)"
                                            if traffic else None),
                         "work_per_launch": dom_work / dom_n if dom_n else None,
                         "share_of_step": (dom_ms / prof_moves) / prof_move_ms,
                         "timing": f"CUDA events around each launch, {prof_moves} moves with "
                                   "the rows run serially (ms_per_step there: "
                                   f"{prof_move_ms:.2f})"},
            "e2e": {"value": e2e_value, "unit": "moves/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h, "steps": e2e_steps},
            # graph replays run the captured launches of the eager moves
            "gpu_launches": int(launches) if not args.graph else
            int(round(launches / args.steps * args.steps_timed)),
            "execution": ("cuda_graph" if args.graph else "eager"),
            "qr_fallbacks_in_timed_moves": qr_fallbacks,
            "eager": eager,
            "comparison": compare,
            "breakdown_ms_per_step": {k: v[0] / prof_moves for k, v in prof.items() if v[2]},
            "clocks": clk,
        }
        if world == 1 and not args.no_cpu_baseline:
            st_np = type("S", (), {})
            from oracle import ctm_oracle as orc
            ost = orc.OracleState(
                {s: {"A": st[s]["A"].cpu().numpy(), "C": [c.cpu().numpy() for c in st[s]["C"]],
                     "E": [e.cpu().numpy() for e in st[s]["E"]]} for s in st.site_list}, 2, 2, CHI)
            times = oracle_moves(ost, args.cpu_moves)
            line["cpu_baseline"] = {"value": len(times) / sum(times), "unit": "moves/s",
                                    "cores": cpu_cores(), "kind": "port",
                                    "sample": f"{len(times)} oracle moves from the GPU run's "
                                              f"saturated chi={CHI} state",
                                    "cpu_model": cpu_model()}
    return line


def clone_state(gb, st):
    c = gb.IpepsState(st.nx, st.ny, st.dims, st.device)
    for s in st.site_list:
        v = st[s]
        c[s] = {"A": v["A"].clone(), "C": [t.clone() for t in v["C"]],
                "E": [t.clone() for t in v["E"]]}
    return c


def compare_paths(gb, st, cfg, dev, precision):
    """From the benchmark's saturated state: moves/s of this library's plain
    FP64 path (the drop-in), and the energy after one move in each precision
    with the same rSVD test matrices, next to the FP64 path's own spread
    between two draws of the test matrices (the rSVD's noise)."""
    import dataclasses
    import torch
    order = gb.sweep_order(2, 2)
    cfg64 = dataclasses.replace(cfg, precision="fp64")

    def seeded(seed):
        g = torch.Generator(device=dev)
        g.manual_seed(seed)
        return lambda n, q, device: torch.randn(n, q, dtype=torch.float64, device=device,
                                               generator=g)

    # FP64 path timing: two moves (one warm), CUDA events
    s64 = clone_state(gb, st)
    mover = gb.DirectionalMover(cfg64, omega_source=seeded(1))
    mover.move(s64, *order[0])
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize(dev)
    a.record()
    for k, idx in order[1:3]:
        mover.move(s64, k, idx)
    b.record()
    torch.cuda.synchronize(dev)
    fp64_ms = a.elapsed_time(b) / 2
    del s64
    # one-move energies
    model = gb.HeisenbergModel(1.0, device=dev)
    energies = {}
    for tag, c, seed in (("fp64", cfg64, 7), ("fp64_other_draw", cfg64, 8),
                         (precision, cfg, 7)):
        s1 = clone_state(gb, st)
        gb.DirectionalMover(c, omega_source=seeded(seed)).move(s1, *order[0])
        energies[tag] = float(gb.measure(s1, model, verbose=False)["Energy"])
        del s1
    e64 = energies["fp64"]
    return {"fp64_path": {"moves_per_s": 1e3 / fp64_ms, "ms_per_step": fp64_ms},
            "one_move_energy": energies,
            "rel_err_vs_fp64": abs(energies[precision] - e64) / abs(e64),
            "fp64_rsvd_draw_spread": abs(energies["fp64_other_draw"] - e64) / abs(e64)}


def aggregate(total_s, steps, world, device="cpu"):
    """Whole-job throughput of `world` independent replicas: every rank ran
    `steps` moves in `total_s` seconds; the job's time is the slowest rank's.
    Returns (max seconds over ranks, moves/s of the whole job)."""
    import torch
    import torch.distributed as dist
    t = torch.tensor([total_s], dtype=torch.float64, device=device)
    if world > 1:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        dist.barrier()
    total_max = float(t.item())
    return total_max, world * steps / total_max


_FP64_PEAK = {}


def fp64_peak_tflops(dev):
    import torch
    if dev in _FP64_PEAK:
        return _FP64_PEAK[dev]
    n = 4096
    a = torch.randn(n, n, dtype=torch.float64, device=dev)
    b = torch.randn(n, n, dtype=torch.float64, device=dev)
    for _ in range(2):
        torch.matmul(a, b)
    torch.cuda.synchronize(dev)
    best = 1e9
    for _ in range(3):
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record()
        torch.matmul(a, b)
        e.record()
        torch.cuda.synchronize(dev)
        best = min(best, s.elapsed_time(e) / 1e3)
    _FP64_PEAK[dev] = 2.0 * n**3 / best / 1e12
    return _FP64_PEAK[dev]


def run_profile_case(args):
    """The small case for kernel captures: a synthetic saturated environment
    (C, E at chi with seeded normal entries, unit Frobenius norm) and one
    left move (both projector pairs and both boundary triples), repeated
    ``--steps`` times, with a few hundred launches in total.  No growth
    iterations: the spectra are those of random tensors, not of a converged
    environment (the Jacobi sweep count depends on them)."""
    import torch

    gb = package()
    gb.build()
    dev = torch.device("cuda", 0)
    g = torch.Generator().manual_seed(SEED)
    st = gb.IpepsState(2, 2, {"phys": PHYS, "bond": D, "chi": CHI}, dev)
    ref = gb.random_state(D, CHI, SEED, d=PHYS, device=dev)

    def rnd(*shape):
        t = torch.randn(*shape, generator=g, dtype=torch.float64)
        return (t / t.norm()).to(dev)

    for s in ref.site_list:
        st[s] = {"A": ref[s]["A"], "C": [rnd(CHI, CHI) for _ in range(4)],
                 "E": [rnd(CHI, CHI, D, D) for _ in range(4)]}
    gen = torch.Generator(device=dev)
    gen.manual_seed(SEED)
    cfg = gb.CTMRGConfig(projectors="half-system", svd_type="rsvd",
                         rsvd_oversampling=OVERSAMPLING, rsvd_niter=NITER, svd_cutoff=1e-12,
                         precision=args.precision, disable_progressbar=True)
    mover = gb.DirectionalMover(cfg, omega_source=lambda n, q, device: torch.randn(
        n, q, dtype=torch.float64, device=device, generator=gen))
    mover.concurrent = False
    for _ in range(args.steps):
        mover.move(st, 0, 0)
    torch.cuda.synchronize(dev)
    return {"profile_case": "left move on a synthetic chi-saturated state", "moves": args.steps,
            "device_status": gb._abi.device_status()}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=8)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--precision", choices=["fp64", "mixed"], default="mixed")
    ap.add_argument("--graph", action="store_true",
                    help="time replays of one CUDA-graph-captured CTMRG iteration (8 moves)")
    ap.add_argument("--no-compare", action="store_true",
                    help="skip the FP64-path timing and the one-move accuracy check")
    ap.add_argument("--cpu-moves", type=int, default=2)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--profile-case", action="store_true",
                    help="run --steps moves on a synthetic saturated state and exit "
                         "(the small case for ncu kernel captures; prints no bench line)")
    args = ap.parse_args()
    if args.profile_case:
        print(json.dumps(run_profile_case(args)), flush=True)
        return
    if args.warmup < 3:
        ap.error("--warmup must be >= 3")
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        line = run_reference(args, rank)
    else:
        if world > 1:
            import torch
            import torch.distributed as dist
            torch.cuda.set_device(local_rank)
            dist.init_process_group("nccl")
        line = run_gb300(args, rank, world, local_rank)
        if world > 1:
            import torch.distributed as dist
            dist.destroy_process_group()
    if rank == 0 and line is not None:
        print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
