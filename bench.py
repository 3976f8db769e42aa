"""CTMRG moves/s of the GB300 library at D=6, chi=144 (Heisenberg J=1, 2x2 unit
cell, d=2, half-system rSVD projectors, oversampling 16, 2 power iterations).

A step is one directional move (projectors of both rows/columns of the move,
then the boundary renormalization of both).  Moves run as the pairs of one
CTMRG iteration (left with right, up with down: data-independent moves whose
rows all run at once on side streams; the result equals the sequential order
bit for bit), so K is rounded up to an even count.  The environment is first
grown for 50 untimed CTMRG iterations (the iteration count of this
workload), then W untimed moves, then K timed moves, each pair bracketed by
CUDA events on the launching stream with an L2 flush (a 256 MiB write)
between pairs outside the events.

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
GROW_ITERS = 50
N_Q = CHI * D * D
METRIC = "CTMRG moves/s at D=6, chi=144 (Heisenberg, 2x2, half-system rSVD os=16 niter=2)"
WORKLOAD = {"workload": f"heisenberg_2x2_D{D}_chi{CHI}_rsvd_os{OVERSAMPLING}_niter{NITER}",
            "D": D, "chi": CHI, "phys": PHYS, "projectors": "half-system", "svd_type": "rsvd",
            "seed": SEED, "iterations_before_timing": GROW_ITERS}
# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) of one launch of a
# kernel class at this workload, from one ncu capture of `bench.py
# --profile-case --steps 1` (`ncu --set full --clock-control none -k
# regex:tc_gemm_persistent -s 0 -c 2`: the K = chi step 20.3 MB read + 60.0
# MB written, the double-layer step 125.1 MB read + 62.7 MB written);
# classes without a capture report null.
NCU_DRAM_BYTES = {
    "tc_gemm_persistent_kernel (enlarged corner, edge step)": 20.297472e6 + 59.953152e6,
    "tc_gemm_persistent_kernel (enlarged corner, double-layer step)": 125.144064e6 + 62.710784e6,
}


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
    sampled every 20 ms from before the region starts (start() waits for the
    first sample), each sample stamped on arrival; stop() keeps the samples
    that arrived inside the window set by mark_start() / mark_end() (plus one
    sampling interval), or the nearest one when the region is shorter than
    the interval."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    INTERVAL_MS = 20

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


REF_INSTALL = os.path.join(ROOT, "baseline", "_ref")


def reference_modules():
    """The reference itself (installed by pip into baseline/_ref, pure
    Python), or None.  Its ``toml`` import (logging only) is served by a
    stand-in on the standard library's ``tomllib``."""
    if not os.path.isdir(os.path.join(REF_INSTALL, "acetn")):
        return None
    import tomllib
    import types
    if "toml" not in sys.modules:
        mod = types.ModuleType("toml")
        mod.load = lambda f: tomllib.load(open(f, "rb") if isinstance(f, str) else f)
        mod.loads = tomllib.loads
        mod.dumps = lambda d: repr(d) + "\n"
        sys.modules["toml"] = mod
    if REF_INSTALL not in sys.path:
        sys.path.append(REF_INSTALL)
    tn = importlib.import_module("acetn.ipeps.tensor_network")
    cfgm = importlib.import_module("acetn.ipeps.ipeps_config")
    dm = importlib.import_module("acetn.renormalization.directional_mover")
    return tn, cfgm, dm


def reference_network(mods, sites):
    """A reference TensorNetwork on the CPU (float64) holding the given site
    arrays {site: {"A", "C", "E"}} (the reference's site dictionary is
    shared by all its networks; this one replaces its contents)."""
    import numpy as np
    import torch
    tn, cfgm, _ = mods
    net = tn.TensorNetwork(None, cfgm.TNConfig(nx=2, ny=2, dims={"phys": PHYS, "bond": D, "chi": CHI}),
                           torch.float64, torch.device("cpu"))
    for s, v in sites.items():
        st = net[s]
        st["A"] = torch.from_numpy(np.ascontiguousarray(v["A"]))
        st["C"] = [torch.from_numpy(np.ascontiguousarray(c)) for c in v["C"]]
        st["E"] = [torch.from_numpy(np.ascontiguousarray(e)) for e in v["E"]]
    net.rank, net.is_distributed = 0, False
    return net


def reference_moves(mods, net, moves, start=0):
    """Times ``moves`` directional moves of the reference's own CPU path
    (DirectionalMover of acetn/renormalization/directional_mover.py, torch on
    all host threads); returns seconds per move."""
    import torch
    _, cfgm, dm = mods
    torch.set_num_threads(cpu_cores())
    cfg = cfgm.CTMRGConfig(projectors="half-system", svd_type="rsvd",
                           rsvd_oversampling=OVERSAMPLING, rsvd_niter=NITER, svd_cutoff=1e-12)
    mover = dm.DirectionalMover(cfg)
    order = [(0, 0), (2, 1), (0, 1), (2, 0), (1, 1), (3, 0), (1, 0), (3, 1)]
    times = []
    for i in range(moves):
        k, idx = order[(start + i) % len(order)]
        t0 = time.perf_counter()
        (mover.left_move, mover.up_move, mover.right_move, mover.down_move)[k](net, idx)
        times.append(time.perf_counter() - t0)
    return times


def run_reference(args, rank):
    """--impl reference: the reference's own CPU path (its DirectionalMover
    on torch CPU tensors, all host threads) when it is installed in
    baseline/_ref, else the oracle's numpy restatement of it; same
    workload, metric and unit."""
    if rank != 0:
        return None
    from oracle import ctm_oracle as orc
    st = orc.random_state(D, CHI, seed=SEED)
    mods = reference_modules()
    t0 = time.perf_counter()
    if mods is not None:
        net = reference_network(mods, st.sites)
        reference_moves(mods, net, 16)  # two iterations: grow the environment to chi
        grow_s = time.perf_counter() - t0
        reference_moves(mods, net, args.warmup, start=0)
        times = reference_moves(mods, net, args.steps, start=args.warmup)
        kind = "reference"
    else:
        cfg = dict(projectors="half-system", svd_type="rsvd", rsvd_oversampling=OVERSAMPLING,
                   rsvd_niter=NITER, svd_cutoff=1e-12)
        orc.ctmrg(st, cfg, orc.OmegaStream(SEED), steps=2)  # grow the environment to chi
        grow_s = time.perf_counter() - t0
        oracle_moves(st, args.warmup, seed=SEED + 1)
        times = oracle_moves(st, args.steps, seed=SEED + 2)
        kind = "port"
    total = sum(times)
    value = args.steps / total
    q = CHI + OVERSAMPLING
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "moves/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * total / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": dict(WORKLOAD),
        "cpu_baseline": {"value": value, "unit": "moves/s", "cores": cpu_cores(), "kind": kind,
                         "sample": f"{args.steps} moves after 2 growth iterations "
                                   f"({grow_s:.1f} s; chi saturated: the per-move cost of the "
                                   f"{GROW_ITERS}-iteration state) and {args.warmup} warm-up moves",
                         "cpu_model": cpu_model(),
                         "code": ("the reference's DirectionalMover on torch CPU tensors"
                                  if kind == "reference" else "the oracle (numpy restatement)")},
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
    import torch
    import torch.distributed as dist

    gb = package()
    gb.build()
    gb._abi.set_mixed_contraction(args.contraction)
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
    # the environment is grown with the mixed path (seconds; the FP64 path
    # would take minutes), whatever --precision times afterwards
    import dataclasses
    grower = gb.DirectionalMover(dataclasses.replace(cfg, precision="mixed"), omega_source=omega)
    order = gb.sweep_order(2, 2)
    t_grow = time.perf_counter()
    for _ in range(GROW_ITERS):
        for kind, i1, i2 in gb.pair_order(2, 2):
            grower.move_pair(st, kind, i1, i2)
    torch.cuda.synchronize(dev)
    t_grow = time.perf_counter() - t_grow
    mover = gb.DirectionalMover(cfg, omega_source=omega)
    pairs = gb.pair_order(2, 2)
    pos = 0

    def next_pair(mv, state):
        nonlocal pos
        kind, i1, i2 = pairs[pos % len(pairs)]
        mv.move_pair(state, kind, i1, i2)
        pos += 1

    # the tile-plan autotuner, when asked for, tunes the saturated shapes in
    # the warm-up pairs (tuning synchronises) and is off in the timed region
    if args.autotune:
        gb.autotune(True, reset=True)
    for _ in range(max(1, -(-args.warmup // 2))):
        next_pair(mover, st)
    tune_line = None
    if args.autotune:
        gb.autotune(False)
        table = gb.autotune_table()
        tune_line = {"shapes": len(table),
                     "changed": sum(1 for r in table if r["choice"] != 0),
                     "default_ms": round(sum(r["default_ms"] for r in table), 4),
                     "tuned_ms": round(sum(r["best_ms"] for r in table), 4)}
    n_pairs = max(1, -(-args.steps // 2))
    steps = 2 * n_pairs
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    torch.cuda.synchronize(dev)
    if world > 1:
        dist.barrier()
    clocks = ClockSampler(local_rank)
    clocks.start()
    launches0 = gb._abi.kernel_launches()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(n_pairs)]
    torch.cuda.synchronize(dev)
    clocks.mark_start()
    for i in range(n_pairs):
        flush.zero_()
        ev[i][0].record(stream)
        next_pair(mover, st)
        ev[i][1].record(stream)
    torch.cuda.synchronize(dev)
    clocks.mark_end()
    launches = gb._abi.kernel_launches() - launches0
    qr_fallbacks = gb._abi.qr_fallbacks(dev)
    clk = clocks.stop()
    ms = [a.elapsed_time(b) for a, b in ev]
    total_s = sum(ms) / 1e3
    total_max, value = aggregate(total_s, steps, world, dev)

    # per-kernel timing (CUDA events inside the library) on a separate,
    # untimed pass with the rows of each move run one after the other, so
    # that no two kernels of the pass share the GPU
    prof_pairs = 2
    prof_moves = 2 * prof_pairs
    mover.concurrent = False
    pev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
           for _ in range(prof_pairs)]
    gb._abi.profile_begin()
    for i in range(prof_pairs):
        flush.zero_()
        pev[i][0].record(stream)
        next_pair(mover, st)
        pev[i][1].record(stream)
    torch.cuda.synchronize(dev)
    prof = gb._abi.profile_end()
    kernels = gb._abi.profile_kernels()
    prof_move_ms = sum(a.elapsed_time(b) for a, b in pev) / prof_moves
    mover.concurrent = True

    # one CTMRG iteration (8 moves) captured as a CUDA graph and replayed
    graph_line = None
    if not args.no_graph:
        gst = clone_state(gb, st)
        graph = gb.CTMRGGraph(gst, cfg).capture(warmup=1)
        graph.replay(1)
        replays = max(1, -(-steps // len(order)))
        gev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
               for _ in range(replays)]
        torch.cuda.synchronize(dev)
        for i in range(replays):
            flush.zero_()
            gev[i][0].record(stream)
            graph.replay(1)
            gev[i][1].record(stream)
        torch.cuda.synchronize(dev)
        g_s = sum(a.elapsed_time(b) for a, b in gev) / 1e3
        g_total, g_value = aggregate(g_s, replays * len(order), world, dev)
        graph_line = {"value": g_value, "unit": "moves/s",
                      "ms_per_step": 1e3 * g_total / (replays * len(order)),
                      "steps": replays * len(order), "truncated_below_chi": graph.truncated()}
        del graph, gst

    # ---- e2e: host buffers through the public API, copies inside the timed region
    # The state lives in one pinned host buffer (every site's A, C[0..3],
    # E[0..3] back to back).  Every pair copies that buffer to the device in
    # one transfer, runs the two moves on views of the device copy, and reads
    # the tensors it replaced back into their places in the host buffer, which
    # is the next pair's input.  One untimed pair first; wall clock over the
    # timed pairs.
    tensors = [(s, key, n, st[s][key] if key == "A" else st[s][key][n])
               for s in st.site_list for key, count in (("A", 1), ("C", 4), ("E", 4))
               for n in range(count)]
    offsets, total = [], 0
    for _, _, _, t in tensors:
        offsets.append(total)
        total += (t.numel() + 63) // 64 * 64  # every view 512-byte aligned, as allocations are
    host_flat = torch.empty(total, dtype=torch.float64, pin_memory=True)
    for (_, _, _, t), off in zip(tensors, offsets):
        host_flat[off:off + t.numel()].copy_(t.reshape(-1).cpu())
    where = {(s, key, n): (off, t.shape) for (s, key, n, t), off in zip(tensors, offsets)}
    e2e_pairs = 6
    e2e_steps = 2 * e2e_pairs
    h2d = d2h = 0

    def e2e_pair():
        flat = host_flat.to(dev, non_blocking=True)
        dst = gb.IpepsState(2, 2, st.dims, dev)

        def view(s, key, n):
            off, shape = where[(s, key, n)]
            return flat[off:off + shape.numel()].view(shape)

        for s in st.site_list:
            dst[s] = {"A": view(s, "A", 0), "C": [view(s, "C", n) for n in range(4)],
                      "E": [view(s, "E", n) for n in range(4)]}
        before = {s: (list(dst[s]["C"]), list(dst[s]["E"])) for s in st.site_list}
        next_pair(mover, dst)
        # read back the step's result: the tensors the pair replaced (two
        # corners and one edge per renormalised site and move, found by
        # identity) into their places in the host buffer
        moved = 0
        for s in st.site_list:
            for key, old_list in zip(("C", "E"), before[s]):
                for n, t in enumerate(dst[s][key]):
                    if t is not old_list[n]:
                        off, shape = where[(s, key, n)]
                        if tuple(t.shape) != tuple(shape):
                            raise RuntimeError("e2e: a replaced tensor changed its shape")
                        host_flat[off:off + t.numel()].view(shape).copy_(t, non_blocking=True)
                        moved += t.numel() * t.element_size()
        torch.cuda.synchronize(dev)
        return total * 8, moved

    e2e_pair()
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    for i in range(e2e_pairs):
        h2d, d2h = e2e_pair()
    e2e_s = time.perf_counter() - t0
    e2e_value = world * e2e_steps / e2e_s

    compare = None
    if rank == 0 and not args.no_compare:
        compare = compare_paths(gb, st, cfg, dev, args.precision, args.compare_moves)
    sweep = None
    if rank == 0 and not args.no_batched:
        sweep = batched_sweep(gb, dev)
    meas = None
    if rank == 0 and not args.no_measure:
        meas = measure_timing(gb, st, dev)
    als = None
    if rank == 0 and not args.no_als:
        als = als_timing(gb, dev)
    large = None
    if rank == 0 and not args.no_large:
        large = large_instance(gb, dev)

    peaks = {}
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            peaks = json.load(fh)
    except OSError:
        pass
    table = kernel_table(kernels, prof_moves, prof_move_ms, peaks, dev)
    roof = next((k for k in table if k["bound"] in ("tensor", "hbm") and k["achieved"]), None)
    q = CHI + OVERSAMPLING
    line = None
    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "moves/s", "n_gpus": world,
            "steps": steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * total_max / steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64" if args.precision == "fp64" else "bf16/3xbf16+f32+f64",
            "precision": args.precision,
            "contraction": args.contraction,
            "data": "synthetic",
            "config": dict(WORKLOAD),
            "l2": "256 MiB flush between timed moves; quarter tensors 215 MB each",
            "parallelism": f"replicas x{world}",
            "tflops": move_flops(D, CHI, q) / (total_max / steps) / 1e12,
            "roofline": None if roof is None else {
                "bound": roof["bound"], "kernel": roof["name"], "achieved": roof["achieved"],
                "peak": roof["peak"], "unit": roof["achieved_unit"], "frac": roof["frac"],
                "traffic": NCU_DRAM_BYTES.get(roof["name"]),
                "launches_per_step": roof["launches_per_step"],
                "work_per_launch": roof["work_per_launch"], "work_unit": roof["unit"],
                "share_of_step": roof["share"], "peak_source": roof["peak_source"],
                "timing": f"CUDA events around each launch, {prof_moves} moves with the rows "
                          f"run serially (ms_per_step there: {prof_move_ms:.2f})"},
            "dominant_kernel_by_time": None if not table else {
                "kernel": table[0]["name"], "share_of_step": table[0]["share"],
                "bound": table[0]["bound"]},
            "kernels": table[:12],
            "e2e": {"value": e2e_value, "unit": "moves/s", "h2d_bytes_per_step": h2d / 2,
                    "d2h_bytes_per_step": d2h / 2, "steps": e2e_steps,
                    "note": "whole state copied from one pinned host buffer in one transfer "
                            "per pair (two moves), replaced tensors read back into their "
                            "places in it; wall clock over 6 pairs after one untimed pair"},
            "gpu_launches": int(launches),
            "execution": "eager, left/right and up/down pairs of moves",
            "graph": graph_line,
            "autotune": tune_line,
            "qr_fallbacks_in_timed_moves": qr_fallbacks,
            "grow_seconds": t_grow,
            "comparison": compare,
            "batched_sweep": sweep,
            "measure": meas,
            "full_update_als": als,
            "large_instance": large,
            "spans_ms_per_step": {k: v[0] / prof_moves for k, v in prof.items() if v[2]},
            "clocks": clk,
        }
        if world == 1 and not args.no_cpu_baseline:
            arrays = {s: {"A": st[s]["A"].cpu().numpy(), "C": [c.cpu().numpy() for c in st[s]["C"]],
                          "E": [e.cpu().numpy() for e in st[s]["E"]]} for s in st.site_list}
            mods = reference_modules()
            if mods is not None:
                times = reference_moves(mods, reference_network(mods, arrays), args.cpu_moves)
                kind, code = "reference", "the reference's DirectionalMover on torch CPU tensors"
            else:
                from oracle import ctm_oracle as orc
                times = oracle_moves(orc.OracleState(arrays, 2, 2, CHI), args.cpu_moves)
                kind, code = "port", "the oracle (numpy restatement)"
            line["cpu_baseline"] = {"value": len(times) / sum(times), "unit": "moves/s",
                                    "cores": cpu_cores(), "kind": kind, "code": code,
                                    "sample": f"{len(times)} moves from the GPU run's "
                                              f"{GROW_ITERS}-iteration chi={CHI} state",
                                    "cpu_model": cpu_model()}
    return line


def batched_sweep(gb, dev, iterations=3):
    """Parameter sweep of 32 independent transverse-field Ising iPEPS (hx
    uniform in [2.5, 3.5], D from {3, 4, 5}, chi from {48, 64, 80, 100}, one
    seeded generator; float32 storage, FP64 projectors, half-system rSVD with
    the reference's default oversampling 2): moves/s of BatchedCTMRG (every
    instance on its own stream, one iteration of all 32 captured as one CUDA
    graph) against the same 32 instances solved one after another (the plain
    eager path, the reference's move order).  Environments are first grown
    to chi, untimed."""
    import numpy as np
    import torch
    rng = np.random.default_rng(SEED)
    inst = [(float(rng.uniform(2.5, 3.5)), int(rng.choice([3, 4, 5])),
             int(rng.choice([48, 64, 80, 100]))) for _ in range(32)]
    cfg = gb.CTMRGConfig(projectors="half-system", svd_type="rsvd", rsvd_oversampling=2,
                         rsvd_niter=2, svd_cutoff=1e-12, precision="fp64",
                         disable_progressbar=True)

    def f32_state(D, chi, seed):
        st = gb.random_state(D, chi, seed, bias=1e-2, device=dev)
        for s in st.site_list:
            v = st[s]
            st[s] = {"A": v["A"].float(), "C": [t.float() for t in v["C"]],
                     "E": [t.float() for t in v["E"]]}
        return st

    states = [f32_state(D, chi, SEED + i) for i, (_, D, chi) in enumerate(inst)]
    b = gb.BatchedCTMRG(states, cfg)
    t0 = time.perf_counter()
    b.grow()
    grow_s = time.perf_counter() - t0
    seq = [clone_state(gb, st) for st in states]
    a, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize(dev)
    a.record()
    for st in seq:  # one iteration of each instance, one instance after another
        gb.ctmrg(st, cfg, steps=1, pairs=False)
    e.record()
    torch.cuda.synchronize(dev)
    seq_s = a.elapsed_time(e) / 1e3
    del seq
    t0 = time.perf_counter()
    b.capture(warmup=1)
    capture_s = time.perf_counter() - t0
    b.replay(1)
    torch.cuda.synchronize(dev)
    a.record()
    b.replay(iterations)
    e.record()
    torch.cuda.synchronize(dev)
    bat_s = a.elapsed_time(e) / 1e3
    moves = b.moves_per_iteration()
    truncated = b.truncated()
    # the same sweep with the mixed-precision contractions (FP64 spectrum,
    # truncation and scaling), from the grown states
    import dataclasses
    mstates = [clone_state(gb, st) for st in states]
    del b
    bm = gb.BatchedCTMRG(mstates, dataclasses.replace(cfg, precision="mixed"))
    bm.capture(warmup=1)
    bm.replay(1)
    torch.cuda.synchronize(dev)
    a.record()
    bm.replay(iterations)
    e.record()
    torch.cuda.synchronize(dev)
    mix_s = a.elapsed_time(e) / 1e3
    mixed_truncated = bm.truncated()
    del bm, mstates
    return {"instances": len(inst), "D": [x[1] for x in inst], "chi": [x[2] for x in inst],
            "hx_range": [min(x[0] for x in inst), max(x[0] for x in inst)],
            "storage": "float32", "projectors": "fp64 half-system rSVD os=2 niter=2",
            "batched_moves_per_s": moves * iterations / bat_s,
            "sequential_moves_per_s": moves / seq_s,
            "speedup": (moves * iterations / bat_s) / (moves / seq_s),
            "truncated_below_chi": truncated,
            "batched_mixed_moves_per_s": moves * iterations / mix_s,
            "mixed_truncated_below_chi": mixed_truncated,
            "grow_seconds": grow_s, "capture_seconds": capture_s,
            "timing": f"CUDA events; batched: {iterations} graph replays of one iteration of "
                      "all instances; sequential: one eager iteration per instance"}


def large_instance(gb, dev, D8=8, chi8=256, grow=3, pairs=2):
    """The large single instance: Heisenberg, D=8, chi=256 (enlarged corner
    16384 x 16384), half-system rSVD with oversampling 16 and 2 power
    iterations, mixed precision (the site-tensor steps as one-layer
    tensor-core GEMMs, no D^8 double-layer matrix), against one move of the
    FP64 path.  The environment is grown to chi first (untimed); moves run
    as left/right and up/down pairs."""
    import dataclasses
    import torch
    cfg = gb.CTMRGConfig(projectors="half-system", svd_type="rsvd", rsvd_oversampling=16,
                         rsvd_niter=2, svd_cutoff=1e-12, precision="mixed",
                         disable_progressbar=True)
    gen = torch.Generator(device=dev)
    gen.manual_seed(SEED)
    omega = lambda n, q, device: torch.randn(n, q, dtype=torch.float64, device=device,
                                             generator=gen)
    st = gb.random_state(D8, chi8, SEED, d=PHYS, device=dev)
    mover = gb.DirectionalMover(cfg, omega_source=omega)
    order = gb.pair_order(2, 2)
    t0 = time.perf_counter()
    for _ in range(grow):
        for kind, i1, i2 in order:
            mover.move_pair(st, kind, i1, i2)
    torch.cuda.synchronize(dev)
    grow_s = time.perf_counter() - t0
    kind, i1, i2 = order[0]
    mover.move_pair(st, kind, i1, i2)  # warm
    a, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize(dev)
    a.record()
    for i in range(pairs):
        kind, i1, i2 = order[(1 + i) % len(order)]
        mover.move_pair(st, kind, i1, i2)
    e.record()
    torch.cuda.synchronize(dev)
    ms = a.elapsed_time(e) / (2 * pairs)
    gb._abi.profile_begin()
    mover.concurrent = False
    kind, i1, i2 = order[0]
    mover.move_pair(st, kind, i1, i2)
    torch.cuda.synchronize(dev)
    gb._abi.profile_end()
    mover.concurrent = True
    kernels = gb._abi.profile_kernels()
    tc = [k for k in kernels if k["name"].startswith("tc_gemm")]
    tc_ms = sum(k["ms"] for k in tc) / 2
    tc_work = sum(k["work"] for k in tc) / 2
    # one move of the FP64 path on the same state
    s64 = clone_state(gb, st)
    m64 = gb.DirectionalMover(dataclasses.replace(cfg, precision="fp64"), omega_source=omega)
    a.record()
    m64.move(s64, 0, 0)
    e.record()
    torch.cuda.synchronize(dev)
    fp64_ms = a.elapsed_time(e)
    del s64
    q = chi8 + 16
    flops = move_flops(D8, chi8, q)
    return {"workload": f"heisenberg_2x2_D{D8}_chi{chi8}_rsvd_os16_niter2", "precision": "mixed",
            "contraction": "one-layer site-tensor steps", "moves_per_s": 1e3 / ms,
            "ms_per_move": ms, "tflops": flops / (ms / 1e3) / 1e12,
            "tensor_core_ms_per_move_serial": tc_ms,
            "tensor_core_algorithmic_tflops": tc_work / (tc_ms / 1e3) / 1e12 if tc_ms else None,
            "fp64_path_moves_per_s": 1e3 / fp64_ms, "ratio_vs_fp64": fp64_ms / ms,
            "grow_iterations": grow, "grow_seconds": grow_s,
            "timing": f"CUDA events over {pairs} pairs of moves after one warm pair; FP64: one move"}


def measure_timing(gb, st, dev):
    """Wall time of measure() (4 site RDMs, 8 bond RDMs, energy) on the
    benchmark's state: the mixed RDMs (bond RDMs on tensor cores), the FP64
    path, and the reference's own RDM on the host cores for one site and one
    bond (scaled to the 4 + 8 of a measurement), with the energy difference
    of the mixed measurement from the FP64 one."""
    import torch
    model = gb.HeisenbergModel(1.0, device=dev)
    out = {}
    for prec, reps in (("mixed", 3), ("fp64", 1)):
        gb.measure(st, model, verbose=False, precision=prec)  # warm (workspaces)
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        for _ in range(reps):
            e = float(gb.measure(st, model, verbose=False, precision=prec)["Energy"])
        torch.cuda.synchronize(dev)
        out[f"{prec}_ms"] = 1e3 * (time.perf_counter() - t0) / reps
        out[f"{prec}_energy"] = e
    out["mixed_rel_err_vs_fp64"] = (abs(out["mixed_energy"] - out["fp64_energy"])
                                    / abs(out["fp64_energy"]))
    mods = reference_modules()
    arrays = {s: {"A": st[s]["A"].cpu().numpy(), "C": [c.cpu().numpy() for c in st[s]["C"]],
                  "E": [e.cpu().numpy() for e in st[s]["E"]]} for s in st.site_list}
    if mods is not None:
        net = reference_network(mods, arrays)
        rdm_mod = importlib.import_module("acetn.measurement.rdm")
        bond_mod = importlib.import_module("acetn.ipeps.bond")
        torch.set_num_threads(cpu_cores())
        r = rdm_mod.RDM(net)
        t0 = time.perf_counter()
        r[(0, 0)]
        t_site = time.perf_counter() - t0
        t0 = time.perf_counter()
        r[bond_mod.Bond((0, 0), (1, 0), 2)]
        t_bond = time.perf_counter() - t0
        kind = "reference"
    else:
        from oracle import ctm_oracle as orc
        ost = orc.OracleState(arrays, 2, 2, CHI)
        t0 = time.perf_counter()
        orc.site_rdm(ost[(0, 0)])
        t_site = time.perf_counter() - t0
        t0 = time.perf_counter()
        orc.bond_rdm(ost, (0, 0), (1, 0), 2)
        t_bond = time.perf_counter() - t0
        kind = "port"
    out["cpu_ms"] = 1e3 * (4 * t_site + 8 * t_bond)
    out["cpu"] = {"kind": kind, "cores": cpu_cores(),
                  "sample": "one site RDM and one bond RDM, scaled to 4 + 8"}
    return out


def als_timing(gb, dev, nD=12, bD=6, pD=2, reps=3):
    """One ALS solve of the full update (D=6, d=2 bond: reduced tensors
    (12, 6, 2)) with the reference's default config (100 iterations, tol
    1e-15, Cholesky): the GPU solver against the reference's own ALSSolver
    on torch CPU tensors with all host cores (the oracle port without the
    reference install), on the same seeded, positive-definite input."""
    import numpy as np
    import torch
    g = np.random.default_rng(77)
    nz = g.standard_normal((nD, nD, nD * nD))
    n12 = np.einsum("yxz,YXz->yxYX", nz, nz) + 1e-3 * np.einsum(
        "yY,xX->yxYX", np.eye(nD), np.eye(nD))
    a1, a2 = g.random((nD, bD, pD)), g.random((nD, bD, pD))
    gate = (np.eye(pD * pD) + 0.3 * g.random((pD * pD, pD * pD))).reshape(pD, pD, pD, pD)
    a12g = np.einsum("yxpq,pqrs->yxrs", np.einsum("yup,xuq->yxpq", a1, a2), gate)

    class Cfg:
        als_niter, als_tol, als_method, als_epsilon, backend = 100, 1e-15, "cholesky", 1e-12, "torch"

    n12_d = torch.from_numpy(n12).to(dev)
    a12g_d = torch.from_numpy(a12g).to(dev)
    solver = gb.ALSSolver(n12_d, a12g_d, (nD, bD, pD), Cfg())
    solver.solve()  # warm (workspace)
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    for _ in range(reps):
        r1, r2 = solver.solve()
    torch.cuda.synchronize(dev)
    gpu_ms = 1e3 * (time.perf_counter() - t0) / reps
    cost = float(gb.ALSSolver.calculate_cost(r1, r2, a12g_d, n12_d))
    out = {"shape": [nD, bD, pD], "method": "cholesky", "gpu_ms": gpu_ms,
           "gpu_iterations": solver.iterations, "gpu_cost": cost}
    mods = reference_modules()
    if mods is not None:
        als_mod = importlib.import_module("acetn.evolution.als_solver")
        torch.set_num_threads(cpu_cores())
        ref = als_mod.ALSSolver(torch.from_numpy(n12), torch.from_numpy(a12g), (nD, bD, pD), Cfg())
        t0 = time.perf_counter()
        q1, q2 = ref.solve()
        cpu_ms = 1e3 * (time.perf_counter() - t0)
        ref_cost = float(als_mod.ALSSolver.calculate_cost(q1, q2, torch.from_numpy(a12g),
                                                          torch.from_numpy(n12)))
        kind = "reference"
    else:
        from oracle import ctm_oracle as orc
        t0 = time.perf_counter()
        q1, q2, _ = orc.als_solve(n12, a12g, (nD, bD, pD))
        cpu_ms = 1e3 * (time.perf_counter() - t0)
        ref_cost = orc.als_cost(q1, q2, a12g, n12)
        kind = "port"
    out.update({"cpu_ms": cpu_ms, "cpu_cost": ref_cost,
                "cost_rel_diff": abs(cost - ref_cost) / abs(ref_cost),
                "cpu": {"kind": kind, "cores": cpu_cores()}})
    return out


def sm_fp32_peak_tflops(dev):
    """FP32 FMA peak of the SIMT units: SMs x 128 lanes x 2 FLOP x max clock."""
    import torch
    p = torch.cuda.get_device_properties(dev)
    mhz = 2070.0
    try:
        out = subprocess.run(["nvidia-smi", "--query-gpu=clocks.max.sm", "--format=csv,noheader,nounits",
                              "-i", str(dev.index or 0)], capture_output=True, text=True, timeout=10)
        mhz = float(out.stdout.strip().splitlines()[0])
    except (OSError, ValueError, IndexError, subprocess.TimeoutExpired):
        pass
    return p.multi_processor_count * 128 * 2 * mhz * 1e6 / 1e12


def kernel_table(kernels, moves, move_ms, peaks, dev):
    """Kernel classes of the profiled moves sorted by time: share of the
    (serial-rows) move, launches and algorithmic work per launch, achieved
    rate and the fraction of the roof that bounds the class: tensor cores
    (BF16 peak; the work is the algorithmic FLOP count of the contraction the
    launch performs, not the split-precision passes), HBM (algorithmic bytes),
    FP64 or FP32 SIMT FMA; iterative kernels (Jacobi sweeps) have no work
    figure and report time only."""
    bf16 = peaks.get("bf16_tflops") or 1900.0
    hbm = peaks.get("hbm_gbs") or 6800.0
    src = "MEASURED_PEAKS.json" if peaks else "fallback"
    out = []
    for k in kernels:
        name = k["name"]
        if name.startswith("tc_gemm") and k["unit"] == "flop":
            bound, peak, unit, psrc = "tensor", bf16, "TFLOP/s", f"{src} bf16_tflops (burst)"
        elif k["unit"] == "byte":
            bound, peak, unit, psrc = "hbm", hbm, "GB/s", f"{src} hbm_gbs"
        elif "double" in name:
            bound, peak, unit, psrc = "fp64", fp64_peak_tflops(dev), "TFLOP/s", "cuBLAS DGEMM on this GPU"
        else:
            bound, peak, unit, psrc = "fp32", sm_fp32_peak_tflops(dev), "TFLOP/s", "SMs x 128 x 2 x max clock"
        sec = k["ms"] / 1e3
        achieved = None
        if k["work"] > 0 and sec > 0:
            achieved = k["work"] / sec / (1e9 if unit == "GB/s" else 1e12)
        out.append({"name": name, "share": (k["ms"] / moves) / move_ms if move_ms else None,
                    "ms_per_step": k["ms"] / moves, "launches_per_step": k["launches"] / moves,
                    "work_per_launch": k["work"] / k["launches"] if k["launches"] else None,
                    "unit": k["unit"], "bound": bound, "achieved": achieved,
                    "achieved_unit": unit, "peak": peak,
                    "frac": achieved / peak if achieved else None, "peak_source": psrc})
    out.sort(key=lambda x: -x["ms_per_step"])
    return out


def clone_state(gb, st):
    c = gb.IpepsState(st.nx, st.ny, st.dims, st.device)
    for s in st.site_list:
        v = st[s]
        c[s] = {"A": v["A"].clone(), "C": [t.clone() for t in v["C"]],
                "E": [t.clone() for t in v["E"]]}
    return c


def bond_energies(gb, st, model):
    """Per-bond energies <h_b> from trace-normalised bond RDMs (FP64)."""
    import torch
    rdm = gb.RDM(st)
    out = []
    for b in st.bond_list:
        r = rdm[b]
        h2 = model.two_site_hamiltonian(b).reshape(2, 2, 2, 2)
        out.append(float(torch.einsum("PQpq,pqPQ->", r, h2) / torch.einsum("pqpq->", r)))
    return out


def compare_paths(gb, st, cfg, dev, precision, nmoves):
    """From the benchmark's grown state: moves/s of this library's plain FP64
    path (the drop-in), and, for one move of each direction, the energy per
    site and per bond after the move in each precision with the same rSVD
    test matrices, next to the FP64 path's own spread between two draws of
    the test matrices (the rSVD's noise).  Energies use FP64 bond RDMs."""
    import dataclasses
    import statistics as stats
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
    model = gb.HeisenbergModel(1.0, device=dev)
    rows = []
    # one move of each direction (left, right, up, down) from the same state
    for k, idx in [order[i] for i in (0, 1, 2, 3)][:nmoves]:
        e = {}
        runs = [("fp64", cfg64, 7 + k), ("fp64_other_draw", cfg64, 107 + k),
                (precision, cfg, 7 + k)]
        if precision == "mixed":
            # the same mixed move with the reference's cutoff alone (no
            # mixed_svd_floor): the truncation rule of the FP64 path
            runs.append(("mixed_ref_cutoff",
                         dataclasses.replace(cfg, mixed_svd_floor=cfg.svd_cutoff), 7 + k))
        for tag, c, seed in runs:
            s1 = clone_state(gb, st)
            gb.DirectionalMover(c, omega_source=seeded(seed)).move(s1, k, idx)
            e[tag] = bond_energies(gb, s1, model)
            del s1
        ref = e["fp64"]
        e_ref = sum(ref) / 4
        scale = max(abs(x) for x in ref)

        def rel(v):
            return abs(sum(v) / 4 - e_ref) / abs(e_ref)

        def per_bond(v):
            return max(abs(x - y) for x, y in zip(v, ref)) / scale

        row = {"move": [k, idx], "energy_fp64": e_ref,
               "rel_err": rel(e[precision]), "bond_err": per_bond(e[precision]),
               "fp64_draw_rel": rel(e["fp64_other_draw"]),
               "fp64_draw_bond": per_bond(e["fp64_other_draw"])}
        if "mixed_ref_cutoff" in e:
            row["rel_err_ref_cutoff"] = rel(e["mixed_ref_cutoff"])
        rows.append(row)
    errs = [r["rel_err"] for r in rows]
    draws = [r["fp64_draw_rel"] for r in rows]
    return {"fp64_path": {"moves_per_s": 1e3 / fp64_ms, "ms_per_step": fp64_ms},
            "state": f"after {GROW_ITERS} iterations",
            "rel_err_vs_fp64": stats.median(errs), "rel_err_vs_fp64_max": max(errs),
            "fp64_rsvd_draw_spread": stats.median(draws),
            "fp64_rsvd_draw_spread_max": max(draws),
            "rel_err_vs_fp64_ref_cutoff": (
                stats.median(r["rel_err_ref_cutoff"] for r in rows)
                if rows and "rel_err_ref_cutoff" in rows[0] else None),
            "rel_err_vs_fp64_ref_cutoff_max": (
                max(r["rel_err_ref_cutoff"] for r in rows)
                if rows and "rel_err_ref_cutoff" in rows[0] else None),
            "cutoffs": {"mixed_svd_floor": cfg.mixed_svd_floor, "svd_cutoff": cfg.svd_cutoff},
            "moves": rows}


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
    gb._abi.set_mixed_contraction(args.contraction)
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
    if args.profile_measure:
        # one mixed measurement (site RDMs in FP32, bond RDMs on tensor cores)
        gb.measure(st, gb.HeisenbergModel(1.0, device=dev), verbose=False, precision="mixed")
    torch.cuda.synchronize(dev)
    return {"profile_case": "left move on a synthetic chi-saturated state", "moves": args.steps,
            "measure": bool(args.profile_measure), "device_status": gb._abi.device_status()}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=40)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--precision", choices=["fp64", "mixed"], default="mixed")
    ap.add_argument("--no-graph", action="store_true",
                    help="skip the replays of one CUDA-graph-captured CTMRG iteration")
    ap.add_argument("--no-compare", action="store_true",
                    help="skip the FP64-path timing and the one-move accuracy check")
    ap.add_argument("--contraction", choices=["auto", "double-layer", "one-layer"],
                    default="auto", help="form of the mixed path's site-tensor steps")
    ap.add_argument("--profile-measure", action="store_true",
                    help="with --profile-case: one mixed-precision measure() after the moves")
    ap.add_argument("--autotune", action="store_true",
                    help="tune the tensor-core GEMM tile plans in the warm-up pairs")
    ap.add_argument("--no-large", action="store_true",
                    help="skip the D=8, chi=256 instance")
    ap.add_argument("--no-als", action="store_true",
                    help="skip the timing of one full-update ALS solve")
    ap.add_argument("--no-measure", action="store_true",
                    help="skip the measure() timing")
    ap.add_argument("--no-batched", action="store_true",
                    help="skip the 32-instance parameter sweep")
    ap.add_argument("--compare-moves", type=int, default=4,
                    help="moves (one per direction) of the accuracy check")
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
