"""Benchmark of the short-range nonbonded path on one GB300.

Workload (one "step" = one force + energy + virial evaluation):
  288,000-atom SPC water box (96,000 molecules, 14.21 nm), rc 0.9 nm,
  rlist 1.0 nm, Ewald beta from rtol 1e-5, potential-shift LJ; a fresh
  grid + pair list every 100 steps, rolling dynamic pruning every 10 steps
  (rlist_inner 0.95 nm, 5 parts pruned on alternate steps); coordinates
  perturbed by N(0, 0.002 nm) per coordinate and step; forces FP32,
  energies and virial reduced in FP64.

Metric: useful pair interactions per second, useful pairs per evaluation =
N/2 * (rho * 4/3 pi rc^3 + 1) like gmx nonbonded-benchmark
(src/gromacs/nbnxm/benchmark/bench_setup.cpp:272-276).

  python bench.py [--steps K] [--warmup W] [--gpus N] [--impl ours|reference]
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import tempfile
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "useful pair-interactions/s (288k-atom SPC water, F+E+virial, rc 0.9, rlist 1.0)"
RC, RLIST, RLIST_INNER = 0.9, 1.0, 0.95
NSTLIST, NSTPRUNE = 100, 10
SIGMA_STEP = 0.002
# Ewald-analytic + LJ flops per pair with energies (src/gromacs/gmxlib/nrnb.cpp:106)
FLOPS_PER_PAIR_VF = 107
# dram__bytes_read.sum + dram__bytes_write.sum of one k_force launch on this workload, from an
# ncu --set full capture (list, coordinates and the exclusion items' lists; forces stay in L2)
FORCE_KERNEL_DRAM_BYTES = 27.38e6


def useful_pairs(n: int, box) -> float:
    rho = n / float(np.prod(box))
    return n * 0.5 * (rho * 4.0 / 3.0 * math.pi * RC**3 + 1.0)


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def replica_throughput(total_ms: float, units_per_step: float, steps: int, world: int, device=None):
    """Whole-job throughput of `world` independent replicas (one per GPU, no data-path collective):
    the slowest rank's timed region (max over ranks) and world x units x steps / that time.  The
    only collective is this max over the default process group (NCCL on GPUs, gloo in the CPU test)."""
    if world > 1:
        import torch
        import torch.distributed as dist

        t = torch.tensor([total_ms], dtype=torch.float64, device=device)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_ms = float(t.item())
    return total_ms, world * units_per_step * steps / (total_ms * 1e-3)


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 50 ms during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = os.path.join(tempfile.gettempdir(), f"nbx_clocks_{os.getpid()}.csv")

    def __enter__(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "50"], stdout=self.fh, stderr=subprocess.DEVNULL)
            # the timed region starts once the sampler has produced its first line (start-up ~0.1 s)
            t0 = time.perf_counter()
            while time.perf_counter() - t0 < 3.0 and self.proc.poll() is None:
                self.fh.flush()
                if os.path.getsize(self.path) > 0:
                    break
                time.sleep(0.01)
            self.skip = sum(1 for _ in open(self.path))
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.fh.close()

    def summary(self) -> dict:
        if self.proc is None or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        lines = open(self.path).readlines()
        # the lines written before the timed region began are dropped, unless nothing came after
        timed = lines[getattr(self, "skip", 0):] or lines[-1:]
        for line in timed:
            p = [t.strip() for t in line.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                smax.append(float(p[2]))
            except ValueError:
                continue
            for nm, val in zip(names, p[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


def host_threads() -> int:
    return len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else (os.cpu_count() or 1)


def cpu_port_setup():
    """The 288k-atom box in the reference's CPU layout: 4-atom-cluster grid and the simple 4x4
    list (makeClusterListSimple) at rlist, built once (oracle/nbnxm_cpu_oracle.c)."""
    from gmxapi_gb300 import systems
    from oracle import oracle as O

    s = systems.water_large()
    c = O.CpuOracle(s, rc=RC, rlist=RLIST)
    c.grid()
    c.search()
    return s, c


def cpu_baseline_port(budget_s: float = 12.0) -> dict:
    """The CPU port of the reference's SIMD cluster-pair kernel (4-wide vectors, the 4x4 CPU list)
    on the 288k-atom box: F+E evaluations on all host threads and on one, within a time budget."""
    s, c = cpu_port_setup()
    up = useful_pairs(s.n, s.box)
    out = {}
    for threads in (host_threads(), 1):
        c.force(True, threads=threads)  # warm-up
        reps, t0 = 0, time.perf_counter()
        while True:
            c.force(True, threads=threads)
            reps += 1
            if time.perf_counter() - t0 > budget_s / 2 or reps >= 20:
                break
        out[threads] = (up * reps / (time.perf_counter() - t0), reps)
    th = host_threads()
    return {"value": out[th][0], "unit": "pairs/s", "cores": th, "kind": "port",
            "single_thread_value": out[1][0],
            "sample": f"{out[th][1]} (all {th} threads) and {out[1][1]} (1 thread) F+E evaluations of the "
                      "288k-atom SPC box on the reference's CPU list (4-atom clusters, makeClusterListSimple, "
                      "rlist 1.0, built once) by the 4-wide port of its SIMD 4xM kernel "
                      "(oracle/nbnxm_cpu_oracle.c: GCC vector extensions, NEON on the Arm host)"}


def run_reference(args) -> None:
    """--impl reference: the CPU port of the reference's SIMD cluster-pair kernel on this workload,
    on all host threads; each step one F+E evaluation of the whole 288k-atom box."""
    world, rank, _ = dist_env()
    if rank != 0:
        return
    s, c = cpu_port_setup()
    threads = host_threads()
    up = useful_pairs(s.n, s.box)
    elapsed = 0.0
    for it in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        c.force(True, threads=threads)
        dt = time.perf_counter() - t0
        if it >= args.warmup:
            elapsed += dt
    value = up * args.steps / elapsed
    sz = c.sizes()
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "pairs/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": elapsed / args.steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic", "config": workload_config(),
        "cpu_baseline": {"value": value, "unit": "pairs/s", "cores": threads, "kind": "port",
                         "sample": f"each step: one F+E evaluation of the 288k-atom box ({sz['entries']} "
                                   f"i-entries, {sz['j_entries']} j-clusters of the reference's 4x4 CPU list at "
                                   f"rlist 1.0, built once and not timed) by the 4-wide port of the "
                                   f"reference's SIMD 4xM kernel (NEON on the Arm host), {threads} threads "
                                   "with private force buffers summed after each step"},
        "e2e": {"value": value, "unit": "pairs/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def measure_ensemble(dev: int, steps: int = 30, warmup: int = 3) -> dict:
    """256 uneven SPC water boxes (500..20,000 atoms, log-uniform): the batched step
    (autotuned tile, stage depth, launch shape and prune interval, CUDA graph) against the same step as
    256 sequential single-system steps.  Each step is F + E + virial for every system."""
    import torch

    from gmxapi_gb300 import nblib, systems
    from gmxapi_gb300.batch import BatchForceCalculator

    ens = systems.uneven_ensemble(256, seed=3)
    opts = nblib.NBKernelOptions(coulomb_type=nblib.CoulombType.Pme, pairlist_cutoff=RLIST, rcoulomb=RC,
                                 rlist_inner=RLIST_INNER, nstlist=NSTLIST, nstlist_prune=NSTPRUNE,
                                 compute_virial_and_energy=True)
    b = BatchForceCalculator(ens, opts, device=dev)
    stream = torch.cuda.current_stream(dev)
    b.set_stream(stream.cuda_stream)
    n = b.total_atoms
    total = warmup + steps
    gen = torch.Generator(device=f"cuda:{dev}").manual_seed(99)
    frames = torch.empty((total, 3 * n), dtype=torch.float32, device=f"cuda:{dev}")
    frames[0] = torch.from_numpy(np.concatenate([s.x.reshape(-1) for s in ens])).to(frames.device)
    for t in range(1, total):
        frames[t] = frames[t - 1] + SIGMA_STEP * torch.randn(3 * n, generator=gen, device=frames.device)
    space = {"tiles": ((0, 2), (1, 2), (1, 3)), "variants": (0, 1, 2, 3), "prune_intervals": (4, 10, 20)}
    best, tune = b.autotune(frames[: min(total, 12)], **space)
    f = torch.empty(3 * n, dtype=torch.float32, device=frames.device)
    e = torch.empty(2 * len(ens), dtype=torch.float64, device=frames.device)
    v = torch.empty(9 * len(ens), dtype=torch.float64, device=frames.device)

    def timed(fn):
        for t in range(warmup):
            fn(t, frames[t].data_ptr(), f.data_ptr(), e.data_ptr(), v.data_ptr())
        torch.cuda.synchronize()
        a, z = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for k in range(steps):
            fn(warmup + k, frames[warmup + k].data_ptr(), f.data_ptr(), e.data_ptr(), v.data_ptr())
        z.record(stream)
        torch.cuda.synchronize()
        return a.elapsed_time(z) / steps

    seq_ms = timed(b.sequential_md_step_device)
    bat_ms = timed(b.md_step_device)
    # the list search of the whole ensemble (the systems' searches spread over streams, two host
    # reads of the list sizes), wall clock; the timed steps above hold none, so whole search steps
    # of both paths are timed too (wall clock, best of two) and amortized over nstlist steps
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for k in range(3):
        b.search_device(frames[k].data_ptr())
    torch.cuda.synchronize()
    search_ms = (time.perf_counter() - t0) * 1e3 / 3

    def search_step_ms(fn):
        best = None
        for k in range(2):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            fn(NSTLIST * (k + 1), frames[k].data_ptr(), f.data_ptr(), e.data_ptr(), v.data_ptr())
            torch.cuda.synchronize()
            ms = (time.perf_counter() - t0) * 1e3
            best = ms if best is None else min(best, ms)
        return best

    seq_search_step = search_step_ms(b.sequential_md_step_device)
    bat_search_step = search_step_ms(b.md_step_device)
    b.close()
    bat_amortized = bat_ms + (bat_search_step - bat_ms) / NSTLIST
    seq_amortized = seq_ms + (seq_search_step - seq_ms) / NSTLIST
    return {"workload": "256 SPC water boxes, 500..20000 atoms log-uniform (seed 3)", "atoms": n,
            "steps": steps, "batched_ms_per_step": bat_ms, "sequential_ms_per_step": seq_ms,
            "speedup": seq_ms / bat_ms,
            "search_ms": search_ms, "search_atoms_per_s": n / (search_ms * 1e-3),
            "search_step_ms": {"batched": bat_search_step, "sequential": seq_search_step},
            "batched_ms_per_step_with_search": bat_amortized,
            "sequential_ms_per_step_with_search": seq_amortized,
            "speedup_with_search": seq_amortized / bat_amortized,
            "force_evals_per_s_batched": len(ens) / (bat_ms * 1e-3),
            "force_evals_per_s_sequential": len(ens) / (seq_ms * 1e-3),
            "autotuned": best,
            "search_space": {"tile_stage_depth": space["tiles"], "launch_shape": "0: 256x2, 1: 128x4, 2: 512x1, "
                             "3: 64x8 threads x blocks per SM", "prune_intervals": space["prune_intervals"],
                             "tile": "0: one atom pair per lane (8x4 atoms per warp instruction), 1: two pairs per "
                                     "lane (8x8, packed FP32x2)", "candidates": len(tune),
                             "best_ms_per_step": min(tune.values()), "worst_ms_per_step": max(tune.values())},
            "note": "each step: F+E+virial of all systems; search every 100 steps (none inside the timed steps; "
                    "the _with_search figures add one search step per 100 steps of each path), rolling "
                    "prune as autotuned"}


def measure_adjoint(dev: int, steps: int = 20, warmup: int = 3) -> dict:
    """Force-matching gradient on the 24,000-atom random LJ + Coulomb liquid (8 types,
    Lorentz-Berthelot): loss sum |F - F_target|^2 with F_target at parameters perturbed
    by up to 5 %; one step = forward (F + E) + backward kernel (dL/dx, dL/dq, dL/dsigma,
    dL/depsilon).  Reported: the forward alone, the full gradient step, and the
    backward entry point alone, all on the current list (no search inside)."""
    import torch

    from gmxapi_gb300 import nblib, systems
    from gmxapi_gb300.adjoint import (DifferentiableNonbonded, force_matching_loss, lorentz_berthelot_nbfp,
                                      static_list_options)

    s = systems.lj_liquid(n=24000, ntypes=8, seed=4)
    eng = DifferentiableNonbonded(s, static_list_options(RC), device=dev)  # fixed coordinates: list at rc
    d = torch.device("cuda", dev)
    stream = torch.cuda.current_stream(dev)
    rng = np.random.default_rng(12)
    x = torch.tensor(s.x, device=d, requires_grad=True)
    q = torch.tensor(s.q, device=d, requires_grad=True)
    sig = torch.tensor(s.sigma, dtype=torch.float64, device=d, requires_grad=True)
    eps = torch.tensor(s.epsilon, dtype=torch.float64, device=d, requires_grad=True)
    with torch.no_grad():
        qt = q * torch.tensor(rng.uniform(0.95, 1.05, s.n), dtype=torch.float32, device=d)
        nbt = lorentz_berthelot_nbfp(sig * torch.tensor(rng.uniform(0.95, 1.05, s.ntypes), device=d),
                                     eps * torch.tensor(rng.uniform(0.95, 1.05, s.ntypes), device=d))
        f_target, _ = eng(x, qt, nbt)

    def forward():
        with torch.no_grad():
            eng(x, q, lorentz_berthelot_nbfp(sig, eps), search=False)

    def grad_step():
        for t in (x, q, sig, eps):
            t.grad = None
        f, _e = eng(x, q, lorentz_berthelot_nbfp(sig, eps), search=False)
        force_matching_loss(f, f_target).backward()

    def grad_step_torch_loss():
        # the same step with the loss written as a torch expression (three element-wise kernels
        # each way instead of the fused loss kernel)
        for t in (x, q, sig, eps):
            t.grad = None
        f, _e = eng(x, q, lorentz_berthelot_nbfp(sig, eps), search=False)
        ((f - f_target) ** 2).sum().backward()

    gf = torch.randn(s.n, 3, device=d)
    ge = torch.tensor([0.5, 0.5], dtype=torch.float64, device=d)
    gx = torch.empty(s.n, 3, device=d)
    gq = torch.empty(s.n, device=d)
    gp = torch.empty(s.ntypes, s.ntypes, 2, dtype=torch.float64, device=d)

    fe = torch.empty(2, dtype=torch.float64, device=d)
    fo = torch.empty(s.n, 3, device=d)

    def forward_only():
        eng.calc.compute_device(x.data_ptr(), fo.data_ptr(), fe.data_ptr(), None)

    def backward_only():
        eng.calc.backward_device(x.data_ptr(), gf.data_ptr(), ge.data_ptr(), gx.data_ptr(), gq.data_ptr(),
                                 gp.data_ptr())

    def timed(fn):
        for _ in range(warmup):
            fn()
        torch.cuda.synchronize()
        a, z = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for _ in range(steps):
            fn()
        z.record(stream)
        torch.cuda.synchronize()
        return a.elapsed_time(z) / steps

    def graph_timed(fn):
        """Device time of `steps` calls captured in one CUDA graph (no host launch gaps: the
        24,000-atom entries are short enough for Python and launch overhead to dominate)."""
        for _ in range(warmup):
            fn()
        torch.cuda.synchronize()
        side = torch.cuda.Stream(d)
        eng.calc.set_stream(side.cuda_stream)
        try:
            g = torch.cuda.CUDAGraph()
            with torch.cuda.graph(g, stream=side):
                for _ in range(steps):
                    fn()
            for _ in range(2):
                g.replay()
            torch.cuda.synchronize()
            a, z = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            g.replay()
            z.record(stream)
            torch.cuda.synchronize()
            return a.elapsed_time(z) / steps
        finally:
            eng.calc.set_stream(stream.cuda_stream)

    def graph_replay_ms(fn, params):
        """Device time of one call of `fn` -- the user-level autograd code, every torch op and
        engine launch included -- captured once in a CUDA graph and replayed (PyTorch's
        whole-step capture: warm-up on a side stream, gradients set to None before the capture
        so that backward allocates them from the graph's pool)."""
        side = torch.cuda.Stream(d)
        side.wait_stream(stream)
        with torch.cuda.stream(side):
            for _ in range(warmup):
                fn()
        stream.wait_stream(side)
        torch.cuda.synchronize()
        for t in params:
            t.grad = None
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            fn()
        for _ in range(warmup):
            g.replay()
        torch.cuda.synchronize()
        a, z = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for _ in range(steps):
            g.replay()
        z.record(stream)
        torch.cuda.synchronize()
        eng.calc.set_stream(stream.cuda_stream)
        return a.elapsed_time(z) / steps

    fwd_ms = timed(forward)
    step_ms = timed(grad_step)
    fwd_call_ms = timed(forward_only)
    bwd_call_ms = timed(backward_only)
    try:
        fwd_entry_ms, bwd_ms, entry_timing = graph_timed(forward_only), graph_timed(backward_only), "graph"
    except Exception as exc:  # capture unavailable: the per-call times stand
        fwd_entry_ms, bwd_ms, entry_timing = fwd_call_ms, bwd_call_ms, f"per call ({type(exc).__name__}: {exc})"
    try:
        fwd_graph_ms = graph_replay_ms(forward, ())
        step_graph_ms = graph_replay_ms(grad_step, (x, q, sig, eps))
        step_torch_graph_ms = graph_replay_ms(grad_step_torch_loss, (x, q, sig, eps))
        graph_note = "replayed from a CUDA graph"
    except Exception as exc:  # capture unavailable: report the eager ratio only
        fwd_graph_ms = step_graph_ms = step_torch_graph_ms = None
        graph_note = f"eager (capture failed: {type(exc).__name__}: {exc})"
    eng.close()
    return {"workload": "random LJ+Coulomb liquid, 24000 atoms, 8 types, Lorentz-Berthelot, "
                        "rejection at 0.5 sigma (seed 4)", "atoms": s.n, "steps": steps,
            "forward_graph_ms": fwd_graph_ms, "gradient_step_graph_ms": step_graph_ms,
            "gradient_step_vs_forward": (step_graph_ms / fwd_graph_ms) if step_graph_ms else step_ms / fwd_ms,
            "gradient_step_vs_forward_timing": graph_note,
            "gradient_step_torch_loss_graph_ms": step_torch_graph_ms,
            "gradient_step_torch_loss_vs_forward": (step_torch_graph_ms / fwd_graph_ms) if step_torch_graph_ms else None,
            "gradient_steps_per_s": 1e3 / (step_graph_ms or step_ms),
            "forward_eager_ms": fwd_ms, "gradient_step_eager_ms": step_ms,
            "gradient_step_vs_forward_eager": step_ms / fwd_ms,
            "forward_entry_ms": fwd_entry_ms,
            "backward_entry_ms": bwd_ms, "adjoint_cost_vs_forward": bwd_ms / fwd_entry_ms,
            "entry_timing": entry_timing, "forward_entry_call_ms": fwd_call_ms,
            "backward_entry_call_ms": bwd_call_ms,
            "note": "forward = the autograd forward (Lorentz-Berthelot table, parameter upload, F+E); "
                    "gradient step = autograd forward + loss (gmxapi_gb300.adjoint.force_matching_loss: one "
                    "kernel each way; the torch_loss figures write it as ((f - f_t) ** 2).sum()) + backward "
                    "(adjoint kernel and the table's chain rule); the graph figures replay the same Python step captured once in a CUDA "
                    "graph, the eager ones call it from Python every step (host-bound at 24,000 atoms); "
                    "forward entry = C-ABI F+E (convert, force, reduce, energies); backward entry = C-ABI "
                    "adjoint (convert, gradient prepare, adjoint kernel, finish, FP64 table gradients); "
                    "inputs fit in L2"}


def min_pair_distances(ens) -> dict:
    """The closest pair of each liquid of the ensemble (periodic), over all systems: the smallest
    distance in nm and the smallest distance in units of the pair's sigma_ij (Lorentz-Berthelot)."""
    from scipy.spatial import cKDTree

    best_r, best_ratio = np.inf, np.inf
    for s in ens:
        box = float(s.box[0])
        x = np.mod(np.asarray(s.x, np.float64), box)
        pairs = cKDTree(x, boxsize=box).query_pairs(0.5 * float(np.max(s.sigma)), output_type="ndarray")
        if len(pairs) == 0:
            continue
        d = x[pairs[:, 0]] - x[pairs[:, 1]]
        d -= box * np.round(d / box)
        r = np.sqrt((d ** 2).sum(1))
        sij = 0.5 * (s.sigma[s.type[pairs[:, 0]]] + s.sigma[s.type[pairs[:, 1]]])
        best_r = min(best_r, float(r.min()))
        best_ratio = min(best_ratio, float((r / sij).min()))
    return {"min_nm": best_r, "min_over_sigma_ij": best_ratio,
            "construction": "pairs closer than 0.5 sigma_ij rejected and redrawn (0.8 sigma_ij at 100 atoms/nm^3 "
                            "packs beyond random close packing)"}


def measure_force_matching(dev: int, iters: int = 50, warmup: int = 3) -> dict:
    """Batched differentiable force matching: 64 random LJ + Coulomb liquids (8 types,
    2,000-50,000 atoms log-uniform, shared sigma / epsilon / per-type charge scales).
    Targets are the engine's forces at parameters perturbed by up to 5 %; each Adam step
    (lr 1e-3) is one CUDA-graph launch (parameters -> forces, energies, virials -> loss
    -> adjoint) plus the parameter update.  Baseline: the same gradient by central
    differences of plain per-system forward evaluations (2 x 24 parameters x 64 systems)."""
    import torch

    from gmxapi_gb300 import nblib, systems
    from gmxapi_gb300.adjoint import BatchForceMatcher, TypeScaledCharges, lorentz_berthelot_nbfp, static_list_options
    from gmxapi_gb300.batch import BatchForceCalculator

    procs = max(1, min(16, (len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else 4)))
    t_build = time.perf_counter()
    ens = systems.force_matching_ensemble(64, processes=procs)
    t_build = time.perf_counter() - t_build
    d = torch.device("cuda", dev)
    stream = torch.cuda.current_stream(dev)
    ntypes = 8
    sig0 = torch.tensor(ens[0].sigma, dtype=torch.float64, device=d)
    eps0 = torch.tensor(ens[0].epsilon, dtype=torch.float64, device=d)
    q0 = torch.cat([torch.as_tensor(s.q, dtype=torch.float64) for s in ens]).to(d)
    types = torch.cat([torch.as_tensor(s.type, dtype=torch.long) for s in ens]).to(d)
    n = int(q0.numel())
    rng = np.random.default_rng(21)
    opts = static_list_options(RC)  # fixed frames: the list holds exactly the pairs within rc
    opts.compute_virial_and_energy = True
    # targets at perturbed parameters
    ref = BatchForceCalculator(ens, opts, device=dev)
    ref.set_stream(stream.cuda_stream)
    x = torch.cat([torch.as_tensor(s.x, dtype=torch.float32).reshape(-1) for s in ens]).to(d)
    ref.search_device(x.data_ptr())
    pert = [torch.tensor(rng.uniform(0.95, 1.05, ntypes), device=d) for _ in range(3)]
    q_t = (q0 * pert[2][types]).float().contiguous()
    nb_t = lorentz_berthelot_nbfp(sig0 * pert[0], eps0 * pert[1]).float().contiguous()
    ref.set_parameters_device(q_t.data_ptr(), nb_t.data_ptr())
    f_target = torch.empty_like(x)
    ref.compute_device(x.data_ptr(), f_target.data_ptr())
    torch.cuda.synchronize()

    m = BatchForceMatcher(ens, f_target, opts, device=dev)
    sig = sig0.clone().requires_grad_(True)
    eps = eps0.clone().requires_grad_(True)
    qs = torch.ones(ntypes, dtype=torch.float64, device=d, requires_grad=True)
    opt = torch.optim.Adam([sig, eps, qs], lr=1e-3)

    charges = TypeScaledCharges(q0, types, ntypes)

    def loss_at(s_, e_, k_):
        return m(charges(k_), lorentz_berthelot_nbfp(s_, e_))

    def step():
        opt.zero_grad(set_to_none=True)
        loss = loss_at(sig, eps, qs)
        loss.backward()
        opt.step()
        return loss

    for _ in range(warmup):
        step()
    torch.cuda.synchronize()
    losses = []
    a, z = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record(stream)
    for _ in range(iters):
        losses.append(step())
    z.record(stream)
    torch.cuda.synchronize()
    step_ms = a.elapsed_time(z) / iters
    # the graph launch alone (parameters -> forces -> loss -> adjoint), fixed inputs
    with torch.no_grad():
        qg = charges(qs).detach()
        nbg = lorentz_berthelot_nbfp(sig, eps).detach()
    a.record(stream)
    for _ in range(iters):
        m._run(qg, nbg)
    z.record(stream)
    torch.cuda.synchronize()
    graph_ms = a.elapsed_time(z) / iters

    # baseline: central differences of plain sequential per-system forward evaluations
    # the adjoint gradient at the final parameters, compared with central differences there
    opt.zero_grad(set_to_none=True)
    loss_at(sig, eps, qs).backward()
    g_adj = torch.cat([sig.grad, eps.grad, qs.grad]).detach().clone()
    base = torch.cat([sig.detach(), eps.detach(), qs.detach()]).clone()
    fseq = torch.empty_like(x)

    def seq_loss(pv):
        qv = (q0 * pv[16:24][types]).float().contiguous()
        nb = lorentz_berthelot_nbfp(pv[0:8], pv[8:16]).float().contiguous()
        ref.set_parameters_device(qv.data_ptr(), nb.data_ptr())
        ref.sequential_md_step_device(1, x.data_ptr(), fseq.data_ptr())
        return ((fseq.double() - f_target.double()) ** 2).sum()

    ref.set_graph(False)
    seq_loss(base)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    g_fd = torch.empty(24, dtype=torch.float64, device=d)
    for i in range(24):
        h = 1e-3 * float(base[i].abs()) + 1e-6
        pp, pm = base.clone(), base.clone()
        pp[i] += h
        pm[i] -= h
        g_fd[i] = (seq_loss(pp) - seq_loss(pm)) / (2 * h)
    torch.cuda.synchronize()
    fd_ms = (time.perf_counter() - t0) * 1e3
    fd_vs_adj = float(torch.linalg.norm(g_fd - g_adj) / torch.linalg.norm(g_adj))
    m.close()
    ref.close()
    return {"workload": "64 random LJ+Coulomb liquids, 2000..50000 atoms log-uniform, 8 types shared, "
                        "rejection at 0.5 sigma (seed 5)", "atoms": n, "adam_steps": iters, "lr": 1e-3,
            "gradient_step_ms": step_ms, "graph_launch_ms": graph_ms, "force_evals_per_s": 64 * 1e3 / step_ms,
            "loss_first": float(losses[0].detach()), "loss_last": float(losses[-1].detach()),
            "fd_gradient_step_ms": fd_ms, "fd_force_evals_per_s": 64 * 48 * 1e3 / fd_ms,
            "speedup_vs_fd": fd_ms / step_ms, "fd_vs_adjoint_rel_diff": fd_vs_adj,
            "gradient_vs_fp64": "the two smallest systems of this batch (2,007 + 2,095 atoms, same targets): "
                                "loss and sigma / epsilon / charge-scale gradients within 2e-5 relative of FP64 "
                                "autograd over all pairs (tests/test_gpu_batch_adjoint.py::"
                                "test_benchmarked_force_matching_batch_subset_vs_fp64); the whole batch against "
                                "central differences: fd_vs_adjoint_rel_diff",
            "min_pair_distance": min_pair_distances(ens),
            "build_s": t_build,
            "note": "adjoint step = one graph launch (set parameters, forces+energies+virials, loss, adjoint) "
                    "+ Adam on 24 shared parameters; FD = 48 evaluations x 64 sequential per-system "
                    "launches, central differences with step 1e-3 relative"}


def hbm_peak_gbs() -> float:
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "MEASURED_PEAKS.json")
    try:
        return float(json.load(open(path))["hbm_gbs"])
    except (OSError, KeyError, ValueError):
        return 6800.0  # fallback: one earlier GB300 copy measurement


def measure_memory_kernels(calc, frames, flush, stream, reps: int = 8) -> dict:
    """Gridding, search and prune passes of the 288k-atom workload, each after an L2
    flush, timed by the engine's phase events; bytes are the algorithmic bytes per pass:
    grid 39 B/atom (x 12, xq 16, atom index 4, cell 4, bounding boxes 3); search (lower
    bound) = bounding boxes read once (24 B/cluster) + list written (16 B/entry, 32 B/cj4,
    128 B/exclusion mask); prune = 48 B per cj4 examined (cj4 32, outer mask 8, inner mask 8;
    +8 for the outer mask on a fresh list) + 16 B per i-atom and per j-atom read once."""
    import torch

    peak = hbm_peak_gbs()
    sz = calc.sizes()
    calc.phase_timings(reset=True)
    calc.set_timing(True)
    for k in range(reps):
        flush.zero_()
        calc.search_device(frames[k % frames.shape[0]].data_ptr())
    torch.cuda.synchronize()
    t = calc.phase_timings(reset=True)
    sz = calc.sizes()
    nparts = max(1, NSTPRUNE // 2)
    for k in range(reps):
        flush.zero_()
        calc.prune_device(k % nparts)
    torch.cuda.synchronize()
    tr = calc.phase_timings(reset=True)
    for k in range(reps):
        flush.zero_()
        calc.prune_device(-1)
    torch.cuda.synchronize()
    tf = calc.phase_timings(reset=True)
    calc.set_timing(False)
    n, npad, ncj4, nsci, nexcl = sz["num_atoms"], sz["npad"], sz["num_cj4"], sz["num_sci"], sz["num_excl"]
    nclusters = npad // 8

    def entry(ms_count, nbytes, what):
        ms, cnt = ms_count
        avg = ms / max(1, cnt)
        gbs = nbytes / (avg * 1e-3) / 1e9 if avg > 0 else None
        return {"ms": avg, "bytes": nbytes, "GB/s": gbs, "frac": gbs / peak if gbs else None,
                "peak": peak, "bytes_rule": what}

    grid_b = 39 * n
    search_b = 24 * nclusters + 16 * nsci + 32 * ncj4 + 128 * nexcl
    prune_fresh_b = 56 * ncj4 + 16 * npad + 16 * npad
    prune_roll_b = (48 * ncj4 + 16 * npad) / nparts + 16 * npad
    return {
        "grid": entry(t["grid"], grid_b, "39 B/atom"),
        "search_count": entry(t["search_count"], search_b, "lower bound: bb once + list size"),
        "search_write": entry(t["search_write"], search_b, "lower bound: bb once + list written"),
        "prune_fresh": entry(tf["prune"], prune_fresh_b, "56 B/cj4 + 16 B/i-atom + 16 B/j-atom"),
        "prune_rolling": entry(tr["prune"], prune_roll_b,
                               f"(48 B/cj4 + 16 B/i-atom) / {nparts} parts + 16 B/j-atom"),
        "list": {"atoms": n, "npad": npad, "num_sci": nsci, "num_cj4": ncj4, "num_excl": nexcl},
        "note": "each pass after a 256 MB L2 flush; peak = MEASURED_PEAKS.json hbm_gbs (of measured)",
    }


PME_SPACING = 0.12


def measure_pme(dev: int, calc=None, frames=None, flush=None, stream=None, steps: int = 20) -> dict:
    """Smooth-PME reciprocal space for the same 288k-atom box (120^3 grid at 0.12 nm, beta
    from rc 0.9 / rtol 1e-5, pme_order 4): the whole reciprocal step with energy and
    virial, the spread and gather stages alone, the full electrostatics step (cluster-pair
    real space + PME) on one stream, the host-array call, parity against the PME oracle
    and the oracle's own time on the host.  Each timed pass follows a 256 MB L2 flush."""
    import torch

    from gmxapi_gb300 import nblib, systems
    from gmxapi_gb300 import pme as pm
    from oracle import pme_oracle

    s = systems.water_large()
    if calc is None:
        opts = nblib.NBKernelOptions(coulomb_type=nblib.CoulombType.Pme, pairlist_cutoff=RLIST, rcoulomb=RC,
                                     rlist_inner=RLIST_INNER, nstlist=NSTLIST, nstlist_prune=NSTPRUNE,
                                     compute_virial_and_energy=True)
        calc = nblib.ForceCalculator(s, opts, device=dev)
        stream = torch.cuda.current_stream(dev)
        calc.set_stream(stream.cuda_stream)
        x0 = torch.from_numpy(s.x.reshape(-1)).to(f"cuda:{dev}")
        gen = torch.Generator(device=f"cuda:{dev}").manual_seed(99)
        frames = torch.stack([x0 + SIGMA_STEP * k * torch.randn(x0.shape, generator=gen, device=x0.device)
                              for k in range(4)])
        flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=x0.device)
    box = [float(b) for b in s.box]
    grid = pm.grid_size(box, PME_SPACING)
    beta = pm.ewald_coefficient(RC, 1e-5)
    p = pm.Pme(box, grid, beta, device=dev)
    p.set_stream(stream.cuda_stream)
    n = s.n
    q = torch.from_numpy(s.q).to(frames.device)
    f = torch.zeros(n * 3, dtype=torch.float32, device=frames.device)
    ev = torch.zeros(12, dtype=torch.float64, device=frames.device)
    g = torch.zeros(grid, dtype=torch.float32, device=frames.device)

    def timed(fn):
        for k in range(3):
            fn(k)
        torch.cuda.synchronize()
        ms = []
        for k in range(steps):
            flush.zero_()
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record(stream)
            fn(k)
            b.record(stream)
            torch.cuda.synchronize()
            ms.append(a.elapsed_time(b))
        return statistics.median(ms)

    nf = frames.shape[0]
    full = timed(lambda k: p.compute_device(n, frames[k % nf].data_ptr(), q.data_ptr(), f.data_ptr(),
                                            ev.data_ptr(), ev[3:].data_ptr()))
    forces_only = timed(lambda k: p.compute_device(n, frames[k % nf].data_ptr(), q.data_ptr(), f.data_ptr()))
    spread = timed(lambda k: p.spread_device(n, frames[k % nf].data_ptr(), q.data_ptr(), g.data_ptr()))
    gather = timed(lambda k: p.gather_device(n, frames[k % nf].data_ptr(), q.data_ptr(), g.data_ptr(),
                                             f.data_ptr()))

    def electrostatics(k):
        x = frames[k % nf].data_ptr()
        calc.compute_device(x, f.data_ptr(), ev[1:].data_ptr(), ev[3:].data_ptr())
        p.compute_device(n, x, q.data_ptr(), f.data_ptr(), ev.data_ptr(), ev[3:].data_ptr())

    calc.search_device(frames[0].data_ptr())
    step_ms = timed(electrostatics)

    # host arrays: H2D of x and q, D2H of forces, energy and virial inside the call
    x0 = frames[0].cpu().numpy().reshape(-1, 3)
    p2 = pm.Pme(box, grid, beta, device=dev)
    p2.compute(x0, s.q)
    e2e = []
    for _ in range(5):
        t0 = time.perf_counter()
        fh = p2.compute(x0, s.q)
        e2e.append((time.perf_counter() - t0) * 1e3)
    e2e_ms = statistics.median(e2e)

    # parity and the oracle on the host (FP64 numpy, one thread for the spread / gather)
    t0 = time.perf_counter()
    ref_f, ref_e, ref_v = pme_oracle.compute(x0, s.q, box, grid, beta, single=True)
    cpu_ms = (time.perf_counter() - t0) * 1e3
    rel = float(np.sqrt(((fh - ref_f) ** 2).sum() / (ref_f ** 2).sum()))
    p.close()
    p2.close()
    red_ops = n * 4 * 4 * 1.75  # 16-byte reductions: per atom 4 x-points x 4 y-rows x 1.75 aligned blocks
    return {
        "grid": list(grid), "beta": beta, "atoms": n,
        "ms_energy_virial": full, "ms_forces_only": forces_only,
        "atoms_per_s": n / (full * 1e-3),
        "stages_ms": {"spread": spread, "gather": gather,
                      "ffts_solve_memset": forces_only - spread - gather},
        "spread": {"weighted_adds_per_s": n * 64 / (spread * 1e-3),
                   "vector_reductions_per_s": red_ops / (spread * 1e-3),
                   "note": "64 weighted grid adds per atom as 16-byte red.global.add.v4.f32; the 6.9 MB "
                           "grid stays in L2, so the bound is L2 reduction throughput, not HBM"},
        "electrostatics_step_ms": step_ms,
        "electrostatics_note": "cluster-pair LJ + Ewald real space (F+E+virial) then PME (F+E+virial) "
                               "on one stream, list fixed",
        "e2e_ms": e2e_ms,
        "parity": {"force_rel_rms_vs_oracle": rel,
                   "energy_rel_vs_oracle": abs(p2.energy - ref_e) / abs(ref_e),
                   "virial_max_rel_vs_oracle": float(np.abs(p2.virial - ref_v).max() / np.abs(ref_v).max())},
        "cpu_baseline": {"ms": cpu_ms, "kind": "port", "cores": 1,
                         "sample": "one PME evaluation of the full 288k-atom box (numpy oracle)"},
    }


def measure_md(dev: int, steps: int = 200, warmup: int = 20) -> dict:
    """GPU-resident MD steps (nbx_md_run_device): cluster-pair LJ + Ewald real space, PME
    reciprocal space and leap-frog on one stream, for 296,352 argon-like atoms with charges
    +-0.1 e (fcc start at 120 K, box 22.08 nm, rc 0.9, rlist 1.0, nstlist 10, dynamic pruning to
    rlist_inner 0.92 every 4 steps in 2 rolling parts as mdrun does on a GPU, PME grid at 0.12 nm,
    dt 2 fs), energies every 100 steps.  Reports the step time and the NVE drift (the inner radius
    leaves 0.02 nm for 4 steps, ~10x the relative motion of two atoms at 120 K)."""
    import torch

    from gmxapi_gb300 import md, nblib, systems

    s = systems.lj_fcc(cells=42, lattice=0.5256, charge=0.1, seed=1)
    rng = np.random.default_rng(2)
    v0 = (rng.standard_normal((s.n, 3)) * math.sqrt(0.00831446 * 120.0 / systems.ARGON_MASS)).astype(np.float32)
    opts = nblib.NBKernelOptions(pairlist_cutoff=1.0, rcoulomb=0.9, rlist_inner=0.92, nstlist=10,
                                 nstlist_prune=4, compute_virial_and_energy=True)
    run = md.MdRunner(s, np.full(s.n, systems.ARGON_MASS, np.float32), opts, dt=0.002, velocities=v0, pme=True,
                      fourier_spacing=PME_SPACING, device=dev)
    run.run(warmup, nstcalcenergy=warmup)
    torch.cuda.synchronize()
    a = torch.cuda.Event(enable_timing=True)
    b = torch.cuda.Event(enable_timing=True)
    t0 = time.perf_counter()
    a.record(run.stream)
    rows = run.run(steps, nstcalcenergy=100)
    b.record(run.stream)
    torch.cuda.synchronize()
    wall = (time.perf_counter() - t0) * 1e3
    ms = a.elapsed_time(b)
    etot = rows.sum(axis=1)
    out = {
        "atoms": s.n, "box_nm": float(s.box[0]), "pme_grid": list(run.pme.grid), "steps": steps,
        "ms_per_step": ms / steps, "wall_ms_per_step": wall / steps,
        "ns_per_day": 0.002 * steps / (ms * 1e-3) * 86400 / 1000,
        "atom_steps_per_s": s.n * steps / (ms * 1e-3),
        "energy_rows": rows.tolist(),
        "drift_kj_mol": float(etot[-1] - etot[0]), "mean_ekin_kj_mol": float(rows[:, 3].mean()),
        "note": "device-timed over the whole loop (searches every 10 steps and rolling prunes included); "
                "ns/day at dt 2 fs",
    }
    run.close()
    return out


def measure_fep(dev: int, num_perturbed: int = 256, steps: int = 20) -> dict:
    """The perturbed-pair (free-energy) kernel on the 288k-atom water box: num_perturbed atoms
    (seeded choice) change charge and become uncharged in state B, soft-core alpha 0.5,
    lambda 0.5.  Times the force + energy evaluation with and without the perturbation (the
    list is the same size: perturbed atoms stay in the cluster lists with zero parameters)."""
    import torch

    from gmxapi_gb300 import nblib, systems

    s = systems.water_large()
    opts = nblib.NBKernelOptions(coulomb_type=nblib.CoulombType.Pme, pairlist_cutoff=RLIST, rcoulomb=RC,
                                 compute_virial_and_energy=True)
    calc = nblib.ForceCalculator(s, opts, device=dev)
    stream = torch.cuda.current_stream(dev)
    calc.set_stream(stream.cuda_stream)
    x = torch.from_numpy(s.x.reshape(-1)).to(f"cuda:{dev}")
    f = torch.zeros_like(x)
    ev = torch.zeros(11, dtype=torch.float64, device=x.device)
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=x.device)

    def timed():
        for _ in range(3):
            calc.compute_device(x.data_ptr(), f.data_ptr(), ev.data_ptr(), ev[2:].data_ptr())
        torch.cuda.synchronize()
        ms = []
        for _ in range(steps):
            flush.zero_()
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record(stream)
            calc.compute_device(x.data_ptr(), f.data_ptr(), ev.data_ptr(), ev[2:].data_ptr())
            b.record(stream)
            torch.cuda.synchronize()
            ms.append(a.elapsed_time(b))
        return statistics.median(ms)

    calc.search_device(x.data_ptr())
    plain = timed()
    rng = np.random.default_rng(11)
    pert = np.sort(rng.choice(s.n, num_perturbed, replace=False)).astype(np.int32)
    calc.set_free_energy(pert, np.zeros(num_perturbed, np.float32), s.type[pert], lambda_coul=0.5,
                         lambda_vdw=0.5)
    calc.search_device(x.data_ptr())
    with_fep = timed()
    terms = calc.free_energy_terms()
    calc.close()
    return {"atoms": s.n, "perturbed": num_perturbed, "ms_plain": plain, "ms_with_perturbed": with_fep,
            "overhead_ms": with_fep - plain, "lambda": 0.5, "terms": terms,
            "note": "force + energy + virial evaluation, L2 flushed between evaluations; the "
                    "perturbed pairs run in one block per perturbed atom after the cluster kernel"}


def schedule_counts(first: int, steps: int) -> tuple[int, int]:
    """Searches and rolling-prune passes the step schedule runs in steps [first, first + steps):
    a search where step % nstlist == 0, otherwise one rolling-prune part (of nstlist_prune / 2)
    at every second step of list age (nbx_md_step_device, pairlistsets.h:106-114), so every
    entry is pruned once per nstlist_prune steps."""
    sched = range(first, first + steps)
    searches = sum(1 for t in sched if t % NSTLIST == 0)
    prunes = sum(1 for t in sched if t % NSTLIST != 0 and (t % NSTLIST) % 2 == 0)
    return searches, prunes


def workload_config() -> dict:
    return {"workload": "spc_water_288k", "atoms": 288000, "box_nm": 14.21, "rc_nm": RC, "rlist_nm": RLIST,
            "rlist_inner_nm": RLIST_INNER, "nstlist": NSTLIST, "nstlist_prune": NSTPRUNE,
            "perturb_sigma_nm": SIGMA_STEP, "coulomb": "ewald", "energy_virial": "fp64 every step",
            "l2": "flushed (256 MB write) between timed steps", "parallelism": "replicas"}


def run_ours(args) -> None:
    import torch

    world, rank, local = dist_env()
    dev = local if world > 1 else 0
    torch.cuda.set_device(dev)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    from gmxapi_gb300 import nblib, systems

    s = systems.water_large()
    n = s.n
    opts = nblib.NBKernelOptions(coulomb_type=nblib.CoulombType.Pme, pairlist_cutoff=RLIST, rcoulomb=RC,
                                 rlist_inner=RLIST_INNER, nstlist=NSTLIST, nstlist_prune=NSTPRUNE,
                                 compute_virial_and_energy=True)
    calc = nblib.ForceCalculator(s, opts, device=dev)
    stream = torch.cuda.current_stream(dev)
    calc.set_stream(stream.cuda_stream)
    total = args.warmup + args.steps
    # schedule steps: the timed window starts on a search step (step % nstlist == 0), so it holds
    # ceil(K / nstlist) searches, and the warm-up steps run the rolling prunes just before it
    first_timed = NSTLIST * -(-args.warmup // NSTLIST)
    sched0 = first_timed - args.warmup
    searches, prunes = schedule_counts(first_timed, args.steps)
    # coordinate frames: a Gaussian random walk, resident in HBM before timing
    gen = torch.Generator(device=f"cuda:{dev}").manual_seed(1234 + rank)
    frames = torch.empty((total, n * 3), dtype=torch.float32, device=f"cuda:{dev}")
    frames[0] = torch.from_numpy(s.x.reshape(-1)).to(frames.device)
    for t in range(1, total):
        frames[t] = frames[t - 1] + SIGMA_STEP * torch.randn(n * 3, generator=gen, device=frames.device)
    f = torch.empty(n * 3, dtype=torch.float32, device=frames.device)
    ev = torch.zeros(11, dtype=torch.float64, device=frames.device)
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=frames.device)  # 256 MB > L2

    def step(t):
        calc.md_step_device(sched0 + t, frames[t].data_ptr(), f.data_ptr(), ev.data_ptr(), ev[2:].data_ptr())

    for t in range(args.warmup):
        step(t)
    torch.cuda.synchronize()
    pairs0 = calc.pair_count()
    calc.timings(reset=True)
    calc.set_timing(True)
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    with ClockSampler(dev) as clk:
        for k in range(args.steps):
            flush.zero_()
            starts[k].record(stream)
            step(args.warmup + k)
            ends[k].record(stream)
        torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    step_ms = [a.elapsed_time(b) for a, b in zip(starts, ends)]
    total_ms = float(sum(step_ms))
    force_ms, force_launches, launches = calc.timings(reset=True)
    calc.set_timing(False)
    pairs1 = calc.pair_count()
    up = useful_pairs(n, s.box)
    total_ms, value = replica_throughput(total_ms, up, args.steps, world, frames.device)
    if args.core_only:
        # profiling runs: the device-timed schedule alone (no e2e, memory passes or baselines)
        if rank == 0:
            print(json.dumps({"metric": METRIC, "value": value, "unit": "pairs/s", "steps": args.steps,
                              "warmup": args.warmup, "ms_per_step": total_ms / args.steps,
                              "force_ms_per_launch": force_ms / max(1, force_launches), "core_only": True}))
        return

    # e2e: the same schedule through the C ABI with host arrays (pinned), H2D x and D2H f/E/virial per step.
    # As in an MD code, the coordinates live in one pinned host array that the host updates before each
    # step (outside the timed region) and the forces in one pinned array; every step's transfers of
    # both are inside the timed region.
    hframes = frames.cpu()
    hx = torch.empty(n * 3, dtype=torch.float32).pin_memory()
    hf = torch.empty(n * 3, dtype=torch.float32).pin_memory()
    he = np.zeros(2)
    hv = np.zeros(9)
    import ctypes as C

    from gmxapi_gb300 import _lib

    L = _lib.load()
    calc2 = nblib.ForceCalculator(s, opts, device=dev)
    fp = C.POINTER(C.c_float)
    dp = C.POINTER(C.c_double)

    def hstep(t):
        _lib.check(L.nbx_md_step(calc2.h, sched0 + t, C.cast(hx.data_ptr(), fp), C.cast(hf.data_ptr(), fp),
                                 he.ctypes.data_as(dp), hv.ctypes.data_as(dp)), calc2.h)

    for t in range(args.warmup):
        hx.copy_(hframes[t])
        hstep(t)
    torch.cuda.synchronize()
    e2e_ms = 0.0
    for k in range(args.steps):
        hx.copy_(hframes[args.warmup + k])  # the host's new coordinates (outside the timed region)
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        hstep(args.warmup + k)
        e2e_ms += (time.perf_counter() - t0) * 1e3
    e2e_value = world * up * args.steps / (e2e_ms * 1e-3)
    calc2.close()
    memory_kernels = measure_memory_kernels(calc, frames, flush, stream) if rank == 0 else None

    if rank != 0:
        return
    from gmxapi_gb300.nblib import measure_fp32_peak

    ensemble = measure_ensemble(dev) if not args.no_extras else None
    adjoint = measure_adjoint(dev) if not args.no_extras else None
    force_matching = measure_force_matching(dev) if not args.no_extras else None
    pme_block = measure_pme(dev, calc, frames, flush, stream) if not args.no_extras else None
    md_block = measure_md(dev) if not args.no_extras else None
    fep_block = measure_fep(dev) if not args.no_extras else None

    peak = measure_fp32_peak(dev)
    pairs_avg = 0.5 * (pairs0 + pairs1)
    flops = pairs_avg * FLOPS_PER_PAIR_VF
    avg_force_ms = force_ms / max(1, force_launches)
    achieved = flops / (avg_force_ms * 1e-3) / 1e12
    clocks = clk.summary()
    line = {
        "metric": METRIC, "value": value, "unit": "pairs/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded SPC water)",
        "config": dict(workload_config(), timed_schedule_steps=[first_timed, first_timed + args.steps - 1],
                       searches_in_timed_window=searches, rolling_prunes_in_timed_window=prunes),
        "force_evals_per_s": world * args.steps / (total_ms * 1e-3),
        "pairs_computed_per_eval": pairs_avg, "useful_pairs_per_eval": up,
        "roofline": {"bound": "fp32", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                     "frac": achieved / peak, "traffic": FORCE_KERNEL_DRAM_BYTES,
                     "kernel": "nbx::k_force<energy, ewald>",
                     "note": f"{FLOPS_PER_PAIR_VF} flops per computed pair (nrnb.cpp:106) x "
                             f"{pairs_avg:.4g} computed pairs / {avg_force_ms:.4f} ms average launch; "
                             "the launch also holds the excluded-pair and self energy work items; "
                             "peak = measured FFMA probe of this run (of measured); traffic = DRAM bytes "
                             "per launch from ncu"},
        "cpu_baseline": cpu_baseline_port(),
        "e2e": {"value": e2e_value, "unit": "pairs/s", "h2d_bytes_per_step": n * 12,
                "d2h_bytes_per_step": n * 12 + 11 * 8,
                "transfer": "nbx_md_step on pinned host arrays (one coordinate array updated by the host "
                            "before each step, one force array): the kernels read x and write f, E, virial "
                            "in place over the host link (search steps copy x); wall clock per call"},
        "gpu_launches": launches,
        "clocks": clocks,
    }
    line["memory_kernels"] = memory_kernels
    if ensemble is not None:
        line["batched_ensemble"] = ensemble
    if adjoint is not None:
        line["adjoint"] = adjoint
    if force_matching is not None:
        line["force_matching"] = force_matching
    if pme_block is not None:
        line["pme"] = pme_block
    if md_block is not None:
        line["md"] = md_block
    if fep_block is not None:
        line["free_energy"] = fep_block
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-extras", action="store_true",
                    help="skip the batched-ensemble, adjoint and force-matching measurements")
    ap.add_argument("--core-only", action="store_true",
                    help="time the force schedule only and print a reduced line (profiling)")
    ap.add_argument("--only", choices=["ensemble", "adjoint", "force_matching", "pme", "md", "fep"],
                    help="run one of the extra measurements alone and print its JSON (profiling)")
    args = ap.parse_args()
    if args.only:
        import torch

        torch.cuda.set_device(0)
        fn = {"ensemble": measure_ensemble, "adjoint": measure_adjoint, "force_matching": measure_force_matching,
              "pme": measure_pme, "md": measure_md, "fep": measure_fep}
        print(json.dumps({args.only: fn[args.only](0)}))
        return
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
