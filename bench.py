"""Benchmark of the hierarchical max-flow (HMF) solve on GB300.

Workload (one step = one complete solve, initialisation + all iterations):
256^3 float32 phantom of 4 seeded ellipsoids, 2-level tree (root -> 2
branches -> 2 leaves each), Gaussian-NLL data terms, per-voxel smoothness
0.2*exp(-|grad I|^2/0.01) shared by every vertex, 500 iterations,
StepSize 0.1, CC 0.25.  Metric: voxel*label*iterations per second.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

`--impl ours` (default) runs libhmf_gb300.so; `--impl reference` runs the
reference's CPU implementation of the path on the host cores (the compiled
reference code where it was built, else the oracle's restatement of it).
Under torchrun (N > 1) every rank solves its own volume (replicas; the path
needs no exchange between independent volumes) and rank 0 prints the line.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOAD = "ellipsoids256_tree4"
METRIC = "HMF voxel*label*iterations/s (256^3, 2-level tree, 4 leaves, per-voxel smoothness, 500 it)"
UNIT = "voxel*label*iter/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--size", type=int, default=256)
    ap.add_argument("--iterations", type=int, default=500)
    ap.add_argument("--cpu-seconds", type=float, default=12.0, help="bound of the CPU baseline sample")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-reference-gpu", action="store_true",
                    help="skip timing the reference's own CUDA kernels on this GPU")
    ap.add_argument("--no-batched", action="store_true", help="skip the batched-vs-sequential measurement")
    ap.add_argument("--batch-count", type=int, default=64)
    ap.add_argument("--batch-iterations", type=int, default=200)
    ap.add_argument("--no-adjoint", action="store_true", help="skip the forward+adjoint measurement")
    ap.add_argument("--adjoint-size", type=int, default=128)
    ap.add_argument("--adjoint-iterations", type=int, default=300)
    ap.add_argument("--no-dag", action="store_true", help="skip the DAG solver measurement")
    ap.add_argument("--no-paged", action="store_true", help="skip the out-of-core solve measurement")
    ap.add_argument("--no-large-forward", action="store_true",
                    help="skip the forward solve of the 512x512x384 tree8 workload")
    ap.add_argument("--paged-planes", type=int, default=96,
                    help="block planes the out-of-core leg's MaxGPUUsage budget is sized for")
    ap.add_argument("--no-dataterm", action="store_true", help="skip the data-term producer measurement")
    ap.add_argument("--dag-size", type=int, default=256)
    ap.add_argument("--dag-iterations", type=int, default=100)
    ap.add_argument("--profile-adjoint", action="store_true",
                    help="two adjoint solves (--adjoint-size, --adjoint-iterations, every state kept): "
                         "the command ncu wraps")
    ap.add_argument("--profile-dag", action="store_true",
                    help="one DAG solve (--dag-size, --dag-iterations): the command ncu wraps")
    ap.add_argument("--profile-planes", type=int, default=0,
                    help="--profile on the first N z planes of the workload (same x-y extent, a smaller capture)")
    ap.add_argument("--profile", action="store_true",
                    help="two solves (one warm, one profiled) and nothing else: the command ncu wraps")
    ap.add_argument("--large", action="store_true",
                    help="the 512x512x384 tree8 workload (400 iterations): forward solve and the adjoint under "
                         "the automatic memory plan, one JSON line, nothing else (minutes)")
    ap.add_argument("--large-iterations", type=int, default=400)
    ap.add_argument("--large-dims", default="512,512,384", help="VX,VY,VZ of --large (a smaller case for profiles)")
    ap.add_argument("--profile-large", action="store_true",
                    help="two forward solves of the --large workload (--large-dims, --large-iterations): the "
                         "command ncu wraps")
    ap.add_argument("--profile-dataterm", action="store_true",
                    help="two calls of each data-term producer on the --size image: the command ncu wraps")
    ap.add_argument("--profile-post", action="store_true",
                    help="one solve, then two votes and two energy evaluations of its labels: the command ncu wraps")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
            # the first sample: nvidia-smi has set up its session before the timed region starts
            t0 = time.time()
            while not self.lines and self.proc.poll() is None and time.time() - t0 < 3.0:
                time.sleep(0.02)
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
            except ValueError:
                continue
            for nm, val in zip(names, parts[4:8]):
                if val.lower().startswith("active"):
                    reasons.add(nm)
        sm.sort()
        return {"sm_mhz": sm[len(sm) // 2] if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peak_hbm():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def ncu_traffic():
    """DRAM bytes per iteration from the committed ncu summary, if present."""
    path = os.path.join(ROOT, "profiles", "dram_traffic_%s.txt" % WORKLOAD)
    try:
        with open(path) as f:
            for line in f:
                line = line.strip()
                if line.startswith("{"):
                    return json.loads(line)
    except OSError:
        pass
    return None


def compulsory_bytes_per_iteration(w):
    """Algorithmic bytes of one iteration, 4*V*(12*N + L + N_S + 2): every
    non-root vertex's three flows, divergence, sink and label read and written
    once, each data term and distinct smoothness image read once, the source
    flow read and written."""
    N, L, NS = w.n_nonroot, len(w.leaves), w.n_smooth_images
    return 4.0 * w.nvox * (12 * N + L + NS + 2)


def kernel_bytes(w):
    """Compulsory bytes of this implementation's two kernels per iteration."""
    N, L = w.n_nonroot, len(w.leaves)
    kids = {v: 0 for v in range(len(w.parent))}
    for p in w.parent:
        if p >= 0:
            kids[p] += 1
    B = sum(1 for v, p in enumerate(w.parent) if p >= 0 and kids[v])
    n_smooth_reads = sum(1 for v in w.smooth)
    flow = 4.0 * w.nvox * (10 * N + n_smooth_reads)          # r: p3 sink label inc (+S); w: p3 div
    tree = 4.0 * w.nvox * (N + N + (B + 1) + L + (N + 1) + N)  # r: div label sinks(B,root) D; w: sinks label
    return flow, tree


def cpu_reference_sample(w, seconds: float, threads: int):
    """Reference CPU HMF on a bounded sample: the full volume for as many
    iterations as fit in ~`seconds`, initialisation subtracted."""
    from oracle import oracle as O

    lib = None
    try:
        lib = O.reference_library()
    except Exception:
        lib = None
    kind = "reference" if lib is not None else "port"

    def run(iters):
        t0 = time.perf_counter()
        if kind == "reference":
            O.solve_reference_cpu(w.dims, w.parent, w.data, w.smooth, w.alpha, iters, w.step, w.cc)
        else:
            O.solve(w.dims, w.parent, w.data, w.smooth, w.alpha, iters, w.step, w.cc, semantics=O.REF_CPU,
                    threads=threads)
        return time.perf_counter() - t0

    t_init = run(0)
    t_one = max(run(1) - t_init, 1e-6)
    iters = max(1, min(50, int(seconds / t_one)))
    t = max(run(iters) - t_init, 1e-6)
    L = len(w.leaves)
    return {"value": w.nvox * L * iters / t, "unit": UNIT, "cores": 1 if kind == "reference" else threads,
            "kind": kind,
            "sample": "full %dx%dx%d volume, %d of %d iterations (initialisation excluded), REF_CPU semantics"
                      % (w.dims[0], w.dims[1], w.dims[2], iters, w.iterations),
            "seconds": t, "iterations": iters}


def cpu_ref_cuda_sample(w, seconds: float, threads: int):
    """The oracle's REF_CUDA restatement (the algorithm the GPU path runs, in
    the reference kernels' pass order) on all host threads: the full volume
    for as many iterations as fit in ~`seconds`, initialisation subtracted."""
    from oracle import oracle as O

    def run(iters):
        t0 = time.perf_counter()
        O.solve(w.dims, w.parent, w.data, w.smooth, w.alpha, iters, w.step, w.cc, threads=threads)
        return time.perf_counter() - t0

    t_init = run(0)
    t_one = max(run(1) - t_init, 1e-6)
    iters = max(1, min(20, int(seconds / t_one)))
    t = max(run(iters) - t_init, 1e-6)
    L = len(w.leaves)
    return {"value": w.nvox * L * iters / t, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": "full %dx%dx%d volume, %d of %d iterations (initialisation excluded), REF_CUDA semantics, "
                      "FP32, OpenMP" % (w.dims[0], w.dims[1], w.dims[2], iters, w.iterations),
            "seconds": t, "iterations": iters}


def reference_gpu_sample(w, iterations: int = 10):
    """The reference's own HMF CUDA kernels (CUDA_hierarchicalmaxflow.cu and
    CUDA_commonKernels.cu, compiled unmodified from the reference sources for
    sm_103a into oracle/_ref/hmf_ref_kernels.cubin) on this GPU, launched in
    the reference host code's order (vtkCudaHierarchicalMaxFlowSegmentation.cxx:106-476)
    with every buffer resident: two untimed iterations, then `iterations`
    timed with CUDA events (back to back, without the reference's
    per-iteration stream synchronisation)."""
    from oracle import ref_kernels

    if not ref_kernels.available():
        return {"unavailable": "the reference kernels' cubin was not built (the reference sources were absent)"}
    r = ref_kernels.solve(w.dims, w.parent, w.data, w.smooth, w.alpha, iterations=2, step=w.step, cc=w.cc,
                          time_iterations=iterations, fetch_outputs=False)
    ms = r["ms_per_iteration"]
    return {"value": w.nvox * len(w.leaves) / (ms / 1000.0), "unit": UNIT, "ms_per_iteration": ms,
            "launches_per_iteration": r["launches_per_iteration"],
            "sample": "full %dx%dx%d volume, %d timed iterations after 2" % (w.dims[0], w.dims[1], w.dims[2],
                                                                            iterations)}


def host_threads():
    try:
        return len(os.sched_getaffinity(0))
    except Exception:
        return os.cpu_count() or 1


def make_workload(args, rank):
    from robartsvtk_gb300 import synthetic
    return synthetic.ellipsoids_tree4(seed=rank, size=args.size, iterations=args.iterations)


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    w = make_workload(args, 0)
    threads = host_threads()
    for _ in range(max(0, args.warmup)):
        cpu_reference_sample(w, 0.5, threads)
    vals = []
    secs = []
    last = None
    for _ in range(max(1, args.steps)):
        last = cpu_reference_sample(w, args.cpu_seconds / max(1, args.steps), threads)
        vals.append(last["value"])
        secs.append(last["seconds"])
    vals.sort()
    value = vals[len(vals) // 2]
    # A step is one bounded sample (a few iterations of the full volume):
    # ms_per_step is its measured time; the full 500-iteration solve at that
    # rate is stated apart.
    out = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
           "steps": args.steps, "warmup": args.warmup,
           "ms_per_step": 1000.0 * sum(secs) / len(secs),
           "step": "one bounded sample: %s" % last["sample"],
           "extrapolated_ms_per_solve": 1000.0 * w.nvox * len(w.leaves) * w.iterations / value,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
           "config": {"workload": WORKLOAD, "volume": list(w.dims), "vertices": len(w.parent),
                      "leaves": len(w.leaves), "iterations": w.iterations, "semantics": "REF_CPU"},
           "cpu_baseline": {k: last[k] for k in ("kind", "cores", "sample")} | {"value": value, "unit": UNIT},
           "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out))
    return 0


def run_ours(args):
    import numpy as np
    import torch

    from robartsvtk_gb300 import HMFSolver, replicas

    rank, world, local = replicas.rank_env()
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    w = make_workload(args, rank)
    L = len(w.leaves)
    units_per_step = w.nvox * L * w.iterations
    stream = torch.cuda.Stream()

    # ---- device-resident inputs -------------------------------------------
    d_data = {leaf: torch.from_numpy(d).cuda() for leaf, d in w.data.items()}
    smooth_dev = {}
    d_smooth = {}
    for v, S in w.smooth.items():
        key = id(S)
        if key not in smooth_dev:
            smooth_dev[key] = torch.from_numpy(S).cuda()
        d_smooth[v] = smooth_dev[key]
    solver = HMFSolver(w.dims, w.parent)
    for leaf, t in d_data.items():
        solver.set_data(leaf, t)
    for v, t in d_smooth.items():
        solver.set_smoothness(v, t)
    for v, a in w.alpha.items():
        solver.set_smoothness_scalar(v, a)
    solver.set_params(w.iterations, w.step, w.cc)
    torch.cuda.synchronize()

    for _ in range(max(3, args.warmup)):
        solver.solve(stream)
    stream.synchronize()
    replicas.barrier()
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    clocks.start()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    launches = 0
    for _ in range(args.steps):
        solver.solve(stream)
        launches += solver.stats()["launches"]
    e1.record(stream)
    stream.synchronize()
    torch.cuda.synchronize()
    replicas.barrier()
    clock_info = clocks.stop()
    ms_rank = e0.elapsed_time(e1) / args.steps
    # every rank solved its own volume: the job's units over its slowest rank's time
    value = replicas.job_throughput(units_per_step, ms_rank, "cuda")
    ms = replicas.max_over_ranks(ms_rank, "cuda")

    # ---- end to end through the public API with pinned host buffers -------
    # (right after the device-resident steps, under its own clock record):
    # every step stages the inputs from pinned host memory inside solve() and
    # reads every leaf's labels back into pinned host memory; an event after
    # solve() splits the step into the solve (with its input copies) and the
    # copy-out (with its synchronisations)
    h_data = {leaf: torch.from_numpy(d).pin_memory() for leaf, d in w.data.items()}
    h_smooth_obj = {}
    h_smooth = {}
    for v, S in w.smooth.items():
        if id(S) not in h_smooth_obj:
            h_smooth_obj[id(S)] = torch.from_numpy(S).pin_memory()
        h_smooth[v] = h_smooth_obj[id(S)]
    h_out = {leaf: torch.empty(w.dims[::-1], dtype=torch.float32).pin_memory() for leaf in w.leaves}
    h2d = sum(t.numel() * 4 for t in h_data.values()) + sum(t.numel() * 4 for t in h_smooth_obj.values())
    d2h = sum(t.numel() * 4 for t in h_out.values())
    split = []

    def e2e_step(mark=None):
        for leaf, t in h_data.items():
            solver.set_data(leaf, t)
        for v, t in h_smooth.items():
            solver.set_smoothness(v, t)
        solver.solve(stream)
        if mark is not None:
            mark.record(stream)
        for leaf in w.leaves:
            solver.labels(leaf, out=h_out[leaf], stream=stream)

    e2e_step()
    replicas.barrier()
    link = host_link_bandwidth(list(h_data.values()) + list(h_smooth_obj.values()), list(h_out.values()), stream)
    e_steps = max(3, min(args.steps, 5))
    marks = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(e_steps)]
    e2 = torch.cuda.Event(enable_timing=True)
    e3 = torch.cuda.Event(enable_timing=True)
    stream.synchronize()
    e2e_clocks = ClockSampler(local)
    e2e_clocks.start()
    e2.record(stream)
    for i in range(e_steps):
        marks[i][0].record(stream)
        e2e_step(marks[i][1])
    e3.record(stream)
    stream.synchronize()
    e2e_clock_info = e2e_clocks.stop()
    e2e_rank_ms = e2.elapsed_time(e3) / e_steps
    e2e_value = replicas.job_throughput(units_per_step, e2e_rank_ms, "cuda")
    e2e_ms = replicas.max_over_ranks(e2e_rank_ms, "cuda")
    e2e_solve_ms = sum(a.elapsed_time(b) for a, b in marks) / e_steps
    for leaf, t in d_data.items():  # device-resident inputs again for the legs below
        solver.set_data(leaf, t)
    for v, t in d_smooth.items():
        solver.set_smoothness(v, t)

    # ---- per-kernel device times (events around every launch) -------------
    solver.set_timing(True)
    solver.solve(stream)
    st = solver.stats()
    solver.set_timing(False)
    t_flow, t_tree, t_init = st["flow_ms"], st["tree_ms"], st["init_ms"]
    post = bench_post(w, solver, stream)

    # ---- the convergence log's cost (max / mean |du| per iteration) -------
    solver.set_convergence_log(True)
    solver.solve(stream)
    stream.synchronize()
    g0 = torch.cuda.Event(enable_timing=True)
    g1 = torch.cuda.Event(enable_timing=True)
    g0.record(stream)
    for _ in range(2):
        solver.solve(stream)
    g1.record(stream)
    stream.synchronize()
    ms_log = g0.elapsed_time(g1) / 2
    conv = solver.convergence()
    solver.set_convergence_log(False)
    convergence = {"ms_per_step_with_log": ms_log, "ms_per_step_without": ms_rank,
                   "overhead_frac": ms_log / ms_rank - 1.0,
                   "final_max_change": float(conv["max"][-1]), "final_mean_change": float(conv["mean"][-1]),
                   "max_change_every_100": [float(x) for x in conv["max"][::100]]}

    # ---- the FP32 labels' distance from the same iteration in FP64 --------
    # (outside the timed region: hmf_solve_fp64 on the same context and
    # inputs, then the comparison on the device)
    t0 = time.perf_counter()
    solver.solve_fp64(stream)
    fp64 = solver.fp64_error(stream)
    fp64["seconds"] = time.perf_counter() - t0
    fp64["what"] = ("max over leaves and voxels of |u_fp32 - u_fp64| after all %d iterations; argmax leaf "
                    "agreement between the two" % w.iterations)

    # ---- roofline -----------------------------------------------------------
    peak, peak_kind = measured_peak_hbm()
    b_iter = compulsory_bytes_per_iteration(w)
    it_ms = t_flow + t_tree
    # One iteration as the timed solve runs it (the replayed graphs, slab
    # pipeline included): the step time less the initialisation, per
    # iteration, CUDA events on the launching stream.
    it_solve_ms = (ms_rank - t_init) / w.iterations
    achieved = b_iter / (it_solve_ms / 1000.0) / 1e9
    flow_b, tree_b = kernel_bytes(w)
    traffic = ncu_traffic()
    roofline = {
        "bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
        "peak_source": peak_kind + " (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured" else peak_kind,
        "traffic": traffic.get("dram_bytes_per_iteration") if traffic else None,
        "unit_of_work": "one iteration (every flow and sweep launch of it; algorithmic bytes 4*V*(12N+L+N_S+2)"
                        " = %.0f B) at the timed solve's rate: (ms_per_step - init) / iterations = %.4f ms"
                        % (b_iter, it_solve_ms),
        "iteration_ms": it_solve_ms,
        "kernels_one_by_one": {"iteration_ms": it_ms, "achieved_gbs": b_iter / it_ms / 1e6,
                               "frac": b_iter / it_ms / 1e6 / peak},
        "pipeline": solver.pipeline,
        "kernels": {
            "flow_kernel": {"avg_ms": t_flow, "own_bytes": flow_b, "achieved_gbs": flow_b / t_flow / 1e6,
                            "share": t_flow / it_ms},
            "tree_kernel": {"avg_ms": t_tree, "own_bytes": tree_b, "achieved_gbs": tree_b / t_tree / 1e6,
                            "share": t_tree / it_ms},
            "init_kernel_ms": t_init,
        },
    }
    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": max(3, args.warmup), "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded phantom per rank)",
        "config": {"workload": WORKLOAD, "volume": list(w.dims), "vertices": len(w.parent), "leaves": L,
                   "iterations": w.iterations, "step": w.step, "cc": w.cc, "semantics": "REF_CUDA",
                   "smoothness": "per-voxel, one image shared by all vertices",
                   "l2": "no flush: inputs + solver state %.1f GB per step >> 129 MB L2"
                         % (solver.device_bytes() / 1e9),
                   "parallelism": "replicas" if world > 1 else "single GPU"},
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "ms_per_step": e2e_ms, "solve_with_input_copies_ms": e2e_solve_ms,
                "copy_out_and_host_gaps_ms": e2e_rank_ms - e2e_solve_ms, "over_device_resident": e2e_rank_ms / ms_rank - 1.0,
                "host_link": link, "clocks": e2e_clock_info},
        "gpu_launches": launches,
        "clocks": clock_info,
        "roofline": roofline,
        "fp64_max_abs_err": fp64["max_abs_err"],
        "argmax_agreement": fp64["argmax_agreement"],
        "fp64": fp64,
        "convergence_log": convergence,
        "post": post,
    }
    if rank == 0 and not args.no_paged:
        out["paged"] = bench_paged(args, w, solver, h_data, h_smooth, value, stream)
    if rank == 0 and not args.no_batched:
        out["batched"] = bench_batched(args, stream)
    if rank == 0 and not args.no_adjoint:
        out["adjoint"] = bench_adjoint(args, stream)
    if rank == 0 and not args.no_dataterm:
        out["dataterm"] = bench_dataterm(args, stream)
    if rank == 0 and not args.no_dag:
        out["dag"] = bench_dag(args, stream, None if args.no_cpu_baseline else host_threads())
    if rank == 0 and not args.no_large_forward:
        out["large_forward"] = bench_large_forward(args)
    if rank == 0:
        out["ref_cpu_semantics_gpu"] = bench_ref_cpu_semantics(w, d_data, d_smooth, stream)
    if rank == 0 and not args.no_cpu_baseline:
        out["cpu_baseline"] = cpu_reference_sample(w, args.cpu_seconds, host_threads())
        out["ref_cpu_semantics_gpu"]["ratio_to_cpu_baseline"] = (out["ref_cpu_semantics_gpu"]["value"]
                                                                 / out["cpu_baseline"]["value"])
        cb = cpu_ref_cuda_sample(w, args.cpu_seconds, host_threads())
        cb["ratio"] = value / cb["value"]
        out["cpu_baseline_ref_cuda"] = cb
    if rank == 0 and not args.no_reference_gpu:
        rg = reference_gpu_sample(w)
        if "value" in rg:
            rg["ratio"] = value / rg["value"]
        out["reference_gpu"] = rg
    if rank == 0:
        print(json.dumps(out))
    solver.close()
    if dist:
        dist.destroy_process_group()
    return 0


def bench_ref_cpu_semantics(w, d_data, d_smooth, device_stream, reps=3):
    """The computation the reference arm times -- the reference CPU class as
    written (REF_CPU semantics) -- on the GPU, same workload and inputs:
    the like-for-like counterpart of cpu_baseline (CUDA events, 3 solves
    after a warm one)."""
    import torch

    from robartsvtk_gb300 import REF_CPU, HMFSolver

    s = HMFSolver(w.dims, w.parent, REF_CPU)
    for leaf, t in d_data.items():
        s.set_data(leaf, t)
    for v, t in d_smooth.items():
        s.set_smoothness(v, t)
    for v, a in w.alpha.items():
        s.set_smoothness_scalar(v, a)
    s.set_params(w.iterations, w.step, w.cc)
    s.solve(device_stream)
    device_stream.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(device_stream)
    for _ in range(reps):
        s.solve(device_stream)
    e1.record(device_stream)
    device_stream.synchronize()
    ms = e0.elapsed_time(e1) / reps
    s.close()
    return {"what": "REF_CPU semantics (the reference CPU class's computation) on the GPU, device-resident inputs",
            "ms_per_solve": ms, "value": w.nvox * len(w.leaves) * w.iterations / (ms / 1000.0), "unit": UNIT}


def host_link_bandwidth(inputs, outputs, stream, reps=2):
    """Host <-> device copy rate of this machine right before the end-to-end leg,
    over the end-to-end step's own pinned buffers: every input copied to the
    device and every output buffer filled from it, `reps` times, CUDA events
    (the end-to-end time depends on it, and it varies between boxes and
    buffers)."""
    import torch

    dev = torch.empty_like(inputs[0], device="cuda")
    e = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
    with torch.cuda.stream(stream):
        for t in inputs:
            dev.copy_(t, non_blocking=True)
        e[0].record(stream)
        for _ in range(reps):
            for t in inputs:
                dev.copy_(t, non_blocking=True)
        e[1].record(stream)
        for _ in range(reps):
            for t in outputs:
                t.copy_(dev, non_blocking=True)
        e[2].record(stream)
    stream.synchronize()
    h2d = reps * sum(t.numel() * 4 for t in inputs)
    d2h = reps * sum(t.numel() * 4 for t in outputs)
    return {"h2d_gbs": h2d / e[0].elapsed_time(e[1]) / 1e6, "d2h_gbs": d2h / e[1].elapsed_time(e[2]) / 1e6,
            "h2d_ms_per_step": e[0].elapsed_time(e[1]) / reps, "d2h_ms_per_step": e[1].elapsed_time(e[2]) / reps,
            "buffers": "the end-to-end step's %d pinned inputs and %d pinned outputs" % (len(inputs), len(outputs))}


def bench_paged(args, w, in_core, h_data, h_smooth, in_core_value, device_stream):
    """The same workload out of core (hmf_create_paged): a MaxGPUUsage budget
    that holds three blocks of --paged-planes planes and the inputs (which
    then stay on the device), the state in pinned host memory, pinned host
    inputs; CUDA events around whole solves.  The labels must equal the
    in-core solve's bit for bit."""
    import numpy as np
    import torch

    from robartsvtk_gb300 import HMFSolver

    total = torch.cuda.get_device_properties(torch.cuda.current_device()).total_memory
    pitch = (w.dims[0] + 3) // 4 * 4
    n_inputs = len(w.leaves) + len({id(S) for S in w.smooth.values()})
    per_plane = (9 * (len(w.parent) - 1) + 1 + n_inputs) * pitch * w.dims[1] * 4
    inputs = n_inputs * w.nvox * 4
    budget = 3 * (16 << 20) + inputs + 3 * args.paged_planes * per_plane
    usage = budget / total
    s = HMFSolver(w.dims, w.parent, max_gpu_usage=usage)
    for leaf, t in h_data.items():
        s.set_data(leaf, t)
    for v, t in h_smooth.items():
        s.set_smoothness(v, t)
    for v, a in w.alpha.items():
        s.set_smoothness_scalar(v, a)
    s.set_params(w.iterations, w.step, w.cc)
    s.solve(device_stream)  # warm: block contexts, pinned host state, graphs
    device_stream.synchronize()
    reps = 2
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(device_stream)
    for _ in range(reps):
        s.solve(device_stream)
    e1.record(device_stream)
    device_stream.synchronize()
    ms = e0.elapsed_time(e1) / reps
    plan = s.paged_plan()
    same = all(np.array_equal(s.labels(leaf, stream=device_stream), in_core.labels(leaf, stream=device_stream))
               for leaf in w.leaves)
    units = w.nvox * len(w.leaves) * w.iterations
    out = {
        "workload": "the benchmark workload out of core: state in pinned host memory, pinned host inputs",
        "max_gpu_usage": usage, "budget_bytes": budget, "device_bytes": s.device_bytes(),
        "plan": plan, "ms_per_solve": ms, "value": units / (ms / 1000.0), "unit": UNIT,
        "fraction_of_in_core": units / (ms / 1000.0) / in_core_value,
        "link_gbs": plan["link_bytes"] / (ms / 1000.0) / 1e9,
        "labels_identical_to_in_core": bool(same), "repetitions": reps,
    }
    s.close()
    return out


def bench_post(w, solver, device_stream):
    """The solved benchmark volume's label vote (hmf_get_vote into a device
    int32 buffer) and energy decomposition (hmf_get_energy), CUDA events on
    the launching stream.  Algorithmic bytes: vote 4V(L+1) (each leaf label
    read once, the label map written); energy 4V(2L+N_S) (each leaf label and
    data term, each distinct smoothness image read once)."""
    import torch

    V = w.dims[0] * w.dims[1] * w.dims[2]
    L = len(w.leaves)
    n_s = len({id(S) for S in w.smooth.values()})
    peak, _ = measured_peak_hbm()
    out = torch.empty(w.dims[::-1], dtype=torch.int32, device="cuda")

    def timed(fn, reps):
        fn()
        device_stream.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(device_stream)
        for _ in range(reps):
            fn()
        e1.record(device_stream)
        device_stream.synchronize()
        return e0.elapsed_time(e1) / reps

    t_vote = timed(lambda: solver.vote(out=out, stream=device_stream), 10)
    # hmf_get_energy runs on the context's stream and synchronises it
    t_energy = timed(lambda: solver.energy(), 3)
    b_vote = 4.0 * V * (L + 1)
    b_energy = 4.0 * V * (2 * L + n_s)
    res = {}
    for name, t, b in (("vote", t_vote, b_vote), ("energy", t_energy, b_energy)):
        gbs = b / t / 1e6
        res[name] = {"ms": t, "bytes": b, "achieved_gbs": gbs, "frac": gbs / peak}
    res["energy"]["note"] = "one call: the sums zeroed, one kernel, the 8-byte-per-vertex sums read back, a stream sync"
    return res


def dataterm_inputs(n):
    """The data-term producers' inputs, on the device: an n^3 image of
    integers 0..199 and four int32 label maps (each voxel 1 with p = 0.3),
    from a seeded torch generator."""
    import torch

    g = torch.Generator(device="cuda")
    g.manual_seed(0)
    img = (torch.rand((n, n, n), generator=g, device="cuda") * 200.0).floor()
    maps = [(torch.rand((n, n, n), generator=g, device="cuda") < 0.3).to(torch.int32) for _ in range(4)]
    return img, maps


def run_profile_dataterm(args):
    """Two calls of each data-term producer on the --size image (the Gaussian
    entropy cost, normalised, and the 4-map log-likelihood cost), device
    resident: the command ncu wraps."""
    import torch

    from robartsvtk_gb300 import data_term, log_likelihood

    img, maps = dataterm_inputs(args.size)
    out = torch.empty_like(img)
    for _ in range(2):
        data_term(2, img, k1=20.0, c1=100.0, entropy=True, normalize=True, out=out)
    for _ in range(2):
        log_likelihood(img, maps, label_id=1, resolution=1.0, required_agreement=0.5, out=out)
    torch.cuda.synchronize()
    print(json.dumps({"profile_dataterm": "%d^3 float image, 4 int32 label maps" % args.size,
                      "checksum": float(out.double().sum().item())}))
    return 0


def bench_dataterm(args, device_stream):
    """The data-term producers on the 256^3 phantom image, device-resident:
    a Gaussian entropy cost of one image, normalised (hmf_data_term; bytes 8V:
    one float read, one written, plus one read for the range), and the
    log-likelihood cost from 4 int32 label maps (hmf_log_likelihood; bytes
    4V(3 + 2*4): the maps and the image read in the seed scan and the
    histogram pass, the image read and the cost written in the last pass).
    CUDA events, the best of 3 calls."""
    import torch

    from robartsvtk_gb300 import data_term, log_likelihood

    n = args.size
    img, maps = dataterm_inputs(n)
    peak, _ = measured_peak_hbm()
    V = n ** 3

    def best(fn):
        fn()
        torch.cuda.synchronize()
        times = []
        for _ in range(3):
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record()
            fn()
            e1.record()
            torch.cuda.synchronize()
            times.append(e0.elapsed_time(e1))
        return min(times)

    out = torch.empty_like(img)
    t_dt = best(lambda: data_term(2, img, k1=20.0, c1=100.0, entropy=True, normalize=True, out=out))
    t_ll = best(lambda: log_likelihood(img, maps, label_id=1, resolution=1.0, required_agreement=0.5, out=out))
    b_dt = 12.0 * V
    b_ll = 4.0 * V * (3 + 2 * 4)
    return {"workload": "%d^3 float image, 4 int32 label maps" % n,
            "data_term_gaussian_entropy_normalised": {"ms": t_dt, "bytes": b_dt, "achieved_gbs": b_dt / t_dt / 1e6,
                                                      "frac": b_dt / t_dt / 1e6 / peak,
                                                      "note": "double-precision exp/log as the reference computes"},
            "log_likelihood": {"ms": t_ll, "bytes": b_ll, "achieved_gbs": b_ll / t_ll / 1e6,
                               "frac": b_ll / t_ll / 1e6 / peak,
                               "note": "three passes with two host synchronisations (range, histogram size)"}}


def dag_workload(size, iterations):
    """The 256^3 tree4 phantom (ellipsoids_tree4) solved as a rooted DAG: the
    tree's edges in vertex order plus B2 -> L1, so leaf L1 has two parents
    (unweighted: push-down weight 1/2 each).  Vertices 0 root, 1 B1, 2 L0,
    3 L1, 4 B2, 5 L2, 6 L3; smoothness image shared, alpha 1 on every vertex."""
    from robartsvtk_gb300 import synthetic

    w = synthetic.ellipsoids_tree4(seed=0, size=size, iterations=iterations)
    edges = [(p, v) for v, p in enumerate(w.parent) if p >= 0] + [(4, 3)]
    return w, edges


def bench_dag(args, device_stream, cpu_threads):
    """DAG solver throughput (voxel.label.iterations/s, device-resident
    inputs, CUDA events) and the per-voxel graph sweep's roofline.  Sweep
    algorithmic bytes per voxel: 4(7N + L + 2) (sink, source, divergence and
    label of each non-root node read; sink, label and source written; each
    data term read; the root's source read and written)."""
    import torch

    from robartsvtk_gb300 import DAGSolver

    w, edges = dag_workload(args.dag_size, args.dag_iterations)
    n = len(w.parent)
    N, L = n - 1, len(w.leaves)
    S = torch.from_numpy(next(iter(w.smooth.values()))).cuda()
    d = {leaf: torch.from_numpy(a).cuda() for leaf, a in w.data.items()}
    s = DAGSolver(w.dims, n, edges)
    for leaf, t in d.items():
        s.set_data(leaf, t)
    for v in range(1, n):
        s.set_smoothness(v, S)
        s.set_smoothness_scalar(v, 1.0)
    s.set_params(w.iterations, w.step, w.cc)
    s.solve(device_stream)
    device_stream.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    reps = 2
    e0.record(device_stream)
    for _ in range(reps):
        s.solve(device_stream)
    e1.record(device_stream)
    device_stream.synchronize()
    ms = e0.elapsed_time(e1) / reps
    s.set_timing(True)
    s.solve(device_stream)
    st = s.stats()
    s.set_timing(False)
    V = w.nvox
    peak, _ = measured_peak_hbm()
    sweep_b = 4.0 * V * (7 * N + L + 2)
    flow_b = 44.0 * V * N
    out = {"workload": "ellipsoids%d_tree4 as a DAG (+ edge B2->L1), %d iterations" % (args.dag_size, w.iterations),
           "value": V * L * w.iterations / (ms / 1000.0), "unit": UNIT, "ms_per_solve": ms,
           "launches": st["launches"],
           "flow_kernel": {"avg_ms": st["flow_ms"], "bytes": flow_b, "achieved_gbs": flow_b / st["flow_ms"] / 1e6,
                           "frac": flow_b / st["flow_ms"] / 1e6 / peak},
           "dag_sweep_kernel": {"avg_ms": st["tree_ms"], "bytes": sweep_b,
                                "achieved_gbs": sweep_b / st["tree_ms"] / 1e6,
                                "frac": sweep_b / st["tree_ms"] / 1e6 / peak},
           "dag_init_kernel_ms": st["init_ms"]}
    s.close()
    if cpu_threads:
        out["cpu_baseline"] = cpu_dag_sample(w, edges, cpu_threads)
    return out


def cpu_dag_sample(w, edges, threads, iters=2):
    """The DAG oracle (the same fixed task order, FP32, OpenMP) on the host
    cores: the full volume for `iters` iterations, initialisation excluded.
    The reference's own CPU DAG class is not a baseline: its flow magnitude
    reads past its buffers."""
    from oracle import oracle as O

    n = len(w.parent)
    alpha = {v: 1.0 for v in range(1, n)}

    def run(k):
        t0 = time.perf_counter()
        O.dag_solve(w.dims, n, edges, w.data, None, w.smooth, alpha, k, w.step, w.cc, threads=threads)
        return time.perf_counter() - t0

    t = max(run(iters) - run(0), 1e-6)
    return {"value": w.nvox * len(w.leaves) * iters / t, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": "full %dx%dx%d volume, %d iterations (initialisation excluded)" % (*w.dims, iters)}


def backward_bytes_per_step(w):
    """Compulsory bytes of one backward step (the sweep reverse and the flow
    reverse): sweep reads per vertex the two sink adjoint parts and the sink
    after, the data term (leaves) or the sink before (others), per non-root
    vertex the label adjoint, gb, the label before and the divergence after,
    per leaf the data gradient (double); writes per vertex the new sink
    adjoint, per non-root vertex the label and divergence adjoints, per leaf
    the data gradient.  Flow reverse per non-root vertex: 10 reads, 4 writes."""
    n, L = len(w.parent), len(w.leaves)
    sweep = (2 * n + n + 4 * (n - 1) + 2 * L) + (n + 2 * (n - 1) + 2 * L)
    flow = 14 * (n - 1)
    return 4.0 * w.nvox * (sweep + flow)


def large_forward(args):
    """The 512x512x384 CT-like phantom, tree root -> 2 -> 4 -> 8 (14 non-root
    vertices, 8 leaves), one shared per-voxel smoothness image, 400
    iterations, solved forward once after a 5-iteration warm-up (inputs
    resident on the device, CUDA events on one stream), with per-kernel
    averages of a 10-iteration solve timed launch by launch.  Returns the
    workload, the solver (still holding the state) and the forward record."""
    import torch

    from robartsvtk_gb300 import HMFSolver, synthetic

    t0 = time.time()
    dims = tuple(int(v) for v in args.large_dims.split(","))
    w = synthetic.ellipsoids_tree8(seed=5, dims=dims, iterations=args.large_iterations)
    gen_s = time.time() - t0
    stream = torch.cuda.Stream()
    peak, peak_kind = measured_peak_hbm()
    d = {leaf: torch.from_numpy(a).cuda() for leaf, a in w.data.items()}
    S = torch.from_numpy(next(iter(w.smooth.values()))).cuda()
    s = HMFSolver(w.dims, w.parent)
    s._bench_inputs = (d, S)  # keep the device inputs alive with the solver
    for leaf, t in d.items():
        s.set_data(leaf, t)
    for v in w.smooth:
        s.set_smoothness(v, S)
    for v, a in w.alpha.items():
        s.set_smoothness_scalar(v, a)
    s.set_params(5, w.step, w.cc)
    s.solve(stream)  # warm-up (tables, first launches)
    s.set_params(w.iterations, w.step, w.cc)
    stream.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    s.solve(stream)
    e1.record(stream)
    stream.synchronize()
    t_fwd = e0.elapsed_time(e1)
    T = w.iterations
    s.set_params(min(T, 10), w.step, w.cc)
    s.set_timing(True)
    s.solve(stream)
    kstats = s.stats()
    s.set_timing(False)
    s.set_params(T, w.step, w.cc)
    vli = w.nvox * len(w.leaves) * T
    b_iter = compulsory_bytes_per_iteration(w)
    fwd = {"workload": "ellipsoids%dx%dx%d_tree8" % tuple(w.dims), "volume": list(w.dims), "vertices": len(w.parent),
           "leaves": len(w.leaves), "iterations": T, "data": "synthetic (seeded phantom)", "generate_s": gen_s,
           "ms": t_fwd, "value": vli / (t_fwd / 1000.0), "unit": "voxel*label*iter/s",
           "bytes_per_iteration": b_iter, "achieved_gbs": b_iter * T / (t_fwd / 1000.0) / 1e9,
           "frac": b_iter * T / (t_fwd / 1000.0) / 1e9 / peak, "peak_gbs": peak, "peak_source": peak_kind,
           "flow_kernel_ms": kstats["flow_ms"], "tree_kernel_ms": kstats["tree_ms"],
           "device_bytes": s.device_bytes()}
    return w, s, stream, fwd


def bench_large_forward(args, adjoint_iterations=40):
    """The large forward solve of `large_forward` inside the default run, with
    the agreement of its label vote with the phantom's classes; then the
    adjoint w.r.t. the data terms on the same volume and tree over
    `adjoint_iterations` iterations (400 take ~100 s: bench.py --large), its
    automatic plan in the free HBM less a margin, to state the backward
    step's throughput and HBM fraction at this shape."""
    import numpy as np
    import torch

    w, s, stream, fwd = large_forward(args)
    vote = torch.empty(w.dims[::-1], dtype=torch.int32, device="cuda")
    s.vote(out=vote, stream=stream)
    stream.synchronize()
    leaf_of_class = torch.tensor(sorted(w.data), dtype=torch.int32, device="cuda")
    truth_leaf = leaf_of_class[torch.from_numpy(w.truth.astype(np.int64)).cuda()]
    fwd["vote_agrees_with_phantom"] = float((vote == truth_leaf).float().mean().item())
    del vote, truth_leaf
    if adjoint_iterations > 0:
        peak, _ = measured_peak_hbm()
        order = np.array([s.leaves.index(leaf) for leaf in sorted(w.data)], dtype=np.int32)
        truth = torch.from_numpy(order[w.truth]).cuda()
        T = adjoint_iterations
        s.set_params(T, w.step, w.cc)
        free_b, _ = torch.cuda.mem_get_info()
        s.set_adjoint_memory(max_bytes=max(0, free_b - (6 << 30)))
        stream.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        s.solve_adjoint(truth, stream=stream)
        e1.record(stream)
        stream.synchronize()
        t_adj = e0.elapsed_time(e1)
        plan = s.adjoint_plan()
        t_it = fwd["ms"] / fwd["iterations"]
        t_bwd = t_adj - plan["forward_iterations"] * t_it
        b_bwd = backward_bytes_per_step(w)
        vli = w.nvox * len(w.leaves) * T
        fwd["adjoint"] = {"iterations": T, "ms": t_adj, **plan, "device_bytes": s.device_bytes(),
                          "backward_ms": t_bwd, "backward_ms_per_step": t_bwd / T,
                          "backward_note": "adjoint time minus the schedule's forward iterations at the forward "
                                           "solve's per-iteration time",
                          "backward_value": vli / (t_bwd / 1000.0), "unit": UNIT,
                          "backward_bytes_per_step": b_bwd,
                          "backward_achieved_gbs": b_bwd * T / (t_bwd / 1000.0) / 1e9,
                          "backward_frac": b_bwd * T / (t_bwd / 1000.0) / 1e9 / peak}
        del truth
    s.close()
    torch.cuda.empty_cache()
    return fwd


def run_large(args):
    """The large forward solve (large_forward), then hmf_solve_adjoint with
    the automatic plan (every state kept if it fits, else the
    fewest-forward-iterations schedule over the state slots that fit in the
    free HBM less a margin).  Times are CUDA events on one stream."""
    import numpy as np
    import torch

    w, s, stream, fwd = large_forward(args)
    peak, peak_kind = measured_peak_hbm()
    # phantom class k is leaf 7 + k; the adjoint's truth indexes s.leaves
    order = np.array([s.leaves.index(leaf) for leaf in sorted(w.data)], dtype=np.int32)
    truth = torch.from_numpy(order[w.truth]).cuda()

    def timed(fn):
        stream.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        r = fn()
        e1.record(stream)
        stream.synchronize()
        return e0.elapsed_time(e1), r

    T = w.iterations
    t_fwd = fwd["ms"]
    vli = w.nvox * len(w.leaves) * T
    # the adjoint may use the free device memory but a margin (the library's
    # default budget is 85% of it): every state slot saves forward passes
    free_b, _ = torch.cuda.mem_get_info()
    s.set_adjoint_memory(max_bytes=max(0, free_b - (6 << 30)))
    t_adj, loss = timed(lambda: s.solve_adjoint(truth, stream=stream))
    plan = s.adjoint_plan()
    t_it = t_fwd / T
    t_bwd = t_adj - plan["forward_iterations"] * t_it
    b_bwd = backward_bytes_per_step(w)
    out = {
        "workload": fwd["workload"], "forward": fwd,
        "adjoint": {"ms": t_adj, "ratio_to_forward": t_adj / t_fwd, "loss": loss, **plan,
                    "device_bytes": s.device_bytes(),
                    "backward_ms": t_bwd,
                    "backward_note": "adjoint time minus the schedule's forward iterations at the forward solve's "
                                     "per-iteration time",
                    "backward_value": vli / (t_bwd / 1000.0),
                    "backward_bytes_per_step": b_bwd,
                    "backward_achieved_gbs": b_bwd * T / (t_bwd / 1000.0) / 1e9,
                    "backward_frac": b_bwd * T / (t_bwd / 1000.0) / 1e9 / peak},
        "peak_gbs": peak, "peak_source": peak_kind,
    }
    s.close()
    print(json.dumps(out))
    return 0


def run_profile_large(args):
    import torch

    from robartsvtk_gb300 import HMFSolver, synthetic

    dims = tuple(int(v) for v in args.large_dims.split(","))
    w = synthetic.ellipsoids_tree8(seed=5, dims=dims, iterations=args.large_iterations)
    d = {leaf: torch.from_numpy(a).cuda() for leaf, a in w.data.items()}
    S = torch.from_numpy(next(iter(w.smooth.values()))).cuda()
    s = HMFSolver(w.dims, w.parent)
    for leaf, t in d.items():
        s.set_data(leaf, t)
    for v in w.smooth:
        s.set_smoothness(v, S)
    for v, a in w.alpha.items():
        s.set_smoothness_scalar(v, a)
    s.set_params(w.iterations, w.step, w.cc)
    for _ in range(2):
        s.solve()
    torch.cuda.synchronize()
    print(json.dumps({"profile_large": list(w.dims), "iterations": w.iterations, "launches": s.stats()["launches"]}))
    s.close()
    return 0


def run_profile_adjoint(args):
    import torch

    from robartsvtk_gb300 import HMFSolver, synthetic

    w = synthetic.ellipsoids_flat4(seed=3, size=args.adjoint_size, iterations=args.adjoint_iterations)
    d = {leaf: torch.from_numpy(a).cuda() for leaf, a in w.data.items()}
    truth = torch.from_numpy(w.truth.astype("int32")).cuda()
    s = HMFSolver(w.dims, w.parent)
    for leaf, t in d.items():
        s.set_data(leaf, t)
    for v, a in w.alpha.items():
        s.set_smoothness_scalar(v, a)
    s.set_params(w.iterations, w.step, w.cc)
    losses = [s.solve_adjoint(truth) for _ in range(2)]
    torch.cuda.synchronize()
    print(json.dumps({"profile_adjoint": list(w.dims), "iterations": w.iterations, "loss": losses[-1],
                      "plan": s.adjoint_plan()}))
    s.close()
    return 0


def run_profile_dag(args):
    import torch

    from robartsvtk_gb300 import DAGSolver

    w, edges = dag_workload(args.dag_size, args.dag_iterations)
    n = len(w.parent)
    s = DAGSolver(w.dims, n, edges)
    keep = [torch.from_numpy(a).cuda() for a in w.data.values()]
    for leaf, t in zip(w.data, keep):
        s.set_data(leaf, t)
    S = torch.from_numpy(next(iter(w.smooth.values()))).cuda()
    for v in range(1, n):
        s.set_smoothness(v, S)
        s.set_smoothness_scalar(v, 1.0)
    s.set_params(w.iterations, w.step, w.cc)
    s.solve()
    torch.cuda.synchronize()
    print(json.dumps({"profile_dag": list(w.dims), "iterations": w.iterations, "launches": s.stats()["launches"]}))
    s.close()
    return 0


def bench_batched(args, device_stream):
    """64 volumes with axes U{48..192}, flat 3 leaves, alpha 0.15, 200
    iterations: one batched solve (autotuned) against the same 64 volumes
    solved one after another, each in its own context.  Inputs are resident
    on the device; times are CUDA events on one stream."""
    import torch

    from robartsvtk_gb300 import HMFBatchSolver, HMFSolver, synthetic

    ws = synthetic.batch_flat3(seed=7, count=args.batch_count, iterations=args.batch_iterations)
    keep = []
    dev = []
    for w in ws:
        d = {leaf: torch.from_numpy(a).cuda() for leaf, a in w.data.items()}
        keep.extend(d.values())
        dev.append(d)
    L = len(ws[0].leaves)
    units = sum(w.nvox for w in ws) * L * ws[0].iterations
    batch = HMFBatchSolver([w.dims for w in ws], ws[0].parent)
    for i, w in enumerate(ws):
        for leaf, t in dev[i].items():
            batch.set_data(i, leaf, t)
    for v, a in ws[0].alpha.items():
        batch.set_smoothness_scalar(v, a)
    batch.set_params(ws[0].iterations, ws[0].step, ws[0].cc)
    batch.autotune(device_stream)
    singles = []
    for i, w in enumerate(ws):
        s = HMFSolver(w.dims, w.parent)
        for leaf, t in dev[i].items():
            s.set_data(leaf, t)
        for v, a in w.alpha.items():
            s.set_smoothness_scalar(v, a)
        s.set_params(w.iterations, w.step, w.cc)
        singles.append(s)

    def timed(fn, reps):
        fn()
        device_stream.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(device_stream)
        for _ in range(reps):
            fn()
        e1.record(device_stream)
        device_stream.synchronize()
        return e0.elapsed_time(e1) / reps

    t_batch = timed(lambda: batch.solve(device_stream), 3)
    t_seq = timed(lambda: [s.solve(device_stream) for s in singles], 3)
    launches = batch.stats()["launches"]
    plan = {"flow_window": batch.flow_window, "zchunk": batch.zchunk(), "pipeline": batch.pipeline}
    # What one persistent launch could save over the replayed graph of two
    # launches per iteration: the time that replay spends outside the kernels
    # (launch gaps), from the kernels' own event times in a solve launched one
    # by one.  (The default replay, pipelined over volume groups, overlaps
    # kernels and is faster than their sum.)
    batch.set_pipeline(False)
    t_two = timed(lambda: batch.solve(device_stream), 2)
    batch.set_timing(True)
    batch.solve(device_stream)
    st = batch.stats()
    batch.set_timing(False)
    batch.set_pipeline(True)
    iters = ws[0].iterations
    kernel_ms = iters * (st["flow_ms"] + st["tree_ms"]) + st["init_ms"]
    for s in singles:
        s.close()
    batch.close()
    return {"workload": "%d volumes, axes U{48..192}, flat 3 leaves, alpha 0.15, %d iterations"
                        % (len(ws), ws[0].iterations),
            "voxels": sum(w.nvox for w in ws),
            "value": units / (t_batch / 1000.0), "sequential_value": units / (t_seq / 1000.0), "unit": UNIT,
            "ms_batched": t_batch, "ms_sequential": t_seq, "speedup_vs_sequential": t_seq / t_batch,
            "repetitions": 3,
            "launches_per_batched_solve": launches,
            "ms_two_launches_per_iteration": t_two,
            "kernel_ms_per_batched_solve": kernel_ms,
            "outside_kernels_frac": max(0.0, 1.0 - kernel_ms / t_two),
            **plan}


def bench_adjoint(args, device_stream):
    """128^3, 4 ellipsoids, sigma 0.1, flat 4 leaves, alpha 0.1, 300
    iterations; loss = voxelwise cross-entropy of the final labels against the
    phantom's classes.  Times the forward solve alone and the forward +
    adjoint (hmf_solve_adjoint) with checkpoints every 30 iterations and with
    every state kept (automatic plan), inputs resident on the device."""
    import torch

    from robartsvtk_gb300 import HMFSolver, synthetic

    w = synthetic.ellipsoids_flat4(seed=3, size=args.adjoint_size, iterations=args.adjoint_iterations)
    d = {leaf: torch.from_numpy(a).cuda() for leaf, a in w.data.items()}
    truth = torch.from_numpy(w.truth.astype("int32")).cuda()
    s = HMFSolver(w.dims, w.parent)
    for leaf, t in d.items():
        s.set_data(leaf, t)
    for v, a in w.alpha.items():
        s.set_smoothness_scalar(v, a)
    s.set_params(w.iterations, w.step, w.cc)

    def timed(fn, reps):
        fn()
        device_stream.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(device_stream)
        for _ in range(reps):
            fn()
        e1.record(device_stream)
        device_stream.synchronize()
        return e0.elapsed_time(e1) / reps

    t_fwd = timed(lambda: s.solve(device_stream), 3)
    res = {}
    for k in (30, 0):
        loss = [0.0]

        def run():
            loss[0] = s.solve_adjoint(truth, checkpoint_every=k, stream=device_stream)

        t = timed(run, 2)
        plan = s.adjoint_plan()
        res["every_state_kept" if k == 0 else "checkpoint_every_%d" % k] = {
            "ms": t, "ratio_to_forward": t / t_fwd, "checkpoint_every": plan["checkpoint_every"],
            "recomputed_segments": plan["recomputed_segments"], "loss": loss[0],
            "launches": s.stats()["launches"]}
    ga = s.alpha_gradient()
    out = {"workload": "ellipsoids%d_flat4, %d iterations, loss = cross-entropy of final labels"
                       % (args.adjoint_size, w.iterations),
           "forward_ms": t_fwd, "device_bytes": s.device_bytes(),
           "dalpha": [float(x) for x in ga[1:]], **res}
    s.close()
    return out


def run_profile(args):
    """Two solves of the benchmark workload with device-resident inputs;
    launches per solve: 1 init_kernel + iterations x (flow_kernel, tree_kernel)."""
    import numpy as np
    import torch

    from robartsvtk_gb300 import HMFSolver

    w = make_workload(args, 0)
    nz = args.profile_planes
    if 0 < nz < w.dims[2]:  # the first nz planes ([z, y, x] arrays)
        w.dims = (w.dims[0], w.dims[1], nz)
        w.data = {leaf: np.ascontiguousarray(d[:nz]) for leaf, d in w.data.items()}
        cut = {}
        w.smooth = {v: cut.setdefault(id(S), np.ascontiguousarray(S[:nz])) for v, S in w.smooth.items()}
    solver = HMFSolver(w.dims, w.parent)
    keep = {}
    for leaf, d in w.data.items():
        keep[("d", leaf)] = torch.from_numpy(d).cuda()
        solver.set_data(leaf, keep[("d", leaf)])
    for v, S in w.smooth.items():
        if ("s", id(S)) not in keep:
            keep[("s", id(S))] = torch.from_numpy(S).cuda()
        solver.set_smoothness(v, keep[("s", id(S))])
    for v, a in w.alpha.items():
        solver.set_smoothness_scalar(v, a)
    solver.set_params(w.iterations, w.step, w.cc)
    for _ in range(2):
        solver.solve()
        torch.cuda.synchronize()
    print(json.dumps({"profile": WORKLOAD, "volume": list(w.dims), "iterations": w.iterations,
                      "launches_per_solve": solver.stats()["launches"]}))
    solver.close()
    return 0


def run_profile_post(args):
    """One solve of the benchmark workload (--size, --iterations), then two
    votes into a device buffer and two energy decompositions of its labels."""
    import torch

    from robartsvtk_gb300 import HMFSolver

    w = make_workload(args, 0)
    solver = HMFSolver(w.dims, w.parent)
    keep = {}
    for leaf, d in w.data.items():
        keep[("d", leaf)] = torch.from_numpy(d).cuda()
        solver.set_data(leaf, keep[("d", leaf)])
    for v, S in w.smooth.items():
        if ("s", id(S)) not in keep:
            keep[("s", id(S))] = torch.from_numpy(S).cuda()
        solver.set_smoothness(v, keep[("s", id(S))])
    for v, a in w.alpha.items():
        solver.set_smoothness_scalar(v, a)
    solver.set_params(w.iterations, w.step, w.cc)
    solver.solve()
    out = torch.empty(w.dims[::-1], dtype=torch.int32, device="cuda")
    for _ in range(2):
        solver.vote(out=out)
    torch.cuda.synchronize()
    energies = [solver.energy() for _ in range(2)]
    print(json.dumps({"profile_post": WORKLOAD, "volume": list(w.dims), "iterations": w.iterations,
                      "f0": energies[-1][0]}))
    solver.close()
    return 0


def main():
    args = parse()
    if args.profile:
        return run_profile(args)
    if args.profile_post:
        return run_profile_post(args)
    if args.profile_dataterm:
        return run_profile_dataterm(args)
    if args.profile_dag:
        return run_profile_dag(args)
    if args.profile_adjoint:
        return run_profile_adjoint(args)
    if args.large:
        return run_large(args)
    if args.profile_large:
        return run_profile_large(args)
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
