"""Python side of the HMF drop-in.

`HMFSolver` owns one C-ABI context (include/hmf.h).  `HierarchicalMaxFlowSegmentation`
mirrors the filter surface of vtkHierarchicalMaxFlowSegmentation /
vtkCudaHierarchicalMaxFlowSegmentation
(Common/vtkRobartsCommon/vtkHierarchicalMaxFlowSegmentation.h:43-204) with
numpy arrays (host) or CUDA torch tensors (device) in place of vtkImageData
and a parent array in place of vtkTree.  Arrays are indexed [z, y, x], x
fastest, which is VTK's scalar layout.
"""
from __future__ import annotations

import ctypes
import sys

import numpy as np

from . import _capi
from ._capi import HMF_DEVICE, HMF_HOST, HMF_SEMANTICS_REF_CPU, HMF_SEMANTICS_REF_CUDA, HMFError, check

__all__ = ["HMFSolver", "HMFBatchSolver", "HierarchicalMaxFlowSegmentation", "REF_CUDA", "REF_CPU", "HMFError",
           "vote", "decomposition_energy", "DAGSolver", "DirectedAcyclicGraphMaxFlowSegmentation"]

REF_CUDA = HMF_SEMANTICS_REF_CUDA
REF_CPU = HMF_SEMANTICS_REF_CPU


def _stream_handle(stream) -> int | None:
    if stream is None:
        return None
    if isinstance(stream, int):
        return stream
    handle = getattr(stream, "cuda_stream", None)
    if handle is None:
        raise TypeError("stream must be None, an int cudaStream_t or a torch.cuda.Stream")
    return int(handle)


def _array_pointer(arr, nvox: int):
    """(pointer, where, keepalive) of a float32 contiguous volume."""
    if isinstance(arr, np.ndarray):
        if arr.dtype != np.float32 or not arr.flags["C_CONTIGUOUS"]:
            raise TypeError("numpy volumes must be C-contiguous float32")
        if arr.size != nvox:
            raise ValueError("volume has %d voxels, expected %d" % (arr.size, nvox))
        return arr.ctypes.data, HMF_HOST, arr
    mod = type(arr).__module__
    if mod.startswith("torch"):
        import torch

        if arr.dtype != torch.float32 or not arr.is_contiguous():
            raise TypeError("torch volumes must be contiguous float32")
        if arr.numel() != nvox:
            raise ValueError("volume has %d voxels, expected %d" % (arr.numel(), nvox))
        where = HMF_DEVICE if arr.is_cuda else HMF_HOST
        return arr.data_ptr(), where, arr
    raise TypeError("volumes must be numpy arrays or torch tensors")


def _truth_pointer(truth, nvox: int):
    """(pointer, where, keepalive) of an int32 class map (numpy or torch)."""
    if isinstance(truth, np.ndarray):
        if truth.dtype != np.int32 or not truth.flags["C_CONTIGUOUS"] or truth.size != nvox:
            raise TypeError("truth must be a C-contiguous int32 array of the volume's size")
        return truth.ctypes.data, HMF_HOST, truth
    import torch

    if truth.dtype != torch.int32 or not truth.is_contiguous() or truth.numel() != nvox:
        raise TypeError("truth must be a contiguous int32 tensor of the volume's size")
    return truth.data_ptr(), HMF_DEVICE if truth.is_cuda else HMF_HOST, truth


class HMFSolver:
    """One solver context: a volume size (vx, vy, vz), a label tree given as a
    parent array, and a semantics (REF_CUDA or REF_CPU)."""

    def __init__(self, dims, parent, semantics: int = REF_CUDA, device: int = 0, max_gpu_usage=None):
        """max_gpu_usage: None solves in core; a fraction of the device's
        memory (the reference's MaxGPUUsage) makes an out-of-core context
        (hmf_create_paged) whose state lives in pinned host memory."""
        self._lib = _capi.load()
        self.dims = tuple(int(d) for d in dims)
        self.parent = [int(p) for p in parent]
        self.nvox = self.dims[0] * self.dims[1] * self.dims[2]
        par = (ctypes.c_int * len(self.parent))(*self.parent)
        ctx = ctypes.c_void_p()
        self.max_gpu_usage = max_gpu_usage
        if max_gpu_usage is None:
            check(self._lib.hmf_create(ctypes.byref(ctx), *self.dims, par, len(self.parent), int(semantics),
                                       int(device)))
        else:
            check(self._lib.hmf_create_paged(ctypes.byref(ctx), *self.dims, par, len(self.parent), int(semantics),
                                             int(device), float(max_gpu_usage)))
        self._ctx = ctx
        self._keep: dict = {}
        n = self._lib.hmf_leaf_order(self._ctx, None, 0)
        buf = (ctypes.c_int * max(n, 1))()
        self._lib.hmf_leaf_order(self._ctx, buf, n)
        self.leaves = [buf[i] for i in range(n)]

    # -- inputs ---------------------------------------------------------
    def set_data(self, node: int, arr) -> None:
        ptr, where, keep = _array_pointer(arr, self.nvox)
        check(self._lib.hmf_set_data(self._ctx, int(node), ptr, where), self._ctx)
        self._keep[("d", node)] = keep

    def set_data_pointer(self, node: int, ptr: int, where: int) -> None:
        check(self._lib.hmf_set_data(self._ctx, int(node), int(ptr), int(where)), self._ctx)

    def set_smoothness(self, node: int, arr) -> None:
        if arr is None:
            check(self._lib.hmf_set_smoothness(self._ctx, int(node), None, HMF_HOST), self._ctx)
            self._keep.pop(("s", node), None)
            return
        ptr, where, keep = _array_pointer(arr, self.nvox)
        check(self._lib.hmf_set_smoothness(self._ctx, int(node), ptr, where), self._ctx)
        self._keep[("s", node)] = keep

    def set_smoothness_scalar(self, node: int, alpha: float) -> None:
        check(self._lib.hmf_set_smoothness_scalar(self._ctx, int(node), float(alpha)), self._ctx)

    def set_params(self, iterations: int = 100, step: float = 0.1, cc: float = 0.25) -> None:
        check(self._lib.hmf_set_params(self._ctx, int(iterations), float(step), float(cc)), self._ctx)

    def set_timing(self, enabled: bool) -> None:
        check(self._lib.hmf_set_timing(self._ctx, 1 if enabled else 0), self._ctx)

    def set_zchunk(self, z: int) -> None:
        """Planes each flow-kernel CTA marches (0: the default plan)."""
        check(self._lib.hmf_set_zchunk(self._ctx, int(z)), self._ctx)

    def zchunk(self) -> int:
        return int(self._lib.hmf_get_zchunk(self._ctx))

    def set_pipeline(self, enabled: bool) -> None:
        """Per-slab graph nodes so that sweeps overlap flows (same results)."""
        check(self._lib.hmf_set_pipeline(self._ctx, 1 if enabled else 0), self._ctx)

    @property
    def pipeline(self) -> bool:
        return check(self._lib.hmf_get_pipeline(self._ctx), self._ctx) == 1

    def set_flow_window(self, rows: int) -> None:
        """Flow-kernel window rows: 32 or 64 (0: default)."""
        check(self._lib.hmf_set_flow_window(self._ctx, int(rows)), self._ctx)

    @property
    def flow_window(self) -> int:
        return check(self._lib.hmf_get_flow_window(self._ctx), self._ctx)

    def set_flow_units(self, units: int) -> None:
        """Window-vertex marches per flow-kernel CTA, 1..64 (0: 1)."""
        check(self._lib.hmf_set_flow_units(self._ctx, int(units)), self._ctx)

    @property
    def flow_units(self) -> int:
        return check(self._lib.hmf_get_flow_units(self._ctx), self._ctx)

    def autotune(self, stream=None) -> None:
        """Time the flow kernel for each candidate z chunk on the current
        inputs and keep the fastest (hmf_autotune)."""
        check(self._lib.hmf_autotune(self._ctx, _stream_handle(stream)), self._ctx)

    # -- run ------------------------------------------------------------
    def solve(self, stream=None) -> None:
        check(self._lib.hmf_solve(self._ctx, _stream_handle(stream)), self._ctx)

    def solve_continue(self, stream=None) -> None:
        """`iterations` more iterations from the state the last solve ended in,
        without re-initialising (hmf_solve_continue): solve(k1) then
        solve_continue(k2) equals solve(k1 + k2) bit for bit."""
        check(self._lib.hmf_solve_continue(self._ctx, _stream_handle(stream)), self._ctx)

    def _fetch(self, fn, node, out, stream):
        if out is None:
            out = np.empty((self.dims[2], self.dims[1], self.dims[0]), dtype=np.float32)
        ptr, where, _ = _array_pointer(out, self.nvox)
        check(fn(self._ctx, int(node), ptr, where, _stream_handle(stream)), self._ctx)
        return out

    def labels(self, node: int, out=None, stream=None):
        """Labelling of a non-root vertex into `out` (numpy / torch), or a new
        numpy array [VZ, VY, VX]."""
        return self._fetch(self._lib.hmf_get_labels, node, out, stream)

    def sink(self, node: int, out=None, stream=None):
        return self._fetch(self._lib.hmf_get_sink, node, out, stream)

    # -- vote and energy --------------------------------------------------
    def vote(self, out=None, stream=None):
        """Label per voxel: the leaf (vertex id) with the largest final label,
        ties as the context's semantics (REF_CUDA: last leaf, REF_CPU: first).
        int32 [VZ, VY, VX] numpy array, or into `out` (numpy or torch int32)."""
        return _fetch_vote(lambda ptr, where, s: self._lib.hmf_get_vote(self._ctx, ptr, where, s),
                           self.dims, out, stream, self._ctx)

    def energy(self):
        """Energy decomposition of the final labels: (f0, f) with f per vertex id."""
        return _fetch_energy(lambda f0, f, n: self._lib.hmf_get_energy(self._ctx, f0, f, n), len(self.parent),
                             self._ctx)

    # -- convergence log ----------------------------------------------------
    def set_convergence_log(self, enabled: bool) -> None:
        """Per-iteration max / mean |u_new - u_old| reduced inside the sweep."""
        check(self._lib.hmf_set_convergence_log(self._ctx, 1 if enabled else 0), self._ctx)

    def convergence(self) -> dict:
        """{"max": [...], "mean": [...]} per iteration of the last solve."""
        n = check(self._lib.hmf_get_convergence(self._ctx, None, None, 0), self._ctx)
        mx = (ctypes.c_double * max(n, 1))()
        mean = (ctypes.c_double * max(n, 1))()
        check(self._lib.hmf_get_convergence(self._ctx, mx, mean, n), self._ctx)
        return {"max": np.array(mx[:n]), "mean": np.array(mean[:n])}

    # -- bounded copy waits --------------------------------------------------
    def set_wait_limit(self, limit_ns: int = 0) -> None:
        """Bound (ns) of the flow kernels' copy waits (0: the default 0.5 s)."""
        check(self._lib.hmf_set_wait_limit(self._ctx, int(limit_ns)), self._ctx)

    def inject_wait_stall(self, kernel: int) -> None:
        """Make one CTA of the next launch of `kernel` (HMF_STALL_*) wait on a
        barrier nothing completes, so its bounded wait runs out (-1 cancels)."""
        check(self._lib.hmf_inject_wait_stall(self._ctx, int(kernel)), self._ctx)

    # -- reference precision (FP64) ----------------------------------------
    def solve_fp64(self, stream=None) -> None:
        """The same REF_CUDA iteration in FP64 on the GPU (hmf_solve_fp64)."""
        check(self._lib.hmf_solve_fp64(self._ctx, _stream_handle(stream)), self._ctx)

    def labels_fp64(self, node: int, stream=None) -> np.ndarray:
        """FP64 labelling of a non-root vertex, float64 [VZ, VY, VX]."""
        out = np.empty((self.dims[2], self.dims[1], self.dims[0]), dtype=np.float64)
        check(self._lib.hmf_get_labels_fp64(self._ctx, int(node), out.ctypes.data, HMF_HOST,
                                            _stream_handle(stream)), self._ctx)
        return out

    def fp64_error(self, stream=None) -> dict:
        """max |u_fp32 - u_fp64| over leaves and voxels between the last solve
        and the last solve_fp64, and the fraction of voxels whose argmax leaf
        agrees."""
        mx = ctypes.c_double()
        agree = ctypes.c_double()
        check(self._lib.hmf_fp64_error(self._ctx, ctypes.byref(mx), ctypes.byref(agree), _stream_handle(stream)),
              self._ctx)
        return {"max_abs_err": mx.value, "argmax_agreement": agree.value}

    def fp64_loss(self, truth, eps: float = 1e-6, stream=None) -> float:
        """The adjoint's cross-entropy loss on the FP64 labels."""
        ptr, where, keep = _truth_pointer(truth, self.nvox)
        loss = ctypes.c_double()
        check(self._lib.hmf_fp64_loss(self._ctx, ptr, where, float(eps), ctypes.byref(loss),
                                      _stream_handle(stream)), self._ctx)
        del keep
        return loss.value

    def set_fp64_probe(self, kind: int = _capi.HMF_FP64_PROBE_NONE, node: int = 0, voxel: int = 0,
                       value: float = 0.0) -> None:
        """Inputs of later FP64 solves that differ from the FP32 inputs (for
        finite differences): a leaf's data term at one dense voxel index, or a
        vertex's alpha, as a double; kind NONE clears them."""
        check(self._lib.hmf_set_fp64_probe(self._ctx, int(kind), int(node), int(voxel), float(value)), self._ctx)

    # -- adjoint ----------------------------------------------------------
    def solve_adjoint(self, truth, checkpoint_every: int = 0, eps: float = 1e-6, stream=None) -> float:
        """Solve, then differentiate L = -(1/V) sum log(max(u_truth, eps)) of
        the final leaf labels.  truth: int32 [VZ, VY, VX] indices into
        `self.leaves` (numpy, or a torch tensor on the host or the device).
        Returns L; gradients via data_gradient() / alpha_gradient()."""
        ptr, where, keep = _truth_pointer(truth, self.nvox)
        loss = ctypes.c_double()
        check(self._lib.hmf_solve_adjoint(self._ctx, ptr, where, int(checkpoint_every), float(eps),
                                          ctypes.byref(loss), _stream_handle(stream)), self._ctx)
        del keep
        return loss.value

    def data_gradient(self, leaf: int, out=None, stream=None):
        """dL/dD of a leaf's data term, float64 [VZ, VY, VX] (numpy, or a
        float64 torch tensor given as `out`)."""
        if out is None:
            out = np.empty((self.dims[2], self.dims[1], self.dims[0]), dtype=np.float64)
            ptr, where = out.ctypes.data, HMF_HOST
        elif isinstance(out, np.ndarray):
            if out.dtype != np.float64 or not out.flags["C_CONTIGUOUS"] or out.size != self.nvox:
                raise TypeError("out must be a C-contiguous float64 array of the volume's size")
            ptr, where = out.ctypes.data, HMF_HOST
        else:
            import torch

            if out.dtype != torch.float64 or not out.is_contiguous() or out.numel() != self.nvox:
                raise TypeError("out must be a contiguous float64 tensor of the volume's size")
            ptr, where = out.data_ptr(), HMF_DEVICE if out.is_cuda else HMF_HOST
        check(self._lib.hmf_get_data_gradient(self._ctx, int(leaf), ptr, where, _stream_handle(stream)), self._ctx)
        return out

    def alpha_gradient(self) -> np.ndarray:
        """dL/dalpha per vertex id (the root reads 0)."""
        buf = (ctypes.c_double * len(self.parent))()
        rc = self._lib.hmf_get_alpha_gradient(self._ctx, buf, len(self.parent))
        check(min(rc, 0), self._ctx)
        return np.array(buf[:], dtype=np.float64)

    def adjoint_plan(self) -> dict:
        """The schedule of the last solve_adjoint: checkpoint interval (0 for
        the fewest-forward-iterations schedule), recomputed segments, state
        slots, forward iterations run (first pass included) and backward
        steps."""
        k = ctypes.c_int()
        r = ctypes.c_int()
        check(self._lib.hmf_get_adjoint_plan(self._ctx, ctypes.byref(k), ctypes.byref(r)), self._ctx)
        slots = ctypes.c_int()
        fwd = ctypes.c_longlong()
        bwd = ctypes.c_longlong()
        check(self._lib.hmf_get_adjoint_schedule(self._ctx, ctypes.byref(slots), ctypes.byref(fwd),
                                                 ctypes.byref(bwd)), self._ctx)
        return {"checkpoint_every": k.value, "recomputed_segments": r.value, "state_slots": slots.value,
                "forward_iterations": fwd.value, "backward_steps": bwd.value}

    def set_adjoint_memory(self, max_bytes: int = 0, max_state_slots: int = 0) -> None:
        """Budget of later automatic (checkpoint_every=0) adjoint plans: device
        bytes for the adjoint's arrays (0: 85% of the free memory) and a cap on
        state slots (0: none)."""
        check(self._lib.hmf_set_adjoint_memory(self._ctx, int(max_bytes), int(max_state_slots)), self._ctx)

    def stats(self):
        launches = ctypes.c_longlong()
        ms = (ctypes.c_double * 3)()
        check(self._lib.hmf_get_stats(self._ctx, ctypes.byref(launches), ms, 3), self._ctx)
        return {"launches": launches.value, "flow_ms": ms[0], "tree_ms": ms[1], "init_ms": ms[2]}

    def device_bytes(self) -> int:
        return int(self._lib.hmf_device_bytes(self._ctx))

    def set_paged_plan(self, block_planes: int = 0, round_iterations: int = 0, inputs: str = "auto") -> None:
        """Out-of-core contexts: planes per block and iterations per round of
        later solves (0: from the budget), and where host inputs are read from
        ("auto", "host": over the link every round, "device": copied to the
        device once per solve)."""
        mode = {"auto": _capi.HMF_PAGED_INPUTS_AUTO, "host": _capi.HMF_PAGED_INPUTS_HOST,
                "device": _capi.HMF_PAGED_INPUTS_DEVICE}[inputs]
        check(self._lib.hmf_set_paged_plan(self._ctx, int(block_planes), int(round_iterations), mode), self._ctx)

    def paged_plan(self) -> dict:
        """Out-of-core contexts: the plan of the last solve and the bytes it
        moved between host and device."""
        vals = [ctypes.c_int() for _ in range(4)]
        link = ctypes.c_longlong()
        check(self._lib.hmf_get_paged_plan(self._ctx, *[ctypes.byref(v) for v in vals], ctypes.byref(link)),
              self._ctx)
        return {"blocks": vals[0].value, "block_planes": vals[1].value, "round_iterations": vals[2].value,
                "rounds": vals[3].value, "link_bytes": link.value}

    def close(self) -> None:
        if getattr(self, "_ctx", None):
            self._lib.hmf_destroy(self._ctx)
            self._ctx = None
            self._keep.clear()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


class HMFBatchSolver:
    """Many volumes of different sizes sharing one label tree, solved together
    (include/hmf.h, hmf_create_batch).  `dims` is a list of (VX, VY, VZ)."""

    def __init__(self, dims, parent, semantics: int = REF_CUDA, device: int = 0):
        self._lib = _capi.load()
        self.dims = [tuple(int(d) for d in dd) for dd in dims]
        self.parent = [int(p) for p in parent]
        flat = (ctypes.c_int * (3 * len(self.dims)))(*[d for dd in self.dims for d in dd])
        par = (ctypes.c_int * len(self.parent))(*self.parent)
        ctx = ctypes.c_void_p()
        check(self._lib.hmf_create_batch(ctypes.byref(ctx), len(self.dims), flat, par, len(self.parent),
                                         int(semantics), int(device)))
        self._ctx = ctx
        self._keep: dict = {}
        n = self._lib.hmf_leaf_order(self._ctx, None, 0)
        buf = (ctypes.c_int * max(n, 1))()
        self._lib.hmf_leaf_order(self._ctx, buf, n)
        self.leaves = [buf[i] for i in range(n)]

    def _nvox(self, b):
        d = self.dims[b]
        return d[0] * d[1] * d[2]

    def set_data(self, volume: int, node: int, arr) -> None:
        ptr, where, keep = _array_pointer(arr, self._nvox(volume))
        check(self._lib.hmf_batch_set_data(self._ctx, int(volume), int(node), ptr, where), self._ctx)
        self._keep[("d", volume, node)] = keep

    def set_smoothness(self, volume: int, node: int, arr) -> None:
        if arr is None:
            check(self._lib.hmf_batch_set_smoothness(self._ctx, int(volume), int(node), None, HMF_HOST), self._ctx)
            self._keep.pop(("s", volume, node), None)
            return
        ptr, where, keep = _array_pointer(arr, self._nvox(volume))
        check(self._lib.hmf_batch_set_smoothness(self._ctx, int(volume), int(node), ptr, where), self._ctx)
        self._keep[("s", volume, node)] = keep

    def set_smoothness_scalar(self, node: int, alpha: float) -> None:
        check(self._lib.hmf_set_smoothness_scalar(self._ctx, int(node), float(alpha)), self._ctx)

    def set_params(self, iterations: int = 100, step: float = 0.1, cc: float = 0.25) -> None:
        check(self._lib.hmf_set_params(self._ctx, int(iterations), float(step), float(cc)), self._ctx)

    def set_timing(self, enabled: bool) -> None:
        check(self._lib.hmf_set_timing(self._ctx, 1 if enabled else 0), self._ctx)

    def set_flow_units(self, units: int) -> None:
        """Window-vertex marches per flow-kernel CTA, 1..64 (0: 1)."""
        check(self._lib.hmf_set_flow_units(self._ctx, int(units)), self._ctx)

    def autotune(self, stream=None) -> None:
        check(self._lib.hmf_autotune(self._ctx, _stream_handle(stream)), self._ctx)

    def solve(self, stream=None) -> None:
        check(self._lib.hmf_solve(self._ctx, _stream_handle(stream)), self._ctx)

    solve_continue = HMFSolver.solve_continue

    # the flow plan's controls, shared with HMFSolver
    set_pipeline = HMFSolver.set_pipeline
    pipeline = HMFSolver.pipeline
    set_flow_window = HMFSolver.set_flow_window
    flow_window = HMFSolver.flow_window
    set_zchunk = HMFSolver.set_zchunk
    zchunk = HMFSolver.zchunk

    def set_convergence_log(self, enabled: bool) -> None:
        """Per-iteration max / mean |u_new - u_old| over all volumes."""
        HMFSolver.set_convergence_log(self, enabled)

    def convergence(self) -> dict:
        return HMFSolver.convergence(self)

    def labels(self, volume: int, node: int, out=None, stream=None):
        if out is None:
            d = self.dims[volume]
            out = np.empty((d[2], d[1], d[0]), dtype=np.float32)
        ptr, where, _ = _array_pointer(out, self._nvox(volume))
        check(self._lib.hmf_batch_get_labels(self._ctx, int(volume), int(node), ptr, where,
                                             _stream_handle(stream)), self._ctx)
        return out

    def sink(self, volume: int, node: int, out=None, stream=None):
        if out is None:
            d = self.dims[volume]
            out = np.empty((d[2], d[1], d[0]), dtype=np.float32)
        ptr, where, _ = _array_pointer(out, self._nvox(volume))
        check(self._lib.hmf_batch_get_sink(self._ctx, int(volume), int(node), ptr, where,
                                           _stream_handle(stream)), self._ctx)
        return out

    def vote(self, volume: int, out=None, stream=None):
        """Label per voxel of one volume (see HMFSolver.vote)."""
        b = int(volume)
        return _fetch_vote(lambda ptr, where, s: self._lib.hmf_batch_get_vote(self._ctx, b, ptr, where, s),
                           self.dims[b], out, stream, self._ctx)

    def energy(self, volume: int):
        """Energy decomposition of one volume's final labels: (f0, f)."""
        b = int(volume)
        return _fetch_energy(lambda f0, f, n: self._lib.hmf_batch_get_energy(self._ctx, b, f0, f, n),
                             len(self.parent), self._ctx)

    def stats(self):
        launches = ctypes.c_longlong()
        ms = (ctypes.c_double * 3)()
        check(self._lib.hmf_get_stats(self._ctx, ctypes.byref(launches), ms, 3), self._ctx)
        return {"launches": launches.value, "flow_ms": ms[0], "tree_ms": ms[1], "init_ms": ms[2]}

    def device_bytes(self) -> int:
        return int(self._lib.hmf_device_bytes(self._ctx))

    def close(self) -> None:
        if getattr(self, "_ctx", None):
            self._lib.hmf_destroy(self._ctx)
            self._ctx = None
            self._keep.clear()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def _fetch_vote(call, dims, out, stream, ctx):
    nvox = dims[0] * dims[1] * dims[2]
    if out is None:
        out = np.empty((dims[2], dims[1], dims[0]), dtype=np.int32)
    if isinstance(out, np.ndarray):
        if out.dtype != np.int32 or not out.flags["C_CONTIGUOUS"] or out.size != nvox:
            raise TypeError("out must be a C-contiguous int32 array of the volume's size")
        ptr, where = out.ctypes.data, HMF_HOST
    else:
        import torch

        if out.dtype != torch.int32 or not out.is_contiguous() or out.numel() != nvox:
            raise TypeError("out must be a contiguous int32 tensor of the volume's size")
        ptr, where = out.data_ptr(), HMF_DEVICE if out.is_cuda else HMF_HOST
    check(call(ptr, where, _stream_handle(stream)), ctx)
    return out


def _fetch_energy(call, n, ctx):
    f0 = ctypes.c_double()
    f = (ctypes.c_double * n)()
    check(call(ctypes.byref(f0), f, n), ctx)
    return f0.value, np.array(f[:], dtype=np.float64)



def adjoint_schedule(iterations: int, state_slots: int = 0, checkpoint_every: int = 0):
    """The adjoint's schedule as a list of (kind, t, a, b) actions (host
    only): kind 0 = forward iteration t from slot a to slot b, 1 = loss on
    x_T in slot a, 2 = backward step of iteration t with x_t in slot a and
    x_{t+1} in slot b.  checkpoint_every > 0: fixed interval; 0: fewest
    forward iterations over `state_slots` slots.  None when infeasible."""
    lib = _capi.load()
    n = lib.hmf_adjoint_schedule(int(iterations), int(state_slots), int(checkpoint_every), None, 0)
    if n < 0:
        return None
    buf = (ctypes.c_int * (4 * n))()
    lib.hmf_adjoint_schedule(int(iterations), int(state_slots), int(checkpoint_every), buf, n)
    return [tuple(buf[4 * i:4 * i + 4]) for i in range(n)]

def vote(inputs, values=None, semantics: int = REF_CUDA, out=None, stream=None):
    """Label vote over equally sized float32 images (numpy on the host or
    torch tensors on the device): out[i] = values[k] of the input with the
    largest value (values default: 0..n-1).  Replaces vtkCudaImageVote
    (REF_CUDA ties: last wins) / vtkImageVote (REF_CPU: first wins)."""
    lib = _capi.load()
    n = len(inputs)
    if n == 0:  # the library reports the error
        check(lib.hmf_vote(0, None, None, 0, int(semantics), None, HMF_HOST, None))
    nvox = int(np.prod(inputs[0].shape))
    keep = []
    ptrs = (ctypes.c_void_p * n)()
    where = None
    for k, a in enumerate(inputs):
        p, w, kp = _array_pointer(a, nvox)
        if where is None:
            where = w
        elif w != where:
            raise ValueError("vote inputs must all be on the host or all on the device")
        ptrs[k] = p
        keep.append(kp)
    vals = np.ascontiguousarray(values if values is not None else np.arange(n), dtype=np.int32)
    if out is None:
        if where == HMF_DEVICE:
            import torch

            out = torch.empty(tuple(inputs[0].shape), dtype=torch.int32, device=inputs[0].device)
        else:
            out = np.empty(tuple(inputs[0].shape), dtype=np.int32)
    optr = out.data_ptr() if where == HMF_DEVICE else out.ctypes.data
    check(lib.hmf_vote(n, ptrs, vals.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), nvox, int(semantics), optr,
                       where, _stream_handle(stream)))
    return out


def decomposition_energy(dims, parent, data, labels, smooth=None, stream=None):
    """Energy decomposition of leaf labellings (dicts by vertex id; numpy on
    the host or CUDA tensors): (f0, f per vertex id).  Replaces
    vtkCudaHierarchicalMaxFlowDecomposition's GetF0 / GetF."""
    lib = _capi.load()
    dims = tuple(int(d) for d in dims)
    nvox = dims[0] * dims[1] * dims[2]
    n = len(parent)
    par = (ctypes.c_int * n)(*[int(p) for p in parent])
    keep = []
    arrays = {}
    where = None
    for name, src in (("d", data), ("l", labels), ("s", smooth or {})):
        arr = (ctypes.c_void_p * n)()
        for v, a in src.items():
            p, w, kp = _array_pointer(a, nvox)
            if where is None:
                where = w
            elif w != where:
                raise ValueError("energy inputs must all be on the host or all on the device")
            arr[int(v)] = p
            keep.append(kp)
        arrays[name] = arr
    f0 = ctypes.c_double()
    f = (ctypes.c_double * n)()
    check(lib.hmf_decomposition_energy(dims[0], dims[1], dims[2], par, n, arrays["d"], arrays["l"], arrays["s"],
                                       where if where is not None else HMF_HOST, ctypes.byref(f0), f,
                                       _stream_handle(stream)))
    return f0.value, np.array(f[:], dtype=np.float64)


class DAGSolver(HMFSolver):
    """One solver context for a directed acyclic graph of labels (the problem
    of vtkCudaDirectedAcyclicGraphMaxFlowSegmentation): `n_nodes` vertices,
    `edges` = [(parent, child), ...] in edge order, optional positive
    per-edge `weights`.  Leaves are numbered in the graph's forward-iterator
    order (`leaves`).  A vertex without set_smoothness_scalar has alpha 0, as
    in the reference class.  The vote works on it; the adjoint, the energy
    decomposition and batches are for trees."""

    def __init__(self, dims, n_nodes, edges, weights=None, device: int = 0):
        self._lib = _capi.load()
        self.dims = tuple(int(d) for d in dims)
        self.nvox = self.dims[0] * self.dims[1] * self.dims[2]
        self.edges = [(int(p), int(c)) for p, c in edges]
        self.weights = None if weights is None else [float(w) for w in weights]
        n_edges = len(self.edges)
        if self.weights is not None and len(self.weights) != n_edges:
            raise ValueError("one weight per edge")
        ep = (ctypes.c_int * max(n_edges, 1))(*[p for p, _ in self.edges])
        ec = (ctypes.c_int * max(n_edges, 1))(*[c for _, c in self.edges])
        ew = (ctypes.c_float * n_edges)(*self.weights) if self.weights is not None else None
        first_parent = [-1] * int(n_nodes)
        for p, c in reversed(self.edges):
            if 0 <= c < len(first_parent):
                first_parent[c] = p
        self.parent = first_parent
        ctx = ctypes.c_void_p()
        check(self._lib.hmf_create_dag(ctypes.byref(ctx), *self.dims, int(n_nodes), n_edges, ep, ec, ew,
                                       REF_CUDA, int(device)))
        self._ctx = ctx
        self._keep: dict = {}
        n = self._lib.hmf_leaf_order(self._ctx, None, 0)
        buf = (ctypes.c_int * max(n, 1))()
        self._lib.hmf_leaf_order(self._ctx, buf, n)
        self.leaves = [buf[i] for i in range(n)]


class HierarchicalMaxFlowSegmentation:
    """Filter-style API with the reference's method names.

    Differences from the VTK class, all forced by the absence of VTK: the tree
    is a parent array (SetStructure / SetHierarchy), images are arrays, and
    GetOutputDataObject returns an array.  Errors are reported the way
    RequestData reports them: Update() returns -1 and the message is printed
    (vtkErrorMacro) and kept in GetLastError()."""

    def __init__(self, semantics: int = REF_CUDA):
        self.Structure = None
        self.SmoothnessScalars: dict[int, float] = {}
        self.NumberOfIterations = 100
        self.CC = 0.25
        self.StepSize = 0.1
        self.Device = 0
        self.MaxGPUUsage = None
        self.Semantics = semantics
        self._data: dict[int, object] = {}
        self._smooth: dict[int, object] = {}
        self._outputs: dict[int, np.ndarray] = {}
        self._solver: HMFSolver | None = None
        self._error = ""

    # vtkSetObjectMacro(Structure, vtkTree) (.h:53-54)
    def SetStructure(self, parent):
        self.Structure = [int(p) for p in parent]

    SetHierarchy = SetStructure

    def GetStructure(self):
        return self.Structure

    # AddSmoothnessScalar (.cxx:93-104): std::map::insert keeps the first value
    def AddSmoothnessScalar(self, node: int, alpha: float):
        if alpha >= 0.0:
            self.SmoothnessScalars.setdefault(int(node), float(alpha))
        else:
            self._report("Cannot use a negative smoothness value.")

    # vtkSetClampMacro (.h:64-77)
    def SetNumberOfIterations(self, n: int):
        self.NumberOfIterations = max(0, min(int(n), 2**31 - 1))

    def GetNumberOfIterations(self) -> int:
        return self.NumberOfIterations

    def SetCC(self, cc: float):
        self.CC = min(1.0, max(0.0, float(cc)))

    def GetCC(self) -> float:
        return self.CC

    def SetStepSize(self, s: float):
        self.StepSize = min(1.0, max(0.0, float(s)))

    def GetStepSize(self) -> float:
        return self.StepSize

    def SetDevice(self, d: int):
        self.Device = int(d)

    # vtkCudaHierarchicalMaxFlowSegmentation::MaxGPUUsage (.h:52), clamped as
    # vtkCudaHierarchicalMaxFlowSegmentation2's vtkSetClampMacro (.h:74-75);
    # None (the default) solves in core, a fraction solves out of core within
    # that share of the device's memory (same results)
    def SetMaxGPUUsage(self, usage):
        self.MaxGPUUsage = None if usage is None else min(1.0, max(0.0, float(usage)))

    def GetMaxGPUUsage(self):
        return self.MaxGPUUsage

    def GetDevice(self) -> int:
        return self.Device

    def SetDataInputDataObject(self, idx: int, image):
        if image is None:
            self._data.pop(int(idx), None)
        else:
            self._data[int(idx)] = image

    def GetDataInputDataObject(self, idx: int):
        return self._data.get(int(idx))

    def SetSmoothnessInputDataObject(self, idx: int, image):
        if image is None:
            self._smooth.pop(int(idx), None)
        else:
            self._smooth[int(idx)] = image

    def GetSmoothnessInputDataObject(self, idx: int):
        return self._smooth.get(int(idx))

    def GetOutputDataObject(self, idx: int):
        return self._outputs.get(int(idx))

    def GetNumberOfOutputPorts(self) -> int:
        return len(self._solver.leaves) if self._solver else 0

    def GetLastError(self) -> str:
        return self._error

    def _report(self, msg: str) -> int:
        self._error = msg
        print("ERROR: HierarchicalMaxFlowSegmentation: " + msg, file=sys.stderr)
        return -1

    def _shape(self, image):
        return tuple(int(s) for s in image.shape)

    # RequestData (.cxx:555-933) with CheckInputConsistancy (:363-505)
    def Update(self, stream=None) -> int:
        return self._run(stream, continued=False)

    def ContinueUpdate(self, stream=None) -> int:
        """NumberOfIterations more iterations from the state the last Update
        or ContinueUpdate ended in (hmf_solve_continue; no counterpart in the
        reference), with the inputs and parameters as set now: Update with k1
        iterations then ContinueUpdate with k2 gives Update(k1 + k2)'s
        outputs.  The hierarchy, extent, semantics, device and MaxGPUUsage must
        be those of that Update."""
        return self._run(stream, continued=True)

    def _run(self, stream, continued: bool) -> int:
        self._error = ""
        if not self.Structure:
            return self._report("Hierarchy must be provided.")
        shape = None
        for image in list(self._data.values()) + list(self._smooth.values()):
            s = self._shape(image)
            if len(s) != 3:
                return self._report("Data type must be FLOAT and only have one component.")
            if shape is None:
                shape = s
            elif s != shape:
                return self._report("Inconsistant object extent.")
        if shape is None:
            return self._report("Missing data prior for leaf node.")
        dims = (shape[2], shape[1], shape[0])
        try:
            if (self._solver is None or self._solver.dims != dims or self._solver.parent != self.Structure
                    or getattr(self._solver, "_semantics", None) != self.Semantics
                    or self._solver.max_gpu_usage != self.MaxGPUUsage):
                if continued:
                    return self._report("ContinueUpdate follows an Update with the same hierarchy, extent, "
                                        "semantics, device and MaxGPUUsage.")
                if self._solver is not None:
                    self._solver.close()
                self._solver = HMFSolver(dims, self.Structure, self.Semantics, self.Device, self.MaxGPUUsage)
                self._solver._semantics = self.Semantics
            sol = self._solver
            for leaf in sol.leaves:
                if leaf not in self._data:
                    return self._report("Missing data prior for leaf node.")
                sol.set_data(leaf, self._data[leaf])
            for v, p in enumerate(self.Structure):
                if p < 0:
                    continue
                sol.set_smoothness_scalar(v, self.SmoothnessScalars.get(v, 1.0))
                sol.set_smoothness(v, self._smooth.get(v))
            sol.set_params(self.NumberOfIterations, self.StepSize, self.CC)
            if continued:
                sol.solve_continue(stream)
            else:
                sol.solve(stream)
            self._outputs = {leaf: sol.labels(leaf, stream=stream) for leaf in sol.leaves}
        except HMFError as e:
            return self._report(str(e))
        return 1


class DirectedAcyclicGraphMaxFlowSegmentation(HierarchicalMaxFlowSegmentation):
    """Filter-style API of vtkCudaDirectedAcyclicGraphMaxFlowSegmentation
    (Common/vtkRobartsCommon/vtkDirectedAcyclicGraphMaxFlowSegmentation.h:52-123)
    with the same stand-ins as HierarchicalMaxFlowSegmentation: the
    vtkRootedDirectedAcyclicGraph is given as (n_nodes, edges, weights) to
    SetStructure, images are arrays.  Vertices without AddSmoothnessScalar
    get alpha 0 (the CUDA class reads its scalar map with operator[])."""

    def __init__(self):
        super().__init__(REF_CUDA)

    def SetStructure(self, n_nodes, edges, weights=None):
        self.Structure = (int(n_nodes), [(int(p), int(c)) for p, c in edges],
                          None if weights is None else [float(w) for w in weights])

    SetHierarchy = SetStructure

    def _report(self, msg: str) -> int:
        self._error = msg
        print("ERROR: DirectedAcyclicGraphMaxFlowSegmentation: " + msg, file=sys.stderr)
        return -1

    def ContinueUpdate(self, stream=None) -> int:
        """Refused: a graph's last iteration runs fewer tasks than the others,
        so a solve cannot be continued (hmf_solve_continue refuses graphs)."""
        return self._report("ContinueUpdate is for label trees, not graphs.")

    # RequestData / CheckInputConsistancy (vtkDirectedAcyclicGraphMaxFlowSegmentation.cxx:387-527, :574-1032)
    def Update(self, stream=None) -> int:
        self._error = ""
        if not self.Structure:
            return self._report("Structure must be provided.")
        shape = None
        for image in list(self._data.values()) + list(self._smooth.values()):
            s = self._shape(image)
            if len(s) != 3:
                return self._report("Data type must be FLOAT and only have one component.")
            if shape is None:
                shape = s
            elif s != shape:
                return self._report("Inconsistant object extent.")
        if shape is None:
            return self._report("Missing data prior for leaf node.")
        dims = (shape[2], shape[1], shape[0])
        n_nodes, edges, weights = self.Structure
        try:
            key = (dims, n_nodes, tuple(edges), None if weights is None else tuple(weights))
            if self._solver is None or getattr(self._solver, "_key", None) != key:
                if self._solver is not None:
                    self._solver.close()
                self._solver = DAGSolver(dims, n_nodes, edges, weights, self.Device)
                self._solver._key = key
            sol = self._solver
            for leaf in sol.leaves:
                if leaf not in self._data:
                    return self._report("Missing data prior for leaf node.")
                sol.set_data(leaf, self._data[leaf])
            for v in range(n_nodes):
                if sol.parent[v] < 0:
                    continue
                sol.set_smoothness_scalar(v, self.SmoothnessScalars.get(v, 0.0))
                sol.set_smoothness(v, self._smooth.get(v))
            sol.set_params(self.NumberOfIterations, self.StepSize, self.CC)
            sol.solve(stream)
            self._outputs = {leaf: sol.labels(leaf, stream=stream) for leaf in sol.leaves}
        except HMFError as e:
            return self._report(str(e))
        return 1
