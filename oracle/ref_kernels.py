"""Runs the reference's own HMF CUDA kernels -- TEST INFRASTRUCTURE ONLY.

oracle/build_oracle.py compiles ImageProcessing/vtkCudaImageAnalytics/CUDA_hierarchicalmaxflow.cu
and Common/vtkCudaCommonStatic/CUDA_commonKernels.cu, unmodified, from the
reference tree into oracle/_ref/hmf_ref_kernels.cubin.  This module loads that
cubin through the CUDA driver API and replays the reference host code's launch
sequence:
    InitializeAlgorithm  vtkCudaHierarchicalMaxFlowSegmentation.cxx:547-658
    PropogateLabels      :63-104
    SolveMaxFlow         :106-427
    UpdateLabel          :429-476
with every buffer resident and padded by VX*VY floats on each side, as the
reference allocates them (:513-538, CUDA_hierarchicalmaxflow.cu:33-60), since
its kernels read up to one plane outside a buffer before masking.  Buffers are
torch CUDA tensors; kernels run on torch's current stream.

It also runs the reference's vote kernel (CUDA_imagevote.cu), the
gradient kernel of its energy decomposition (CUDA_hierarchicalmaxflowdecomp.cu),
and the DAG solver's tasks (vtkCudaMaxFlowSegmentationTask.cxx:309-492) in the
fixed order that oracle/dag_oracle.cpp restates.
It is used only to generate golden vectors (tests/golden/make_golden.py) and
to pin the oracle; nothing in the product imports it.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import build_oracle

CUBIN = os.path.join(build_oracle.REF_OUT, "hmf_ref_kernels.cubin")
NUMTHREADS = 512  # vtkCudaCommon.h:23

_NAMES = {
    "zero": "_Z13ZeroOutBufferIfEvPT_i",
    "setconst": "_Z16SetBufferToConstIfEvPT_S0_i",
    "sum": "_Z10SumBuffersIfEvPT_S1_i",
    "copy": "_Z11CopyBuffersIfEvPT_S1_i",
    "mulstore": "_Z22MultiplyAndStoreBufferIfEvPT_S1_S0_i",
    "min": "_Z15kern_MinBuffersPfS_i",
    "lbl": "_Z8kern_LblPfS_S_i",
    "divbuf": "_Z18kern_DivideBuffersPfS_i",
    "sinkstore": "_Z30kern_FindSinkPotentialAndStorePfS_S_S_fi",
    "sourcestore": "_Z32kern_FindSourcePotentialAndStorePfS_S_S_fi",
    "leafsink": "_Z26kern_FindLeafSinkPotentialPfS_S_S_fi",
    "capacity": "_Z18kern_ApplyCapacityPfS_i",
    "label": "_Z16kern_UpdateLabelPfS_S_S_fi",
    "gradstep": "_Z17kern_CalcGradStepPfS_S_S_ffi",
    "descent": "_Z23kern_DescentSpatialFlowPfS_S_S_4int2i",
    "magvari": "_Z29kern_ComputeFlowMagVariSmoothPfS_S_S_S_f4int2i",
    "magconst": "_Z30kern_ComputeFlowMagConstSmoothPfS_S_S_f4int2i",
    "project": "_Z12kern_ProjectPfS_S_S_4int2i",
    "divergence": "_Z15kern_DivergencePfS_S_S_4int2i",
    # vote (CUDA_imagevote.cu:30, instantiated for float inputs / int labels)
    "civ": "_Z23CUDA_CIV_kernMinWithMapIfiEvPT_S1_PT0_S2_i",
    # energy decomposition (CUDA_hierarchicalmaxflowdecomp.cu:19)
    "ghmfd_grad": "_Z25kern_GHMFD_GradientBufferPfS_4int3i",
    "mul": "_Z15MultiplyBuffersIfEvPT_S1_i",
    # DAG solver tasks (CUDA_hierarchicalmaxflow.cu:610-664, CUDA_commonKernels.cu:96, :419)
    "resetsink": "_Z20kern_ResetSinkBufferPfS_S_S_ffi",
    "pushup": "_Z22kern_PushUpSourceFlowsPfS_S_S_S_ffi",
    "copy2": "_Z17kern_Copy2BuffersPfS_S_i",
    "translate": "_Z15TranslateBufferIfEvPT_S0_S0_i",
    "sumscaled": "_Z16SumScaledBuffersIfEvPT_S1_S0_i",
}


class _Int2(ctypes.Structure):
    _fields_ = [("x", ctypes.c_int), ("y", ctypes.c_int)]


class _Int3(ctypes.Structure):
    _fields_ = [("x", ctypes.c_int), ("y", ctypes.c_int), ("z", ctypes.c_int)]


class _Ptr(int):
    """A device address (kept apart from int kernel arguments)."""


def available() -> bool:
    return os.path.exists(CUBIN)


class ReferenceKernels:
    def __init__(self):
        import torch

        torch.cuda.init()
        torch.zeros(1, device="cuda")  # make the primary context current
        self.torch = torch
        self.cu = ctypes.CDLL("libcuda.so.1")
        self.module = ctypes.c_void_p()
        self._ck(self.cu.cuModuleLoad(ctypes.byref(self.module), CUBIN.encode()), "cuModuleLoad")
        self.fn = {}
        for key, name in _NAMES.items():
            f = ctypes.c_void_p()
            self._ck(self.cu.cuModuleGetFunction(ctypes.byref(f), self.module, name.encode()), name)
            self.fn[key] = f

    @staticmethod
    def _ck(rc, what):
        if rc != 0:
            raise RuntimeError("CUDA driver call %s failed with %d" % (what, rc))

    def launch(self, key, size, *args):
        cargs = []
        for a in args:
            if isinstance(a, (_Int2, _Int3)):
                cargs.append(a)
            elif isinstance(a, _Ptr):
                cargs.append(ctypes.c_void_p(int(a)))
            elif isinstance(a, float):
                cargs.append(ctypes.c_float(a))
            elif isinstance(a, int):
                cargs.append(ctypes.c_int(a))
            else:
                raise TypeError("unsupported kernel argument %r" % (a,))
        ptrs = (ctypes.c_void_p * len(cargs))(*[ctypes.cast(ctypes.pointer(c), ctypes.c_void_p) for c in cargs])
        grid = (size - 1) // NUMTHREADS + 1
        stream = ctypes.c_void_p(self.torch.cuda.current_stream().cuda_stream)
        self._ck(self.cu.cuLaunchKernel(self.fn[key], grid, 1, 1, NUMTHREADS, 1, 1, 0, stream, ptrs, None), key)


def solve(dims, parent, data, smooth=None, alpha=None, iterations=100, step=0.1, cc=0.25, time_iterations=0,
          fetch_outputs=True):
    """REF_CUDA through the reference's own kernels.  Arguments as
    oracle.oracle.solve(); returns {"u": [n, VZ, VY, VX] float32, "sink": ...}.

    time_iterations > 0: after the `iterations` iterations, that many more
    are timed with CUDA events on the launching stream (launched back to
    back, without the per-iteration stream synchronisation of
    vtkCudaHierarchicalMaxFlowSegmentation.cxx:681); the result then holds
    "ms_per_iteration" and "launches_per_iteration"."""
    import torch

    K = ReferenceKernels()
    vx, vy, vz = (int(d) for d in dims)
    V = vx * vy * vz
    pad = vx * vy + 2 * NUMTHREADS
    n = len(parent)
    kids = [[] for _ in range(n)]
    root = -1
    for v, p in enumerate(parent):
        if p < 0:
            root = v
        else:
            kids[p].append(v)
    order = []
    stack = [root]
    while stack:
        v = stack.pop()
        order.append(v)
        stack.extend(reversed(kids[v]))
    leaves = [v for v in order if not kids[v]]
    keep = []

    def buf(init=None):
        t = torch.zeros(V + 2 * pad, dtype=torch.float32, device="cuda")
        if init is not None:
            t[pad:pad + V] = torch.from_numpy(np.ascontiguousarray(init, dtype=np.float32).reshape(-1)).cuda()
        keep.append(t)
        return _Ptr(t.data_ptr() + 4 * pad)

    fx, fy, fz, dv, sink, lab, work = ({} for _ in range(7))
    for v in range(n):
        sink[v] = buf()
        if not kids[v]:
            pass
        else:
            work[v] = buf()
        if v != root:
            fx[v], fy[v], fz[v], dv[v], lab[v] = buf(), buf(), buf(), buf(), buf()
    D = {l: buf(data[l]) for l in leaves}
    S = {}
    for v in range(n):
        if smooth is not None and smooth.get(v) is not None:
            S[v] = buf(smooth[v])
    a = {v: float(np.float32((alpha or {}).get(v, 1.0))) for v in range(n)}
    inc = {v: sink[parent[v]] for v in range(n) if v != root}
    dims2 = _Int2(vx, vy)
    step = float(np.float32(step))
    cc = float(np.float32(cc))
    icc = float(np.float32(1.0) / np.float32(cc))

    # InitializeAlgorithm (.cxx:547-658)
    for v in range(n):
        if v != root:
            for b in (fx[v], fy[v], fz[v], dv[v]):
                K.launch("zero", V, b, V)
    for l in leaves:
        K.launch("copy", V, sink[l], D[l], V)
    for l in leaves[1:]:
        K.launch("min", V, sink[leaves[0]], sink[l], V)
    K.launch("zero", V, work[root], V)
    K.launch("lbl", V, lab[leaves[0]], sink[leaves[0]], D[leaves[0]], V)
    K.launch("sum", V, work[root], lab[leaves[0]], V)
    for l in leaves[1:]:
        K.launch("copy", V, sink[l], sink[leaves[0]], V)
        K.launch("lbl", V, lab[l], sink[l], D[l], V)
        K.launch("sum", V, work[root], lab[l], V)
    for l in leaves:
        K.launch("divbuf", V, lab[l], work[root], V)
    for v in order:
        if v != root and kids[v]:
            K.launch("copy", V, sink[v], sink[leaves[0]], V)
    K.launch("copy", V, sink[root], sink[leaves[0]], V)

    def propagate(v):  # :63-104
        if kids[v] and v != root:
            K.launch("zero", V, lab[v], V)
        for k in kids[v]:
            propagate(k)
        if v == root or parent[v] == root:
            return
        K.launch("sum", V, lab[parent[v]], lab[v], V)

    propagate(root)

    def update_label(v):  # :429-476
        if v == root:
            return
        K.launch("label", V, sink[v], inc[v], dv[v], lab[v], cc, V)

    def solve_node(v):  # :106-427
        is_root, is_leaf = v == root, not kids[v]
        is_branch = not is_root and not is_leaf
        if not is_leaf:
            if is_branch:
                K.launch("zero", V, work[v], V)
            else:
                K.launch("setconst", V, work[v], float(np.float32(1.0) / np.float32(cc)), V)
        if not is_root:
            K.launch("gradstep", V, sink[v], inc[v], dv[v], lab[v], step, icc, V)
            K.launch("descent", V, dv[v], fx[v], fy[v], fz[v], dims2, V)
            if v in S:
                K.launch("magvari", V, dv[v], fx[v], fy[v], fz[v], S[v], a[v], dims2, V)
            else:
                K.launch("magconst", V, dv[v], fx[v], fy[v], fz[v], a[v], dims2, V)
            K.launch("project", V, dv[v], fx[v], fy[v], fz[v], dims2, V)
            K.launch("divergence", V, dv[v], fx[v], fy[v], fz[v], dims2, V)
        for k in kids[v]:
            solve_node(k)
        if is_branch:
            K.launch("sinkstore", V, work[v], inc[v], dv[v], lab[v], icc, V)
            K.launch("mulstore", V, work[v], sink[v], float(np.float32(1.0) / np.float32(len(kids[v]) + 1)), V)
        if is_root:
            K.launch("mulstore", V, work[v], sink[v], float(np.float32(1.0) / np.float32(len(kids[v]))), V)
        if is_leaf:
            K.launch("leafsink", V, sink[v], inc[v], dv[v], lab[v], icc, V)
            K.launch("capacity", V, sink[v], D[v], V)
        for k in reversed(kids[v]):
            update_label(k)
        if not is_root:
            K.launch("sourcestore", V, work[parent[v]], sink[v], dv[v], lab[v], icc, V)

    for _ in range(int(iterations)):
        solve_node(root)
    torch.cuda.synchronize()
    timing = {}
    if time_iterations > 0:
        count = [0]
        launch = K.launch

        def counted(*a):
            count[0] += 1
            launch(*a)

        K.launch = counted
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(int(time_iterations)):
            solve_node(root)
        e1.record()
        torch.cuda.synchronize()
        K.launch = launch
        timing = {"ms_per_iteration": e0.elapsed_time(e1) / time_iterations,
                  "launches_per_iteration": count[0] / time_iterations}
    if not fetch_outputs:
        return timing

    def fetch(p):
        return _as_tensor(keep, p, V, pad).cpu().numpy().reshape(vz, vy, vx)

    u = np.zeros((n, vz, vy, vx), dtype=np.float32)
    s = np.zeros((n, vz, vy, vx), dtype=np.float32)
    for v in range(n):
        s[v] = fetch(sink[v])
        if v != root:
            u[v] = fetch(lab[v])
    return {"u": u, "sink": s, **timing}


def _as_tensor(keep, ptr, V, pad):
    for t in keep:
        base = t.data_ptr() + 4 * pad
        if base == ptr:
            return t[pad:pad + V]
    raise KeyError("unknown buffer")


def _padded(keep, V, pad, init=None, dtype=None):
    import torch

    t = torch.zeros(V + 2 * pad, dtype=dtype or torch.float32, device="cuda")
    if init is not None:
        t[pad:pad + V] = torch.from_numpy(np.ascontiguousarray(init).reshape(-1)).cuda()
    keep.append(t)
    return t, _Ptr(t.data_ptr() + t.element_size() * pad)


def vote(inputs, values):
    """The reference CUDA vote (CUDA_CIV_COMPUTE, CUDA_imagevote.cu:230-268):
    maximum buffer = input 0, then kern_MinWithMap per input in order (its
    kernels read before their bounds check, so buffers are padded).
    Returns int32 labels shaped like the inputs."""
    import torch

    K = ReferenceKernels()
    shape = np.asarray(inputs[0]).shape
    V = int(np.prod(shape))
    pad = 2 * NUMTHREADS
    keep = []
    _, pmx = _padded(keep, V, pad, np.asarray(inputs[0], dtype=np.float32))
    out, pout = _padded(keep, V, pad, dtype=torch.int32)
    for k, a in enumerate(inputs):
        _, pin = _padded(keep, V, pad, np.asarray(a, dtype=np.float32))
        K.launch("civ", V, pin, pmx, pout, int(values[k]), V)
    torch.cuda.synchronize()
    return out[pad:pad + V].cpu().numpy().reshape(shape)


def gradient_terms(label, dims, smooth=None):
    """kern_GHMFD_GradientBuffer of one labelling, times a smoothness image
    by MultiplyBuffers when given, as CUDA_GHMFD_*ForLabel form the per-voxel
    terms (CUDA_hierarchicalmaxflowdecomp.cu:19-38, :88-139).  float32
    [VZ, VY, VX]."""
    import torch

    K = ReferenceKernels()
    vx, vy, vz = (int(d) for d in dims)
    V = vx * vy * vz
    pad = vx * vy + 2 * NUMTHREADS
    keep = []
    _, plab = _padded(keep, V, pad, np.asarray(label, dtype=np.float32))
    g, pg = _padded(keep, V, pad)
    K.launch("ghmfd_grad", V, plab, pg, _Int3(vx, vy, vz), V)
    if smooth is not None:
        sm, psm = _padded(keep, V, pad, np.asarray(smooth, dtype=np.float32))
        K.launch("mul", V, psm, pg, V)
        g = sm
    torch.cuda.synchronize()
    return g[pad:pad + V].cpu().numpy().reshape(vz, vy, vx)


class DagGraph:
    """The rooted DAG bookkeeping of oracle/dag_oracle.cpp (levels, forward
    iterator order, weighted parent and child counts) in float32 as the
    reference computes it (vtkDirectedAcyclicGraphMaxFlowSegmentation.cxx:906-995,
    vtkCudaDirectedAcyclicGraphMaxFlowSegmentation.cxx:343-692)."""

    def __init__(self, n_nodes, edges, weights=None):
        f32 = np.float32
        self.n = n = int(n_nodes)
        self.ep = [int(p) for p, _ in edges]
        self.ec = [int(c) for _, c in edges]
        self.weighted = weights is not None
        self.ew = [f32(w) for w in weights] if weights is not None else [f32(1.0)] * len(edges)
        self.in_e = [[] for _ in range(n)]
        self.out_e = [[] for _ in range(n)]
        for e, (p, c) in enumerate(zip(self.ep, self.ec)):
            self.out_e[p].append(e)
            self.in_e[c].append(e)
        self.root = [v for v in range(n) if not self.in_e[v]][0]
        indeg = [len(self.in_e[v]) for v in range(n)]
        self.level = [0] * n
        topo = [self.root]
        for v in topo:
            for e in self.out_e[v]:
                k = self.ec[e]
                self.level[k] = max(self.level[k], self.level[v] + 1)
                indeg[k] -= 1
                if indeg[k] == 0:
                    topo.append(k)
        seen = {self.root}
        self.forward = [self.root]
        for v in self.forward:
            for e in self.out_e[v]:
                k = self.ec[e]
                if self.level[k] == self.level[v] + 1 and k not in seen:
                    seen.add(k)
                    self.forward.append(k)
        self.n_parents = [f32(0.0)] * n
        for v in range(n):
            acc = f32(0.0)
            for e in self.in_e[v]:
                acc = f32(acc + (self.ew[e] if self.weighted else f32(1.0)))
            self.n_parents[v] = acc
        self.wkids = [f32(0.0)] * n
        for v in range(n):
            acc = f32(0.0)
            for e in self.out_e[v]:
                t = f32((float(self.ew[e]) if self.weighted else 1.0) / float(self.n_parents[self.ec[e]]))
                acc = f32(acc + f32(t * t))
            self.wkids[v] = acc

    def leaf(self, v):
        return not self.out_e[v]

    def wdown(self, e):
        return self.ew[e] if self.weighted else np.float32(1.0 / float(len(self.in_e[self.ec[e]])))

    def wup(self, e):
        f32 = np.float32
        W = self.ew[e] if self.weighted else f32(1.0 / float(len(self.in_e[self.ec[e]])))
        p = self.ep[e]
        return f32(W / self.wkids[p]) if p == self.root else f32(W / f32(self.wkids[p] + f32(1.0)))


def dag_solve(dims, n_nodes, edges, data, weights=None, smooth=None, alpha=None, iterations=100, step=0.1,
              cc=0.25):
    """The DAG solver through the reference's own kernels, tasks in the order of
    oracle/dag_oracle.cpp.  Arguments as oracle.oracle.dag_solve(); returns
    {"u", "sink", "inc"}: [n, VZ, VY, VX] float32."""
    import torch

    K = ReferenceKernels()
    g = DagGraph(n_nodes, edges, weights)
    vx, vy, vz = (int(d) for d in dims)
    V = vx * vy * vz
    pad = vx * vy + 2 * NUMTHREADS
    n = g.n
    keep = []

    def buf(init=None):
        t = torch.zeros(V + 2 * pad, dtype=torch.float32, device="cuda")
        if init is not None:
            t[pad:pad + V] = torch.from_numpy(np.ascontiguousarray(init, dtype=np.float32).reshape(-1)).cuda()
        keep.append(t)
        return _Ptr(t.data_ptr() + 4 * pad)

    leaves = [v for v in g.forward if g.leaf(v)]
    sink = {v: buf() for v in range(n)}
    fx, fy, fz, dv, lab, inc = ({} for _ in range(6))
    for v in range(n):
        if v != g.root:
            fx[v], fy[v], fz[v], dv[v], lab[v], inc[v] = buf(), buf(), buf(), buf(), buf(), buf()
    D = {l: buf(data[l]) for l in leaves}
    S = {v: buf(smooth[v]) for v in range(n) if smooth is not None and smooth.get(v) is not None}
    a = {v: float(np.float32((alpha or {}).get(v, 0.0))) for v in range(n)}
    acc = buf()
    dims2 = _Int2(vx, vy)
    step = float(np.float32(step))
    ccf = float(np.float32(cc))
    icc = float(np.float32(1.0) / np.float32(cc))
    src = sink[g.root]

    # initialisation (vtkCudaDirectedAcyclicGraphMaxFlowSegmentation.cxx:844-1045)
    K.launch("copy", V, src, D[leaves[0]], V)
    for l in leaves[1:]:
        K.launch("min", V, src, D[l], V)
    for v in g.forward:
        if v != g.root:
            K.launch("copy2", V, src, sink[v], inc[v], V)
    for l in leaves:
        K.launch("lbl", V, lab[l], sink[l], D[l], V)
        K.launch("sum", V, acc, lab[l], V)
    for l in leaves:
        K.launch("divbuf", V, lab[l], acc, V)
    for v in reversed(g.forward):
        if v == g.root or g.leaf(v):
            continue
        K.launch("zero", V, lab[v], V)
        for e in g.out_e[v]:
            K.launch("sumscaled", V, lab[v], lab[g.ec[e]], float(g.wdown(e)), V)

    shift = float(np.float32(1.0 / float(np.float32(np.float32(cc) * g.wkids[g.root]))))
    T = int(iterations)
    for t in range(T):
        for v in g.forward:  # (1) UpdateSpatialFlowsTask
            if v == g.root:
                continue
            K.launch("gradstep", V, sink[v], inc[v], dv[v], lab[v], step, icc, V)
            K.launch("descent", V, dv[v], fx[v], fy[v], fz[v], dims2, V)
            if v in S:
                K.launch("magvari", V, dv[v], fx[v], fy[v], fz[v], S[v], a[v], dims2, V)
            else:
                K.launch("magconst", V, dv[v], fx[v], fy[v], fz[v], a[v], dims2, V)
            K.launch("project", V, dv[v], fx[v], fy[v], fz[v], dims2, V)
            K.launch("divergence", V, dv[v], fx[v], fy[v], fz[v], dims2, V)
        K.launch("translate", V, src, 1.0, shift, V)  # (2) ResetSinkFlowRoot
        for v in range(n):
            if v == g.root:
                continue
            if g.leaf(v):  # ApplySinkPotentialLeafTask, UpdateLabelsTask
                K.launch("leafsink", V, sink[v], inc[v], dv[v], lab[v], icc, V)
                K.launch("capacity", V, sink[v], D[v], V)
                K.launch("label", V, sink[v], inc[v], dv[v], lab[v], ccf, V)
            else:  # ResetSinkFlowBranch
                k = float(np.float32(1.0 / (float(g.wkids[v]) + 1.0)))
                K.launch("resetsink", V, sink[v], inc[v], dv[v], lab[v], k, icc, V)
        if t == T - 1:
            break
        for v in reversed(g.forward):  # (3) PushUpSourceFlows, branch UpdateLabelsTask
            if v == g.root:
                continue
            for e in g.in_e[v]:
                K.launch("pushup", V, sink[g.ep[e]], sink[v], inc[v], dv[v], lab[v], float(g.wup(e)), icc, V)
            if not g.leaf(v):
                K.launch("label", V, sink[v], inc[v], dv[v], lab[v], ccf, V)
        for v in range(n):  # (4) ClearSourceBuffer, PushDownSinkFlows
            if v == g.root:
                continue
            K.launch("zero", V, inc[v], V)
            for e in g.in_e[v]:
                K.launch("sumscaled", V, inc[v], sink[g.ep[e]], float(g.wdown(e)), V)
    torch.cuda.synchronize()

    def fetch(p):
        return _as_tensor(keep, p, V, pad).cpu().numpy().reshape(vz, vy, vx)

    out = {k: np.zeros((n, vz, vy, vx), dtype=np.float32) for k in ("u", "sink", "inc")}
    for v in range(n):
        out["sink"][v] = fetch(sink[v])
        if v != g.root:
            out["u"][v] = fetch(lab[v])
            out["inc"][v] = fetch(inc[v])
    return out
