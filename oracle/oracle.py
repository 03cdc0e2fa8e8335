"""ctypes front end of the oracle -- TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py (its cpu_baseline leg and
its reference arm) import this module, and only as the checker or as the CPU
baseline.  The product (robartsvtk_gb300) never does.

`solve()` runs hmf_oracle.cpp (REF_CUDA in FP32/FP64, or the REF_CPU port);
`solve_reference_cpu()` runs the same REF_CPU driver linked against the
reference's own compiled vtkMaxFlowSegmentationUtilities.cxx (only where the
reference sources were available to build it).
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import build_oracle

REF_CUDA = 0
REF_CPU = 1

_libs: dict[str, ctypes.CDLL] = {}


def _load(path: str, entry: str) -> ctypes.CDLL:
    if path in _libs:
        return _libs[path]
    lib = ctypes.CDLL(path)
    fn = getattr(lib, entry)
    fn.restype = ctypes.c_int
    fn.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                   ctypes.c_int, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_void_p),
                   ctypes.POINTER(ctypes.c_void_p), ctypes.POINTER(ctypes.c_double), ctypes.c_int,
                   ctypes.c_float, ctypes.c_float, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    lib.oracle_last_error.restype = ctypes.c_char_p
    _libs[path] = lib
    return lib


def port_library() -> ctypes.CDLL:
    return _load(build_oracle.build_port(), "oracle_hmf_solve")


def reference_library() -> ctypes.CDLL | None:
    path = os.path.join(build_oracle.REF_OUT, "libhmf_ref_cpu.so")
    if not os.path.exists(path):
        if build_oracle.build_reference_cpu() is None:
            return None
    try:
        return _load(path, "oracle_ref_hmf_solve")
    except OSError:
        return None  # e.g. a library built for another host architecture


def _call(lib, entry, semantics, precision, threads, dims, parent, data, smooth, alpha,
          iterations, step, cc, want_sink, want_div):
    vx, vy, vz = (int(d) for d in dims)
    n = len(parent)
    V = vx * vy * vz
    par = (ctypes.c_int * n)(*[int(p) for p in parent])
    keep = []
    dptr = (ctypes.c_void_p * n)()
    sptr = (ctypes.c_void_p * n)()
    for v in range(n):
        d = data.get(v) if data is not None else None
        if d is not None:
            a = np.ascontiguousarray(d, dtype=np.float32).reshape(-1)
            assert a.size == V
            keep.append(a)
            dptr[v] = a.ctypes.data
        s = smooth.get(v) if smooth is not None else None
        if s is not None:
            a = np.ascontiguousarray(s, dtype=np.float32).reshape(-1)
            assert a.size == V
            keep.append(a)
            sptr[v] = a.ctypes.data
    al = (ctypes.c_double * n)(*[float(alpha.get(v, 1.0)) if alpha else 1.0 for v in range(n)])
    u = np.zeros((n, V), dtype=np.float64)
    sink = np.zeros((n, V), dtype=np.float64) if want_sink else None
    div = np.zeros((n, V), dtype=np.float64) if want_div else None
    rc = getattr(lib, entry)(semantics, precision, threads, vx, vy, vz, n, par, dptr, sptr, al,
                             int(iterations), float(step), float(cc), u.ctypes.data,
                             sink.ctypes.data if sink is not None else None,
                             div.ctypes.data if div is not None else None)
    if rc != 0:
        raise RuntimeError("oracle failed (%d): %s" % (rc, lib.oracle_last_error().decode()))
    shape = (n, vz, vy, vx)
    out = {"u": u.reshape(shape)}
    if sink is not None:
        out["sink"] = sink.reshape(shape)
    if div is not None:
        out["div"] = div.reshape(shape)
    return out


def solve(dims, parent, data, smooth=None, alpha=None, iterations=100, step=0.1, cc=0.25,
          semantics=REF_CUDA, precision=32, threads=0, want_sink=False, want_div=False):
    """Run the oracle.  `dims` = (VX, VY, VZ); `parent` = parent id per vertex
    (-1 for the root); `data`/`smooth`/`alpha` = dicts keyed by vertex id.
    Returns {"u": [n, VZ, VY, VX] float64 labels, optional "sink", "div"}."""
    return _call(port_library(), "oracle_hmf_solve", semantics, precision, threads, dims, parent,
                 data, smooth, alpha, iterations, step, cc, want_sink, want_div)


def iterate(dims, parent, data, state, smooth=None, alpha=None, iterations=1, step=0.1, cc=0.25, init=False,
            threads=0):
    """REF_CUDA FP32 iterations from a given state, in place.  `state` = dict
    of float32 arrays [n, VZ, VY, VX]: "fx", "fy", "fz", "div", "u" (non-root
    rows used) and "sink" (every row; the root's is the source flow).  With
    init=True the state is first initialised from the data terms."""
    lib = port_library()
    fn = lib.oracle_hmf_iterate
    fn.restype = ctypes.c_int
    vx, vy, vz = (int(d) for d in dims)
    n = len(parent)
    par = (ctypes.c_int * n)(*[int(p) for p in parent])
    keep = []
    dptr = (ctypes.c_void_p * n)()
    sptr = (ctypes.c_void_p * n)()
    for v in range(n):
        if data.get(v) is not None:
            a = np.ascontiguousarray(data[v], dtype=np.float32).reshape(-1)
            keep.append(a)
            dptr[v] = a.ctypes.data
        if smooth and smooth.get(v) is not None:
            a = np.ascontiguousarray(smooth[v], dtype=np.float32).reshape(-1)
            keep.append(a)
            sptr[v] = a.ctypes.data
    al = (ctypes.c_double * n)(*[float((alpha or {}).get(v, 1.0)) for v in range(n)])
    arrs = []
    for k in ("fx", "fy", "fz", "div", "u", "sink"):
        a = state[k]
        if a.dtype != np.float32 or not a.flags["C_CONTIGUOUS"] or a.shape != (n, vz, vy, vx):
            raise ValueError("state[%r] must be a C-contiguous float32 array of shape %r" % (k, (n, vz, vy, vx)))
        arrs.append(a.ctypes.data_as(ctypes.POINTER(ctypes.c_float)))
    rc = fn(int(threads), vx, vy, vz, n, par, dptr, sptr if smooth else None, al, 1 if init else 0,
            int(iterations), ctypes.c_float(step), ctypes.c_float(cc), *arrs)
    if rc != 0:
        raise RuntimeError("oracle error %d: %s" % (rc, lib.oracle_last_error().decode()))


def new_state(dims, n):
    """Zeroed state arrays for iterate()."""
    vx, vy, vz = (int(d) for d in dims)
    return {k: np.zeros((n, vz, vy, vx), np.float32) for k in ("fx", "fy", "fz", "div", "u", "sink")}


def solve_reference_cpu(dims, parent, data, smooth=None, alpha=None, iterations=100, step=0.1,
                        cc=0.25, want_sink=False, want_div=False):
    """REF_CPU through the reference's own compiled utility loops (single thread)."""
    lib = reference_library()
    if lib is None:
        raise FileNotFoundError("reference CPU library not built (reference sources absent)")
    return _call(lib, "oracle_ref_hmf_solve", REF_CPU, 32, 1, dims, parent, data, smooth, alpha,
                 iterations, step, cc, want_sink, want_div)


def adjoint(dims, parent, data, truth, smooth=None, alpha=None, iterations=20, step=0.1, cc=0.25, eps=1e-6,
            precision=64, threads=0):
    """Loss -(1/V) sum log(max(u_truth, eps)) of the REF_CUDA solve and its
    gradients (oracle restatement of the adjoint).  truth: int32 [VZ, VY, VX]
    class index into the DFS pre-order leaf list.  Returns
    {"loss", "dD": [n, VZ, VY, VX], "dalpha": [n], "u": [n, VZ, VY, VX]}."""
    lib = port_library()
    fn = lib.oracle_hmf_adjoint
    fn.restype = ctypes.c_int
    vx, vy, vz = (int(d) for d in dims)
    n = len(parent)
    V = vx * vy * vz
    par = (ctypes.c_int * n)(*[int(p) for p in parent])
    keep = []
    dptr = (ctypes.c_void_p * n)()
    sptr = (ctypes.c_void_p * n)()
    for v in range(n):
        if data.get(v) is not None:
            a = np.ascontiguousarray(data[v], dtype=np.float32).reshape(-1)
            keep.append(a)
            dptr[v] = a.ctypes.data
        if smooth and smooth.get(v) is not None:
            a = np.ascontiguousarray(smooth[v], dtype=np.float32).reshape(-1)
            keep.append(a)
            sptr[v] = a.ctypes.data
    al = (ctypes.c_double * n)(*[float((alpha or {}).get(v, 1.0)) for v in range(n)])
    tr = np.ascontiguousarray(truth, dtype=np.int32).reshape(-1)
    loss = ctypes.c_double()
    dD = np.zeros((n, V), np.float64)
    da = np.zeros(n, np.float64)
    u = np.zeros((n, V), np.float64)
    rc = fn(int(precision), int(threads), vx, vy, vz, n, par, dptr, sptr, al, int(iterations), ctypes.c_float(step),
            ctypes.c_float(cc), tr.ctypes.data_as(ctypes.c_void_p), ctypes.c_double(eps), ctypes.byref(loss),
            dD.ctypes.data_as(ctypes.c_void_p), da.ctypes.data_as(ctypes.c_void_p),
            u.ctypes.data_as(ctypes.c_void_p))
    if rc != 0:
        raise RuntimeError("oracle adjoint failed (%d): %s" % (rc, lib.oracle_last_error().decode()))
    shape = (n, vz, vy, vx)
    return {"loss": loss.value, "dD": dD.reshape(shape), "dalpha": da, "u": u.reshape(shape)}


def vote(inputs, values=None, semantics=REF_CUDA):
    """Label vote over float images (oracle restatement): returns int32 ids,
    values[k] for the winning input k (default: k)."""
    lib = port_library()
    fn = lib.oracle_vote
    fn.restype = ctypes.c_int
    arrs = [np.ascontiguousarray(a, dtype=np.float32) for a in inputs]
    shape = arrs[0].shape
    n = arrs[0].size
    ptrs = (ctypes.c_void_p * len(arrs))(*[a.ctypes.data for a in arrs])
    vals = np.ascontiguousarray(values if values is not None else np.arange(len(arrs)), dtype=np.int32)
    out = np.zeros(n, np.int32)
    rc = fn(int(semantics), len(arrs), ptrs, vals.ctypes.data_as(ctypes.c_void_p), ctypes.c_longlong(n),
            out.ctypes.data_as(ctypes.c_void_p))
    if rc != 0:
        raise RuntimeError("oracle vote failed (%d): %s" % (rc, lib.oracle_last_error().decode()))
    return out.reshape(shape)


def energy(dims, parent, data, labels, smooth=None, want_terms=False):
    """Energy decomposition of leaf labellings (oracle restatement):
    {"f0": float, "f": [n] per vertex, optional "terms": [n, VZ, VY, VX]}."""
    lib = port_library()
    fn = lib.oracle_energy
    fn.restype = ctypes.c_int
    vx, vy, vz = (int(d) for d in dims)
    n = len(parent)
    V = vx * vy * vz
    par = (ctypes.c_int * n)(*[int(p) for p in parent])
    keep = []
    dp = (ctypes.c_void_p * n)()
    lp = (ctypes.c_void_p * n)()
    sp = (ctypes.c_void_p * n)()
    for v in range(n):
        for src, dst in ((data, dp), (labels, lp), (smooth, sp)):
            if src is not None and src.get(v) is not None:
                a = np.ascontiguousarray(src[v], dtype=np.float32).reshape(-1)
                keep.append(a)
                dst[v] = a.ctypes.data
    f0 = ctypes.c_double()
    f = np.zeros(n, np.float64)
    terms = np.zeros((n, V), np.float32) if want_terms else None
    rc = fn(vx, vy, vz, n, par, dp, lp, sp, ctypes.byref(f0), f.ctypes.data_as(ctypes.c_void_p),
            terms.ctypes.data_as(ctypes.c_void_p) if terms is not None else None)
    if rc != 0:
        raise RuntimeError("oracle energy failed (%d): %s" % (rc, lib.oracle_last_error().decode()))
    out = {"f0": f0.value, "f": f}
    if terms is not None:
        out["terms"] = terms.reshape((n, vz, vy, vx))
    return out


def _dag_edges(edges, weights):
    ep = np.ascontiguousarray([int(p) for p, _ in edges], dtype=np.int32)
    ec = np.ascontiguousarray([int(c) for _, c in edges], dtype=np.int32)
    ew = None if weights is None else np.ascontiguousarray(weights, dtype=np.float32)
    return ep, ec, ew


def dag_solve(dims, n_nodes, edges, data, weights=None, smooth=None, alpha=None, iterations=100, step=0.1,
              cc=0.25, precision=32, threads=0):
    """The DAG max-flow solver as vtkCudaDirectedAcyclicGraphMaxFlowSegmentation
    runs it, in the fixed task order of dag_oracle.cpp.  `edges` = [(parent,
    child), ...] in edge order, `weights` per edge or None; `data`/`smooth`/
    `alpha` dicts keyed by vertex id (a vertex missing from `alpha` has alpha
    0).  Returns {"u", "sink", "inc"}: [n, VZ, VY, VX] float64."""
    lib = port_library()
    fn = lib.oracle_dag_solve
    fn.restype = ctypes.c_int
    lib.oracle_dag_last_error.restype = ctypes.c_char_p
    vx, vy, vz = (int(d) for d in dims)
    n = int(n_nodes)
    V = vx * vy * vz
    ep, ec, ew = _dag_edges(edges, weights)
    keep = []
    dptr = (ctypes.c_void_p * n)()
    sptr = (ctypes.c_void_p * n)()
    for v in range(n):
        if data.get(v) is not None:
            a = np.ascontiguousarray(data[v], dtype=np.float32).reshape(-1)
            keep.append(a)
            dptr[v] = a.ctypes.data
        if smooth and smooth.get(v) is not None:
            a = np.ascontiguousarray(smooth[v], dtype=np.float32).reshape(-1)
            keep.append(a)
            sptr[v] = a.ctypes.data
    al = (ctypes.c_double * n)(*[float((alpha or {}).get(v, float("nan"))) for v in range(n)])
    u = np.zeros((n, V), np.float64)
    sink = np.zeros((n, V), np.float64)
    inc = np.zeros((n, V), np.float64)
    rc = fn(int(precision), int(threads), vx, vy, vz, n, len(ep), ep.ctypes.data_as(ctypes.c_void_p),
            ec.ctypes.data_as(ctypes.c_void_p), ew.ctypes.data_as(ctypes.c_void_p) if ew is not None else None,
            dptr, sptr, al, int(iterations), ctypes.c_float(step), ctypes.c_float(cc),
            u.ctypes.data_as(ctypes.c_void_p), sink.ctypes.data_as(ctypes.c_void_p),
            inc.ctypes.data_as(ctypes.c_void_p))
    if rc != 0:
        raise RuntimeError("oracle DAG solve failed (%d): %s" % (rc, lib.oracle_dag_last_error().decode()))
    shape = (n, vz, vy, vx)
    return {"u": u.reshape(shape), "sink": sink.reshape(shape), "inc": inc.reshape(shape)}


def dag_forward(n_nodes, edges, weights=None):
    """The rooted DAG's forward-iterator vertex order (leaves in it = output order)."""
    lib = port_library()
    fn = lib.oracle_dag_forward
    fn.restype = ctypes.c_int
    lib.oracle_dag_last_error.restype = ctypes.c_char_p
    ep, ec, ew = _dag_edges(edges, weights)
    out = np.zeros(int(n_nodes), np.int32)
    rc = fn(int(n_nodes), len(ep), ep.ctypes.data_as(ctypes.c_void_p), ec.ctypes.data_as(ctypes.c_void_p),
            ew.ctypes.data_as(ctypes.c_void_p) if ew is not None else None, out.ctypes.data_as(ctypes.c_void_p))
    if rc != 0:
        raise RuntimeError("oracle DAG graph rejected (%d): %s" % (rc, lib.oracle_dag_last_error().decode()))
    return [int(v) for v in out]
