"""Generates the golden vectors in this folder from the reference's own code.

  python -m tests.golden.make_golden --ref-cpu     (where the reference sources are)
      REF_CPU outputs of the reference's vtkMaxFlowSegmentationUtilities.cxx,
      compiled from source (oracle/_ref/libhmf_ref_cpu.so), driven by the
      restated recursion of vtkHierarchicalMaxFlowSegmentation.cxx:973-1259.
  python -m tests.golden.make_golden --ref-cuda OUT.npz   (on a GPU)
      REF_CUDA outputs of the reference's own CUDA kernels
      (oracle/_ref/hmf_ref_kernels.cubin, built from CUDA_hierarchicalmaxflow.cu
      and CUDA_commonKernels.cu), replaying the launch order of
      vtkCudaHierarchicalMaxFlowSegmentation.cxx:106-658.
  python -m tests.golden.make_golden --ref-post OUT.npz   (on a GPU)
      the reference's vote kernel (CUDA_imagevote.cu) over seeded images with
      ties, and the per-voxel terms of its energy decomposition
      (CUDA_hierarchicalmaxflowdecomp.cu) of seeded labellings, with and
      without a smoothness image (POST_CASES in tests/golden/cases.py).
  python -m tests.golden.make_golden --ref-dag OUT.npz   (on a GPU)
      the DAG solver through the reference's own kernels, its tasks
      (vtkCudaMaxFlowSegmentationTask.cxx:309-492) in the order that
      oracle/dag_oracle.cpp restates (DAG_CASES in tests/golden/cases.py).
"""
import os
import sys

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__)))))

from tests.golden.cases import CASES, problem  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))


def _pack(out, name, res, n):
    out[name + "/u"] = res["u"].astype(np.float32)
    out[name + "/sink"] = res["sink"].astype(np.float32)


def ref_cpu(path):
    from oracle import oracle as O
    out = {}
    for name in CASES:
        w = problem(name)
        res = O.solve_reference_cpu(w.dims, w.parent, w.data, w.smooth, w.alpha, w.iterations, w.step, w.cc,
                                    want_sink=True)
        _pack(out, name, res, len(w.parent))
    np.savez_compressed(path, **out)


def ref_cuda(path):
    from oracle import ref_kernels
    out = {}
    for name in CASES:
        w = problem(name)
        res = ref_kernels.solve(w.dims, w.parent, w.data, w.smooth, w.alpha, w.iterations, w.step, w.cc)
        _pack(out, name, res, len(w.parent))
    np.savez_compressed(path, **out)


def ref_post(path):
    from oracle import ref_kernels
    from tests.golden.cases import POST_CASES, post_problem
    out = {}
    for name in POST_CASES:
        p = post_problem(name)
        out[name + "/vote_inputs"] = np.stack(p["inputs"])
        out[name + "/vote_values"] = np.asarray(p["values"], np.int32)
        out[name + "/vote"] = ref_kernels.vote(p["inputs"], p["values"])
        out[name + "/label"] = p["label"]
        out[name + "/smooth"] = p["smooth"]
        out[name + "/grad"] = ref_kernels.gradient_terms(p["label"], p["dims"])
        out[name + "/grad_smooth"] = ref_kernels.gradient_terms(p["label"], p["dims"], p["smooth"])
    np.savez_compressed(path, **out)


def ref_dag(path):
    from oracle import ref_kernels
    from tests.golden.cases import DAG_CASES, dag_problem
    out = {}
    for name in DAG_CASES:
        w = dag_problem(name)
        res = ref_kernels.dag_solve(w.dims, w.n, w.edges, w.data, w.weights, w.smooth, w.alpha, w.iterations,
                                    w.step, w.cc)
        for k in ("u", "sink", "inc"):
            out[name + "/" + k] = res[k].astype(np.float32)
    np.savez_compressed(path, **out)


if __name__ == "__main__":
    if "--ref-cpu" in sys.argv:
        ref_cpu(os.path.join(HERE, "ref_cpu_golden.npz"))
    if "--ref-cuda" in sys.argv:
        i = sys.argv.index("--ref-cuda")
        ref_cuda(sys.argv[i + 1] if i + 1 < len(sys.argv) else os.path.join(HERE, "ref_cuda_golden.npz"))
    if "--ref-post" in sys.argv:
        i = sys.argv.index("--ref-post")
        ref_post(sys.argv[i + 1] if i + 1 < len(sys.argv) else os.path.join(HERE, "ref_post_golden.npz"))
    if "--ref-dag" in sys.argv:
        i = sys.argv.index("--ref-dag")
        ref_dag(sys.argv[i + 1] if i + 1 < len(sys.argv) else os.path.join(HERE, "ref_dag_golden.npz"))
