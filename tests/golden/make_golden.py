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


if __name__ == "__main__":
    if "--ref-cpu" in sys.argv:
        ref_cpu(os.path.join(HERE, "ref_cpu_golden.npz"))
    if "--ref-cuda" in sys.argv:
        i = sys.argv.index("--ref-cuda")
        ref_cuda(sys.argv[i + 1] if i + 1 < len(sys.argv) else os.path.join(HERE, "ref_cuda_golden.npz"))
