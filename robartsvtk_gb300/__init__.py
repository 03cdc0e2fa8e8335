"""robartsvtk_gb300 -- GB300-native (sm_103a) hierarchical continuous max-flow
segmentation, a drop-in for RobartsVTK's vtkHierarchicalMaxFlowSegmentation /
vtkCudaHierarchicalMaxFlowSegmentation path.

The compute is libhmf_gb300.so (CUDA kernels + C ABI, include/hmf.h); this
package binds it and mirrors the reference's filter API.
"""
from .segmentation import (REF_CPU, REF_CUDA, HierarchicalMaxFlowSegmentation, HMFBatchSolver,  # noqa: F401
                           HMFError, HMFSolver, decomposition_energy, vote)

__all__ = ["HMFSolver", "HMFBatchSolver", "HierarchicalMaxFlowSegmentation", "REF_CUDA", "REF_CPU", "HMFError",
           "vote", "decomposition_energy"]
