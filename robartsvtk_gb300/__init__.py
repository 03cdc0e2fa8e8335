"""robartsvtk_gb300 -- GB300-native (sm_103a) hierarchical continuous max-flow
segmentation, a drop-in for RobartsVTK's vtkHierarchicalMaxFlowSegmentation /
vtkCudaHierarchicalMaxFlowSegmentation path, with the directed-acyclic-graph
variant (vtkCudaDirectedAcyclicGraphMaxFlowSegmentation), the label vote and
the energy decomposition that follow it.

The compute is libhmf_gb300.so (CUDA kernels + C ABI, include/hmf.h); this
package binds it and mirrors the reference's filter API.
"""
from .segmentation import (REF_CPU, REF_CUDA, DAGSolver, DirectedAcyclicGraphMaxFlowSegmentation,  # noqa: F401
                           HierarchicalMaxFlowSegmentation, HMFBatchSolver, HMFError, HMFSolver,
                           adjoint_schedule, decomposition_energy, vote)

from .dataterm import ImageDataTerm, ImageLogLikelihood, data_term, log_likelihood  # noqa: F401

__all__ = ["HMFSolver", "HMFBatchSolver", "HierarchicalMaxFlowSegmentation", "REF_CUDA", "REF_CPU", "HMFError",
           "vote", "decomposition_energy", "DAGSolver", "DirectedAcyclicGraphMaxFlowSegmentation",
           "data_term", "log_likelihood", "ImageDataTerm", "ImageLogLikelihood", "adjoint_schedule"]
