// TEST INFRASTRUCTURE ONLY.  Translation unit that compiles the reference's
// own HMF CUDA kernels, in place from the reference tree (the include path is
// set by oracle/build_oracle.py), into one sm_103a cubin.  oracle/ref_kernels.py
// loads that cubin on a GPU and replays the reference launch order
// (vtkCudaHierarchicalMaxFlowSegmentation.cxx:106-476, :547-658) to produce
// golden vectors for the REF_CUDA oracle, and runs the vote
// (CUDA_imagevote.cu) and energy-decomposition (CUDA_hierarchicalmaxflowdecomp.cu)
// kernels for theirs.  Nothing in the product uses it.
#include "CUDA_commonKernels.cu"
#include "CUDA_hierarchicalmaxflow.cu"
#include "CUDA_hierarchicalmaxflowdecomp.cu"
#include "CUDA_imagevote.cu"
