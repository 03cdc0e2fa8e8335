// hmf_segmentation.hpp -- VTK-free C++ drop-in for the filter surface of
// vtkHierarchicalMaxFlowSegmentation / vtkCudaHierarchicalMaxFlowSegmentation
// (Common/vtkRobartsCommon/vtkHierarchicalMaxFlowSegmentation.h:43-204,
//  ImageProcessing/vtkCudaImageAnalytics/vtkCudaHierarchicalMaxFlowSegmentation.h:36-85),
// backed by the C ABI of include/hmf.h.
//
// Method names, argument meaning and error behaviour follow the reference:
//  - the tree is a parent array (vertex ids, -1 for the root) instead of a
//    vtkTree; SetStructure and SetHierarchy are the same call;
//  - images are float32 buffers with their dimensions instead of
//    vtkImageData; every input must have the same dimensions;
//  - AddSmoothnessScalar keeps the first value given for a vertex and rejects
//    negative values (vtkHierarchicalMaxFlowSegmentation.cxx:93-104);
//  - the setters clamp as vtkSetClampMacro does (.h:64-77);
//  - Update() returns 1 on success and -1 on failure (RequestData's
//    convention), with the message in GetLastError();
//  - GetOutputDataObject(leaf) returns the leaf's probabilistic labelling,
//    keyed by tree vertex id (.cxx:337-346), owned by the filter.
#pragma once

#include <map>
#include <string>
#include <vector>

#include "../../include/hmf.h"

namespace hmf {

class HierarchicalMaxFlowSegmentation {
 public:
  HierarchicalMaxFlowSegmentation();
  ~HierarchicalMaxFlowSegmentation();
  HierarchicalMaxFlowSegmentation(const HierarchicalMaxFlowSegmentation&) = delete;
  HierarchicalMaxFlowSegmentation& operator=(const HierarchicalMaxFlowSegmentation&) = delete;

  void SetStructure(const std::vector<int>& parent);
  void SetHierarchy(const std::vector<int>& parent) { SetStructure(parent); }
  const std::vector<int>& GetStructure() const { return parent_; }

  void AddSmoothnessScalar(int node, double alpha);

  void SetNumberOfIterations(int n);
  int GetNumberOfIterations() const { return iterations_; }
  void SetCC(float cc);
  float GetCC() const { return cc_; }
  void SetStepSize(float step);
  float GetStepSize() const { return step_; }

  // where = HMF_HOST or HMF_DEVICE; dims = {VX, VY, VZ}; NULL data removes the input.
  void SetDataInputDataObject(int node, const float* data, const int dims[3], int where = HMF_HOST);
  const float* GetDataInputDataObject(int node) const;
  void SetSmoothnessInputDataObject(int node, const float* smooth, const int dims[3], int where = HMF_HOST);
  const float* GetSmoothnessInputDataObject(int node) const;

  // CudaObject::SetDevice (Common/vtkCudaCommon/CudaObject.h:44)
  void SetDevice(int device) { device_ = device; }
  int GetDevice() const { return device_; }
  // vtkCudaHierarchicalMaxFlowSegmentation's MaxGPUUsage (.h:52): the
  // fraction of the device's memory the solve may hold, clamped to [0, 1]
  // as vtkCudaHierarchicalMaxFlowSegmentation2's setter does (.h:74-75).  A
  // negative value (the default) solves in core; otherwise the solve runs
  // out of core (hmf_create_paged) within that budget, with the same
  // results.
  void SetMaxGPUUsage(double usage) { max_gpu_usage_ = usage < 0.0 ? -1.0 : (usage > 1.0 ? 1.0 : usage); }
  double GetMaxGPUUsage() const { return max_gpu_usage_; }
  // HMF_SEMANTICS_REF_CUDA (default) or HMF_SEMANTICS_REF_CPU
  void SetSemantics(int semantics) { semantics_ = semantics; }
  int GetSemantics() const { return semantics_; }

  int Update(void* stream = nullptr);
  // NumberOfIterations more iterations from the state the last Update or
  // ContinueUpdate ended in (hmf_solve_continue; no counterpart in the
  // reference): the inputs and parameters as set now, the hierarchy,
  // extent, semantics, device and MaxGPUUsage unchanged since that Update.
  // Update(k1) then ContinueUpdate(k2) gives Update(k1 + k2)'s outputs.
  int ContinueUpdate(void* stream = nullptr);

  const float* GetOutputDataObject(int node) const;
  int GetNumberOfOutputPorts() const { return (int)leaves_.size(); }
  const std::vector<int>& GetLeafOrder() const { return leaves_; }
  const std::string& GetLastError() const { return error_; }

 private:
  struct Input {
    const float* ptr = nullptr;
    int dims[3] = {0, 0, 0};
    int where = HMF_HOST;
  };
  int Fail(const std::string& msg);
  int Run(void* stream, bool continued);

  std::vector<int> parent_;
  std::map<int, double> scalars_;
  std::map<int, Input> data_, smooth_;
  int iterations_ = 100;
  float cc_ = 0.25f;
  float step_ = 0.1f;
  int device_ = 0;
  int semantics_ = HMF_SEMANTICS_REF_CUDA;
  double max_gpu_usage_ = -1.0;

  hmf_ctx* ctx_ = nullptr;
  int ctx_dims_[3] = {0, 0, 0};
  std::vector<int> ctx_parent_;
  int ctx_semantics_ = -1, ctx_device_ = -1;
  double ctx_usage_ = -1.0;

  std::vector<int> leaves_;
  std::map<int, std::vector<float>> outputs_;
  std::string error_;
};

}  // namespace hmf
