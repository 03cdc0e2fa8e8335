// hmf_segmentation.cpp -- see hmf_segmentation.hpp.
#include "hmf_segmentation.hpp"

#include <algorithm>
#include <climits>

namespace hmf {

HierarchicalMaxFlowSegmentation::HierarchicalMaxFlowSegmentation() = default;

HierarchicalMaxFlowSegmentation::~HierarchicalMaxFlowSegmentation() {
  if (ctx_) hmf_destroy(ctx_);
}

void HierarchicalMaxFlowSegmentation::SetStructure(const std::vector<int>& parent) { parent_ = parent; }

void HierarchicalMaxFlowSegmentation::AddSmoothnessScalar(int node, double alpha) {
  if (alpha >= 0.0) {
    scalars_.insert({node, alpha});  // std::map::insert: the first value stays
  } else {
    error_ = "Cannot use a negative smoothness value.";
  }
}

void HierarchicalMaxFlowSegmentation::SetNumberOfIterations(int n) { iterations_ = std::max(0, n); }
void HierarchicalMaxFlowSegmentation::SetCC(float cc) { cc_ = std::min(1.0f, std::max(0.0f, cc)); }
void HierarchicalMaxFlowSegmentation::SetStepSize(float s) { step_ = std::min(1.0f, std::max(0.0f, s)); }

void HierarchicalMaxFlowSegmentation::SetDataInputDataObject(int node, const float* data, const int dims[3],
                                                             int where) {
  if (!data) {
    data_.erase(node);
    return;
  }
  Input in;
  in.ptr = data;
  in.where = where;
  for (int k = 0; k < 3; ++k) in.dims[k] = dims[k];
  data_[node] = in;
}

const float* HierarchicalMaxFlowSegmentation::GetDataInputDataObject(int node) const {
  auto it = data_.find(node);
  return it == data_.end() ? nullptr : it->second.ptr;
}

void HierarchicalMaxFlowSegmentation::SetSmoothnessInputDataObject(int node, const float* smooth,
                                                                   const int dims[3], int where) {
  if (!smooth) {
    smooth_.erase(node);
    return;
  }
  Input in;
  in.ptr = smooth;
  in.where = where;
  for (int k = 0; k < 3; ++k) in.dims[k] = dims[k];
  smooth_[node] = in;
}

const float* HierarchicalMaxFlowSegmentation::GetSmoothnessInputDataObject(int node) const {
  auto it = smooth_.find(node);
  return it == smooth_.end() ? nullptr : it->second.ptr;
}

int HierarchicalMaxFlowSegmentation::Fail(const std::string& msg) {
  error_ = msg;
  return -1;
}

const float* HierarchicalMaxFlowSegmentation::GetOutputDataObject(int node) const {
  auto it = outputs_.find(node);
  return it == outputs_.end() ? nullptr : it->second.data();
}

// RequestData (vtkHierarchicalMaxFlowSegmentation.cxx:555-933) with
// CheckInputConsistancy (:363-505): validate, then initialise and iterate on
// the device, then fetch the leaf labellings.
int HierarchicalMaxFlowSegmentation::Update(void* stream) { return Run(stream, false); }

int HierarchicalMaxFlowSegmentation::ContinueUpdate(void* stream) { return Run(stream, true); }

int HierarchicalMaxFlowSegmentation::Run(void* stream, bool continued) {
  error_.clear();
  if (parent_.empty()) return Fail("Hierarchy must be provided.");
  const int n = (int)parent_.size();
  // consistent extents across every input (:440-456, :476-491)
  int dims[3] = {-1, -1, -1};
  auto check_dims = [&](const Input& in) {
    if (dims[0] < 0) {
      for (int k = 0; k < 3; ++k) dims[k] = in.dims[k];
      return true;
    }
    return in.dims[0] == dims[0] && in.dims[1] == dims[1] && in.dims[2] == dims[2];
  };
  for (auto& kv : data_)
    if (kv.first >= 0 && kv.first < n && !check_dims(kv.second)) return Fail("Inconsistant object extent.");
  for (auto& kv : smooth_)
    if (kv.first >= 0 && kv.first < n && !check_dims(kv.second)) return Fail("Inconsistant object extent.");
  if (dims[0] <= 0) return Fail("Missing data prior for leaf node.");

  const bool rebuild = !ctx_ || ctx_parent_ != parent_ || ctx_semantics_ != semantics_ ||
                       ctx_device_ != device_ || ctx_usage_ != max_gpu_usage_ || dims[0] != ctx_dims_[0] ||
                       dims[1] != ctx_dims_[1] || dims[2] != ctx_dims_[2];
  if (continued && rebuild)
    return Fail("ContinueUpdate follows an Update with the same hierarchy, extent, semantics, device and "
                "MaxGPUUsage.");
  if (rebuild) {
    if (ctx_) hmf_destroy(ctx_);
    ctx_ = nullptr;
    int rc = max_gpu_usage_ < 0.0
                 ? hmf_create(&ctx_, dims[0], dims[1], dims[2], parent_.data(), n, semantics_, device_)
                 : hmf_create_paged(&ctx_, dims[0], dims[1], dims[2], parent_.data(), n, semantics_, device_,
                                    max_gpu_usage_);
    if (rc != HMF_OK) {
      ctx_ = nullptr;
      return Fail(hmf_last_error(nullptr));
    }
    ctx_parent_ = parent_;
    ctx_semantics_ = semantics_;
    ctx_device_ = device_;
    ctx_usage_ = max_gpu_usage_;
    for (int k = 0; k < 3; ++k) ctx_dims_[k] = dims[k];
    int nl = hmf_leaf_order(ctx_, nullptr, 0);
    leaves_.assign(nl, -1);
    hmf_leaf_order(ctx_, leaves_.data(), nl);
  }
  for (int v = 0; v < n; ++v) {
    if (parent_[v] < 0) continue;
    auto it = scalars_.find(v);
    hmf_set_smoothness_scalar(ctx_, v, it == scalars_.end() ? 1.0 : it->second);
    auto sm = smooth_.find(v);
    hmf_set_smoothness(ctx_, v, sm == smooth_.end() ? nullptr : sm->second.ptr,
                       sm == smooth_.end() ? HMF_HOST : sm->second.where);
  }
  for (int l : leaves_) {
    auto it = data_.find(l);
    if (it == data_.end()) return Fail("Missing data prior for leaf node.");
    if (hmf_set_data(ctx_, l, it->second.ptr, it->second.where) != HMF_OK) return Fail(hmf_last_error(ctx_));
  }
  hmf_set_params(ctx_, iterations_, step_, cc_);
  if ((continued ? hmf_solve_continue(ctx_, stream) : hmf_solve(ctx_, stream)) != HMF_OK)
    return Fail(hmf_last_error(ctx_));
  const size_t V = (size_t)dims[0] * dims[1] * dims[2];
  outputs_.clear();
  for (int l : leaves_) {
    std::vector<float>& out = outputs_[l];
    out.resize(V);
    if (hmf_get_labels(ctx_, l, out.data(), HMF_HOST, stream) != HMF_OK) return Fail(hmf_last_error(ctx_));
  }
  return 1;
}

}  // namespace hmf
