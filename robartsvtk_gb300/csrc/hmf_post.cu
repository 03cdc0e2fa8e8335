// hmf_post.cu -- the label vote and the energy decomposition (include/hmf.h):
// standalone drop-ins for CUDA_CIV_COMPUTE (CUDA_imagevote.h) and the
// CUDA_GHMFD_* launchers (CUDA_hierarchicalmaxflowdecomp.h), and the same
// computations on a solver context's final labels.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstring>
#include <vector>

#include "hmf_ctx.hpp"
#include "hmf_post.cuh"

using namespace hmfi;

namespace {

int grid_for(long long n) {
  int dev = 0, sms = 148;
  if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  return (int)std::max<long long>(1, std::min<long long>((n + hmf::kPostThreads - 1) / hmf::kPostThreads,
                                                         (long long)sms * 16));
}

// Device copies of host arrays (freed at scope end).
struct Scratch {
  std::vector<void*> ptrs;
  ~Scratch() {
    for (void* p : ptrs) cudaFree(p);
  }
  template <class T>
  cudaError_t copy_in(const T* src, size_t count, const T** dst, cudaStream_t s) {
    void* p = nullptr;
    cudaError_t e = cudaMalloc(&p, count * sizeof(T));
    if (e != cudaSuccess) return e;
    ptrs.push_back(p);
    *dst = static_cast<const T*>(p);
    return cudaMemcpyAsync(p, src, count * sizeof(T), cudaMemcpyHostToDevice, s);
  }
};

int launch_vote(hmf_ctx* c, const hmf::VoteInputs& in, const hmf::Geometry& G, int* out, cudaStream_t s) {
  bool quads = G.pitch % 4 == 0;
  for (int k = 0; k < in.n; ++k) quads = quads && (reinterpret_cast<uintptr_t>(in.in[k]) % 16) == 0;
  if (quads) {
    const long long nq = (long long)G.vy * G.vz * (G.pitch / 4);
    hmf::vote4_kernel<<<grid_for(nq), hmf::kPostThreads, 0, s>>>(in, G, out);
    CK(cudaGetLastError(), "vote4_kernel launch");
  } else {
    const long long dense = (long long)G.vx * G.vy * G.vz;
    hmf::vote_kernel<<<grid_for(dense), hmf::kPostThreads, 0, s>>>(in, G, out);
    CK(cudaGetLastError(), "vote_kernel launch");
  }
  return HMF_OK;
}

constexpr size_t kEnergyTableBytes = (sizeof(hmf::EnergyTable) + 255) / 256 * 256;
constexpr size_t kEnergyBuffer = kEnergyTableBytes + sizeof(double) * (1 + hmf::kMaxVertices);

// Energy of leaf labellings over a tree; arrays pitched per G.  Synchronous.
// `buffer` (kEnergyBuffer bytes of device memory) holds the table and the
// sums; null: allocated for this call.
int launch_energy(hmf_ctx* c, const hmf::EnergyTable& tab, const hmf::Geometry& G, double* f0, double* f,
                  int n_nodes, cudaStream_t s, char* buffer) {
  char* own = nullptr;
  if (!buffer) {
    CK(cudaMalloc(&own, kEnergyBuffer), "cudaMalloc(energy buffer)");
    buffer = own;
  }
  hmf::EnergyTable* d_tab = reinterpret_cast<hmf::EnergyTable*>(buffer);
  double* d_sums = reinterpret_cast<double*>(buffer + kEnergyTableBytes);
  std::vector<double> sums(1 + hmf::kMaxVertices, 0.0);
  // persistent grid: as many blocks as are resident at once, each walking rows
  auto grid_of = [&](auto kernel) {
    int dev = 0, sms = 148, per = 1;
    if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, hmf::kPostThreads, 0) != cudaSuccess || per < 1)
      per = 1;
    return std::max(1, std::min(G.vy * G.vz, sms * per));
  };
  cudaError_t e = cudaMemsetAsync(d_sums, 0, sizeof(double) * sums.size(), s);
  if (e == cudaSuccess && tab.n <= hmf::kEnergyRegMax && G.plane <= INT32_MAX) {
    hmf::EnergyRegParams P;
    std::memset(&P, 0, sizeof(P));
    P.sum_index[0] = 0;
    for (int k = 0; k < tab.n; ++k) {
      P.label[k] = tab.label[k];
      P.data[k] = tab.data[k];
      P.smooth[k] = tab.smooth[k];
      if (tab.n_kids[k] == 0) P.leaf_mask |= 1u << k;
      if (tab.parent_entry[k] >= 0) P.kids[tab.parent_entry[k]] |= 1u << k;
      P.sum_index[1 + k] = 1 + tab.vertex[k];
    }
    auto launch = [&](auto kernel) { kernel<<<grid_of(kernel), hmf::kPostThreads, 0, s>>>(P, G, d_sums); };
    switch (tab.n) {
      case 1: launch(hmf::energy_reg_kernel<1>); break;
      case 2: launch(hmf::energy_reg_kernel<2>); break;
      case 3: launch(hmf::energy_reg_kernel<3>); break;
      case 4: launch(hmf::energy_reg_kernel<4>); break;
      case 5: launch(hmf::energy_reg_kernel<5>); break;
      case 6: launch(hmf::energy_reg_kernel<6>); break;
      case 7: launch(hmf::energy_reg_kernel<7>); break;
      default: launch(hmf::energy_reg_kernel<8>); break;
    }
    e = cudaGetLastError();
  } else if (e == cudaSuccess) {
    e = cudaMemcpyAsync(d_tab, &tab, sizeof(tab), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) {
      hmf::energy_kernel<<<grid_of(hmf::energy_kernel), hmf::kPostThreads, 0, s>>>(d_tab, G, d_sums);
      e = cudaGetLastError();
    }
  }
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(sums.data(), d_sums, sizeof(double) * sums.size(), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (own) cudaFree(own);
  if (e != cudaSuccess) return cuda_fail(c, e, "energy_kernel");
  if (f0) *f0 = sums[0];
  for (int v = 0; v < n_nodes && f; ++v) f[v] = sums[1 + v];
  return HMF_OK;
}

// Post-order table of a parent array (children in increasing id order).
int energy_tree(hmf_ctx* c, const int* parent, int n_nodes, hmf::EnergyTable& tab, std::vector<int>& entry) {
  if (!parent || n_nodes < 2 || n_nodes > hmf::kMaxVertices)
    return fail(c, HMF_ERR_TREE, "the tree needs 2..64 vertices given as a parent array");
  int root = -1;
  std::vector<std::vector<int>> kids(n_nodes);
  for (int v = 0; v < n_nodes; ++v) {
    if (parent[v] < 0) {
      if (root >= 0) return fail(c, HMF_ERR_TREE, "the tree has more than one root");
      root = v;
    } else if (parent[v] >= n_nodes || parent[v] == v) {
      return fail(c, HMF_ERR_TREE, "tree parent id out of range");
    } else {
      kids[parent[v]].push_back(v);
    }
  }
  if (root < 0) return fail(c, HMF_ERR_TREE, "the tree has no root");
  std::vector<int> post;
  std::vector<std::pair<int, int>> st{{root, 0}};
  std::vector<char> seen(n_nodes, 0);
  while (!st.empty()) {
    auto& top = st.back();
    if (top.second == 0) {
      if (seen[top.first]) return fail(c, HMF_ERR_TREE, "the tree has a cycle");
      seen[top.first] = 1;
    }
    if (top.second < (int)kids[top.first].size()) {
      const int k = kids[top.first][top.second++];
      st.push_back({k, 0});
    } else {
      post.push_back(top.first);
      st.pop_back();
    }
  }
  if ((int)post.size() != n_nodes) return fail(c, HMF_ERR_TREE, "the tree is not connected");
  std::memset(&tab, 0, sizeof(tab));
  entry.assign(n_nodes, -1);
  int e = 0;
  for (int v : post)
    if (v != root) entry[v] = e++;
  tab.n = e;
  int kp = 0;
  for (int v : post) {
    if (v == root) continue;
    const int i = entry[v];
    tab.vertex[i] = v;
    tab.parent_entry[i] = parent[v] == root ? -1 : entry[parent[v]];
    tab.first_kid[i] = kp;
    tab.n_kids[i] = (int)kids[v].size();
    for (int k : kids[v]) tab.kids[kp++] = entry[k];
  }
  tab.n_kids_total = kp;
  return HMF_OK;
}

}  // namespace

extern "C" {

int hmf_vote(int n_inputs, const float* const* inputs, const int* values, long long n_voxels, int semantics,
             int* out, int where, void* stream) {
  hmf_ctx* c = nullptr;  // errors: hmf_last_error(NULL)
  if (n_inputs < 1 || n_inputs > hmf::kMaxVertices || !inputs || !out || n_voxels < 0 || n_voxels > 0x7fffffffLL)
    return fail(c, HMF_ERR_INVALID_ARGUMENT, "the vote needs 1..64 inputs, an output and < 2^31 voxels");
  if (semantics != HMF_SEMANTICS_REF_CUDA && semantics != HMF_SEMANTICS_REF_CPU)
    return fail(c, HMF_ERR_INVALID_ARGUMENT, "unknown semantics");
  if (where != HMF_HOST && where != HMF_DEVICE) return fail(c, HMF_ERR_INVALID_ARGUMENT, "bad `where`");
  for (int k = 0; k < n_inputs; ++k)
    if (!inputs[k]) return fail(c, HMF_ERR_MISSING_INPUT, "a vote input is NULL");
  if (where == HMF_DEVICE) {
    for (int k = 0; k < n_inputs; ++k)
      if (int rc = check_device_pointer(c, inputs[k], "vote input")) return rc;
    if (int rc = check_device_pointer(c, out, "vote output")) return rc;
  }
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  Scratch scratch;
  hmf::VoteInputs in;
  std::memset(&in, 0, sizeof(in));
  in.n = n_inputs;
  in.semantics = semantics;
  for (int k = 0; k < n_inputs; ++k) {
    in.values[k] = values ? values[k] : k;
    if (where == HMF_DEVICE) in.in[k] = inputs[k];
    else CK(scratch.copy_in(inputs[k], (size_t)n_voxels, &in.in[k], s), "vote input copy");
  }
  int* dout = out;
  if (where == HMF_HOST) {
    void* p = nullptr;
    CK(cudaMalloc(&p, sizeof(int) * std::max<long long>(n_voxels, 1)), "cudaMalloc(vote output)");
    scratch.ptrs.push_back(p);
    dout = static_cast<int*>(p);
  }
  // one dense row of n voxels
  hmf::Geometry G{(int)n_voxels, 1, 1, (int)n_voxels, n_voxels, n_voxels};
  if (n_voxels > 0) {
    int rc = launch_vote(c, in, G, dout, s);
    if (rc) return rc;
  }
  if (where == HMF_HOST) {
    CK(cudaMemcpyAsync(out, dout, sizeof(int) * n_voxels, cudaMemcpyDeviceToHost, s), "vote output copy");
    CK(cudaStreamSynchronize(s), "vote");
  }
  return HMF_OK;
}

int hmf_decomposition_energy(int vx, int vy, int vz, const int* parent, int n_nodes, const float* const* data,
                             const float* const* labels, const float* const* smooth, int where, double* f0,
                             double* f, void* stream) {
  hmf_ctx* c = nullptr;  // errors: hmf_last_error(NULL)
  if (vx <= 0 || vy <= 0 || vz <= 0) return fail(c, HMF_ERR_INVALID_ARGUMENT, "volume dimensions must be positive");
  if (vx > (1 << 30) || vy > (1 << 30) || vz > (1 << 30))
    return fail(c, HMF_ERR_INVALID_ARGUMENT, "volume dimensions above 2^30 are not supported");
  if (where != HMF_HOST && where != HMF_DEVICE) return fail(c, HMF_ERR_INVALID_ARGUMENT, "bad `where`");
  hmf::EnergyTable tab;
  std::vector<int> entry;
  int rc = energy_tree(c, parent, n_nodes, tab, entry);
  if (rc) return rc;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  const size_t V = (size_t)vx * vy * vz;
  Scratch scratch;
  for (int v = 0; v < n_nodes; ++v) {
    const int e = entry[v];
    if (e < 0) continue;
    const bool leaf = tab.n_kids[e] == 0;
    if (leaf && (!data || !data[v] || !labels || !labels[v]))
      return fail(c, HMF_ERR_MISSING_INPUT, "a leaf's data term or labelling is NULL");
    auto bring = [&](const float* src, const float** dst) -> int {
      if (where == HMF_DEVICE) {
        if (int rc = check_device_pointer(c, src, "energy input")) return rc;
        *dst = src;
      } else {
        CK(scratch.copy_in(src, V, dst, s), "energy input copy");
      }
      return HMF_OK;
    };
    if (leaf) {
      if ((rc = bring(labels[v], &tab.label[e]))) return rc;
      if ((rc = bring(data[v], &tab.data[e]))) return rc;
    }
    if (smooth && smooth[v] && (rc = bring(smooth[v], &tab.smooth[e]))) return rc;
  }
  hmf::Geometry G{vx, vy, vz, vx, (long long)vx * vy, (long long)V};
  return launch_energy(c, tab, G, f0, f, n_nodes, s, nullptr);
}

int hmf_batch_get_vote(hmf_ctx* c, int volume, int* out, int where, void* stream) {
  if (!c) return HMF_ERR_INVALID_ARGUMENT;
  if (int rc = refuse_paged(c, "hmf_get_vote")) return rc;
  if (!valid_volume(c, volume)) return fail(c, HMF_ERR_INVALID_ARGUMENT, "volume index out of range");
  if (!out) return fail(c, HMF_ERR_INVALID_ARGUMENT, "output pointer is NULL");
  if (where != HMF_HOST && where != HMF_DEVICE) return fail(c, HMF_ERR_INVALID_ARGUMENT, "bad `where`");
  if (!c->solved) return fail(c, HMF_ERR_STATE, "hmf_solve has not run");
  DeviceGuard dg(c->device);
  if (where == HMF_DEVICE)
    if (int rc = check_device_pointer(c, out, "vote output")) return rc;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  const auto& V = c->vols[volume];
  hmf::VoteInputs in;
  std::memset(&in, 0, sizeof(in));
  in.n = (int)c->leaves.size();
  in.semantics = c->semantics == HMF_SEMANTICS_REF_CPU ? 1 : 0;
  for (int j = 0; j < in.n; ++j) {
    in.in[j] = c->label[c->leaves[j]] + V.off;
    in.values[j] = c->leaves[j];
  }
  hmf::Geometry G{V.vx, V.vy, V.vz, V.pitch, V.plane, V.vol};
  const size_t dense = (size_t)V.vx * V.vy * V.vz;
  int* dout = out;
  void* tmp = nullptr;
  if (where == HMF_HOST) {
    CK(cudaMalloc(&tmp, sizeof(int) * dense), "cudaMalloc(vote output)");
    dout = static_cast<int*>(tmp);
  }
  int rc = launch_vote(c, in, G, dout, s);
  if (rc) {
    if (tmp) cudaFree(tmp);
    return rc;
  }
  if (where == HMF_HOST) {
    cudaError_t e = cudaMemcpyAsync(out, dout, sizeof(int) * dense, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    cudaFree(tmp);
    if (e != cudaSuccess) return cuda_fail(c, e, "vote output copy");
    return check_error_flag(c);
  }
  return HMF_OK;
}

int hmf_get_vote(hmf_ctx* c, int* out, int where, void* stream) { return hmf_batch_get_vote(c, 0, out, where, stream); }

int hmf_batch_get_energy(hmf_ctx* c, int volume, double* f0, double* f, int n) {
  if (!c) return HMF_ERR_INVALID_ARGUMENT;
  if (int rc = refuse_paged(c, "hmf_get_energy")) return rc;
  if (!valid_volume(c, volume)) return fail(c, HMF_ERR_INVALID_ARGUMENT, "volume index out of range");
  if (c->dag) return fail(c, HMF_ERR_INVALID_ARGUMENT, "the energy decomposition is defined for trees, not graphs");
  if (!c->solved) return fail(c, HMF_ERR_STATE, "hmf_solve has not run");
  DeviceGuard dg(c->device);
  hmf::EnergyTable tab;
  std::vector<int> entry;
  int rc = energy_tree(c, c->parent.data(), c->n, tab, entry);
  if (rc) return rc;
  const auto& V = c->vols[volume];
  for (int v = 0; v < c->n; ++v) {
    const int e = entry[v];
    if (e < 0) continue;
    if (tab.n_kids[e] == 0) {
      tab.label[e] = c->label[v] + V.off;
      tab.data[e] = c->st_data[v] + V.off;
    }
    if (c->st_smooth[v] && c->smooth[volume][v].ptr) tab.smooth[e] = c->st_smooth[v] + V.off;
  }
  hmf::Geometry G{V.vx, V.vy, V.vz, V.pitch, V.plane, V.vol};
  std::vector<double> fv(c->n, 0.0);
  if (!c->d_post) CK(cudaMalloc(&c->d_post, kEnergyBuffer), "cudaMalloc(energy buffer)");
  rc = launch_energy(c, tab, G, f0, fv.data(), c->n, c->stream, c->d_post);
  if (rc) return rc;
  for (int v = 0; v < n && v < c->n && f; ++v) f[v] = fv[v];
  return c->n;
}

int hmf_get_energy(hmf_ctx* c, double* f0, double* f, int n) { return hmf_batch_get_energy(c, 0, f0, f, n); }

}  // extern "C"
