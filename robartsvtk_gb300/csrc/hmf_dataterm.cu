// hmf_dataterm.cu -- the data-term producers that precede a solve:
//
//  hmf_data_term       vtkImageDataTerm (Common/vtkRobartsCommon/vtkImageDataTerm.cxx:62-470):
//                      per voxel a constant, logistic, Gaussian or spike cost
//                      of one or two images, as a probability or an entropy,
//                      optionally normalised by the first image's range.
//  hmf_log_likelihood  vtkImageLogLikelihood (vtkImageLogLikelihood.cxx:140-250):
//                      a histogram of the image over the voxels that enough
//                      label maps mark with one label, and per voxel the
//                      negative log of its bin's frequency.
//
// Both evaluate the reference's expressions in its precision (double for the
// data term, float for the histogram) and order of operations (the library is
// built without contraction, as the reference's x86 build computes), with
// CUDA's double exp / log where the reference calls the C library's.  Images
// are float32 (the reference templates over VTK scalar types and writes the
// input's type; a float cost is what the solver takes).
#include <cuda_runtime.h>

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <initializer_list>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/hmf.h"
#include "hmf_ctx.hpp"

using namespace hmfi;

namespace {

constexpr int kThreads = 256;

int grid_for(long long n) {
  int dev = 0, sms = 148;
  if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const long long blocks = (n + kThreads - 1) / kThreads;
  return (int)std::max<long long>(1, std::min<long long>(blocks, (long long)sms * 16));
}

// Order-preserving map of a float to an unsigned int (for atomic min / max).
__device__ __forceinline__ unsigned int float_key(float f) {
  const unsigned int u = __float_as_uint(f);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__host__ __device__ inline float key_float(unsigned int k) {
  const unsigned int u = (k & 0x80000000u) ? (k & 0x7fffffffu) : ~k;
#ifdef __CUDA_ARCH__
  return __uint_as_float(u);
#else
  float f;
  std::memcpy(&f, &u, sizeof(f));
  return f;
#endif
}

// mm[0] = key of the minimum, mm[1] = key of the maximum (NaN skipped, as
// vtkDataArray's range ignores it).
__global__ void range_kernel(const float* __restrict__ in, long long n, unsigned int* mm) {
  unsigned int lo = 0xffffffffu, hi = 0u;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const float v = in[i];
    if (v != v) continue;
    const unsigned int k = float_key(v);
    lo = min(lo, k);
    hi = max(hi, k);
  }
  for (int s = 16; s > 0; s >>= 1) {
    lo = min(lo, __shfl_down_sync(0xffffffffu, lo, s));
    hi = max(hi, __shfl_down_sync(0xffffffffu, hi, s));
  }
  if ((threadIdx.x & 31) == 0) {
    atomicMin(&mm[0], lo);
    atomicMax(&mm[1], hi);
  }
}

struct TermParams {
  int op, entropy, two;
  double k1, c1, k2, c2;
  int normalize;
  double off, mul;
};

// vtkImageDataTermExecute1 (:62-249) and vtkImageDataTermExecute2 (:255-390).
__global__ void data_term_kernel(const TermParams P, const float* __restrict__ in1, const float* __restrict__ in2,
                                 long long n, float* __restrict__ out) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const double x1 = (double)in1[i];
    double v;
    if (P.op == HMF_DATA_TERM_CONSTANT) {
      v = P.c1;
    } else if (P.op == HMF_DATA_TERM_LOGISTIC) {
      const double a = 1.0 + exp(-(P.k1 * (x1 - P.c1)));
      if (P.two) {
        const double b = 1.0 + exp(-(P.k2 * ((double)in2[i] - P.c2)));
        v = P.entropy ? log(a * b) : 1.0 / (a * b);
      } else {
        v = P.entropy ? log(a) : 1.0 / a;
      }
    } else if (P.op == HMF_DATA_TERM_GAUSSIAN) {
      const double q1 = (x1 - P.c1) / P.k1;
      if (P.two) {
        const double q2 = ((double)in2[i] - P.c2) / P.k2;
        v = P.entropy ? 0.5 * q1 * q1 + 0.5 * q2 * q2 : exp(-0.5 * q1 * q1 - 0.5 * (q2 * q2));
      } else {
        v = P.entropy ? 0.5 * q1 * q1 : exp(-0.5 * q1 * q1);
      }
    } else {  // spike (one image)
      v = (x1 == P.k1) ? P.c1 : P.c2;
    }
    float o = (float)v;
    if (P.normalize) o = (float)(((double)o + P.off) * P.mul);
    out[i] = o;
  }
}

struct LLParams {
  int comps, n_maps, actual_maps, label_id;
  int min_agree;  // smallest agreeing count k with (double)k >= agreement * (double)actual_maps
  float resolution;
};

struct LLMaps {
  const int* map[HMF_MAX_LABEL_MAPS];
};

// A seed: enough label maps mark voxel i with the label.  The reference's
// test, (double)agree >= agreement * (double)actual_maps, is monotone in the
// integer count, so the host turns it into the threshold min_agree.
__device__ __forceinline__ bool ll_sample(const LLParams& P, const LLMaps& M, long long i) {
  int agree = 0;
  for (int k = 0; k < P.n_maps; ++k)
    if (M.map[k] && M.map[k][i] == P.label_id) ++agree;
  return agree >= P.min_agree;
}

// sums: [0] samples; keys: [0..1] min, [2..3] max per component
__global__ void ll_scan_kernel(const LLParams P, const LLMaps M, const float* __restrict__ img, long long n,
                               unsigned long long* count, unsigned int* keys) {
  unsigned long long c = 0;
  unsigned int lo0 = 0xffffffffu, lo1 = 0xffffffffu, hi0 = 0u, hi1 = 0u;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    if (!ll_sample(P, M, i)) continue;
    ++c;
    const unsigned int k0 = float_key(img[P.comps * i]);
    lo0 = min(lo0, k0);
    hi0 = max(hi0, k0);
    if (P.comps == 2) {
      const unsigned int k1 = float_key(img[2 * i + 1]);
      lo1 = min(lo1, k1);
      hi1 = max(hi1, k1);
    }
  }
  for (int s = 16; s > 0; s >>= 1) {
    c += __shfl_down_sync(0xffffffffu, c, s);
    lo0 = min(lo0, __shfl_down_sync(0xffffffffu, lo0, s));
    hi0 = max(hi0, __shfl_down_sync(0xffffffffu, hi0, s));
    lo1 = min(lo1, __shfl_down_sync(0xffffffffu, lo1, s));
    hi1 = max(hi1, __shfl_down_sync(0xffffffffu, hi1, s));
  }
  if ((threadIdx.x & 31) == 0) {
    if (c) atomicAdd(count, c);
    atomicMin(&keys[0], lo0);
    atomicMin(&keys[1], lo1);
    atomicMax(&keys[2], hi0);
    atomicMax(&keys[3], hi1);
  }
}

struct Hist {
  float mn0, mn1;
  int sz0, sz1;
};

__device__ __forceinline__ int ll_bin(float x, float mn, float res) { return (int)((x - mn) / res); }

__device__ __forceinline__ int ll_seed_bin(const LLParams& P, const Hist& H, const float* __restrict__ img,
                                           long long i) {
  int b = ll_bin(img[P.comps * i], H.mn0, P.resolution);
  if (P.comps == 2) b = b * H.sz1 + ll_bin(img[2 * i + 1], H.mn1, P.resolution);
  return b;  // < bins: the host checked the seeds' range against the bin counts
}

// Histograms of up to kSharedBins bins (48 KB, the default dynamic shared
// memory limit): each CTA counts its voxels in shared memory and adds its non-zero bins to the global histogram once (integer
// counts, so the totals do not depend on the order).
constexpr int kSharedBins = 12288;
__global__ void ll_hist_shared_kernel(const LLParams P, const LLMaps M, const Hist H, const float* __restrict__ img,
                                      long long n, int bins, unsigned int* hist) {
  extern __shared__ unsigned int sh[];  // bins entries
  for (int b = threadIdx.x; b < bins; b += blockDim.x) sh[b] = 0u;
  __syncthreads();
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    if (ll_sample(P, M, i)) atomicAdd(&sh[ll_seed_bin(P, H, img, i)], 1u);
  __syncthreads();
  for (int b = threadIdx.x; b < bins; b += blockDim.x) {
    const unsigned int v = sh[b];
    if (v) atomicAdd(&hist[b], v);
  }
}

// Larger histograms: global atomics.
__global__ void ll_hist_kernel(const LLParams P, const LLMaps M, const Hist H, const float* __restrict__ img,
                               long long n, unsigned int* hist) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    if (ll_sample(P, M, i)) atomicAdd(&hist[ll_seed_bin(P, H, img, i)], 1u);
}

// The cost of a voxel depends on its bin only, so it is evaluated once per
// bin: frequency hist[i] / (float)szSample + 1.0e-10 (the counts kept as the
// reference's float increments keep them: they stop growing at 2^24), cost
// -log(frequency), divided by the cost of an empty bin, -log(1.0e-10), when
// normalised.  cost[bins] is the cost of a voxel outside the histogram.
__global__ void ll_cost_kernel(const unsigned int* __restrict__ hist, int bins, unsigned long long samples,
                               int normalize, float* __restrict__ cost) {
  const double floor_cost = -log(1.0e-10);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i <= bins; i += gridDim.x * blockDim.x) {
    float o;
    if (i < bins) {
      const float cnt = (float)min(hist[i], 16777216u);
      const float freq = (float)((double)(cnt / (float)(int)samples) + 1.0e-10);
      o = (float)(-log((double)freq));
    } else {
      o = (float)floor_cost;
    }
    if (normalize) o = (float)((double)o / floor_cost);
    cost[i] = o;
  }
}

__global__ void ll_out_kernel(const LLParams P, const Hist H, const float* __restrict__ img,
                              const float* __restrict__ cost, int bins, long long n, float* __restrict__ out) {
  const float outside = cost[bins];
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const float x0 = img[P.comps * i];
    const int b0 = ll_bin(x0, H.mn0, P.resolution);
    float o;
    if (x0 < H.mn0 || b0 >= H.sz0) {
      o = outside;
    } else if (P.comps == 1) {
      o = cost[b0];
    } else {
      const float x1 = img[2 * i + 1];
      const int b1 = ll_bin(x1, H.mn1, P.resolution);
      o = (x1 < H.mn1 || b1 >= H.sz1) ? outside : cost[b0 * H.sz1 + b1];
    }
    out[i] = o;
  }
}

// Device copies of host inputs for one call.
// Scratch of one call, drawn from a memory pool of the library's own (one
// per device, keeping up to 256 MB between calls) and returned to it in
// stream order: no cudaMalloc / cudaFree per call, whose implicit device
// synchronisation would also stall the caller's other streams.
cudaMemPool_t scratch_pool() {
  static std::mutex mu;
  static std::map<int, cudaMemPool_t> pools;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return nullptr;
  std::lock_guard<std::mutex> lock(mu);
  auto it = pools.find(dev);
  if (it != pools.end()) return it->second;
  cudaMemPoolProps props;
  std::memset(&props, 0, sizeof(props));
  props.allocType = cudaMemAllocationTypePinned;
  props.location.type = cudaMemLocationTypeDevice;
  props.location.id = dev;
  cudaMemPool_t pool = nullptr;
  if (cudaMemPoolCreate(&pool, &props) != cudaSuccess) {
    cudaGetLastError();
    pool = nullptr;  // plain cudaMalloc then
  } else {
    unsigned long long keep = 256ull << 20;
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
  }
  pools[dev] = pool;
  return pool;
}

struct Scratch {
  explicit Scratch(cudaStream_t s) : stream(s), pool(scratch_pool()) {}
  cudaStream_t stream;
  cudaMemPool_t pool;
  std::vector<void*> bufs;
  ~Scratch() {
    for (void* p : bufs) pool ? cudaFreeAsync(p, stream) : cudaFree(p);
  }
  template <class T>
  cudaError_t alloc(T** out, size_t count) {
    void* p = nullptr;
    cudaError_t e = pool ? cudaMallocFromPoolAsync(&p, count * sizeof(T), pool, stream)
                         : cudaMalloc(&p, count * sizeof(T));
    if (e == cudaSuccess) bufs.push_back(p);
    *out = static_cast<T*>(p);
    return e;
  }
  template <class T>
  cudaError_t bring(const T* src, size_t count, int where, const T** dst, cudaStream_t s) {
    if (where == HMF_DEVICE) {
      *dst = src;
      return cudaSuccess;
    }
    T* d = nullptr;
    cudaError_t e = alloc(&d, count);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d, src, count * sizeof(T), cudaMemcpyHostToDevice, s);
    *dst = d;
    return e;
  }
};

hmf_ctx* const kNoCtx = nullptr;

}  // namespace

extern "C" {

int hmf_data_term(int op, int entropy, int normalize, double k1, double c1, double k2, double c2, const float* in1,
                  const float* in2, long long n_voxels, float* out, int where, void* stream) {
  hmf_ctx* c = kNoCtx;
  if (!in1 || !out || n_voxels < 1) return fail(c, HMF_ERR_INVALID_ARGUMENT, "an image or the output is missing");
  if (where != HMF_HOST && where != HMF_DEVICE) return fail(c, HMF_ERR_INVALID_ARGUMENT, "bad `where`");
  if (op < HMF_DATA_TERM_CONSTANT || op > HMF_DATA_TERM_SPIKE)
    return fail(c, HMF_ERR_INVALID_ARGUMENT, "unknown data-term operation");
  if (in2 && op == HMF_DATA_TERM_SPIKE)
    return fail(c, HMF_ERR_INVALID_ARGUMENT,
                "the spike operation takes one image (the reference's two-image form writes no output)");
  if (where == HMF_DEVICE)
    for (const void* q : {(const void*)in1, (const void*)in2, (const void*)out})
      if (int rc = check_device_pointer(c, q, "data-term buffer")) return rc;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  TermParams P{};
  P.op = op;
  P.entropy = entropy != 0;
  P.two = in2 != nullptr;
  P.k1 = k1;
  P.k2 = k2;
  // constants as Execute1 / Execute2 derive them (note: Execute1's second
  // constant is C1 unless it is a logarithm; Execute2 takes logarithms for
  // the constant operation only and never normalises)
  if (!P.two) {
    const bool lg = (op == HMF_DATA_TERM_CONSTANT || op == HMF_DATA_TERM_SPIKE) && P.entropy;
    P.c1 = lg ? -std::log(c1) : c1;
    P.c2 = lg ? -std::log(c2) : c1;
  } else {
    const bool lg = op == HMF_DATA_TERM_CONSTANT && P.entropy;
    P.c1 = lg ? -std::log(c1) : c1;
    P.c2 = lg ? -std::log(c2) : c2;
  }
  Scratch sc(s);
  const float* d1 = nullptr;
  const float* d2 = nullptr;
  float* dout = out;
  cudaError_t e = sc.bring(in1, (size_t)n_voxels, where, &d1, s);
  if (e == cudaSuccess && in2) e = sc.bring(in2, (size_t)n_voxels, where, &d2, s);
  if (e == cudaSuccess && where == HMF_HOST) e = sc.alloc(&dout, (size_t)n_voxels);
  if (e != cudaSuccess) return cuda_fail(c, e, "data-term input copy");
  if (normalize && !P.two) {
    // vtkImageDataTermExecute1's normalisation (:187-249) by the first image's range
    unsigned int* mm = nullptr;
    e = sc.alloc(&mm, 2);
    const unsigned int init[2] = {0xffffffffu, 0u};
    unsigned int h[2] = {0, 0};
    if (e == cudaSuccess) e = cudaMemcpyAsync(mm, init, sizeof(init), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) {
      range_kernel<<<grid_for(n_voxels), kThreads, 0, s>>>(d1, n_voxels, mm);
      e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(h, mm, sizeof(h), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cuda_fail(c, e, "data-term range");
    const double R0 = key_float(h[0]), R1 = key_float(h[1]);
    const double K1 = P.k1, C1 = P.c1;
    double off = 0.0, mul = 1.0 / C1;
    if (op == HMF_DATA_TERM_GAUSSIAN && P.entropy) {
      const double vmax = 0.5 * ((R1 - C1) / K1) * ((R1 - C1) / K1);
      const double vmin = 0.5 * ((R0 - C1) / K1) * ((R0 - C1) / K1);
      const double mx = (vmax >= vmin) ? vmax : vmin;
      double mn = (vmax < vmin) ? vmax : vmin;
      if (C1 > R0 && C1 < R1) mn = 0.0f;
      off = -mn;
      mul = 1.0 / (mx - mn);
    } else if (op == HMF_DATA_TERM_GAUSSIAN) {
      const double vmax = std::exp(-0.5 * ((R1 - C1) / K1) * ((R1 - C1) / K1));
      const double vmin = std::exp(-0.5 * ((R0 - C1) / K1) * ((R0 - C1) / K1));
      const double mn = std::exp(-((vmax >= vmin) ? vmax : vmin));
      double mx = std::exp(-((vmax < vmin) ? vmax : vmin));
      if (C1 > R0 && C1 < R1) mx = 1.0f;
      off = -mn;
      mul = 1.0 / (mx - mn);
    } else if (op == HMF_DATA_TERM_LOGISTIC && P.entropy) {
      const double vmax = std::log(1.0 + std::exp(-(K1 * (R1 - C1))));
      const double vmin = std::log(1.0 + std::exp(-(K1 * (R0 - C1))));
      const double mx = (vmax >= vmin) ? vmax : vmin;
      const double mn = (vmax < vmin) ? vmax : vmin;
      off = -mn;
      mul = 1.0 / (mx - mn);
    } else if (op == HMF_DATA_TERM_LOGISTIC) {
      const double vmax = 1.0 / (1.0 + std::exp(-(K1 * (R1 - C1))));
      const double vmin = 1.0 / (1.0 + std::exp(-(K1 * (R0 - C1))));
      const double mx = (vmax >= vmin) ? vmax : vmin;
      const double mn = (vmax < vmin) ? vmax : vmin;
      off = -mn;
      mul = 1.0 / (mx - mn);
    }
    P.normalize = 1;
    P.off = off;
    P.mul = mul;
  }
  data_term_kernel<<<grid_for(n_voxels), kThreads, 0, s>>>(P, d1, d2, n_voxels, dout);
  e = cudaGetLastError();
  if (e == cudaSuccess && where == HMF_HOST) {
    e = cudaMemcpyAsync(out, dout, sizeof(float) * (size_t)n_voxels, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  }
  if (e != cudaSuccess) return cuda_fail(c, e, "data_term_kernel");
  return HMF_OK;
}

int hmf_log_likelihood(const float* image, int components, const int* const* label_maps, int n_label_maps,
                       long long n_voxels, int label_id, float resolution, double required_agreement, int normalize,
                       float* out, int where, void* stream) {
  hmf_ctx* c = kNoCtx;
  if (!image || !out || n_voxels < 1) return fail(c, HMF_ERR_INVALID_ARGUMENT, "the image or the output is missing");
  if (where != HMF_HOST && where != HMF_DEVICE) return fail(c, HMF_ERR_INVALID_ARGUMENT, "bad `where`");
  if (components != 1 && components != 2)
    return fail(c, HMF_ERR_INVALID_ARGUMENT, "the image must have one or two components");
  if (n_label_maps < 0 || n_label_maps > HMF_MAX_LABEL_MAPS || (n_label_maps && !label_maps))
    return fail(c, HMF_ERR_INVALID_ARGUMENT, "bad label-map list");
  if (!(resolution >= FLT_MIN)) return fail(c, HMF_ERR_INVALID_ARGUMENT, "histogram resolution must be positive");
  if (!(required_agreement >= 0.0 && required_agreement <= 1.0))
    return fail(c, HMF_ERR_INVALID_ARGUMENT, "required agreement must lie in [0, 1]");
  if (where == HMF_DEVICE) {
    if (int rc = check_device_pointer(c, image, "log-likelihood image")) return rc;
    if (int rc = check_device_pointer(c, out, "log-likelihood output")) return rc;
    for (int k = 0; k < n_label_maps; ++k)
      if (int rc = check_device_pointer(c, label_maps[k], "label map")) return rc;
  }
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  LLParams P{};
  P.comps = components;
  P.n_maps = n_label_maps;
  P.label_id = label_id;
  P.resolution = resolution;
  LLMaps M{};
  Scratch sc(s);
  const float* img = nullptr;
  float* dout = out;
  cudaError_t e = sc.bring(image, (size_t)n_voxels * components, where, &img, s);
  for (int k = 0; k < n_label_maps && e == cudaSuccess; ++k) {
    if (!label_maps[k]) continue;
    ++P.actual_maps;
    e = sc.bring(label_maps[k], (size_t)n_voxels, where, &M.map[k], s);
  }
  P.min_agree = n_label_maps + 1;  // no count qualifies
  for (int k = 0; k <= n_label_maps; ++k)
    if ((double)k >= required_agreement * (double)P.actual_maps) {
      P.min_agree = k;
      break;
    }
  if (e == cudaSuccess && where == HMF_HOST) e = sc.alloc(&dout, (size_t)n_voxels);
  unsigned long long* cnt = nullptr;
  unsigned int* keys = nullptr;
  if (e == cudaSuccess) e = sc.alloc(&cnt, 1);
  if (e == cudaSuccess) e = sc.alloc(&keys, 4);
  if (e != cudaSuccess) return cuda_fail(c, e, "log-likelihood input copy");
  const unsigned int kinit[4] = {0xffffffffu, 0xffffffffu, 0u, 0u};
  e = cudaMemsetAsync(cnt, 0, sizeof(*cnt), s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(keys, kinit, sizeof(kinit), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) {
    ll_scan_kernel<<<grid_for(n_voxels), kThreads, 0, s>>>(P, M, img, n_voxels, cnt, keys);
    e = cudaGetLastError();
  }
  unsigned long long samples = 0;
  unsigned int hk[4] = {0, 0, 0, 0};
  if (e == cudaSuccess) e = cudaMemcpyAsync(&samples, cnt, sizeof(samples), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(hk, keys, sizeof(hk), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return cuda_fail(c, e, "log-likelihood scan");
  if (samples == 0) {
    // no seed voxel: every cost 1 (std::fill_n, vtkImageLogLikelihood.cxx:193-197)
    std::vector<float> ones;
    if (where == HMF_HOST) {
      for (long long i = 0; i < n_voxels; ++i) out[i] = 1.0f;
      return HMF_OK;
    }
    ones.assign((size_t)n_voxels, 1.0f);
    e = cudaMemcpyAsync(out, ones.data(), sizeof(float) * ones.size(), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cuda_fail(c, e, "log-likelihood output");
    return HMF_OK;
  }
  // min starts at FLT_MAX and max at FLT_MIN (:169-170), compared as floats
  Hist H{};
  float mn[2] = {FLT_MAX, FLT_MAX}, mx[2] = {FLT_MIN, FLT_MIN};
  for (int k = 0; k < components; ++k) {
    const float lo = key_float(hk[k]), hi = key_float(hk[2 + k]);
    mn[k] = (mn[k] < lo) ? mn[k] : lo;
    mx[k] = (mx[k] > hi) ? mx[k] : hi;
  }
  H.mn0 = mn[0];
  H.mn1 = mn[1];
  // the reference's bin counts, precedence as written: (int)(max - min/resolution) + 1
  const float s0 = mx[0] - mn[0] / resolution;
  if (!(s0 > -1.0f && s0 < 2.0e9f)) return fail(c, HMF_ERR_INVALID_ARGUMENT, "histogram size out of range");
  H.sz0 = (int)s0 + 1;
  H.sz1 = 1;
  if (components == 2) {
    const float s1 = mx[1] - mn[1] / resolution;
    if (!(s1 > -1.0f && s1 < 2.0e9f)) return fail(c, HMF_ERR_INVALID_ARGUMENT, "histogram size out of range");
    H.sz1 = (int)s1 + 1;
  }
  // the reference writes past its histogram when a seed's bin exceeds that
  // count (its bin count divides only the minimum by the resolution)
  if ((int)((mx[0] - mn[0]) / resolution) >= H.sz0 ||
      (components == 2 && (int)((mx[1] - mn[1]) / resolution) >= H.sz1))
    return fail(c, HMF_ERR_INVALID_ARGUMENT,
                "seed values span more bins than the reference's histogram holds "
                "((int)(max - min/resolution) + 1 bins): it would write past its histogram");
  const long long bins = (long long)H.sz0 * H.sz1;
  if (bins > (1LL << 28)) return fail(c, HMF_ERR_INVALID_ARGUMENT, "histogram of more than 2^28 bins");
  unsigned int* hist = nullptr;
  float* cost = nullptr;
  e = sc.alloc(&hist, (size_t)bins);
  if (e == cudaSuccess) e = sc.alloc(&cost, (size_t)bins + 1);
  if (e == cudaSuccess) e = cudaMemsetAsync(hist, 0, sizeof(unsigned int) * (size_t)bins, s);
  if (e == cudaSuccess) {
    if (bins <= kSharedBins)
      ll_hist_shared_kernel<<<grid_for(n_voxels), kThreads, sizeof(unsigned int) * (size_t)bins, s>>>(
          P, M, H, img, n_voxels, (int)bins, hist);
    else
      ll_hist_kernel<<<grid_for(n_voxels), kThreads, 0, s>>>(P, M, H, img, n_voxels, hist);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) {
    ll_cost_kernel<<<grid_for(bins + 1), kThreads, 0, s>>>(hist, (int)bins, samples, normalize != 0, cost);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) {
    ll_out_kernel<<<grid_for(n_voxels), kThreads, 0, s>>>(P, H, img, cost, (int)bins, n_voxels, dout);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess && where == HMF_HOST)
    e = cudaMemcpyAsync(out, dout, sizeof(float) * (size_t)n_voxels, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);  // the call is synchronous
  if (e != cudaSuccess) return cuda_fail(c, e, "log-likelihood kernels");
  return HMF_OK;
}

}  // extern "C"
