// Conformation statistics of the -distr files on the device (the reference
// computes them on the host with O(N_cha x range) loops, common/ensemble.cu:
// 356-484): histograms of Z over chains and of N over strands (block-private
// shared-memory counters, then one global add per bin), and the lengths |Q| of
// the internal strands sorted on the device (CUB radix sort) for the Q
// distribution.
#include <cstdint>
#include <vector>

#include <cub/device/device_radix_sort.cuh>
#include <cuda_runtime.h>

#include "../../include/dsm.h"
#include "dsm_host.h"
#include "dsm_internal.h"

namespace {

using dsm::ChainState;
using dsm::EnsDev;

// One warp per chain: Z into hz[Z], N of every strand into hn[N]
__global__ void k_hist_zn(const EnsDev* __restrict__ ensp, unsigned long long* hz, unsigned long long* hn,
                          int zbins, int nbins) {
  extern __shared__ unsigned int sh[];
  const EnsDev& E = *ensp;
  unsigned int* sz = sh;
  unsigned int* sn = sh + zbins;
  for (int i = threadIdx.x; i < zbins + nbins; i += blockDim.x) sh[i] = 0u;
  __syncthreads();
  const int lane = threadIdx.x & 31, wpb = blockDim.x >> 5;
  for (int c = blockIdx.x * wpb + (threadIdx.x >> 5); c < E.n_chains; c += gridDim.x * wpb) {
    const int Z = E.cs[c].Z;
    if (lane == 0 && Z >= 0 && Z < zbins) atomicAdd(&sz[Z], 1u);
    const float4* q = E.QN + (size_t)c * E.cap;
    for (int s = lane; s < Z; s += 32) {
      const int n = (int)q[s].w;
      if (n >= 0 && n < nbins) atomicAdd(&sn[n], 1u);
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < zbins; i += blockDim.x)
    if (sz[i]) atomicAdd(&hz[i], (unsigned long long)sz[i]);
  for (int i = threadIdx.x; i < nbins; i += blockDim.x)
    if (sn[i]) atomicAdd(&hn[i], (unsigned long long)sn[i]);
}

// |Q| of the internal strands 1..Z-2 of chain c at out[off[c] ..]
// (ensemble.cu:439-455: the dangling end strands have no vector)
__global__ void k_qlen(const EnsDev* __restrict__ ensp, const long long* __restrict__ off, float* out) {
  const EnsDev& E = *ensp;
  const int lane = threadIdx.x & 31, wpb = blockDim.x >> 5;
  for (int c = blockIdx.x * wpb + (threadIdx.x >> 5); c < E.n_chains; c += gridDim.x * wpb) {
    const int Z = E.cs[c].Z;
    const float4* q = E.QN + (size_t)c * E.cap;
    for (int s = 1 + lane; s < Z - 1; s += 32) {
      const float4 v = q[s];
      out[off[c] + s - 1] = __fsqrt_rn(__fmaf_rn(v.z, v.z, __fmaf_rn(v.y, v.y, __fmul_rn(v.x, v.x))));
    }
  }
}

int fail(dsm_sim* s, int code, const char* msg) {
  if (s) s->err = msg;
  return code;
}

}  // namespace

#define CKD(call)                                                            \
  do {                                                                       \
    cudaError_t e_ = (call);                                                 \
    if (e_ != cudaSuccess) return fail(s, DSM_ERR_CUDA, cudaGetErrorString(e_)); \
  } while (0)

extern "C" int dsm_zn_hist(dsm_sim* s, uint64_t* z_counts, int32_t z_bins, uint64_t* n_counts, int32_t n_bins) {
  if (!s || !s->ready || z_bins < 1 || n_bins < 1 || !z_counts || !n_counts) return DSM_ERR_INVALID;
  const size_t shm = (size_t)(z_bins + n_bins) * sizeof(unsigned int);
  if (shm > 200 * 1024) return fail(s, DSM_ERR_INVALID, "histogram ranges too large for shared memory");
  unsigned long long* d = nullptr;
  CKD(cudaMallocAsync((void**)&d, (size_t)(z_bins + n_bins) * sizeof(unsigned long long), s->st));
  CKD(cudaMemsetAsync(d, 0, (size_t)(z_bins + n_bins) * sizeof(unsigned long long), s->st));
  // one fixed limit (the attribute is process-wide; threads must not lower it)
  if (shm > 48 * 1024)
    CKD(cudaFuncSetAttribute((const void*)k_hist_zn, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
  const int grid = s->sm_count * 2;
  k_hist_zn<<<grid, 256, shm, s->st>>>(s->d_ens, d, d + z_bins, z_bins, n_bins);
  CKD(cudaGetLastError());
  CKD(cudaMemcpyAsync(z_counts, d, (size_t)z_bins * sizeof(uint64_t), cudaMemcpyDeviceToHost, s->st));
  CKD(cudaMemcpyAsync(n_counts, d + z_bins, (size_t)n_bins * sizeof(uint64_t), cudaMemcpyDeviceToHost, s->st));
  CKD(cudaFreeAsync(d, s->st));
  CKD(cudaStreamSynchronize(s->st));
  return DSM_OK;
}

extern "C" int dsm_q_sorted(dsm_sim* s, float* q, int64_t* n) {
  if (!s || !s->ready || !n) return DSM_ERR_INVALID;
  const int nc = s->P.n_chains;
  std::vector<ChainState> cs(nc);
  CKD(cudaMemcpyAsync(cs.data(), s->d_cs, (size_t)nc * sizeof(ChainState), cudaMemcpyDeviceToHost, s->st));
  CKD(cudaStreamSynchronize(s->st));
  std::vector<long long> off(nc);
  long long tot = 0;
  for (int i = 0; i < nc; ++i) {
    off[i] = tot;
    tot += cs[i].Z > 2 ? cs[i].Z - 2 : 0;
  }
  if (!q) { *n = tot; return DSM_OK; }
  if (*n < tot) { *n = tot; return fail(s, DSM_ERR_INVALID, "output capacity too small"); }
  *n = tot;
  if (tot == 0) return DSM_OK;
  long long* d_off = nullptr;
  float *d_a = nullptr, *d_b = nullptr;
  void* d_tmp = nullptr;
  size_t tmp = 0;
  CKD(cub::DeviceRadixSort::SortKeys(nullptr, tmp, d_a, d_b, (int)tot, 0, 32, s->st));
  CKD(cudaMallocAsync((void**)&d_off, (size_t)nc * sizeof(long long), s->st));
  CKD(cudaMallocAsync((void**)&d_a, (size_t)tot * sizeof(float), s->st));
  CKD(cudaMallocAsync((void**)&d_b, (size_t)tot * sizeof(float), s->st));
  CKD(cudaMallocAsync(&d_tmp, tmp, s->st));
  CKD(cudaMemcpyAsync(d_off, off.data(), (size_t)nc * sizeof(long long), cudaMemcpyHostToDevice, s->st));
  k_qlen<<<s->sm_count * 4, 256, 0, s->st>>>(s->d_ens, d_off, d_a);
  CKD(cudaGetLastError());
  CKD(cub::DeviceRadixSort::SortKeys(d_tmp, tmp, d_a, d_b, (int)tot, 0, 32, s->st));
  CKD(cudaMemcpyAsync(q, d_b, (size_t)tot * sizeof(float), cudaMemcpyDeviceToHost, s->st));
  for (void* p : {(void*)d_off, (void*)d_a, (void*)d_b, d_tmp}) cudaFreeAsync(p, s->st);
  CKD(cudaStreamSynchronize(s->st));
  return DSM_OK;
}
