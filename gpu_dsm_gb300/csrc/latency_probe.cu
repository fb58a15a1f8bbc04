// Latency probe of the operations on the step kernel's event path (sm_103a).
//
// One warp runs dependent chains of each operation and times them with
// clock64(); the result is cycles per operation (latency for the dependent
// chains, issue cost for the independent ones).  Built and run by
// gpu_dsm_gb300/phases.py --probe; not part of libgpudsm.so.
//
// Every access stays inside its buffer: the shared chase indexes a 256-entry
// array with values below 256, the global chase a 1024-entry array with values
// below 1024.  No loop waits on anything but its own count.
#include <cstdio>
#include <cuda_runtime.h>

namespace {

constexpr int N = 512;   // chain length of the single-precision and integer probes
constexpr int ND = 64;   // chain length of the FP64 probes

// the step kernel's 32-bit form of llrint (dsm_kernels.cu, f2u64_rn)
__device__ __forceinline__ unsigned long long f2u64_rn(float y) {
  const unsigned b = __float_as_uint(y) & 0x7fffffffu;
  const int e = (int)(b >> 23) - 150;
  const unsigned small = __float_as_uint(__fadd_rn(__uint_as_float(b), 8388608.0f)) - 0x4B000000u;
  const unsigned long long big = (unsigned long long)((b & 0x7fffffu) | 0x800000u) << (e & 63);
  return e < 0 ? (unsigned long long)small : big;
}

struct Probe {
  const char* name;
  int ops;
};

constexpr Probe kProbes[] = {
    {"fadd (dependent)", N},
    {"ffma (dependent)", N},
    {"u64 add + shift (dependent)", N},
    {"float -> int64 conversion, hardware (+1 int op)", N},
    {"float -> u64, 32-bit form f2u64_rn (+1 int op)", N},
    {"int64 -> float conversion, hardware (+1 shift)", N},
    {"float -> int64 hardware, 8 independent per step", N},
    {"float -> u64 32-bit form, 8 independent per step", N},
    {"shfl (full warp)", N},
    {"shfl (16-lane tile, width 16)", N},
    {"shared load chase", N},
    {"global load chase, L1 hit", N},
    {"fdiv_rn (+fadd)", N},
    {"ballot (+add)", N},
    {"umul64hi (+or, add)", N},
    {"syncwarp (+add)", N},
    {"fp64 add (dependent)", ND},
    {"fp64 fma (dependent)", ND},
    {"fp64 div_rn (+fp64 add)", ND},
};
constexpr int kNumProbes = sizeof(kProbes) / sizeof(kProbes[0]);

__global__ void probe(const int* __restrict__ gtab, long long* out, float seedf, int seedi) {
  __shared__ int stab[256];
  const int lane = threadIdx.x;
  for (int i = lane; i < 256; i += 32) stab[i] = (i * 97 + 13) & 255;
  __syncwarp();
  float x = seedf + lane;
  int k = seedi + lane;
  unsigned long long u = (unsigned long long)(seedi + 3) << 20;
  double dd = (double)seedf + lane;
  long long t0, t1;
  int slot = 0;
#define PROBE(mask, body)                   \
  __syncwarp(mask);                         \
  t0 = clock64();                           \
  body;                                     \
  t1 = clock64();                           \
  if (lane == 0) out[slot] = t1 - t0;       \
  ++slot;
#define PROBE_ALL(body) PROBE(0xffffffffu, body)
  PROBE_ALL(for (int i = 0; i < N; ++i) x = __fadd_rn(x, 1.0f));
  PROBE_ALL(for (int i = 0; i < N; ++i) x = __fmaf_rn(x, 0.999f, 1.0f));
  PROBE_ALL(for (int i = 0; i < N; ++i) u = u + (u >> 7) + 1);
  PROBE_ALL(for (int i = 0; i < N; ++i) x = __int_as_float(__float_as_int(x) ^ (int)(__float2ll_rn(x) & 1)));
  PROBE_ALL(for (int i = 0; i < N; ++i) x = __int_as_float(__float_as_int(x) ^ (int)(f2u64_rn(x) & 1)));
  PROBE_ALL(for (int i = 0; i < N; ++i) u = (unsigned long long)__float_as_uint(__ll2float_rn((long long)u)) << 20);
  {
    float y0 = x, y1 = x + 1, y2 = x + 2, y3 = x + 3, y4 = x + 4, y5 = x + 5, y6 = x + 6, y7 = x + 7;
    long long s = 0;
    PROBE_ALL(for (int i = 0; i < N / 8; ++i) {
      s += __float2ll_rn(y0) + __float2ll_rn(y1) + __float2ll_rn(y2) + __float2ll_rn(y3) + __float2ll_rn(y4) +
           __float2ll_rn(y5) + __float2ll_rn(y6) + __float2ll_rn(y7);
      y0 = __fadd_rn(y0, 1.0f); y1 = __fadd_rn(y1, 1.0f); y2 = __fadd_rn(y2, 1.0f); y3 = __fadd_rn(y3, 1.0f);
      y4 = __fadd_rn(y4, 1.0f); y5 = __fadd_rn(y5, 1.0f); y6 = __fadd_rn(y6, 1.0f); y7 = __fadd_rn(y7, 1.0f);
    });
    k += (int)s;
  }
  {
    float y0 = x, y1 = x + 1, y2 = x + 2, y3 = x + 3, y4 = x + 4, y5 = x + 5, y6 = x + 6, y7 = x + 7;
    unsigned long long s = 0;
    PROBE_ALL(for (int i = 0; i < N / 8; ++i) {
      s += f2u64_rn(y0) + f2u64_rn(y1) + f2u64_rn(y2) + f2u64_rn(y3) + f2u64_rn(y4) + f2u64_rn(y5) + f2u64_rn(y6) +
           f2u64_rn(y7);
      y0 = __fadd_rn(y0, 1.0f); y1 = __fadd_rn(y1, 1.0f); y2 = __fadd_rn(y2, 1.0f); y3 = __fadd_rn(y3, 1.0f);
      y4 = __fadd_rn(y4, 1.0f); y5 = __fadd_rn(y5, 1.0f); y6 = __fadd_rn(y6, 1.0f); y7 = __fadd_rn(y7, 1.0f);
    });
    k += (int)s;
  }
  PROBE_ALL(for (int i = 0; i < N; ++i) k = __shfl_sync(0xffffffffu, k, (lane + 1) & 31));
  if (lane < 16) {
    PROBE(0x0000ffffu, for (int i = 0; i < N; ++i) k = __shfl_sync(0x0000ffffu, k, (lane + 1) & 15, 16));
  } else {
    ++slot;
  }
  PROBE_ALL(for (int i = 0; i < N; ++i) k = stab[k & 255]);
  PROBE_ALL(for (int i = 0; i < N; ++i) k = __ldg(&gtab[k & 1023]));
  PROBE_ALL(for (int i = 0; i < N; ++i) x = __fdiv_rn(1.0f, __fadd_rn(x, 1.5f)));
  PROBE_ALL(for (int i = 0; i < N; ++i) k = __ballot_sync(0xffffffffu, (k & 1) != 0) + lane);
  PROBE_ALL(for (int i = 0; i < N; ++i) u = __umul64hi(u, 0x9E3779B97F4A7C15ull) + (u | 1));
  PROBE_ALL(for (int i = 0; i < N; ++i) { __syncwarp(); k += 1; });
  PROBE_ALL(for (int i = 0; i < ND; ++i) dd = __dadd_rn(dd, 1.0));
  PROBE_ALL(for (int i = 0; i < ND; ++i) dd = __fma_rn(dd, 0.999, 1.0));
  PROBE_ALL(for (int i = 0; i < ND; ++i) dd = __ddiv_rn(1.0, __dadd_rn(dd, 1.5)));
#undef PROBE_ALL
#undef PROBE
  // keep every chain live
  if (lane == 0) out[kNumProbes] = (long long)k + (long long)u + (long long)__float_as_int(x) + (long long)dd;
}

}  // namespace

int main() {
  int* gtab = nullptr;
  long long* out = nullptr;
  if (cudaMalloc(&gtab, 1024 * sizeof(int)) != cudaSuccess || cudaMalloc(&out, 64 * sizeof(long long)) != cudaSuccess) {
    std::printf("{\"error\": \"cudaMalloc\"}\n");
    return 1;
  }
  int h[1024];
  for (int i = 0; i < 1024; ++i) h[i] = (i * 389 + 7) & 1023;
  cudaMemcpy(gtab, h, sizeof(h), cudaMemcpyHostToDevice);
  cudaMemset(out, 0, 64 * sizeof(long long));
  for (int rep = 0; rep < 3; ++rep) {  // the last repetition runs warm
    probe<<<1, 32>>>(gtab, out, 1.25f, 5);
    const cudaError_t e = cudaDeviceSynchronize();
    if (e != cudaSuccess) {
      std::printf("{\"error\": \"%s\"}\n", cudaGetErrorString(e));
      return 1;
    }
  }
  long long r[64];
  cudaMemcpy(r, out, sizeof(r), cudaMemcpyDeviceToHost);
  std::printf("{");
  for (int i = 0; i < kNumProbes; ++i)
    std::printf("%s\"%s\": %.2f", i ? ", " : "", kProbes[i].name, (double)r[i] / kProbes[i].ops);
  std::printf("}\n");
  cudaFree(gtab);
  cudaFree(out);
  return 0;
}
