// ORACLE — test infrastructure only.  Nothing in the product includes this file.
//
// Host stand-ins for the CUDA constructs used by the reference's two kernel
// files, common/ensemble_kernel.cu and common/eq_ensemble_kernel.cu of
// ktaletsk/gpu_dsm, so that those files compile unchanged with g++ and their
// kernels run on the CPU (oracle/ref_step.cpp drives them).  This directory is
// put first on the include path, so the reference's `#include "cuda_runtime.h"`
// (eq_ensemble_kernel.cu:22) finds this header and no CUDA header is used.
//
// What each construct becomes:
//  * __global__/__device__/__constant__/__launch_bounds__: nothing; kernels are
//    plain functions that the host loop calls once per (block, thread) index,
//    with blockDim = 1 so that blockIdx carries the thread's index.
//  * texture<T,2,...> references (common/textures_surfaces.h:28-36): a 2-D
//    host array bound by the host loop; tex2D does point sampling at the
//    unnormalised coordinate with clamp addressing, as the reference's
//    textures do by default.  The three random-number textures are bound to
//    hooks instead, which hand out the oracle's shared random stream.
//  * surface<void,2> references (textures_surfaces.h:31,38-44): a 2-D byte
//    array; surf2Dwrite/surf2Dread address x in bytes.  An access out of
//    range, which traps on a GPU, is recorded in refshim_error and skipped.
//  * __fdividef/__powf/__expf/__fsqrt_rn: IEEE single-precision a/b, powf,
//    expf, sqrtf from the host libm (the GPU's approximate intrinsics have no
//    host definition); the oracle's reference-arithmetic mode uses the same.
//  * fdivide(a, b): called at eq_ensemble_kernel.cu:395 but defined nowhere
//    in the reference tree; here (float)(a / b) with the division in double,
//    the precision of its double argument sumW.
#pragma once
#include <cmath>
#include <cstddef>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <sys/types.h>

#define __global__
#define __device__
#define __host__
#define __constant__
#define __shared__
#define __forceinline__ inline
#define __launch_bounds__(...)

struct float2 { float x, y; };
struct alignas(16) float4 { float x, y, z, w; };
struct uint3 { unsigned int x, y, z; };
struct dim3 {
  unsigned int x, y, z;
  dim3(unsigned int a = 1, unsigned int b = 1, unsigned int c = 1) : x(a), y(b), z(c) {}
};
inline float2 make_float2(float x, float y) { return float2{x, y}; }
inline float4 make_float4(float x, float y, float z, float w) { return float4{x, y, z, w}; }

// thread indices of the kernel call in progress (set by the host loop)
extern uint3 threadIdx, blockIdx;
extern dim3 blockDim, gridDim;

// first out-of-range surface access since the last reset (0: none)
extern int refshim_error;

enum cudaTextureReadMode { cudaReadModeElementType = 0 };
struct cudaArray;
struct cudaPitchedPtr {
  void* ptr;
  size_t pitch, xsize, ysize;
};

template <class T, int dim = 1, cudaTextureReadMode mode = cudaReadModeElementType>
struct texture {
  const T* data = nullptr;       // row-major, height rows of width elements
  int width = 0, height = 0;
  T (*hook)(int x, int y) = nullptr;  // element source for the random textures
};

template <class T, int d, cudaTextureReadMode m>
inline T tex2D(const texture<T, d, m>& t, float x, float y) {
  int ix = (int)std::floor(x), iy = (int)std::floor(y);
  if (t.hook) return t.hook(ix, iy);
  if (ix < 0) ix = 0;
  if (ix >= t.width) ix = t.width - 1;
  if (iy < 0) iy = 0;
  if (iy >= t.height) iy = t.height - 1;
  return t.data[(size_t)iy * t.width + ix];
}

template <class T, int dim>
struct surface {
  unsigned char* data = nullptr;  // row-major, height rows of width_bytes bytes
  int width_bytes = 0, height = 0;
};

template <class T, class V>
inline void surf2Dwrite(T val, surface<V, 2>& s, int xb, int y) {
  if (xb < 0 || y < 0 || y >= s.height || xb + (int)sizeof(T) > s.width_bytes) {
    if (!refshim_error) refshim_error = 1;
    return;
  }
  std::memcpy(s.data + (size_t)y * s.width_bytes + xb, &val, sizeof(T));
}

template <class T, class V>
inline void surf2Dread(T* out, surface<V, 2>& s, int xb, int y) {
  if (xb < 0 || y < 0 || y >= s.height || xb + (int)sizeof(T) > s.width_bytes) {
    if (!refshim_error) refshim_error = 2;
    std::memset(out, 0, sizeof(T));
    return;
  }
  std::memcpy(out, s.data + (size_t)y * s.width_bytes + xb, sizeof(T));
}

template <class T, class V>
inline void surf1Dwrite(T val, surface<V, 1>& s, int xb) {
  if (xb < 0 || xb + (int)sizeof(T) > s.width_bytes) {
    if (!refshim_error) refshim_error = 3;
    return;
  }
  std::memcpy(s.data + xb, &val, sizeof(T));
}

inline float __fdividef(float a, float b) { return a / b; }
inline float __powf(float a, float b) { return powf(a, b); }
inline float __expf(float a) { return expf(a); }
inline float __fsqrt_rn(float a) { return sqrtf(a); }
inline float fdivide(float a, double b) { return (float)((double)a / b); }
