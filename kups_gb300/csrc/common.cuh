// Shared device helpers of the kups_gb300 kernels (sm_103a).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/kups_gb300.h"

#define KUPS_CUDA_TRY(expr)                      \
  do {                                           \
    cudaError_t _e = (expr);                     \
    if (_e != cudaSuccess) return KUPS_ERR_CUDA; \
  } while (0)

namespace kups {

// Multiprocessor count of the current device, looked up once per device.
inline int device_sm_count() {
  constexpr int kDevices = 64;
  static int sms[kDevices] = {};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) dev = 0;
  int n = dev >= 0 && dev < kDevices ? sms[dev] : 0;
  if (n <= 0) {
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) n = 1;
    if (dev >= 0 && dev < kDevices) sms[dev] = n;
  }
  return n;
}

// ----------------------------------------------------------------- status word
// First error wins; capacity errors keep the largest requirement seen.
__device__ inline void status_capacity(kups_status *st, int32_t which, int64_t required,
                                       int64_t first_bad) {
  if (st == nullptr) return;
  atomicCAS(reinterpret_cast<int *>(&st->code), KUPS_OK, KUPS_ERR_CAPACITY);
  if (st->code == KUPS_ERR_CAPACITY) {
    atomicExch(reinterpret_cast<int *>(&st->detail), which);
    atomicMax(reinterpret_cast<long long *>(&st->required), (long long)required);
    atomicCAS(reinterpret_cast<unsigned long long *>(&st->first_bad),
              (unsigned long long)(-1LL), (unsigned long long)first_bad);
  }
}

__device__ inline void status_error(kups_status *st, int32_t code, int64_t first_bad) {
  if (st == nullptr) return;
  if (atomicCAS(reinterpret_cast<int *>(&st->code), KUPS_OK, code) == KUPS_OK)
    atomicExch(reinterpret_cast<unsigned long long *>(&st->first_bad),
               (unsigned long long)first_bad);
}

// ----------------------------------------------------------------- float64 cell math
// Written with explicit _rn intrinsics so no fused multiply-add changes the
// rounding: the membership test d^2 < rc^2 must agree bit for bit with the
// float64 CPU restatement (same operation order).
struct Tril64 {
  double t[6];  // L00, L10, L11, L20, L21, L22
};

__device__ inline Tril64 load_tril64(const double *p) {
  Tril64 r;
#pragma unroll
  for (int k = 0; k < 6; ++k) r.t[k] = p[k];
  return r;
}

// Inverse of the lower-triangular lattice by forward substitution.
__device__ inline Tril64 inverse_tril64(const Tril64 &L) {
  const double a = L.t[0], b = L.t[1], c = L.t[2], d = L.t[3], e = L.t[4], f = L.t[5];
  Tril64 r;
  const double i00 = __ddiv_rn(1.0, a);
  const double i11 = __ddiv_rn(1.0, c);
  const double i22 = __ddiv_rn(1.0, f);
  const double i10 = __ddiv_rn(-__dmul_rn(b, i00), c);
  const double i21 = __ddiv_rn(-__dmul_rn(e, i11), f);
  const double i20 = __ddiv_rn(-__dadd_rn(__dmul_rn(d, i00), __dmul_rn(e, i10)), f);
  r.t[0] = i00; r.t[1] = i10; r.t[2] = i11; r.t[3] = i20; r.t[4] = i21; r.t[5] = i22;
  return r;
}

// y = x @ L for lower-triangular L.
__device__ inline void row_times_tril64(const double x[3], const Tril64 &L, double y[3]) {
  y[0] = __dadd_rn(__dadd_rn(__dmul_rn(x[0], L.t[0]), __dmul_rn(x[1], L.t[1])),
                   __dmul_rn(x[2], L.t[3]));
  y[1] = __dadd_rn(__dmul_rn(x[1], L.t[2]), __dmul_rn(x[2], L.t[4]));
  y[2] = __dmul_rn(x[2], L.t[5]);
}

__device__ inline double norm2_64(const double v[3]) {
  return __dadd_rn(__dadd_rn(__dmul_rn(v[0], v[0]), __dmul_rn(v[1], v[1])),
                   __dmul_rn(v[2], v[2]));
}

// Face-to-face widths V/|b x c|, V/|a x c|, V/|a x b| of the cell.
__device__ inline void perpendicular_widths64(const Tril64 &L, double w[3]) {
  const double L00 = L.t[0], L10 = L.t[1], L11 = L.t[2], L20 = L.t[3], L21 = L.t[4],
               L22 = L.t[5];
  const double v = fabs(L00 * L11 * L22);
  const double c0 = L11 * L22, c1 = L10 * L22, c2 = L10 * L21 - L11 * L20;
  const double bxc = sqrt(c0 * c0 + c1 * c1 + c2 * c2);
  const double axc = sqrt((L00 * L22) * (L00 * L22) + (L00 * L21) * (L00 * L21));
  const double axb = fabs(L00 * L11);
  w[0] = v / bxc;
  w[1] = v / axc;
  w[2] = v / axb;
}

// ----------------------------------------------------------------- Philox4x32-10
// Counter-based generator of Salmon, Moraes, Dror & Shaw, "Parallel random
// numbers: as easy as 1, 2, 3" (SC'11): 10 rounds of the Philox-4x32 bijection
// with the paper's multipliers and Weyl key increments.
struct U4 {
  uint32_t x, y, z, w;
};

__device__ inline U4 philox4x32_10(U4 ctr, uint32_t k0, uint32_t k1) {
  const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u;
  const uint32_t W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    const uint32_t hi0 = __umulhi(M0, ctr.x), lo0 = M0 * ctr.x;
    const uint32_t hi1 = __umulhi(M1, ctr.z), lo1 = M1 * ctr.z;
    U4 n;
    n.x = hi1 ^ ctr.y ^ k0;
    n.y = lo1;
    n.z = hi0 ^ ctr.w ^ k1;
    n.w = lo0;
    ctr = n;
    k0 += W0;
    k1 += W1;
  }
  return ctr;
}

// Uniform in (0, 1] from 32 random bits.
__device__ inline float u01_open0(uint32_t v) {
  return (float)(v >> 8) * (1.0f / 16777216.0f) + (1.0f / 16777216.0f);
}

// Four standard normals by the Box-Muller transform.
__device__ inline void normal4(uint64_t seed, uint64_t stream, uint64_t counter, float out[4]) {
  U4 c{(uint32_t)counter, (uint32_t)(counter >> 32), (uint32_t)stream, (uint32_t)(stream >> 32)};
  U4 r = philox4x32_10(c, (uint32_t)seed, (uint32_t)(seed >> 32));
  const float u1 = u01_open0(r.x), u2 = u01_open0(r.y);
  const float u3 = u01_open0(r.z), u4 = u01_open0(r.w);
  const float m1 = sqrtf(-2.0f * logf(u1)), m2 = sqrtf(-2.0f * logf(u3));
  float s1, c1, s2, c2;
  sincospif(2.0f * u2, &s1, &c1);
  sincospif(2.0f * u4, &s2, &c2);
  out[0] = m1 * c1;
  out[1] = m1 * s1;
  out[2] = m2 * c2;
  out[3] = m2 * s2;
}

// ----------------------------------------------------------------- reductions
__device__ inline double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__device__ inline float warp_sum(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// erfc(x) for x >= 0 by the Chebyshev-fitted formula of Numerical Recipes in C, 2nd ed.,
// section 6.2 ("erfcc"): t = 1 / (1 + x / 2), erfc(x) = t exp(-x^2 + P(t)) with a degree-9
// polynomial P; fractional error below 1.2e-7 everywhere in exact arithmetic (float32
// evaluation adds a few ulp plus |x^2| * 2^-24 through the exponential).  One reciprocal,
// nine FMAs and one fast exponential.
__device__ __forceinline__ float erfc_cheb(float x) {
  float t;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(t) : "f"(fmaf(0.5f, x, 1.0f)));  // 1 ulp
  float p = 0.17087277f;
  p = fmaf(p, t, -0.82215223f);
  p = fmaf(p, t, 1.48851587f);
  p = fmaf(p, t, -1.13520398f);
  p = fmaf(p, t, 0.27886807f);
  p = fmaf(p, t, -0.18628806f);
  p = fmaf(p, t, 0.09678418f);
  p = fmaf(p, t, 0.37409196f);
  p = fmaf(p, t, 1.00002368f);
  p = fmaf(p, t, -1.26551223f);
  return t * __expf(fmaf(-x, x, p));
}

// arr[sys * stride + comp] += v from every lane of a full warp (sys < 0: nothing);
// one atomic per warp when the whole warp works on one system.
__device__ inline void add_system(double *arr, int stride, int comp, int sys, double v) {
  const unsigned full = 0xffffffffu;
  const int s0 = __shfl_sync(full, sys, 0);
  if (__all_sync(full, sys == s0)) {
    v = warp_sum(v);
    if ((threadIdx.x & 31) == 0 && sys >= 0) atomicAdd(&arr[(int64_t)sys * stride + comp], v);
  } else if (sys >= 0) {
    atomicAdd(&arr[(int64_t)sys * stride + comp], v);
  }
}

// Block-wide sum of a double; every thread gets the result.  `scratch` holds
// at least 33 doubles; the call contains two __syncthreads().
__device__ inline double block_sum(double v, double *scratch) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int nw = (blockDim.x + 31) >> 5;
  v = warp_sum(v);
  if (lane == 0) scratch[wid] = v;
  __syncthreads();
  if (wid == 0) {
    double s = lane < nw ? scratch[lane] : 0.0;
    s = warp_sum(s);
    if (lane == 0) scratch[32] = s;
  }
  __syncthreads();
  const double r = scratch[32];
  return r;
}

// Block-wide sum of per-thread float partials, returned to every thread as a double:
// warps add in float, warp 0 adds the warp partials in double (float64 issue is
// scarce on this part, so a double shuffle tree over the whole block is avoided).
// `scratch` holds at least 33 doubles; two __syncthreads() inside.
__device__ inline double block_sum_f(float v, double *scratch) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int nw = (blockDim.x + 31) >> 5;
  v = warp_sum(v);
  if (lane == 0) scratch[wid] = (double)v;
  __syncthreads();
  if (wid == 0) {
    double s = lane < nw ? scratch[lane] : 0.0;
    s = warp_sum(s);
    if (lane == 0) scratch[32] = s;
  }
  __syncthreads();
  return scratch[32];
}

// Block-wide exclusive scan; returns this thread's exclusive prefix and writes
// the block total to *total.  `scratch` holds at least 32 T; two
// __syncthreads() inside, and the caller syncs before reusing `scratch`.
template <typename T>
__device__ inline T block_exclusive_scan(T v, T *scratch, T *total) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int nw = (blockDim.x + 31) >> 5;
  T x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const T y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) scratch[wid] = x;
  __syncthreads();
  if (wid == 0) {
    T s = lane < nw ? scratch[lane] : T(0);
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const T y = __shfl_up_sync(0xffffffffu, s, o);
      if (lane >= o) s += y;
    }
    scratch[lane] = s;  // inclusive prefix of the warp totals
  }
  __syncthreads();
  const T warp_prefix = wid > 0 ? scratch[wid - 1] : T(0);
  *total = scratch[nw - 1];
  return warp_prefix + x - v;
}

}  // namespace kups
