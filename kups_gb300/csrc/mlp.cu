// Tensor-core (tcgen05) GEMM and the learned insertion-proposal MLP.
//
// The learned proposal has no counterpart in the reference; it plugs into the
// ChangesFn log-ratio hook of the insertion move (src/kups/mcmc/moves.py:92-98,
// src/kups/core/propagator.py:330-334).
//
// GEMM: C[M, N] = act(alpha * A[M, K] . B[N, K]^T + bias[N]) with arbitrary
// element strides for A, B and C (so transposed operands need no copies).
// One CTA computes a 128 x BN tile: four warps stage K-chunks of 64 from
// global memory into shared memory in the canonical no-swizzle K-major
// layout (8-row x 16-byte core matrices), one thread issues
// tcgen05.mma.cta_group::1.kind::f16 (BF16 inputs, FP32 accumulation in
// tensor memory) and tcgen05.commit to an mbarrier, and the epilogue reads
// the accumulator back with tcgen05.ld.32x32b.  Every mbarrier wait is
// bounded; on time-out the kernel records KUPS_ERR_UNSUPPORTED, frees its
// tensor memory and returns.
#include <cuda_bf16.h>

#include "common.cuh"

namespace kups {
namespace {

constexpr int kBM = 128;
constexpr int kBK = 64;
constexpr int kGemmThreads = 128;
constexpr long long kWaitLimit = 1LL << 26;

__device__ inline uint32_t smem_u32(const void *p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// Shared-memory matrix descriptor (no swizzle, K-major): start >> 4 in
// [0, 14), leading byte offset >> 4 in [16, 30) (next core matrix along K),
// stride byte offset >> 4 in [32, 46) (next 8-row group), descriptor version
// 1 in [46, 48), swizzle mode 0 in [61, 64).
__device__ inline uint64_t make_sdesc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr >> 4) & 0x3FFFu);
  d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
  d |= (uint64_t)1 << 46;
  return d;
}

// Instruction descriptor, kind::f16: D = F32 (bits 4-5 = 1), A = B = BF16
// (bits 7-9 = 1, 10-12 = 1), both K-major, N >> 3 in [17, 23), M >> 4 in [24, 29).
__device__ inline uint32_t make_idesc(int m, int n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}

__device__ inline void mbar_init(uint32_t addr, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(addr), "r"(count));
}

__device__ inline bool mbar_wait(uint32_t addr, uint32_t phase) {
  for (long long i = 0; i < kWaitLimit; ++i) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(done)
        : "r"(addr), "r"(phase)
        : "memory");
    if (done) return true;
  }
  return false;
}

__device__ inline float act_fn(float x, int act) {
  if (act == 1) return fmaxf(x, 0.f);                      // ReLU
  if (act == 2) return x > 20.f ? x : log1pf(expf(x));     // softplus
  return x;
}

// Strided element access: element (r, c) of a matrix at p + r * sr + c * sc.
template <typename T>
__device__ inline float ld_el(const T *p, int64_t r, int64_t c, int64_t sr, int64_t sc) {
  return (float)p[r * sr + c * sc];
}
template <>
__device__ inline float ld_el<__nv_bfloat16>(const __nv_bfloat16 *p, int64_t r, int64_t c, int64_t sr, int64_t sc) {
  return __bfloat162float(p[r * sr + c * sc]);
}

struct GemmArgs {
  const void *a;
  const void *b;
  void *c;
  void *c2;           // optional second output (same tile, its own strides)
  const float *bias;  // [N] or null
  const float *gate;  // optional: C *= act'(pre) mask source (same layout as c, fp32) or null
  int64_t sar, sac, sbr, sbc, scr, scc, sc2r, sc2c, sgr, sgc;
  int m, n, k;
  float alpha, beta;  // C = alpha * AB^T (+ beta * C)
  int act;            // 0 none, 1 relu, 2 softplus
  int a_bf16, b_bf16, c_bf16, c2_bf16;
  int gate_kind;      // 0 none, 1: multiply by relu'(gate) (gate > 0), 2: by softplus'(gate) = sigmoid
};

template <int BN>
__global__ void __launch_bounds__(kGemmThreads) gemm_tcgen05_kernel(GemmArgs g, kups_status *status) {
  extern __shared__ __align__(1024) unsigned char smem[];
  __nv_bfloat16 *sa = reinterpret_cast<__nv_bfloat16 *>(smem);                      // 128 x 64
  __nv_bfloat16 *sb = reinterpret_cast<__nv_bfloat16 *>(smem + kBM * kBK * 2);      // BN x 64
  uint64_t *mbar = reinterpret_cast<uint64_t *>(smem + (kBM + BN) * kBK * 2);
  uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(mbar + 1);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int m0 = blockIdx.x * kBM, n0 = blockIdx.y * BN;
  if (warp == 0) {
    const uint32_t cols = BN < 32 ? 32 : BN;
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(cols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (tid == 0) mbar_init(smem_u32(mbar), 1);
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tmem_slot;
  const uint32_t idesc = make_idesc(kBM, BN);
  uint32_t phase = 0;
  bool ok = true;
  const int nk = (g.k + kBK - 1) / kBK;
  for (int kc = 0; kc < nk && ok; ++kc) {
    const int k0 = kc * kBK;
    // stage A (128 x 64) and B (BN x 64) as bf16 core matrices: element (r, kk) at
    // ((r / 8) * 8 + kk / 8) * 64 + (r % 8) * 8 + kk % 8   (elements)
    for (int e = tid; e < kBM * kBK; e += kGemmThreads) {
      const int r = e / kBK, kk = e % kBK;
      const int gr = m0 + r, gk = k0 + kk;
      float v = 0.f;
      if (gr < g.m && gk < g.k)
        v = g.a_bf16 ? ld_el((const __nv_bfloat16 *)g.a, gr, gk, g.sar, g.sac) : ld_el((const float *)g.a, gr, gk, g.sar, g.sac);
      sa[((r >> 3) * (kBK / 8) + (kk >> 3)) * 64 + (r & 7) * 8 + (kk & 7)] = __float2bfloat16(v);
    }
    for (int e = tid; e < BN * kBK; e += kGemmThreads) {
      const int r = e / kBK, kk = e % kBK;
      const int gr = n0 + r, gk = k0 + kk;
      float v = 0.f;
      if (gr < g.n && gk < g.k)
        v = g.b_bf16 ? ld_el((const __nv_bfloat16 *)g.b, gr, gk, g.sbr, g.sbc) : ld_el((const float *)g.b, gr, gk, g.sbr, g.sbc);
      sb[((r >> 3) * (kBK / 8) + (kk >> 3)) * 64 + (r & 7) * 8 + (kk & 7)] = __float2bfloat16(v);
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
    if (tid == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      for (int ks = 0; ks < kBK / 16; ++ks) {
        // K step of 16 = two core matrices along K = 256 bytes
        const uint64_t ad = make_sdesc(smem_u32(sa) + ks * 256, 128, (kBK / 8) * 128);
        const uint64_t bd = make_sdesc(smem_u32(sb) + ks * 256, 128, (kBK / 8) * 128);
        const uint32_t accumulate = (kc > 0 || ks > 0) ? 1u : 0u;
        asm volatile(
            "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
            " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(tmem),
            "l"(ad), "l"(bd), "r"(idesc), "r"(accumulate));
      }
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                       smem_u32(mbar))
                   : "memory");
    }
    ok = mbar_wait(smem_u32(mbar), phase);
    phase ^= 1u;
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    __syncthreads();
  }
  if (!ok) {
    if (tid == 0) status_error(status, KUPS_ERR_UNSUPPORTED, blockIdx.x);
  } else {
    // epilogue: warp w reads TMEM lanes 32w .. 32w + 31 (rows), 16 columns at a time
    const int row = m0 + warp * 32 + lane;
    for (int c0 = 0; c0 < BN; c0 += 16) {
      uint32_t r[16];
      const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0;
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, "
          "%14, %15}, [%16];"
          : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
            "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
          : "r"(taddr));
      asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
      if (row < g.m) {
        for (int i = 0; i < 16; ++i) {
          const int col = n0 + c0 + i;
          if (col >= g.n) break;
          float v = g.alpha * __uint_as_float(r[i]);
          if (g.beta != 0.f) {
            const int64_t o = (int64_t)row * g.scr + (int64_t)col * g.scc;
            v += g.beta * (g.c_bf16 ? __bfloat162float(((__nv_bfloat16 *)g.c)[o]) : ((float *)g.c)[o]);
          }
          if (g.bias) v += g.bias[col];
          if (g.gate_kind) {
            const float pre = g.gate[(int64_t)row * g.sgr + (int64_t)col * g.sgc];
            v *= g.gate_kind == 1 ? (pre > 0.f ? 1.f : 0.f) : 1.f / (1.f + expf(-pre));
          }
          v = act_fn(v, g.act);
          const int64_t o = (int64_t)row * g.scr + (int64_t)col * g.scc;
          if (g.c_bf16) ((__nv_bfloat16 *)g.c)[o] = __float2bfloat16(v);
          else ((float *)g.c)[o] = v;
          if (g.c2) {
            const int64_t o2 = (int64_t)row * g.sc2r + (int64_t)col * g.sc2c;
            if (g.c2_bf16) ((__nv_bfloat16 *)g.c2)[o2] = __float2bfloat16(v);
            else ((float *)g.c2)[o2] = v;
          }
        }
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) {
    const uint32_t cols = BN < 32 ? 32 : BN;
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(cols));
  }
}

template <int BN>
int32_t launch_gemm(const GemmArgs &g, kups_status *status, cudaStream_t stream) {
  const size_t smem = (size_t)(kBM + BN) * kBK * 2 + 64;
  KUPS_CUDA_TRY(cudaFuncSetAttribute(gemm_tcgen05_kernel<BN>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  dim3 grid((g.m + kBM - 1) / kBM, (g.n + BN - 1) / BN);
  gemm_tcgen05_kernel<BN><<<grid, kGemmThreads, smem, stream>>>(g, status);
  return cudaGetLastError() == cudaSuccess ? KUPS_OK : KUPS_ERR_CUDA;
}

}  // namespace
}  // namespace kups

using namespace kups;

extern "C" int32_t kups_gemm_bf16(const void *a, int32_t a_bf16, int64_t sa_row, int64_t sa_col,
                                  const void *b, int32_t b_bf16, int64_t sb_row, int64_t sb_col,
                                  void *c, int32_t c_bf16, int64_t sc_row, int64_t sc_col, void *c2,
                                  int32_t c2_bf16, int64_t sc2_row, int64_t sc2_col, const float *bias,
                                  const float *gate, int32_t gate_kind, int64_t sg_row, int64_t sg_col,
                                  int32_t m, int32_t n, int32_t k, float alpha, float beta, int32_t act,
                                  kups_status *status, void *stream) {
  if (m <= 0 || n <= 0 || k <= 0 || act < 0 || act > 2 || gate_kind < 0 || gate_kind > 2) return KUPS_ERR_INVALID;
  GemmArgs g;
  g.a = a; g.b = b; g.c = c; g.c2 = c2; g.bias = bias; g.gate = gate;
  g.sar = sa_row; g.sac = sa_col; g.sbr = sb_row; g.sbc = sb_col; g.scr = sc_row; g.scc = sc_col;
  g.sc2r = sc2_row; g.sc2c = sc2_col; g.sgr = sg_row; g.sgc = sg_col;
  g.m = m; g.n = n; g.k = k; g.alpha = alpha; g.beta = beta; g.act = act;
  g.a_bf16 = a_bf16; g.b_bf16 = b_bf16; g.c_bf16 = c_bf16; g.c2_bf16 = c2_bf16; g.gate_kind = gate_kind;
  cudaStream_t st = (cudaStream_t)stream;
  if (n <= 64) return launch_gemm<64>(g, status, st);
  if (n <= 128) return launch_gemm<128>(g, status, st);
  return launch_gemm<256>(g, status, st);
}
