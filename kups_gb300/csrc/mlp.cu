// Tensor-core (tcgen05) GEMM and the learned insertion-proposal MLP.
//
// The learned proposal has no counterpart in the reference; it plugs into the
// ChangesFn log-ratio hook of the insertion move (src/kups/mcmc/moves.py:92-98,
// src/kups/core/propagator.py:330-334).
//
// GEMM: C[M, N] = act(alpha * A[M, K] . B[N, K]^T + bias[N]) with arbitrary
// element strides for A, B and C (so transposed operands need no copies);
// split-K (grid z) for the weight gradients, whose K is the batch.
// One CTA computes a 128 x BN tile.  Bfloat16 operands with K contiguous are
// loaded by TMA (cp.async.bulk.tensor, 128-byte swizzle) into a ring of
// stages (gemm_tma_kernel); other layouts are staged by the threads with
// 16-byte copies or element-wise into the canonical no-swizzle K-major layout
// (8-row x 16-byte core matrices, gemm_tcgen05_kernel).  One thread issues
// tcgen05.mma.cta_group::1.kind::f16 (BF16 inputs, FP32 accumulation in
// tensor memory) and tcgen05.commit to an mbarrier, and the epilogue reads
// the accumulator back with tcgen05.ld.32x32b.  Every mbarrier wait is
// bounded; on time-out the kernel records KUPS_ERR_UNSUPPORTED, frees its
// tensor memory and returns.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cudaTypedefs.h>

#include <algorithm>

#include "common.cuh"
#include "proposal.cuh"

namespace kups {
namespace {

constexpr int kBM = 128;
constexpr int kBK = 64;
constexpr int kGemmThreads = 256;  // 8 warps: warps w and w + 4 share TMEM lanes 32 (w % 4) ..
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

// softplus(x) = max(x, 0) + ln(1 + exp(-|x|)) with SFU exp / log (no overflow; the absolute
// error, a few 1e-8, is far below the bfloat16 rounding that follows)
__device__ inline float softplus_fast(float x) { return fmaxf(x, 0.f) + __logf(1.0f + __expf(-fabsf(x))); }

// One 32-byte store (a whole L2 sector) of eight 32-bit values.
__device__ inline void st_v8(void *p, const uint32_t (&w)[8]) {
  asm volatile("st.global.v8.b32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8};" ::"l"(p), "r"(w[0]), "r"(w[1]), "r"(w[2]),
               "r"(w[3]), "r"(w[4]), "r"(w[5]), "r"(w[6]), "r"(w[7])
               : "memory");
}

__device__ inline void red_add_v4(float *p, float a, float b, float c, float d) {
  asm volatile("red.relaxed.gpu.global.add.v4.f32 [%0], {%1, %2, %3, %4};" ::"l"(p), "f"(a), "f"(b), "f"(c), "f"(d)
               : "memory");
}

__device__ inline float act_fn(float x, int act) {
  if (act == 1) return fmaxf(x, 0.f);                      // ReLU
  if (act == 2) return x > 20.f ? x : log1pf(__expf(x));  // softplus (SFU exp)
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
  int gate_kind;      // 0 none, 1: multiply by relu'(gate) (gate > 0), 2: by softplus'(gate) = sigmoid,
                      // 3: by softplus' expressed through its output h = softplus(z): 1 - exp(-h)
  int split_k;        // > 1: blockIdx.z takes a slice of K and atomically adds alpha * partial to C
  void *c3;           // optional third output, bfloat16, its own strides (a transposed copy)
  int64_t sc3r, sc3c;
  int row_epi;        // set by dispatch_gemm: the register (lane = row) epilogue applies
  int row_v8;         // ... and C (and c2) rows are 32-byte aligned: whole-sector 32-byte stores
  int fast_math;      // softplus and the gates through SFU exp / log (the network's own calls)
};

__device__ inline void cp_async16(uint32_t dst, const void *src, uint32_t src_bytes) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(dst), "l"(src), "r"(src_bytes) : "memory");
}
__device__ inline void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ inline void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

// Stages rows [r0, r0 + ROWS) x columns [k0, k0 + 64) of an operand into the
// no-swizzle K-major core-matrix layout: element (r, kk) at
//   ((r / 8) * 8 + kk / 8) * 64 + (r % 8) * 8 + kk % 8.
// Fast path (bfloat16, unit K stride, 16-byte rows): one 16-byte cp.async per
// core-matrix row; thread e copies row (e / 64) * 8 + e % 8, K group (e / 8) % 8,
// whose shared-memory destination is element 8 e (a warp fills 512 contiguous
// bytes and reads 64 contiguous bytes of each of 8 rows).  Rows past the end
// are zero-filled (source size 0).  Otherwise every element is loaded,
// converted and stored.
template <int ROWS>
__device__ inline void stage_operand(__nv_bfloat16 *s, const void *p, int is_bf16, int64_t sr, int64_t sc, bool fast,
                                     int r0, int nrows, int k0, int k, int tid) {
  if (fast) {
    const __nv_bfloat16 *base = (const __nv_bfloat16 *)p;
    const uint32_t s0 = smem_u32(s);
    for (int e = tid; e < ROWS * (kBK / 8); e += kGemmThreads) {
      const int r = (e >> 6) * 8 + (e & 7), kg = (e >> 3) & 7;
      const int gr = r0 + r, gk = k0 + kg * 8;
      const bool in = gr < nrows && gk < k;
      const __nv_bfloat16 *src = in ? base + (int64_t)gr * sr + gk : base;
      cp_async16(s0 + (uint32_t)e * 16u, src, in ? 16u : 0u);
    }
  } else {
    const bool rows_fast = sr == 1 && sc != 1;  // walk along the unit-stride index
    for (int e = tid; e < ROWS * kBK; e += kGemmThreads) {
      const int r = rows_fast ? e % ROWS : e / kBK, kk = rows_fast ? e / ROWS : e % kBK;
      const int gr = r0 + r, gk = k0 + kk;
      float v = 0.f;
      if (gr < nrows && gk < k)
        v = is_bf16 ? ld_el((const __nv_bfloat16 *)p, gr, gk, sr, sc) : ld_el((const float *)p, gr, gk, sr, sc);
      s[((r >> 3) * (kBK / 8) + (kk >> 3)) * 64 + (r & 7) * 8 + (kk & 7)] = __float2bfloat16(v);
    }
  }
}

__device__ inline bool fast_operand(const void *p, int is_bf16, int64_t sr, int64_t sc, int k) {
  return is_bf16 && sc == 1 && (sr % 8) == 0 && (k % 8) == 0 && (((uintptr_t)p) & 15) == 0;
}

// Register epilogue of a 128 x BN accumulator tile in tensor memory (row-major float32 C with
// 16-byte aligned rows, N a multiple of 32, beta = 0 or split K): warp w reads TMEM lanes
// 32 (w % 4) .. + 31, so lane l holds row m0 + 32 (w % 4) + l, 32 columns at a time of the
// column half w / 4, and applies every term in registers: 16-byte loads of bias and gate,
// 16-byte stores of C and of the bfloat16 copy (c2), vector reductions for split K, and the
// transposed bfloat16 copy (c3, element (row, col) at col * sc3c + row) written with
// lane = row (64 contiguous bytes per warp instruction).
template <int BN>
__device__ inline void register_epilogue(const GemmArgs &g, uint32_t tmem, int m0, int n0, int warp, int lane) {
  const int quarter = warp & 3, half = warp >> 2;
  const int row = m0 + quarter * 32 + lane;
  const bool rin = row < g.m;
  for (int c0 = half * (BN / 2); c0 < (half + 1) * (BN / 2); c0 += 32) {
    uint32_t r[32];
    const uint32_t taddr = tmem + ((uint32_t)(quarter * 32) << 16) + (uint32_t)c0;
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, "
        "%14, %15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
          "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
    const int col0 = n0 + c0;
    if (col0 >= g.n) continue;  // N is a multiple of 32: the chunk is wholly in or out
    float v[32];
#pragma unroll
    for (int i = 0; i < 32; ++i) v[i] = g.alpha * __uint_as_float(r[i]);
    if (g.split_k > 1) {
      if (rin) {
        float *dst = (float *)g.c + (int64_t)row * g.scr + col0;
#pragma unroll
        for (int q = 0; q < 8; ++q) red_add_v4(dst + 4 * q, v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
      }
      continue;
    }
    if (g.bias != nullptr) {
      const float4 *b4 = reinterpret_cast<const float4 *>(g.bias + col0);
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        const float4 b = __ldg(b4 + q);
        v[4 * q] += b.x;
        v[4 * q + 1] += b.y;
        v[4 * q + 2] += b.z;
        v[4 * q + 3] += b.w;
      }
    }
    if (g.gate_kind != 0 && rin) {
      const float4 *g4 = reinterpret_cast<const float4 *>(g.gate + (int64_t)row * g.sgr + col0);
      const int kind = g.gate_kind + (g.fast_math ? 3 : 0);
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        const float4 t = g4[q];
        const float pre[4] = {t.x, t.y, t.z, t.w};
#pragma unroll
        for (int e = 0; e < 4; ++e) {
          const float x = pre[e];
          float f;
          if (kind == 1 || kind == 4) f = x > 0.f ? 1.f : 0.f;
          else if (kind == 2) f = 1.f / (1.f + expf(-x));
          else if (kind == 5) f = __frcp_rn(1.f + __expf(-x));
          else if (kind == 3) f = -expm1f(-x);
          else f = 1.f - __expf(-x);
          v[4 * q + e] *= f;
        }
      }
    }
    if (g.act == 1) {
#pragma unroll
      for (int i = 0; i < 32; ++i) v[i] = fmaxf(v[i], 0.f);
    } else if (g.act == 2) {
      if (g.fast_math) {
#pragma unroll
        for (int i = 0; i < 32; ++i) v[i] = softplus_fast(v[i]);
      } else {
#pragma unroll
        for (int i = 0; i < 32; ++i) v[i] = act_fn(v[i], 2);
      }
    }
    if (rin) {
      float *cr = (float *)g.c + (int64_t)row * g.scr + col0;
      if (g.row_v8) {  // each lane writes whole 32-byte sectors of its row
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          uint32_t w[8];
#pragma unroll
          for (int e = 0; e < 8; ++e) w[e] = __float_as_uint(v[8 * q + e]);
          st_v8(cr + 8 * q, w);
        }
      } else {
        float4 *cp = reinterpret_cast<float4 *>(cr);
#pragma unroll
        for (int q = 0; q < 8; ++q) cp[q] = make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
      }
      if (g.c2 != nullptr) {
        __nv_bfloat16 *c2r = (__nv_bfloat16 *)g.c2 + (int64_t)row * g.sc2r + col0;
        uint32_t w[16];
#pragma unroll
        for (int e = 0; e < 16; ++e) {
          const __nv_bfloat162 h = __floats2bfloat162_rn(v[2 * e], v[2 * e + 1]);
          w[e] = *reinterpret_cast<const uint32_t *>(&h);
        }
        if (g.row_v8) {
          st_v8(c2r, *reinterpret_cast<const uint32_t(*)[8]>(&w[0]));
          st_v8(c2r + 16, *reinterpret_cast<const uint32_t(*)[8]>(&w[8]));
        } else {
          uint4 *c2p = reinterpret_cast<uint4 *>(c2r);
#pragma unroll
          for (int q = 0; q < 4; ++q) c2p[q] = make_uint4(w[4 * q], w[4 * q + 1], w[4 * q + 2], w[4 * q + 3]);
        }
      }
      if (g.c3 != nullptr) {
        __nv_bfloat16 *c3p = (__nv_bfloat16 *)g.c3 + (int64_t)col0 * g.sc3c + row;
#pragma unroll
        for (int i = 0; i < 32; ++i) {
          *c3p = __float2bfloat16(v[i]);
          c3p += g.sc3c;
        }
      }
    }
  }
}

// Two-stage pipeline: the 16-byte copies of K chunk c + 1 are in flight while
// the tensor cores work on chunk c; a stage is refilled only after the
// mbarrier of the MMAs that read it has completed.
template <int BN>
__global__ void __launch_bounds__(kGemmThreads, 4) gemm_tcgen05_kernel(GemmArgs g, kups_status *status) {
  extern __shared__ __align__(1024) unsigned char smem[];
  constexpr int kStageBytes = (kBM + BN) * kBK * 2;
  uint64_t *mbar = reinterpret_cast<uint64_t *>(smem + 2 * kStageBytes);  // [2]
  uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(mbar + 2);
  auto sa = [&](int st) { return reinterpret_cast<__nv_bfloat16 *>(smem + st * kStageBytes); };
  auto sb = [&](int st) { return reinterpret_cast<__nv_bfloat16 *>(smem + st * kStageBytes + kBM * kBK * 2); };
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int m0 = blockIdx.x * kBM, n0 = blockIdx.y * BN;
  if (warp == 0) {
    const uint32_t cols = BN < 32 ? 32 : BN;
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(cols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (tid == 0) {
    mbar_init(smem_u32(&mbar[0]), 1);
    mbar_init(smem_u32(&mbar[1]), 1);
  }
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tmem_slot;
  const uint32_t idesc = make_idesc(kBM, BN);
  const int nk_all = (g.k + kBK - 1) / kBK;
  const int per_split = (nk_all + g.split_k - 1) / g.split_k;
  const int kc_begin = blockIdx.z * per_split;
  const int kc_end = min(nk_all, kc_begin + per_split);
  const bool fa = fast_operand(g.a, g.a_bf16, g.sar, g.sac, g.k);
  const bool fb = fast_operand(g.b, g.b_bf16, g.sbr, g.sbc, g.k);
  // per stage (bit st): parity of the next completion to wait for, and whether MMAs reading it are
  // in flight (bit fields, not arrays: the stage index is dynamic)
  uint32_t phase = 0u, pending = 0u;
  bool ok = true;
  if (kc_begin < kc_end) {
    stage_operand<kBM>(sa(0), g.a, g.a_bf16, g.sar, g.sac, fa, m0, g.m, kc_begin * kBK, g.k, tid);
    stage_operand<BN>(sb(0), g.b, g.b_bf16, g.sbr, g.sbc, fb, n0, g.n, kc_begin * kBK, g.k, tid);
    cp_async_commit();
  }
  for (int kc = kc_begin; kc < kc_end; ++kc) {
    const int st = (kc - kc_begin) & 1, nx = st ^ 1;
    if (kc + 1 < kc_end) {
      if ((pending >> nx) & 1u) {  // the MMAs of chunk kc - 1 read stage nx
        ok = mbar_wait(smem_u32(&mbar[nx]), (phase >> nx) & 1u);
        if (ok) {  // after a time-out the clean-up below waits for these MMAs again
          phase ^= 1u << nx;
          pending &= ~(1u << nx);
        }
      }
      if (!__syncthreads_and(ok)) {
        ok = false;
        break;
      }
      stage_operand<kBM>(sa(nx), g.a, g.a_bf16, g.sar, g.sac, fa, m0, g.m, (kc + 1) * kBK, g.k, tid);
      stage_operand<BN>(sb(nx), g.b, g.b_bf16, g.sbr, g.sbc, fb, n0, g.n, (kc + 1) * kBK, g.k, tid);
      cp_async_commit();
      cp_async_wait<1>();  // chunk kc has landed (this thread's copies)
    } else {
      cp_async_wait<0>();
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
    if (tid == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      for (int ks = 0; ks < kBK / 16; ++ks) {
        // K step of 16 = two core matrices along K = 256 bytes
        const uint64_t ad = make_sdesc(smem_u32(sa(st)) + ks * 256, 128, (kBK / 8) * 128);
        const uint64_t bd = make_sdesc(smem_u32(sb(st)) + ks * 256, 128, (kBK / 8) * 128);
        const uint32_t accumulate = (kc > kc_begin || ks > 0) ? 1u : 0u;
        asm volatile(
            "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
            " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(tmem),
            "l"(ad), "l"(bd), "r"(idesc), "r"(accumulate));
      }
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                       smem_u32(&mbar[st]))
                   : "memory");
    }
    pending |= 1u << st;
  }
  cp_async_wait<0>();
  // every MMA in flight completes (bounded waits) before the accumulator is read or freed
  for (int st = 0; st < 2; ++st)
    if ((pending >> st) & 1u) ok = mbar_wait(smem_u32(&mbar[st]), (phase >> st) & 1u) && ok;
  ok = __syncthreads_and(ok);
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  if (!ok) {
    if (tid == 0) status_error(status, KUPS_ERR_UNSUPPORTED, blockIdx.x);
  } else if (kc_begin < kc_end && g.row_epi) {
    register_epilogue<BN>(g, tmem, m0, n0, warp, lane);
  } else if (kc_begin < kc_end) {  // an empty K slice holds no accumulator
    // epilogue: warp w reads TMEM lanes 32 (w % 4) .. + 31 (rows) and the column half
    // w / 4, 32 columns at a time, into a padded 32 x 33 shared-memory block.  The
    // elementwise terms run with lane = column (coalesced bias / gate / C loads and
    // row-major stores, 128 contiguous bytes of one row per instruction); the transposed
    // bfloat16 copy (c3) is written back with lane = row (coalesced as well).
    const int quarter = warp & 3, half = warp >> 2;
    const int rbase = m0 + quarter * 32;
    float *blk = reinterpret_cast<float *>(smem) + warp * 32 * 33;  // pipeline stages are free now
    for (int c0 = half * (BN / 2); c0 < (half + 1) * (BN / 2); c0 += 32) {
      uint32_t r[32];
      const uint32_t taddr = tmem + ((uint32_t)(quarter * 32) << 16) + (uint32_t)c0;
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, "
          "%14, %15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
          : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
            "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
            "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
            "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
          : "r"(taddr));
      asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
      for (int i = 0; i < 32; ++i) blk[lane * 33 + i] = __uint_as_float(r[i]);
      __syncwarp();
      const int col = n0 + c0 + lane;
      if (col < g.n) {
        const float bias = g.bias ? g.bias[col] : 0.f;
        // unrolled so that the gate loads of several rows are in flight together
#pragma unroll 8
        for (int rr = 0; rr < 32; ++rr) {
          const int row = rbase + rr;
          if (row >= g.m) continue;
          float v = g.alpha * blk[rr * 33 + lane];
          const int64_t o = (int64_t)row * g.scr + (int64_t)col * g.scc;
          if (g.split_k > 1) {
            atomicAdd((float *)g.c + o, v);
            continue;
          }
          if (g.beta != 0.f) v += g.beta * (g.c_bf16 ? __bfloat162float(((__nv_bfloat16 *)g.c)[o]) : ((float *)g.c)[o]);
          v += bias;
          if (g.gate_kind) {
            const float pre = g.gate[(int64_t)row * g.sgr + (int64_t)col * g.sgc];
            v *= g.gate_kind == 1 ? (pre > 0.f ? 1.f : 0.f)
                 : g.gate_kind == 2 ? 1.f / (1.f + expf(-pre))
                                    : -expm1f(-pre);
          }
          v = act_fn(v, g.act);
          if (g.c_bf16) ((__nv_bfloat16 *)g.c)[o] = __float2bfloat16(v);
          else ((float *)g.c)[o] = v;
          if (g.c2) {
            const int64_t o2 = (int64_t)row * g.sc2r + (int64_t)col * g.sc2c;
            if (g.c2_bf16) ((__nv_bfloat16 *)g.c2)[o2] = __float2bfloat16(v);
            else ((float *)g.c2)[o2] = v;
          }
          blk[rr * 33 + lane] = v;
        }
      }
      __syncwarp();
      if (g.c3 != nullptr && g.split_k == 1) {
        const int row = rbase + lane;
        if (row < g.m) {
#pragma unroll 8
          for (int i = 0; i < 32; ++i) {
            const int cc = n0 + c0 + i;
            if (cc >= g.n) continue;
            ((__nv_bfloat16 *)g.c3)[(int64_t)row * g.sc3r + (int64_t)cc * g.sc3c] =
                __float2bfloat16(blk[lane * 33 + i]);
          }
        }
      }
      __syncwarp();
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
  const size_t smem = (size_t)2 * (kBM + BN) * kBK * 2 + 64;
  KUPS_CUDA_TRY(cudaFuncSetAttribute(gemm_tcgen05_kernel<BN>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  dim3 grid((g.m + kBM - 1) / kBM, (g.n + BN - 1) / BN, g.split_k);
  gemm_tcgen05_kernel<BN><<<grid, kGemmThreads, smem, stream>>>(g, status);
  return cudaGetLastError() == cudaSuccess ? KUPS_OK : KUPS_ERR_CUDA;
}

// ---------------------------------------------------------------------------
// TMA-fed variant for bfloat16 operands with K contiguous (every GEMM of the network's
// training step): one thread issues cp.async.bulk.tensor loads of 64-wide K chunks (128-byte
// rows, 128-byte swizzle) into a ring of STAGES stages, each completing on its mbarrier, and
// the MMAs of a chunk as soon as it has landed; the ring holds the whole K extent of the
// network's GEMMs (K <= 256), so every load of a tile is in flight at once.  A stage is
// refilled only after the commit of the MMAs that read it.  The other threads wait at the
// block barrier, then all run the register epilogue.  Every wait is bounded; on time-out the
// thread waits (bounded) for the loads and MMAs it issued, records KUPS_ERR_UNSUPPORTED, and
// the tile frees its tensor memory without writing C.

// Shared-memory matrix descriptor, K-major with 128-byte swizzle: 8-row groups of 128-byte
// rows 1024 bytes apart (stride byte offset), leading byte offset unused (1), version 1,
// layout type 2 (128-byte swizzle) in [61, 64).  The tile base is 1024-byte aligned; a K step
// of 16 elements advances the start address by 32 bytes.
__device__ inline uint64_t make_sdesc_sw128(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr >> 4) & 0x3FFFu);
  d |= (uint64_t)1 << 16;
  d |= (uint64_t)(1024 >> 4) << 32;
  d |= (uint64_t)1 << 46;
  d |= (uint64_t)2 << 61;
  return d;
}

__device__ inline void mbar_expect_tx(uint32_t mbar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(mbar), "r"(bytes) : "memory");
}

// 2-D tiled load of the box at (x = c0 along K, y = c1 along rows) into shared memory.
__device__ inline void tma_load_2d(uint32_t dst, const CUtensorMap *map, int c0, int c1, uint32_t mbar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
          dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(mbar)
      : "memory");
}

template <int BN, int STAGES, int MINB>
__global__ void __launch_bounds__(kGemmThreads, MINB)
    gemm_tma_kernel(const __grid_constant__ CUtensorMap ta, const __grid_constant__ CUtensorMap tb, GemmArgs g,
                    kups_status *status) {
  extern __shared__ unsigned char smem_raw[];
  unsigned char *smem = reinterpret_cast<unsigned char *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) &
                                                          ~uintptr_t(1023));
  constexpr uint32_t kABytes = kBM * kBK * 2, kBBytes = BN * kBK * 2, kStage = kABytes + kBBytes;
  uint64_t *full = reinterpret_cast<uint64_t *>(smem + STAGES * kStage);  // [STAGES]: chunk landed
  uint64_t *freed = full + STAGES;                                        // [STAGES]: its MMAs done
  uint64_t *done = freed + STAGES;                                        // every MMA of the tile done
  uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(done + 1);
  int *ok_flag = reinterpret_cast<int *>(tmem_slot + 1);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int m0 = blockIdx.x * kBM, n0 = blockIdx.y * BN;
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"((uint32_t)BN));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (tid == 0) {
    for (int st = 0; st < STAGES; ++st) {
      mbar_init(smem_u32(&full[st]), 1);
      mbar_init(smem_u32(&freed[st]), 1);
    }
    mbar_init(smem_u32(done), 1);
    *ok_flag = 1;
  }
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tmem_slot;
  const int nk_all = (g.k + kBK - 1) / kBK;
  const int per_split = (nk_all + g.split_k - 1) / g.split_k;
  const int kc_begin = blockIdx.z * per_split;
  const int kc_end = min(nk_all, kc_begin + per_split);
  const int nk = max(0, kc_end - kc_begin);
  if (tid == 0) {
    const uint32_t idesc = make_idesc(kBM, BN);
    auto sa = [&](int st) { return smem_u32(smem + st * kStage); };
    auto sb = [&](int st) { return smem_u32(smem + st * kStage + kABytes); };
    auto load = [&](int j) {  // chunk j of this tile's K range into stage j % STAGES
      const int st = j % STAGES, k0 = (kc_begin + j) * kBK;
      mbar_expect_tx(smem_u32(&full[st]), kStage);
      tma_load_2d(sa(st), &ta, k0, m0, smem_u32(&full[st]));
      tma_load_2d(sb(st), &tb, k0, n0, smem_u32(&full[st]));
    };
    bool ok = true;
    int issued = 0, consumed = 0;
    for (; issued < min(STAGES, nk); ++issued) load(issued);
    for (int i = 0; i < nk && ok; ++i) {
      const int st = i % STAGES;
      const uint32_t par = (uint32_t)(i / STAGES) & 1u;
      ok = mbar_wait(smem_u32(&full[st]), par);
      if (!ok) break;
      consumed = i + 1;
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      for (int ks = 0; ks < kBK / 16; ++ks) {
        const uint64_t ad = make_sdesc_sw128(sa(st) + ks * 32);
        const uint64_t bd = make_sdesc_sw128(sb(st) + ks * 32);
        const uint32_t accumulate = (i > 0 || ks > 0) ? 1u : 0u;
        asm volatile(
            "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
            " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(tmem),
            "l"(ad), "l"(bd), "r"(idesc), "r"(accumulate));
      }
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                       smem_u32(&freed[st]))
                   : "memory");
      if (issued < nk) {  // refill this stage once its MMAs are done
        ok = mbar_wait(smem_u32(&freed[st]), par);
        if (!ok) break;
        load(issued++);
      }
    }
    // every MMA issued so far completes before the accumulator is read or freed
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(done))
                 : "memory");
    const bool mma_done = mbar_wait(smem_u32(done), 0u);
    if (!ok) {  // loads still in flight land before the tile exits
      for (int j = consumed; j < issued; ++j)
        mbar_wait(smem_u32(&full[j % STAGES]), (uint32_t)(j / STAGES) & 1u);
    }
    *ok_flag = (ok && mma_done) ? 1 : 0;
  }
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  if (!*ok_flag) {
    if (tid == 0) status_error(status, KUPS_ERR_UNSUPPORTED, blockIdx.x);
  } else if (nk > 0) {
    register_epilogue<BN>(g, tmem, m0, n0, warp, lane);
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"((uint32_t)BN));
}

bool encode_operand_map(PFN_cuTensorMapEncodeTiled_v12000 enc, CUtensorMap *m, const void *p, int64_t rows,
                        int64_t k, int64_t sr, int box_rows);

PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = [] {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      p = nullptr;
    return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  }();
  return fn;
}

// Tensor map of a bfloat16 [rows, k] operand with row stride sr elements (K contiguous), boxes
// of 64 x box_rows, 128-byte swizzle; out-of-range elements read as zero.  The last maps made
// are kept (a training step passes the same workspace operands every step), so encoding runs
// once per distinct operand; the cache is per host thread.
bool operand_map(CUtensorMap *m, const void *p, int64_t rows, int64_t k, int64_t sr, int box_rows) {
  struct Entry {
    const void *p;
    int64_t rows, k, sr;
    int box;
    CUtensorMap map;
  };
  constexpr int kCache = 32;
  static thread_local Entry cache[kCache];
  static thread_local int next = 0;
  for (int i = 0; i < kCache; ++i) {
    const Entry &e = cache[i];
    if (e.p == p && e.rows == rows && e.k == k && e.sr == sr && e.box == box_rows) {
      *m = e.map;
      return true;
    }
  }
  PFN_cuTensorMapEncodeTiled_v12000 enc = tensor_map_encoder();
  if (enc == nullptr || !encode_operand_map(enc, m, p, rows, k, sr, box_rows)) return false;
  cache[next] = Entry{p, rows, k, sr, box_rows, *m};
  next = (next + 1) % kCache;
  return true;
}

bool encode_operand_map(PFN_cuTensorMapEncodeTiled_v12000 enc, CUtensorMap *m, const void *p, int64_t rows,
                        int64_t k, int64_t sr, int box_rows) {
  cuuint64_t dims[2] = {(cuuint64_t)k, (cuuint64_t)rows};
  cuuint64_t strides[1] = {(cuuint64_t)sr * 2};
  cuuint32_t box[2] = {(cuuint32_t)kBK, (cuuint32_t)box_rows};
  cuuint32_t es[2] = {1, 1};
  return enc(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void *>(p), dims, strides, box, es,
             CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
             CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// Whether the TMA-fed kernel applies: both operands bfloat16 with K contiguous, 16-byte aligned
// bases and row strides of at least K elements that are multiples of 8, and the register epilogue.
bool tma_operands(const GemmArgs &g) {
  auto al16 = [](const void *q) { return (((uintptr_t)q) & 15) == 0; };
  return g.a_bf16 && g.b_bf16 && g.sac == 1 && g.sbc == 1 && g.sar % 8 == 0 && g.sbr % 8 == 0 && g.sar >= g.k &&
         g.sbr >= g.k && al16(g.a) && al16(g.b) && g.row_epi;
}

template <int BN, int STAGES, int MINB>
int32_t launch_gemm_tma(const GemmArgs &g, kups_status *status, cudaStream_t stream, bool &launched) {
  launched = false;
  CUtensorMap ta, tb;
  if (!operand_map(&ta, g.a, g.m, g.k, g.sar, kBM) || !operand_map(&tb, g.b, g.n, g.k, g.sbr, BN)) return KUPS_OK;
  const size_t smem = (size_t)STAGES * (kBM + BN) * kBK * 2 + 1024 + 256;
  static int set_device = -1;  // the attribute is per device: set it once for each device in turn
  int dev = 0;
  KUPS_CUDA_TRY(cudaGetDevice(&dev));
  if (set_device != dev) {
    KUPS_CUDA_TRY(cudaFuncSetAttribute(gemm_tma_kernel<BN, STAGES, MINB>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    set_device = dev;
  }
  dim3 grid((g.m + kBM - 1) / kBM, (g.n + BN - 1) / BN, g.split_k);
  gemm_tma_kernel<BN, STAGES, MINB><<<grid, kGemmThreads, smem, stream>>>(ta, tb, g, status);
  launched = true;
  return cudaGetLastError() == cudaSuccess ? KUPS_OK : KUPS_ERR_CUDA;
}

// Tile width: 128 (64 for N <= 64), narrowed to 64 while the grid would leave SMs idle
// (fewer than two CTAs per SM of 148).  128-wide tiles (64 KB of pipeline buffers, three
// CTAs per SM) beat 256-wide ones (two CTAs per SM) on the network's K <= 256 GEMMs.
// Whether the register epilogue of gemm_tcgen05_kernel applies: float32 C (and the optional
// bias, gate and bfloat16 copy) row-major with unit column stride and 16-byte aligned rows,
// N a multiple of 32, no beta term; the transposed copy (c3) with unit row stride.
bool row_epilogue(const GemmArgs &g) {
  auto al16 = [](const void *q) { return (((uintptr_t)q) & 15) == 0; };
  if (g.c_bf16 || g.scc != 1 || g.scr % 4 != 0 || !al16(g.c) || g.n % 32 != 0) return false;
  if (g.split_k > 1) return true;  // alpha * partial added into C
  if (g.beta != 0.f) return false;
  if (g.bias != nullptr && !al16(g.bias)) return false;
  if (g.gate_kind != 0 && (g.sgc != 1 || g.sgr % 4 != 0 || !al16(g.gate))) return false;
  if (g.c2 != nullptr && (!g.c2_bf16 || g.sc2c != 1 || g.sc2r % 8 != 0 || !al16(g.c2))) return false;
  if (g.c3 != nullptr && g.sc3r != 1) return false;
  return true;
}

int32_t dispatch_gemm(const GemmArgs &g0, kups_status *status, cudaStream_t st) {
  GemmArgs g = g0;
  g.row_epi = row_epilogue(g) ? 1 : 0;
  auto al32 = [](const void *q) { return (((uintptr_t)q) & 31) == 0; };
  g.row_v8 = g.row_epi && g.scr % 8 == 0 && al32(g.c) &&
             (g.c2 == nullptr || (g.sc2r % 16 == 0 && al32(g.c2)));
  if (tma_operands(g)) {  // one tile column per 256 of N; the tile ring holds K <= 256 whole
    // tiles as wide as N (up to 256, one CTA per SM) with a four-stage ring: measured against
    // 128 x 128 and 128 x 64 tiles with two stages (three and four CTAs per SM) and with four
    // stages, it was the fastest on the network's training step (0.194 against 0.196-0.214 ms)
    bool launched = false;
    const int32_t rc = g.n <= 64    ? launch_gemm_tma<64, 4, 1>(g, status, st, launched)
                       : g.n <= 128 ? launch_gemm_tma<128, 4, 1>(g, status, st, launched)
                                    : launch_gemm_tma<256, 4, 1>(g, status, st, launched);
    if (launched || rc != KUPS_OK) return rc;
  }
  const int64_t rows = ((int64_t)g.m + kBM - 1) / kBM * g.split_k;
  int bn = g.n <= 64 ? 64 : 128;
  while (bn > 64 && rows * ((g.n + bn - 1) / bn) < 2 * 148) bn >>= 1;
  if (bn == 64) return launch_gemm<64>(g, status, st);
  if (bn == 128) return launch_gemm<128>(g, status, st);
  return launch_gemm<256>(g, status, st);
}

// Row-major operand helper for the network's own GEMM calls.
struct Op {
  const void *p;
  int bf16;
  int64_t sr, sc;
};

// c: float32 with strides (scr, scc); c2: bfloat16 copy, same strides; c3: bfloat16
// transposed copy (element (r, col) at col * m + r).
int32_t gemm_call(Op a, Op b, void *c, int64_t scr, int64_t scc, void *c2, const float *bias, const float *gate,
                  int gate_kind, int m, int n, int k, float beta, int act, int split, kups_status *status,
                  cudaStream_t st, void *c3 = nullptr) {
  GemmArgs g;
  g.a = a.p; g.b = b.p; g.c = c; g.c2 = c2; g.bias = bias; g.gate = gate;
  g.c3 = c3; g.sc3r = 1; g.sc3c = m;
  g.sar = a.sr; g.sac = a.sc; g.sbr = b.sr; g.sbc = b.sc; g.scr = scr; g.scc = scc;
  g.sc2r = scr; g.sc2c = scc; g.sgr = scr; g.sgc = scc;
  g.m = m; g.n = n; g.k = k; g.alpha = 1.f; g.beta = beta; g.act = act;
  g.a_bf16 = a.bf16; g.b_bf16 = b.bf16; g.c_bf16 = 0; g.c2_bf16 = 1; g.gate_kind = gate_kind;
  g.split_k = split;
  g.fast_math = 1;
  return dispatch_gemm(g, status, st);
}

// ============================================================================
// Learned insertion proposal: network, training and grid density.
//
// Fixed architecture: 64 Fourier features of the fractional position f,
// (sin, cos)(2 pi m_j . f) for 32 integer vectors m_j, three softplus layers of
// width 256 (tensor-core GEMMs, bfloat16 operands, float32 accumulation) and
// a linear output g(f).  Parameters are one flat float32 array at the kOff*
// offsets plus a bfloat16 copy read by the GEMMs.  Each layer's output h is
// stored in float32 (the head and the gates read it) and, where it is the
// next GEMM's operand, in bfloat16.  Training minimises the noise-contrastive
// loss with equal halves of data and uniform points,
//   L = (1/n) [sum_data softplus(-g) + sum_uniform softplus(g)],
// whose minimiser is g(f) = ln p_data(f) for f uniform on the unit cube.
constexpr int kFreq = 32, kIn = 2 * kFreq, kHid = 256;
constexpr int64_t kOffW1 = 0, kOffB1 = kOffW1 + kHid * kIn, kOffW2 = kOffB1 + kHid, kOffB2 = kOffW2 + kHid * kHid,
                  kOffW3 = kOffB2 + kHid, kOffB3 = kOffW3 + kHid * kHid, kOffW4 = kOffB3 + kHid,
                  kOffB4 = kOffW4 + kHid, kParams = kOffB4 + 1;
static_assert(kParams == KUPS_MLP_PARAMS, "parameter layout");
constexpr int64_t kChunk = 65536;  // points per forward pass over the workspace

inline size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

// Activations of c points: float32 (the head and the gates read them), bfloat16
// row-major (the next layer's A operand) and bfloat16 transposed [width, c]
// (the weight-gradient GEMMs' operands, K = points contiguous).
struct MlpWork {
  __nv_bfloat16 *feat, *featT, *h1b, *h1T, *h2b, *h2T, *dzab, *dzaT, *dzbb, *dzbT;
  float *h1, *h2, *h3, *dza, *dzb, *g;
};

MlpWork carve(void *ws, int64_t c) {
  char *p = (char *)(((uintptr_t)ws + 255) & ~uintptr_t(255));
  MlpWork w;
  auto take = [&](size_t bytes) {
    char *q = p;
    p += align256(bytes);
    return (void *)q;
  };
  w.feat = (__nv_bfloat16 *)take(2 * (size_t)c * kIn);
  w.featT = (__nv_bfloat16 *)take(2 * (size_t)c * kIn);
  w.h1b = (__nv_bfloat16 *)take(2 * (size_t)c * kHid);
  w.h1T = (__nv_bfloat16 *)take(2 * (size_t)c * kHid);
  w.h2b = (__nv_bfloat16 *)take(2 * (size_t)c * kHid);
  w.h2T = (__nv_bfloat16 *)take(2 * (size_t)c * kHid);
  w.dzab = (__nv_bfloat16 *)take(2 * (size_t)c * kHid);
  w.dzaT = (__nv_bfloat16 *)take(2 * (size_t)c * kHid);
  w.dzbb = (__nv_bfloat16 *)take(2 * (size_t)c * kHid);
  w.dzbT = (__nv_bfloat16 *)take(2 * (size_t)c * kHid);
  w.h1 = (float *)take(4 * (size_t)c * kHid);
  w.h2 = (float *)take(4 * (size_t)c * kHid);
  w.h3 = (float *)take(4 * (size_t)c * kHid);
  w.dza = (float *)take(4 * (size_t)c * kHid);
  w.dzb = (float *)take(4 * (size_t)c * kHid);
  w.g = (float *)take(4 * (size_t)c);
  return w;
}

size_t work_bytes(int64_t c) {
  return 2 * align256(2 * (size_t)c * kIn) + 8 * align256(2 * (size_t)c * kHid) + 5 * align256(4 * (size_t)c * kHid) +
         align256(4 * (size_t)c) + 256;
}

__device__ inline float warp_sum(float v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__device__ inline float softplus(float x) { return x > 20.f ? x : log1pf(expf(x)); }

// sin and cos of 2 pi (m . f) for a point whose coordinates, reduced to [-0.5, 0.5), are the
// float pairs fh + fl.  The phase is carried as a float pair (the products' rounding errors
// recovered by fma, the sums' by two-sum) and reduced modulo one before its single rounding
// to float, so the phase reaching sincospi is within 3e-8 of a turn of the float64 phase and
// the features round to the same bfloat16 values as the float64 features almost always.
__device__ inline void phase_sincos(const int32_t *m, const float fh[3], const float fl[3], float &sn, float &cs) {
  const float m0 = (float)m[0], m1 = (float)m[1], m2 = (float)m[2];
  const float p0 = __fmul_rn(m0, fh[0]), p1 = __fmul_rn(m1, fh[1]), p2 = __fmul_rn(m2, fh[2]);
  float lo = __fadd_rn(__fadd_rn(fmaf(m0, fh[0], -p0), fmaf(m1, fh[1], -p1)), fmaf(m2, fh[2], -p2));
  lo = fmaf(m0, fl[0], fmaf(m1, fl[1], fmaf(m2, fl[2], lo)));
  const float s1 = __fadd_rn(p0, p1);
  float b = __fsub_rn(s1, p0);
  lo = __fadd_rn(lo, __fadd_rn(__fsub_rn(p0, __fsub_rn(s1, b)), __fsub_rn(p1, b)));
  const float s2 = __fadd_rn(s1, p2);
  b = __fsub_rn(s2, s1);
  lo = __fadd_rn(lo, __fadd_rn(__fsub_rn(s1, __fsub_rn(s2, b)), __fsub_rn(p2, b)));
  float t = __fadd_rn(__fsub_rn(s2, rintf(s2)), lo);
  t = __fsub_rn(t, rintf(t));
  sincospif(2.0f * t, &sn, &cs);
}

// Features of point row0 + r: from x (fractional, f64 [., 3]) or, with x null,
// of grid node row0 + r of a grid^3 lattice.
__global__ void features_kernel(const double *x, int64_t row0, int64_t n, int grid, const int32_t *freq,
                                __nv_bfloat16 *feat, __nv_bfloat16 *featT) {
  const int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (r >= n) return;
  double f[3];
  if (x != nullptr) {
    for (int a = 0; a < 3; ++a) f[a] = x[3 * (row0 + r) + a];
  } else {
    const int64_t v = row0 + r, g2 = (int64_t)grid * grid;
    f[0] = (double)(v / g2) / grid;
    f[1] = (double)((v / grid) % grid) / grid;
    f[2] = (double)(v % grid) / grid;
  }
  // coordinates reduced to [-0.5, 0.5) once in float64 and split into float pairs, phases
  // as float pairs (phase_sincos), as the fused forward pass computes them
  float fh[3], fl[3];
  for (int a = 0; a < 3; ++a) {
    const double red = f[a] - rint(f[a]);
    fh[a] = (float)red;
    fl[a] = (float)(red - (double)fh[a]);
  }
  __nv_bfloat162 *o = reinterpret_cast<__nv_bfloat162 *>(feat + r * kIn);
  for (int j = 0; j < kFreq; ++j) {
    float sn, cs;
    phase_sincos(freq + 3 * j, fh, fl, sn, cs);
    o[j] = __floats2bfloat162_rn(sn, cs);
    if (featT != nullptr) {
      featT[(int64_t)(2 * j) * n + r] = __float2bfloat16(sn);
      featT[(int64_t)(2 * j + 1) * n + r] = __float2bfloat16(cs);
    }
  }
}

// Equal halves: rows [0, batch/2) are data points drawn with replacement,
// rows [batch/2, batch) uniform points; Philox keyed by (seed, step, row).
__global__ void nce_batch_kernel(const double *data, int64_t n_data, int64_t batch, uint64_t seed, uint64_t step,
                                 double *x, float *label) {
  const int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (r >= batch) return;
  const U4 c{(uint32_t)r, (uint32_t)(r >> 32), (uint32_t)step, (uint32_t)(step >> 32)};
  const U4 w = philox4x32_10(c, (uint32_t)seed, (uint32_t)(seed >> 32));
  if (r < batch / 2) {
    const uint64_t idx = ((((uint64_t)w.x) << 32) | w.y) % (uint64_t)n_data;
    for (int a = 0; a < 3; ++a) x[3 * r + a] = data[3 * idx + a];
    label[r] = 1.f;
  } else {
    x[3 * r] = w.x * (1.0 / 4294967296.0);
    x[3 * r + 1] = w.y * (1.0 / 4294967296.0);
    x[3 * r + 2] = w.z * (1.0 / 4294967296.0);
    label[r] = 0.f;
  }
}

// g = h3 . w4 + b4, one warp per row.
__global__ void head_kernel(const float *h, int64_t n, const float *w4, const float *b4, float *g) {
  const int lane = threadIdx.x & 31;
  const int64_t row = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  if (row >= n) return;
  float acc = 0.f;
  for (int j = lane; j < kHid; j += 32) acc = fmaf(h[row * kHid + j], w4[j], acc);
  acc = warp_sum(acc);
  if (lane == 0) g[row] = acc + b4[0];
}

// Head forward + loss + first backward step, 8 warps per block, a warp per row:
//   dL/dg = (sigmoid(g) - y) / n,  dz3 = dL/dg * w4 * (1 - exp(-h3)),
//   grad_w4 += sum_rows dL/dg h3,  grad_b4 += sum_rows dL/dg,  loss += L.
__global__ void __launch_bounds__(256) head_nce_kernel(const float *h, int64_t n, const float *w4, const float *b4,
                                                       const float *label, float *dz, __nv_bfloat16 *dzb,
                                                       __nv_bfloat16 *dzT, float *grad_w4, float *grad_b4,
                                                       float *loss) {
  __shared__ float red_w[8][kHid];
  __shared__ float red_b[8], red_l[8];
  // a tile of 32 rows of dz in bfloat16, written out transposed (dzT[col, row]) with consecutive
  // threads on consecutive rows, so the transposed copy's stores coalesce
  __shared__ __nv_bfloat16 tile[32][kHid + 8];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  float wl[8], dw[8];
  for (int j = 0; j < 8; ++j) {
    wl[j] = w4[lane + 32 * j];
    dw[j] = 0.f;
  }
  float db = 0.f, ls = 0.f;
  const float inv_n = 1.f / (float)n;
  for (int64_t r0 = (int64_t)blockIdx.x * 32; r0 < n; r0 += (int64_t)gridDim.x * 32) {
    // warp w takes rows r0 + 4 w .. r0 + 4 w + 3, all four rows' loads issued first
    float hk[4][8];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const int64_t row = r0 + warp * 4 + k;
#pragma unroll
      for (int j = 0; j < 8; ++j) hk[k][j] = row < n ? h[row * kHid + lane + 32 * j] : 0.f;
    }
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const int rl = warp * 4 + k;
      const int64_t row = r0 + rl;
      if (row >= n) break;
      const float *hv = hk[k];
      float acc = 0.f;
      for (int j = 0; j < 8; ++j) acc = fmaf(hv[j], wl[j], acc);
      const float gg = warp_sum(acc) + b4[0];
      const float y = label[row];
      const float dg = (1.f / (1.f + expf(-gg)) - y) * inv_n;
      if (lane == 0) {
        ls += y > 0.5f ? softplus(-gg) : softplus(gg);
        db += dg;
      }
      for (int j = 0; j < 8; ++j) {
        dw[j] = fmaf(dg, hv[j], dw[j]);
        const float d = dg * wl[j] * (1.f - __expf(-hv[j]));  // softplus' through its output (SFU exp)
        const int col = lane + 32 * j;
        dz[row * kHid + col] = d;
        const __nv_bfloat16 db16 = __float2bfloat16(d);
        dzb[row * kHid + col] = db16;
        tile[rl][col] = db16;
      }
    }
    __syncthreads();
    const int nr = n - r0 < 32 ? (int)(n - r0) : 32;
    for (int e = threadIdx.x; e < 32 * kHid; e += blockDim.x) {
      const int col = e >> 5, rl = e & 31;
      if (rl < nr) dzT[(int64_t)col * n + r0 + rl] = tile[rl][col];
    }
    __syncthreads();
  }
  for (int j = 0; j < 8; ++j) red_w[warp][lane + 32 * j] = dw[j];
  if (lane == 0) {
    red_b[warp] = db;
    red_l[warp] = ls;
  }
  __syncthreads();
  for (int c = threadIdx.x; c < kHid; c += blockDim.x) {
    float s = 0.f;
    for (int w = 0; w < 8; ++w) s += red_w[w][c];
    atomicAdd(&grad_w4[c], s);
  }
  if (threadIdx.x == 0) {
    float s = 0.f, l = 0.f;
    for (int w = 0; w < 8; ++w) {
      s += red_b[w];
      l += red_l[w];
    }
    atomicAdd(grad_b4, s);
    if (loss != nullptr) atomicAdd(loss, l * inv_n);
  }
}

// Column sums of z [n, 256] (float32) added into out: thread t reads columns 4 (t % 64) .. + 3
// (16-byte loads, a warp reads 512 contiguous bytes of a row) of every fourth row of the
// block's slab, and the four row groups meet in shared memory.
__global__ void __launch_bounds__(kHid) colsum_kernel(const float *z, int64_t n, float *out) {
  __shared__ float4 part[4][kHid / 4];
  const int t = threadIdx.x, q = t & (kHid / 4 - 1), grp = t / (kHid / 4);
  const int64_t per = (n + gridDim.x - 1) / gridDim.x;
  const int64_t r0 = (int64_t)blockIdx.x * per, r1 = min(n, r0 + per);
  const float4 *z4 = reinterpret_cast<const float4 *>(z);
  float4 s = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll 4
  for (int64_t r = r0 + grp; r < r1; r += 4) {
    const float4 v = z4[r * (kHid / 4) + q];
    s.x += v.x;
    s.y += v.y;
    s.z += v.z;
    s.w += v.w;
  }
  part[grp][q] = s;
  __syncthreads();
  const float *pf = reinterpret_cast<const float *>(part);
  if (r0 < r1) atomicAdd(&out[t], (pf[t] + pf[kHid + t]) + (pf[2 * kHid + t] + pf[3 * kHid + t]));
}

// Adam (Kingma & Ba 2015) with bias corrections c1 = 1 / (1 - beta1^t),
// c2 = 1 / (1 - beta2^t); refreshes the bfloat16 copy and zeroes the gradient.
// bfloat16 copies of a parameter: the flat copy, and for W2 / W3 the transposed copy
// (W^T[in][out]) that the backward GEMMs read as a K-contiguous operand.
__device__ inline void store_bf16(__nv_bfloat16 *pb, __nv_bfloat16 *pbt, int64_t i, float v) {
  const __nv_bfloat16 b = __float2bfloat16(v);
  pb[i] = b;
  if (i >= kOffW2 && i < kOffB2) {
    const int64_t l = i - kOffW2;
    pbt[(l % kHid) * kHid + l / kHid] = b;
  } else if (i >= kOffW3 && i < kOffB3) {
    const int64_t l = i - kOffW3;
    pbt[kHid * kHid + (l % kHid) * kHid + l / kHid] = b;
  }
}

__global__ void adam_kernel(float *p, __nv_bfloat16 *pb, __nv_bfloat16 *pbt, float *g, float *m, float *v, int64_t n,
                            float lr, float b1, float b2, float eps, float c1, float c2) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float gi = g[i];
  const float mi = b1 * m[i] + (1.f - b1) * gi;
  const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
  m[i] = mi;
  v[i] = vi;
  const float pi = p[i] - lr * (mi * c1) / (sqrtf(vi * c2) + eps);
  p[i] = pi;
  store_bf16(pb, pbt, i, pi);
  g[i] = 0.f;
}

// Weights uniform with variance 1 / fan_in (Philox keyed by (seed, index)),
// biases zero; optimiser state and gradients zero.
__global__ void init_kernel(float *p, __nv_bfloat16 *pb, __nv_bfloat16 *pbt, float *g, float *m, float *v,
                            uint64_t seed) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= kParams) return;
  float fan = 0.f;
  if (i < kOffB1) fan = kIn;
  else if ((i >= kOffW2 && i < kOffB2) || (i >= kOffW3 && i < kOffB3) || (i >= kOffW4 && i < kOffB4)) fan = kHid;
  float val = 0.f;
  if (fan > 0.f) {
    const U4 c{(uint32_t)i, (uint32_t)(i >> 32), 0x6d6c70u, 0u};
    const U4 w = philox4x32_10(c, (uint32_t)seed, (uint32_t)(seed >> 32));
    const float u = (float)(w.x >> 8) * (1.0f / 16777216.0f);
    val = (2.f * u - 1.f) * sqrtf(3.f / fan);
  }
  p[i] = val;
  store_bf16(pb, pbt, i, val);
  g[i] = 0.f;
  m[i] = 0.f;
  v[i] = 0.f;
}

__device__ inline float block_max1024(float v, float *red) {
  for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x < 32) {
    float w = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : -INFINITY;
    for (int o = 16; o > 0; o >>= 1) w = fmaxf(w, __shfl_xor_sync(0xffffffffu, w, o));
    if (threadIdx.x == 0) red[0] = w;
  }
  __syncthreads();
  const float r = red[0];
  __syncthreads();
  return r;
}

__device__ inline double block_sum_d(double v, double *red) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x < 32) {
    double w = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.0;
    for (int o = 16; o > 0; o >>= 1) w += __shfl_xor_sync(0xffffffffu, w, o);
    if (threadIdx.x == 0) red[0] = w;
  }
  __syncthreads();
  const double r = red[0];
  __syncthreads();
  return r;
}

// node holds g on entry; on exit d = exp(temper (g - max g)) + floor_frac * mean(exp(temper (g - max g))).
// Two launches over the whole GPU: each block of grid_partials_kernel reduces a grid-stride
// share of the nodes to (its max m_b, sum exp(temper (g - m_b)) in float64, a non-finite flag);
// every block of grid_apply_kernel combines the partials (M = max m_b,
// Z = sum_b s_b exp(temper (m_b - M))) and rewrites its share of the nodes.
constexpr int kNormBlocks = 152, kNormThreads = 1024;

__global__ void __launch_bounds__(kNormThreads) grid_partials_kernel(const float *node, int64_t n, float temper,
                                                                     double *partial, kups_status *status) {
  __shared__ float redf[32];
  __shared__ double redd[32];
  float mx = -INFINITY;
  int bad = 0;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    const float v = node[i];
    if (!isfinite(v)) bad = 1;
    mx = fmaxf(mx, v);
  }
  bad = __syncthreads_or(bad);
  mx = block_max1024(mx, redf);
  double s = 0.0;
  if (!bad && mx > -INFINITY)
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
      s += expf(temper * (node[i] - mx));
  s = block_sum_d(s, redd);
  if (threadIdx.x == 0) {
    partial[3 * blockIdx.x] = (double)mx;
    partial[3 * blockIdx.x + 1] = s;
    partial[3 * blockIdx.x + 2] = bad ? 1.0 : 0.0;
    if (bad) status_error(status, KUPS_ERR_NONFINITE, -1);
  }
}

__global__ void __launch_bounds__(256) grid_apply_kernel(float *node, int64_t n, float temper, float floor_frac,
                                                         const double *partial, int n_partial) {
  // thread b < n_partial (<= 256) holds partial b: block max, then the rescaled sums
  __shared__ float redf[32];
  __shared__ double redd[32];
  const int b = threadIdx.x;
  const bool has = b < n_partial;
  const float mb = has ? (float)partial[3 * b] : -INFINITY;
  const int bad = __syncthreads_or(has && partial[3 * b + 2] != 0.0);
  if (bad) return;
  const float M = block_max1024(mb, redf);
  const double zb = has && mb > -INFINITY ? partial[3 * b + 1] * (double)expf(temper * (mb - M)) : 0.0;
  const float fl = (float)(floor_frac * (block_sum_d(zb, redd) / (double)n));
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    node[i] = expf(temper * (node[i] - M)) + fl;
}

// cdf[c] = sum_{c' < c} mass(c'), mass = mean of the cell's 8 corners (float64),
// in three passes: each block of 256 threads scans kCdfPerBlock cells (8 per thread)
// and records its total, one block scans the totals, and the block offsets are added.
constexpr int kCdfThreads = 256, kCdfPerThread = 8, kCdfPerBlock = kCdfThreads * kCdfPerThread;

__device__ inline double cell_mass(const float *node, int g, int64_t c) {
  const int i = (int)(c / ((int64_t)g * g)), j = (int)((c / g) % g), k = (int)(c % g);
  double d[8];
  grid_corners(node, g, i, j, k, d);
  double s = 0.0;
  for (int b = 0; b < 8; ++b) s += d[b];
  return s * 0.125;
}

// inclusive scan of one double per thread over a block of kCdfThreads threads
__device__ inline double block_inclusive_scan(double v, double *sh) {
  sh[threadIdx.x] = v;
  __syncthreads();
  for (int o = 1; o < kCdfThreads; o <<= 1) {
    const double add = threadIdx.x >= (unsigned)o ? sh[threadIdx.x - o] : 0.0;
    __syncthreads();
    sh[threadIdx.x] += add;
    __syncthreads();
  }
  const double r = sh[threadIdx.x];
  __syncthreads();
  return r;
}

__global__ void __launch_bounds__(kCdfThreads) grid_cdf_local_kernel(const float *node, int g, double *cdf,
                                                                      double *block_total) {
  __shared__ double sh[kCdfThreads];
  const int64_t n = (int64_t)g * g * g;
  const int64_t c0 = (int64_t)blockIdx.x * kCdfPerBlock + (int64_t)threadIdx.x * kCdfPerThread;
  double m[kCdfPerThread], local = 0.0;
  for (int t = 0; t < kCdfPerThread; ++t) {
    m[t] = c0 + t < n ? cell_mass(node, g, c0 + t) : 0.0;
    local += m[t];
  }
  double run = block_inclusive_scan(local, sh) - local;
  for (int t = 0; t < kCdfPerThread; ++t) {
    if (c0 + t < n) cdf[c0 + t] = run;
    run += m[t];
  }
  if (threadIdx.x == kCdfThreads - 1) block_total[blockIdx.x] = run;
}

// exclusive scan of the block totals (one block; offsets written in place), cdf[n] = total
__global__ void __launch_bounds__(kCdfThreads) grid_cdf_totals_kernel(double *block_total, int n_blocks, double *cdf,
                                                                       int64_t n) {
  __shared__ double sh[kCdfThreads];
  __shared__ double round_total;
  double carry = 0.0;
  for (int b0 = 0; b0 < n_blocks; b0 += kCdfThreads) {
    const int b = b0 + threadIdx.x;
    const double v = b < n_blocks ? block_total[b] : 0.0;
    const double inc = block_inclusive_scan(v, sh);
    if (b < n_blocks) block_total[b] = carry + inc - v;
    if (threadIdx.x == kCdfThreads - 1) round_total = inc;
    __syncthreads();
    carry += round_total;
    __syncthreads();
  }
  if (threadIdx.x == 0) cdf[n] = carry;
}

__global__ void grid_cdf_offset_kernel(double *cdf, int64_t n, const double *block_offset) {
  const int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (c < n) cdf[c] += block_offset[c / kCdfPerBlock];
}

__global__ void proposal_sample_kernel(const float *node, const double *cdf, int g, int64_t n, uint64_t seed,
                                       double *f, double *lnq) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const U4 a = philox4x32_10(U4{(uint32_t)i, (uint32_t)(i >> 32), 1u, 0u}, (uint32_t)seed, (uint32_t)(seed >> 32));
  const U4 b = philox4x32_10(U4{(uint32_t)i, (uint32_t)(i >> 32), 2u, 0u}, (uint32_t)seed, (uint32_t)(seed >> 32));
  const double ua[3] = {u32_open0(b.x), u32_open0(b.y), u32_open0(b.z)};
  double x[3];
  const double l = grid_sample(node, cdf, g, u53(a.x, a.y), u53(a.z, a.w), ua, x);
  for (int k = 0; k < 3; ++k) f[3 * i + k] = x[k];
  lnq[i] = l;
}

__global__ void proposal_density_kernel(const float *node, const double *cdf, int g, const double *f, int64_t n,
                                        double *lnq) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double x[3] = {f[3 * i], f[3 * i + 1], f[3 * i + 2]};
  lnq[i] = grid_log_q(node, cdf, g, x);
}

// ============================================================================
// Fused forward pass (inference: kups_mlp_fwd and the grid refresh).  A persistent
// CTA (16 warps, one per SM) takes tiles of 256 points, two 128-row halves that share
// every weight chunk:
//   * features: each point's fractional coordinates reduced to [-0.5, 0.5) once in
//     float64 and split into float pairs, the 32 phases m_j . f as float pairs
//     (phase_sincos), written
//     straight into shared memory as the first layer's A operand (bfloat16,
//     no-swizzle K-major core matrices);
//   * weights: K-chunks of 64 columns of W [256, K] (32 KB) stream through a two-stage
//     ring of 16-byte cp.async copies; the chunk after the current one is in flight
//     while the tensor cores work on the current one (the copies run ahead across
//     layer and tile boundaries: they never depend on the activations);
//   * one thread issues tcgen05.mma (128 x 256 x 16, BF16 in, FP32 accumulate) for both
//     halves per K step into two accumulators of 256 tensor-memory columns each (all
//     512 columns) and commits each chunk to its stage's mbarrier;
//   * the epilogue (all warps: warp w reads TMEM lanes 32 (w % 4) .. + 31 of both halves,
//     64 columns w / 4 ..) adds the bias and applies softplus through the SFU
//     (exp2 / log2: the result is rounded to bfloat16), writes the next layer's A operand
//     into shared memory, and after the last layer folds in the head (w4 . h3 + b4).
// Every mbarrier wait is bounded; on time-out the kernel records KUPS_ERR_UNSUPPORTED,
// waits (bounded) for its own copies, frees its tensor memory and returns.
constexpr int kFwdThreads = 512, kFwdRows = 256, kFwdHalf = 128, kFwdKc = 64;

constexpr size_t kFwdA = (size_t)kFwdRows * kHid * 2;           // 128 KB: A operand, K up to 256
constexpr size_t kFwdStage = (size_t)kHid * kFwdKc * 2;          // 32 KB: one weight chunk
// shared memory: A operand | two weight stages | head partials [4][256] | coordinates [6][256] |
// biases b1 b2 b3 and head weights w4 [4][256] | frequencies [32][3] | b4 | mbarriers, TMEM slot
constexpr size_t kFwdOffPart = kFwdA + 2 * kFwdStage;
constexpr size_t kFwdOffFr = kFwdOffPart + 4 * kFwdRows * 4;
constexpr size_t kFwdOffPar = kFwdOffFr + 6 * kFwdRows * 4;
constexpr size_t kFwdOffFreq = kFwdOffPar + 4 * kHid * 4;
constexpr size_t kFwdOffB4 = kFwdOffFreq + 3 * kFreq * 4;
constexpr size_t kFwdOffBar = kFwdOffB4 + 16;
constexpr size_t kFwdSmem = kFwdOffBar + 64;
static_assert(kFwdOffBar % 8 == 0, "mbarriers are 8-byte aligned");

__device__ inline int fwd_core(int r, int kk, int K) {
  return ((r >> 3) * (K / 8) + (kk >> 3)) * 64 + (r & 7) * 8 + (kk & 7);
}

// Chunk q of the per-tile sequence W1 (1 chunk of 64 columns), W2 (4), W3 (4).
constexpr int kFwdChunks = 1 + 4 + 4;
__device__ inline void fwd_chunk_of(int q, int &layer, int &kc) {
  layer = q == 0 ? 0 : (q <= 4 ? 1 : 2);
  kc = q == 0 ? 0 : (q <= 4 ? q - 1 : q - 5);
}

// columns [64 kc, 64 kc + 64) of W [256, K] -> core-matrix layout of 256 rows x 64; copy e
// takes row (e / 64) * 8 + e % 8, column group (e / 8) % 8 and lands at element 8 e
__device__ inline void fwd_stage_chunk(__nv_bfloat16 *sB, const __nv_bfloat16 *pb, int q, int tid) {
  int layer, kc;
  fwd_chunk_of(q, layer, kc);
  const __nv_bfloat16 *W = pb + (layer == 0 ? kOffW1 : layer == 1 ? kOffW2 : kOffW3);
  const int K = layer == 0 ? kIn : kHid;
  const uint32_t s0 = smem_u32(sB);
  for (int e = tid; e < kHid * (kFwdKc / 8); e += kFwdThreads) {
    const int lo = e & 7, kg = (e >> 3) & 7, rb = e >> 6;
    cp_async16(s0 + (uint32_t)e * 16u, W + (size_t)(rb * 8 + lo) * K + kc * kFwdKc + kg * 8, 16u);
  }
}

__global__ void __launch_bounds__(kFwdThreads, 1)
mlp_forward_kernel(const __nv_bfloat16 *pb, const float *p, const int32_t *freq, const double *x, int64_t n,
                   int grid, float *g_out, kups_status *status) {
  extern __shared__ __align__(1024) unsigned char smem[];
  __nv_bfloat16 *sA = reinterpret_cast<__nv_bfloat16 *>(smem);
  auto sB = [&](int st) { return reinterpret_cast<__nv_bfloat16 *>(smem + kFwdA + st * kFwdStage); };
  float *part = reinterpret_cast<float *>(smem + kFwdOffPart);  // [4][256] head partials
  float *fr = reinterpret_cast<float *>(smem + kFwdOffFr);       // [6][256] coordinates hi, lo
  float *spar = reinterpret_cast<float *>(smem + kFwdOffPar);    // [4][256] b1, b2, b3, w4
  int32_t *sfreq = reinterpret_cast<int32_t *>(smem + kFwdOffFreq);
  float *sb4 = reinterpret_cast<float *>(smem + kFwdOffB4);
  uint64_t *mbar = reinterpret_cast<uint64_t *>(smem + kFwdOffBar);  // [2]
  uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(mbar + 2);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  for (int e = tid; e < 4 * kHid; e += kFwdThreads) {
    const int which = e / kHid;
    const int64_t off = which == 0 ? kOffB1 : which == 1 ? kOffB2 : which == 2 ? kOffB3 : kOffW4;
    spar[e] = p[off + e % kHid];
  }
  for (int e = tid; e < 3 * kFreq; e += kFwdThreads) sfreq[e] = freq[e];
  if (tid == 0) sb4[0] = p[kOffB4];
  const int quarter = warp & 3, cq = warp >> 2;  // TMEM lanes 32 quarter .., columns 64 cq .. of each half
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(2 * kHid));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (tid == 0) {
    mbar_init(smem_u32(&mbar[0]), 1);
    mbar_init(smem_u32(&mbar[1]), 1);
  }
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tmem_slot;
  const uint32_t idesc = make_idesc(kFwdHalf, kHid);
  // per stage (bit st): parity of the next completion to wait for, and whether MMAs reading it are
  // in flight (bit fields, not arrays: the stage index is dynamic)
  uint32_t phase = 0u, pending = 0u;
  bool ok = true;
  const int64_t n_tiles = (n + kFwdRows - 1) / kFwdRows;
  const int64_t my_tiles = blockIdx.x < n_tiles ? (n_tiles - 1 - blockIdx.x) / gridDim.x + 1 : 0;
  const int64_t total_chunks = my_tiles * kFwdChunks;
  int64_t qg = 0;  // this CTA's chunk counter; stage qg & 1
  if (total_chunks > 0) {
    fwd_stage_chunk(sB(0), pb, 0, tid);
    cp_async_commit();
  }
  for (int64_t t = 0; t < my_tiles && ok; ++t) {
    const int64_t tile = blockIdx.x + t * gridDim.x;
    // coordinates of the tile's points reduced to [-0.5, 0.5) in float64, kept in float32
    if (tid < kFwdRows) {
      const int64_t pt = tile * kFwdRows + tid;
      double f[3] = {0.0, 0.0, 0.0};
      if (pt < n) {
        if (x != nullptr) {
          for (int a = 0; a < 3; ++a) f[a] = x[3 * pt + a];
        } else {
          const int64_t g2 = (int64_t)grid * grid;
          f[0] = (double)(pt / g2) / grid;
          f[1] = (double)((pt / grid) % grid) / grid;
          f[2] = (double)(pt % grid) / grid;
        }
      }
      for (int a = 0; a < 3; ++a) {
        const double red = f[a] - rint(f[a]);
        const float hi = (float)red;
        fr[a * kFwdRows + tid] = hi;
        fr[(3 + a) * kFwdRows + tid] = (float)(red - (double)hi);
      }
    }
    __syncthreads();
    for (int e = tid; e < kFwdRows * kFreq; e += kFwdThreads) {
      const int r = e % kFwdRows, j = e / kFwdRows;
      const int64_t pt = tile * kFwdRows + r;
      float sn = 0.f, cs = 0.f;
      if (pt < n) {
        const float fh[3] = {fr[r], fr[kFwdRows + r], fr[2 * kFwdRows + r]};
        const float fl[3] = {fr[3 * kFwdRows + r], fr[4 * kFwdRows + r], fr[5 * kFwdRows + r]};
        phase_sincos(sfreq + 3 * j, fh, fl, sn, cs);
      }
      *reinterpret_cast<__nv_bfloat162 *>(sA + fwd_core(r, 2 * j, kIn)) = __floats2bfloat162_rn(sn, cs);
    }
    for (int layer = 0; layer < 3 && ok; ++layer) {
      const int K = layer == 0 ? kIn : kHid;
      const int nch = K / kFwdKc;
      for (int c = 0; c < nch && ok; ++c, ++qg) {
        const int st = (int)(qg & 1), nx = st ^ 1;
        if (qg + 1 < total_chunks) {
          if ((pending >> nx) & 1u) {  // the MMAs of chunk qg - 1 read stage nx
            ok = mbar_wait(smem_u32(&mbar[nx]), (phase >> nx) & 1u);
            if (ok) {  // after a time-out the clean-up waits for these MMAs again
              phase ^= 1u << nx;
              pending &= ~(1u << nx);
            }
          }
          if (!__syncthreads_and(ok)) {
            ok = false;
            break;
          }
          fwd_stage_chunk(sB(nx), pb, (int)((qg + 1) % kFwdChunks), tid);
          cp_async_commit();
          cp_async_wait<1>();  // chunk qg has landed (this thread's copies)
        } else {
          cp_async_wait<0>();
        }
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // A written by the generic proxy
        __syncthreads();
        if (tid == 0) {
          asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
          for (int ks = 0; ks < kFwdKc / 16; ++ks) {
            const uint64_t bd = make_sdesc(smem_u32(sB(st)) + ks * 256, 128, (kFwdKc / 8) * 128);
            const uint32_t accumulate = (c > 0 || ks > 0) ? 1u : 0u;
            for (int h = 0; h < 2; ++h) {
              const uint64_t ad = make_sdesc(smem_u32(sA) + (uint32_t)(h * kFwdHalf * K * 2) + (c * 4 + ks) * 256,
                                             128, (K / 8) * 128);
              asm volatile(
                  "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
                  " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(tmem + (uint32_t)(h * kHid)),
                  "l"(ad), "l"(bd), "r"(idesc), "r"(accumulate));
            }
          }
          asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                           smem_u32(&mbar[st]))
                       : "memory");
        }
        pending |= 1u << st;
        if (c == nch - 1) {  // the layer's accumulators are complete once its last chunk is
          ok = mbar_wait(smem_u32(&mbar[st]), (phase >> st) & 1u);
          if (ok) {
            phase ^= 1u << st;
            pending &= ~(1u << st);
          }
        }
      }
      if (!__syncthreads_and(ok)) {
        ok = false;
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const float *bias = spar + layer * kHid;
      const float *w4 = spar + 3 * kHid;
      for (int h = 0; h < 2; ++h) {
        const int row = h * kFwdHalf + quarter * 32 + lane;
        float head = 0.f;
        for (int c0 = cq * (kHid / 4); c0 < (cq + 1) * (kHid / 4); c0 += 32) {
          uint32_t r[32];
          const uint32_t taddr = tmem + ((uint32_t)(quarter * 32) << 16) + (uint32_t)(h * kHid + c0);
          asm volatile(
              "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, "
              "%13, %14, %15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
              : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
                "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
                "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
              : "r"(taddr));
          asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
          if (layer < 2) {
            // next layer's A operand: 4 core-matrix rows of 8 bfloat16 (16 bytes each)
#pragma unroll
            for (int q = 0; q < 4; ++q) {
              __nv_bfloat162 hv[4];
#pragma unroll
              for (int u = 0; u < 4; ++u) {
                const int i = q * 8 + 2 * u;
                hv[u] = __floats2bfloat162_rn(softplus_fast(__uint_as_float(r[i]) + bias[c0 + i]),
                                              softplus_fast(__uint_as_float(r[i + 1]) + bias[c0 + i + 1]));
              }
              *reinterpret_cast<uint4 *>(sA + fwd_core(row, c0 + q * 8, kHid)) = *reinterpret_cast<uint4 *>(hv);
            }
          } else {
#pragma unroll
            for (int i = 0; i < 32; ++i)
              head = fmaf(softplus_fast(__uint_as_float(r[i]) + bias[c0 + i]), w4[c0 + i], head);
          }
        }
        if (layer == 2) part[cq * kFwdRows + row] = head;
      }
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      __syncthreads();
      if (layer == 2 && tid < kFwdRows) {
        const int64_t pt = tile * kFwdRows + tid;
        if (pt < n)
          g_out[pt] = ((part[tid] + part[kFwdRows + tid]) + (part[2 * kFwdRows + tid] + part[3 * kFwdRows + tid])) +
                      sb4[0];
      }
    }
  }
  cp_async_wait<0>();
  // a time-out leaves MMAs possibly in flight: wait for them (bounded) before freeing TMEM
  for (int st = 0; st < 2; ++st)
    if ((pending >> st) & 1u) {
      (void)mbar_wait(smem_u32(&mbar[st]), (phase >> st) & 1u);
      pending &= ~(1u << st);
    }
  if (!ok && tid == 0) status_error(status, KUPS_ERR_UNSUPPORTED, blockIdx.x);
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(2 * kHid));
}

int32_t fused_forward(const kups_mlp *net, const double *x, int64_t n, int grid, float *g, kups_status *status,
                      cudaStream_t st) {
  if (n <= 0) return KUPS_OK;
  KUPS_CUDA_TRY(cudaFuncSetAttribute(mlp_forward_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kFwdSmem));
  const int sms = device_sm_count();
  const int64_t tiles = (n + kFwdRows - 1) / kFwdRows;
  const unsigned ctas = (unsigned)std::min<int64_t>(tiles, sms);
  mlp_forward_kernel<<<ctas, kFwdThreads, kFwdSmem, st>>>((const __nv_bfloat16 *)net->param_bf16, net->param,
                                                          net->freq, x, n, grid, g, status);
  return cudaGetLastError() == cudaSuccess ? KUPS_OK : KUPS_ERR_CUDA;
}

inline unsigned blocks(int64_t n, int t) { return (unsigned)((n + t - 1) / t); }

// Forward pass of rows [row0, row0 + c) into w (activations) and g_out; ``train``
// also writes the transposed copies the weight gradients need.
int32_t forward_chunk(const kups_mlp *net, const double *x, int64_t row0, int64_t c, int grid, const MlpWork &w,
                      float *g_out, kups_status *status, cudaStream_t st, bool train = false) {
  const __nv_bfloat16 *pb = (const __nv_bfloat16 *)net->param_bf16;
  const float *p = net->param;
  features_kernel<<<blocks(c, 256), 256, 0, st>>>(x, row0, c, grid, net->freq, w.feat, train ? w.featT : nullptr);
  int32_t rc;
  rc = gemm_call(Op{w.feat, 1, kIn, 1}, Op{pb + kOffW1, 1, kIn, 1}, w.h1, kHid, 1, w.h1b, p + kOffB1, nullptr, 0,
                 (int)c, kHid, kIn, 0.f, 2, 1, status, st, train ? w.h1T : nullptr);
  if (rc) return rc;
  rc = gemm_call(Op{w.h1b, 1, kHid, 1}, Op{pb + kOffW2, 1, kHid, 1}, w.h2, kHid, 1, w.h2b, p + kOffB2, nullptr, 0,
                 (int)c, kHid, kHid, 0.f, 2, 1, status, st, train ? w.h2T : nullptr);
  if (rc) return rc;
  rc = gemm_call(Op{w.h2b, 1, kHid, 1}, Op{pb + kOffW3, 1, kHid, 1}, w.h3, kHid, 1, nullptr, p + kOffB3, nullptr, 0,
                 (int)c, kHid, kHid, 0.f, 2, 1, status, st);
  if (rc) return rc;
  if (g_out != nullptr) head_kernel<<<blocks(c * 32, 256), 256, 0, st>>>(w.h3, c, p + kOffW4, p + kOffB4, g_out);
  return cudaGetLastError() == cudaSuccess ? KUPS_OK : KUPS_ERR_CUDA;
}

int split_for(int64_t k) {
  const int64_t chunks = (k + kBK - 1) / kBK;
  return (int)std::max<int64_t>(1, std::min<int64_t>(74, chunks / 4));
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
                                  int32_t split_k, kups_status *status, void *stream) {
  if (m <= 0 || n <= 0 || k <= 0 || act < 0 || act > 2 || gate_kind < 0 || gate_kind > 3 || split_k < 1 ||
      split_k > 65535)
    return KUPS_ERR_INVALID;
  // split-K accumulates into float32 C with atomics: no epilogue terms but alpha
  if (split_k > 1 && (c_bf16 || c2 || bias || gate_kind || act || beta != 1.f)) return KUPS_ERR_INVALID;
  GemmArgs g;
  g.a = a; g.b = b; g.c = c; g.c2 = c2; g.bias = bias; g.gate = gate;
  g.sar = sa_row; g.sac = sa_col; g.sbr = sb_row; g.sbc = sb_col; g.scr = sc_row; g.scc = sc_col;
  g.sc2r = sc2_row; g.sc2c = sc2_col; g.sgr = sg_row; g.sgc = sg_col;
  g.m = m; g.n = n; g.k = k; g.alpha = alpha; g.beta = beta; g.act = act;
  g.a_bf16 = a_bf16; g.b_bf16 = b_bf16; g.c_bf16 = c_bf16; g.c2_bf16 = c2_bf16; g.gate_kind = gate_kind;
  g.split_k = split_k;
  g.c3 = nullptr;
  g.sc3r = g.sc3c = 0;
  g.fast_math = 0;
  return dispatch_gemm(g, status, (cudaStream_t)stream);
}

extern "C" size_t kups_mlp_workspace_bytes(int64_t n_points) {
  return work_bytes(std::max<int64_t>(1, std::min<int64_t>(n_points, kChunk)));
}

extern "C" int32_t kups_mlp_init(const kups_mlp *net, uint64_t seed, void *stream) {
  if (net == nullptr) return KUPS_ERR_INVALID;
  init_kernel<<<blocks(kParams, 256), 256, 0, (cudaStream_t)stream>>>(
      net->param, (__nv_bfloat16 *)net->param_bf16, (__nv_bfloat16 *)net->param_bf16_t, net->grad, net->adam_m,
      net->adam_v, seed);
  return cudaGetLastError() == cudaSuccess ? KUPS_OK : KUPS_ERR_CUDA;
}

extern "C" int32_t kups_mlp_fwd(const kups_mlp *net, const double *x, int64_t n, float *g, void *workspace,
                                size_t workspace_bytes, kups_status *status, void *stream) {
  if (net == nullptr || n < 0 || (n > 0 && (x == nullptr || g == nullptr))) return KUPS_ERR_INVALID;
  if (workspace_bytes < kups_mlp_workspace_bytes(n)) return KUPS_ERR_INVALID;
  (void)workspace;
  return fused_forward(net, x, n, 0, g, status, (cudaStream_t)stream);
}

extern "C" int32_t kups_mlp_nce_batch(const double *data, int64_t n_data, int32_t batch, uint64_t seed,
                                      uint64_t step, double *x, float *label, void *stream) {
  if (n_data <= 0 || batch <= 0 || (batch & 1)) return KUPS_ERR_INVALID;
  nce_batch_kernel<<<blocks(batch, 256), 256, 0, (cudaStream_t)stream>>>(data, n_data, batch, seed, step, x, label);
  return cudaGetLastError() == cudaSuccess ? KUPS_OK : KUPS_ERR_CUDA;
}

extern "C" int32_t kups_mlp_bwd(const kups_mlp *net, const double *x, const float *label, int32_t n, float *loss,
                                void *workspace, size_t workspace_bytes, kups_status *status, void *stream) {
  if (net == nullptr || n <= 0 || n > kChunk) return KUPS_ERR_INVALID;
  if (workspace_bytes < kups_mlp_workspace_bytes(n)) return KUPS_ERR_INVALID;
  cudaStream_t st = (cudaStream_t)stream;
  const MlpWork w = carve(workspace, n);
  int32_t rc = forward_chunk(net, x, 0, n, 0, w, nullptr, status, st, true);
  if (rc) return rc;
  const __nv_bfloat16 *pbt = (const __nv_bfloat16 *)net->param_bf16_t;  // W2^T, W3^T
  const float *p = net->param;
  float *gr = net->grad;
  const int sms = 148;
  head_nce_kernel<<<std::min<int64_t>(blocks(n, 32), 4 * sms), 256, 0, st>>>(
      w.h3, n, p + kOffW4, p + kOffB4, label, w.dza, w.dzab, w.dzaT, gr + kOffW4, gr + kOffB4, loss);
  const int split = split_for(n);
  const unsigned cs_blocks = (unsigned)std::min<int64_t>(blocks(n, 32), 4 * sms);
  // Every GEMM operand is bfloat16 with K contiguous: the weight gradients read the
  // transposed copies ([width, n], K = points), the input gradients W^T.
  // layer 3: dW3 += dz3^T h2, db3 += colsum dz3, dz2 = (dz3 W3) * (1 - exp(-h2))
  rc = gemm_call(Op{w.dzaT, 1, n, 1}, Op{w.h2T, 1, n, 1}, gr + kOffW3, kHid, 1, nullptr, nullptr, nullptr, 0, kHid,
                 kHid, n, 1.f, 0, split, status, st);
  if (rc) return rc;
  colsum_kernel<<<cs_blocks, kHid, 0, st>>>(w.dza, n, gr + kOffB3);
  rc = gemm_call(Op{w.dzab, 1, kHid, 1}, Op{pbt + kHid * kHid, 1, kHid, 1}, w.dzb, kHid, 1, w.dzbb, nullptr, w.h2, 3,
                 n, kHid, kHid, 0.f, 0, 1, status, st, w.dzbT);
  if (rc) return rc;
  // layer 2
  rc = gemm_call(Op{w.dzbT, 1, n, 1}, Op{w.h1T, 1, n, 1}, gr + kOffW2, kHid, 1, nullptr, nullptr, nullptr, 0, kHid,
                 kHid, n, 1.f, 0, split, status, st);
  if (rc) return rc;
  colsum_kernel<<<cs_blocks, kHid, 0, st>>>(w.dzb, n, gr + kOffB2);
  rc = gemm_call(Op{w.dzbb, 1, kHid, 1}, Op{pbt, 1, kHid, 1}, w.dza, kHid, 1, nullptr, nullptr, w.h1, 3, n, kHid,
                 kHid, 0.f, 0, 1, status, st, w.dzaT);
  if (rc) return rc;
  // layer 1 (no gradient into the features)
  rc = gemm_call(Op{w.dzaT, 1, n, 1}, Op{w.featT, 1, n, 1}, gr + kOffW1, kIn, 1, nullptr, nullptr, nullptr, 0, kHid,
                 kIn, n, 1.f, 0, split, status, st);
  if (rc) return rc;
  colsum_kernel<<<cs_blocks, kHid, 0, st>>>(w.dza, n, gr + kOffB1);
  return cudaGetLastError() == cudaSuccess ? KUPS_OK : KUPS_ERR_CUDA;
}

extern "C" int32_t kups_mlp_adam(const kups_mlp *net, int64_t t, float lr, float beta1, float beta2, float eps,
                                 void *stream) {
  if (net == nullptr || t < 1) return KUPS_ERR_INVALID;
  const float c1 = (float)(1.0 / (1.0 - pow((double)beta1, (double)t)));
  const float c2 = (float)(1.0 / (1.0 - pow((double)beta2, (double)t)));
  adam_kernel<<<blocks(kParams, 256), 256, 0, (cudaStream_t)stream>>>(
      net->param, (__nv_bfloat16 *)net->param_bf16, (__nv_bfloat16 *)net->param_bf16_t, net->grad, net->adam_m,
      net->adam_v, kParams, lr, beta1, beta2, eps, c1, c2);
  return cudaGetLastError() == cudaSuccess ? KUPS_OK : KUPS_ERR_CUDA;
}

extern "C" int32_t kups_mlp_grid_norm(const kups_mlp *net, int32_t grid, float temper, float floor_frac,
                                      float *node, double *cdf, void *workspace, size_t workspace_bytes,
                                      kups_status *status, void *stream) {
  if (net == nullptr || grid < 2 || grid > 256 || !(floor_frac > 0.f) || !(temper > 0.f)) return KUPS_ERR_INVALID;
  const int64_t n = (int64_t)grid * grid * grid;
  if (workspace_bytes < kups_mlp_workspace_bytes(n)) return KUPS_ERR_INVALID;
  cudaStream_t st = (cudaStream_t)stream;
  const MlpWork w = carve(workspace, std::min<int64_t>(n, kChunk));
  const int32_t rc = fused_forward(net, nullptr, n, grid, node, status, st);
  if (rc) return rc;
  // the normaliser's partials and the scan's block totals live in the (unused) activation buffers
  double *partial = reinterpret_cast<double *>(w.h2);
  const int n_norm = (int)std::min<int64_t>(kNormBlocks, (n + kNormThreads - 1) / kNormThreads);
  grid_partials_kernel<<<n_norm, kNormThreads, 0, st>>>(node, n, temper, partial, status);
  grid_apply_kernel<<<4 * kNormBlocks, 256, 0, st>>>(node, n, temper, floor_frac, partial, n_norm);
  // three-pass scan
  const int n_blocks = (int)((n + kCdfPerBlock - 1) / kCdfPerBlock);
  double *totals = reinterpret_cast<double *>(w.h1);
  grid_cdf_local_kernel<<<n_blocks, kCdfThreads, 0, st>>>(node, grid, cdf, totals);
  grid_cdf_totals_kernel<<<1, kCdfThreads, 0, st>>>(totals, n_blocks, cdf, n);
  grid_cdf_offset_kernel<<<blocks(n, 256), 256, 0, st>>>(cdf, n, totals);
  return cudaGetLastError() == cudaSuccess ? KUPS_OK : KUPS_ERR_CUDA;
}

extern "C" int32_t kups_proposal_sample(const float *node, const double *cdf, int32_t grid, int64_t n,
                                        uint64_t seed, double *f, double *log_q, void *stream) {
  if (grid < 2 || n < 0) return KUPS_ERR_INVALID;
  if (n == 0) return KUPS_OK;
  proposal_sample_kernel<<<blocks(n, 128), 128, 0, (cudaStream_t)stream>>>(node, cdf, grid, n, seed, f, log_q);
  return cudaGetLastError() == cudaSuccess ? KUPS_OK : KUPS_ERR_CUDA;
}

extern "C" int32_t kups_proposal_log_density(const float *node, const double *cdf, int32_t grid, const double *f,
                                             int64_t n, double *log_q, void *stream) {
  if (grid < 2 || n < 0) return KUPS_ERR_INVALID;
  if (n == 0) return KUPS_OK;
  proposal_density_kernel<<<blocks(n, 128), 128, 0, (cudaStream_t)stream>>>(node, cdf, grid, f, n, log_q);
  return cudaGetLastError() == cudaSuccess ? KUPS_OK : KUPS_ERR_CUDA;
}
