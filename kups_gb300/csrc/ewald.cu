// Ewald summation: reciprocal-space structure factor, energy, forces and
// cell gradient; self energy; real-space pair terms over an edge list.
//
// Replaces src/kups/potential/classical/ewald.py: EwaldLongRangeInput.kvecs
// (:265-274, k = 2 pi L^-1 n), prefactor (:363-391), _frequency_response /
// _structure_factor_full (:394-439), long_range (:349-360),
// ewald_long_range_energy (:585-601), ewald_self_interaction_energy
// (:277-302), ewald_short_range_energy (:305-325), exclusion_correction_energy
// (:328-346) with coulomb_vacuum_energy (coulomb.py:64-83), and the jax.vjp
// gradients PotentialFromEnergy takes of them (energy.py:264-355).
//
// Reciprocal space, per system s with n_k integer vectors n (zero rows are
// padding, masked like k = 0):
//   theta_ik = 2 pi n_k . f_i  (f = fractional coordinates),
//   S(k) = sum_i q_i (cos, sin)(theta_ik)            [float64 accumulation]
//   P(k) = (2 - [n_x = 0]) 2 pi / V exp(-k^2 / 4 alpha^2) / k^2
//   E = K sum_k P(k) |S(k)|^2
//   dE/dr_i = 2 K q_i sum_k P(k) k (S_s cos - S_c sin)(theta_ik)
//   dE/dL_ab = sum_i f_ia F_ib - sum_k c_k (L^-T k)_a k_b - delta_ab E / L_aa,
//   c_k = K |S|^2 P (-1 / (2 alpha^2) - 2 / k^2)    (F = -dE/dr)
// e^{i theta} is built per atom from per-axis tables e^{2 pi i m f_a},
// m in [-M, M] (the standard Ewald recurrence), so each (atom, k) costs two
// complex products.
#include <algorithm>
#include <mutex>

#include "common.cuh"

namespace kups {
namespace {

constexpr int kMaxM = 16;            // |n_a| <= 16
constexpr int kTab = 2 * kMaxM + 1;  // table entries per axis
constexpr int kAtomsPerChunk = 32;
constexpr int kKPerBlock = 128;

struct Coef {
  double ps_c, ps_s, ck, pad;  // P S_c, P S_s, cell-gradient coefficient
};

struct RecipSys {
  double inv[6];  // L^-1 (tril)
  double L[6];
  double volume;
  int m[3];       // table half-widths actually used
};

__device__ inline void frac64(const double *inv, const double r[3], double f[3]) {
  f[0] = (r[0] * inv[0] + r[1] * inv[1]) + r[2] * inv[3];
  f[1] = r[1] * inv[2] + r[2] * inv[4];
  f[2] = r[2] * inv[5];
}

// k = 2 pi L^-1 n  (column vector), written for the lower-triangular inverse.
__device__ inline void kvec(const double *inv, const int n[3], double k[3]) {
  const double tp = 6.283185307179586476925286766559;
  k[0] = tp * (inv[0] * n[0]);
  k[1] = tp * (inv[1] * n[0] + inv[2] * n[1]);
  k[2] = tp * (inv[3] * n[0] + inv[4] * n[1] + inv[5] * n[2]);
}

// One block per system: cell, inverse, volume, and the largest |n_a| over the
// system's k vectors (block reduction).
__global__ void recip_setup_kernel(const double *tril, const int32_t *kn, int32_t s, int32_t nk,
                                   RecipSys *sys, kups_status *status) {
  __shared__ int mx[3];
  const int i = blockIdx.x;
  if (threadIdx.x < 3) mx[threadIdx.x] = 0;
  __syncthreads();
  int m[3] = {0, 0, 0};
  for (int k = threadIdx.x; k < nk; k += blockDim.x)
    for (int a = 0; a < 3; ++a) m[a] = max(m[a], abs(kn[((int64_t)i * nk + k) * 3 + a]));
  for (int a = 0; a < 3; ++a) atomicMax(&mx[a], m[a]);
  __syncthreads();
  if (threadIdx.x != 0) return;
  RecipSys r;
  const Tril64 L = load_tril64(tril + 6 * (int64_t)i);
  const Tril64 inv = inverse_tril64(L);
  for (int k = 0; k < 6; ++k) {
    r.L[k] = L.t[k];
    r.inv[k] = inv.t[k];
  }
  r.volume = fabs(L.t[0] * L.t[2] * L.t[5]);
  for (int a = 0; a < 3; ++a) {
    int v = mx[a];
    if (v > kMaxM) {
      status_error(status, KUPS_ERR_UNSUPPORTED, i);
      v = kMaxM;
    }
    r.m[a] = v;
  }
  sys[i] = r;
}

// Per-atom tables e^{2 pi i m f_a}, m in [-M, M], from sincospi of the
// fundamental and complex products (error grows ~linearly in |m| <= 16).
__device__ inline void fill_tables(float2 *tab, const double f[3]) {
  for (int a = 0; a < 3; ++a) {
    float s1, c1;
    // reduce f to [-0.5, 0.5) in float64 first so the float32 argument is small
    const double fr = f[a] - rint(f[a]);
    sincospif((float)(2.0 * fr), &s1, &c1);
    float2 *t = tab + a * kTab + kMaxM;
    t[0] = make_float2(1.f, 0.f);
    float cr = 1.f, ci = 0.f;
    for (int m = 1; m <= kMaxM; ++m) {
      const float nr = cr * c1 - ci * s1;
      const float ni = cr * s1 + ci * c1;
      cr = nr;
      ci = ni;
      t[m] = make_float2(cr, ci);
      t[-m] = make_float2(cr, -ci);
    }
  }
}

__device__ inline float2 cmul(float2 a, float2 b) {
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

// S(k): grid (k tiles, atom chunks, systems).  Each block stages the tables of
// 32 atoms in shared memory; each thread owns one k and accumulates the
// chunk in float32, then adds it to S in float64.
__global__ void structure_factor_kernel(const double *pos, const double *q, const int32_t *sys_offset,
                                        const int32_t *kn, int32_t nk, const RecipSys *sysp,
                                        double *sk, double *grad) {
  __shared__ float2 tab[kAtomsPerChunk][3 * kTab];
  __shared__ float qs[kAtomsPerChunk];
  const int s = blockIdx.z;
  const int a0 = sys_offset[s], a1 = sys_offset[s + 1];
  const int c0 = a0 + blockIdx.y * kAtomsPerChunk;
  if (c0 >= a1) return;
  const int na = min(kAtomsPerChunk, a1 - c0);
  const RecipSys &P = sysp[s];
  for (int t = threadIdx.x; t < na; t += blockDim.x) {
    const double r[3] = {pos[3 * (c0 + t)], pos[3 * (c0 + t) + 1], pos[3 * (c0 + t) + 2]};
    double f[3];
    frac64(P.inv, r, f);
    fill_tables(tab[t], f);
    qs[t] = (float)q[c0 + t];
    // the force kernel adds its k-range partials into grad: zero this chunk's rows first
    if (blockIdx.x == 0 && grad != nullptr)
      for (int a = 0; a < 3; ++a) grad[3 * (int64_t)(c0 + t) + a] = 0.0;
  }
  __syncthreads();
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nk) return;
  const int *nv = kn + ((int64_t)s * nk + k) * 3;
  const int nx = nv[0] + kMaxM, ny = nv[1] + kMaxM, nz = nv[2] + kMaxM;
  float sc = 0.f, ss = 0.f;
  for (int t = 0; t < na; ++t) {
    const float2 e = cmul(cmul(tab[t][nx], tab[t][kTab + ny]), tab[t][2 * kTab + nz]);
    sc = fmaf(qs[t], e.x, sc);
    ss = fmaf(qs[t], e.y, ss);
  }
  atomicAdd(&sk[((int64_t)s * nk + k) * 2], (double)sc);
  atomicAdd(&sk[((int64_t)s * nk + k) * 2 + 1], (double)ss);
}

// Per system: energy and the per-k coefficients; one block per system.
//   coef[k] = (P S_c, P S_s, c_k)  with c_k for the cell gradient.
__global__ void recip_energy_kernel(const int32_t *kn, int32_t nk, const double *alpha,
                                    const RecipSys *sysp, const double *sk, double ke,
                                    Coef *coef, double *energy, double *dtril) {
  __shared__ double red[40];
  const int s = blockIdx.y;
  const RecipSys &P = sysp[s];
  const double a = alpha[s];
  const double tp = 6.283185307179586476925286766559;
  double e = 0.0, w[6] = {0, 0, 0, 0, 0, 0};
  // L^-T k: (L^-T)_{ab} = inv_{ba}
  const double *iv = P.inv;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nk; k += gridDim.x * blockDim.x) {
    const int *nv = kn + ((int64_t)s * nk + k) * 3;
    const int n3[3] = {nv[0], nv[1], nv[2]};
    double kv[3];
    kvec(iv, n3, kv);
    const double k2 = kv[0] * kv[0] + kv[1] * kv[1] + kv[2] * kv[2];
    double p = 0.0, ck = 0.0;
    const double sc = sk[((int64_t)s * nk + k) * 2], ss = sk[((int64_t)s * nk + k) * 2 + 1];
    const double s2 = sc * sc + ss * ss;
    if (k2 > 0.0) {
      p = (2.0 - (n3[0] == 0 ? 1.0 : 0.0)) * tp / P.volume * exp(-k2 / (4.0 * a * a)) / k2;
      ck = ke * s2 * p * (-1.0 / (2.0 * a * a) - 2.0 / k2);
    }
    e += ke * p * s2;
    coef[(int64_t)s * nk + k] = Coef{p * sc, p * ss, ck, 0.0};
    // u = L^-T k
    const double u0 = iv[0] * kv[0] + iv[1] * kv[1] + iv[3] * kv[2];
    const double u1 = iv[2] * kv[1] + iv[4] * kv[2];
    const double u2 = iv[5] * kv[2];
    w[0] += ck * u0 * kv[0];
    w[1] += ck * u1 * kv[0];
    w[2] += ck * u1 * kv[1];
    w[3] += ck * u2 * kv[0];
    w[4] += ck * u2 * kv[1];
    w[5] += ck * u2 * kv[2];
  }
  const double et = block_sum(e, red);
  __syncthreads();
  double wt[6];
  for (int c = 0; c < 6; ++c) {
    wt[c] = block_sum(w[c], red);
    __syncthreads();
  }
  // blocks of k vectors add their shares (energy and dtril zeroed by the launcher)
  if (threadIdx.x == 0) {
    atomicAdd(&energy[s], et);
    if (dtril) {
      const int diag[6] = {1, 0, 1, 0, 0, 1};
      const int dk[6] = {0, -1, 2, -1, -1, 5};
      for (int c = 0; c < 6; ++c) {
        double v = -wt[c];
        if (diag[c]) v -= et / P.L[dk[c]];
        atomicAdd(&dtril[6 * (int64_t)s + c], v);  // the sum_i f F part is added by the force kernel
      }
    }
  }
}

// dE/dr_i for every atom of every system (thread per atom; k coefficients
// staged through shared memory), plus the sum_i f_ia F_ib part of dE/dL.
__global__ void recip_force_kernel(const double *pos, const double *q, const int32_t *sys_offset,
                                   const int32_t *kn, int32_t nk, const RecipSys *sysp,
                                   const Coef *coef, double ke, double *grad, double *dtril,
                                   int kblocks_per_split) {
  __shared__ float2 tab[kAtomsPerChunk][3 * kTab];
  __shared__ float4 kc[kKPerBlock];  // (P S_c, P S_s, -, -) as float
  __shared__ int4 kni[kKPerBlock];
  __shared__ double red[40];
  const int s = blockIdx.y;
  const int a0 = sys_offset[s], a1 = sys_offset[s + 1];
  const int c0 = a0 + blockIdx.x * kAtomsPerChunk;
  if (c0 >= a1) return;
  const int na = min(kAtomsPerChunk, a1 - c0);
  const RecipSys &P = sysp[s];
  const int t = threadIdx.x;  // blockDim.x == kAtomsPerChunk * 4: 4 lanes per atom split k
  const int atom = t >> 2, sub = t & 3;
  double f[3] = {0, 0, 0};
  if (t < na) {
    const double r[3] = {pos[3 * (c0 + t)], pos[3 * (c0 + t) + 1], pos[3 * (c0 + t) + 2]};
    frac64(P.inv, r, f);
    fill_tables(tab[t], f);
  }
  __syncthreads();
  // gradient in fractional components: dE/df_a = sum_k 2 K q P 2 pi n_a (Ss c - Sc s)
  float g0 = 0.f, g1 = 0.f, g2 = 0.f;
  // this block's share of the k vectors (blockIdx.z); partials are added into grad
  const int kbeg = blockIdx.z * kblocks_per_split * kKPerBlock;
  const int kfin = min(nk, kbeg + kblocks_per_split * kKPerBlock);
  for (int kb = kbeg; kb < kfin; kb += kKPerBlock) {
    __syncthreads();
    for (int j = threadIdx.x; j < kKPerBlock; j += blockDim.x) {
      if (kb + j < nk) {
        const Coef cc = coef[(int64_t)s * nk + kb + j];
        kc[j] = make_float4((float)cc.ps_c, (float)cc.ps_s, 0.f, 0.f);
        const int *nv = kn + ((int64_t)s * nk + kb + j) * 3;
        kni[j] = make_int4(nv[0], nv[1], nv[2], 0);
      } else {
        kc[j] = make_float4(0.f, 0.f, 0.f, 0.f);
        kni[j] = make_int4(0, 0, 0, 0);
      }
    }
    __syncthreads();
    if (atom < na) {
      const int kend = min(kKPerBlock, kfin - kb);
      for (int j = sub; j < kend; j += 4) {
        const int4 n3 = kni[j];
        const float2 e = cmul(cmul(tab[atom][n3.x + kMaxM], tab[atom][kTab + n3.y + kMaxM]),
                              tab[atom][2 * kTab + n3.z + kMaxM]);
        const float4 c = kc[j];
        const float w = c.y * e.x - c.x * e.y;  // P (S_s cos - S_c sin)
        g0 = fmaf(w, (float)n3.x, g0);
        g1 = fmaf(w, (float)n3.y, g1);
        g2 = fmaf(w, (float)n3.z, g2);
      }
    }
  }
  // reduce the 4 lanes of an atom
  for (int o = 1; o < 4; o <<= 1) {
    g0 += __shfl_xor_sync(0xffffffffu, g0, o);
    g1 += __shfl_xor_sync(0xffffffffu, g1, o);
    g2 += __shfl_xor_sync(0xffffffffu, g2, o);
  }
  double fw[6] = {0, 0, 0, 0, 0, 0};
  if (atom < na && sub == 0) {
    const int i = c0 + atom;
    const double tp = 6.283185307179586476925286766559;
    const double scale = 2.0 * ke * q[i] * tp;
    // dE/df -> dE/dr: r = f L  =>  f = r L^-1, dE/dr_b = sum_a dE/df_a (L^-1)_{ba}
    const double df[3] = {scale * g0, scale * g1, scale * g2};
    const double *iv = P.inv;
    const double gr[3] = {df[0] * iv[0], df[0] * iv[1] + df[1] * iv[2],
                          df[0] * iv[3] + df[1] * iv[4] + df[2] * iv[5]};
    if (kblocks_per_split > 0) {  // k-range partials; the structure-factor kernel zeroed grad
      atomicAdd(&grad[3 * (int64_t)i], gr[0]);
      atomicAdd(&grad[3 * (int64_t)i + 1], gr[1]);
      atomicAdd(&grad[3 * (int64_t)i + 2], gr[2]);
    } else {  // no k vectors (no structure-factor launch): write the zero gradient
      grad[3 * (int64_t)i] = gr[0];
      grad[3 * (int64_t)i + 1] = gr[1];
      grad[3 * (int64_t)i + 2] = gr[2];
    }
    // fractional coordinates of atom i (recomputed: the table owner is lane `atom`)
    const double r[3] = {pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]};
    double fi[3];
    frac64(P.inv, r, fi);
    // sum_i f_ia F_ib, F = -dE/dr
    fw[0] = -fi[0] * gr[0];
    fw[1] = -fi[1] * gr[0];
    fw[2] = -fi[1] * gr[1];
    fw[3] = -fi[2] * gr[0];
    fw[4] = -fi[2] * gr[1];
    fw[5] = -fi[2] * gr[2];
  }
  if (dtril) {
    for (int c = 0; c < 6; ++c) {
      const double v = block_sum(fw[c], red);
      __syncthreads();
      if (threadIdx.x == 0) atomicAdd(&dtril[6 * (int64_t)s + c], v);
    }
  }
  (void)f;
}

__global__ void self_energy_kernel(const double *q, const int32_t *sys_offset, const double *alpha,
                                   double ke, double *energy) {
  __shared__ double red[40];
  const int s = blockIdx.x;
  double acc = 0.0;
  for (int i = sys_offset[s] + threadIdx.x; i < sys_offset[s + 1]; i += blockDim.x) acc += q[i] * q[i];
  const double t = block_sum(acc, red);
  if (threadIdx.x == 0) energy[s] = -t * alpha[s] / sqrt(3.14159265358979323846) * ke;
}

// ---------------------------------------------------------------- real space
// Per directed edge (i, j, shift), d = x_j - x_i + s @ L, r = |d|:
//   LJ    4 eps (c6^2 - c6) [r^2 < rc_lj^2]
//   EWALD K q_i q_j erfc(alpha r) / r [r < rc_ew]
//   VACUUM (exclusion correction, subtracted) K q_i q_j / r, no cutoff
// Each term is summed / 2 per system (directed edges), gradients as in
// kups_lj_edges.  Float64 distance; pair arithmetic in float64.
__global__ void pair_edges_kernel(const double *pos, const int32_t *system, const int32_t *species,
                                  const double *q, int64_t n, const double *tril, int32_t s,
                                  const double *lj_sigma, const double *lj_eps, int32_t nsp,
                                  const double *rc_lj, const double *alpha, const double *rc_ew,
                                  double ke, int32_t terms, const int32_t *edges,
                                  const int32_t *shifts, int64_t n_edges, double *energy,
                                  double *grad, double *dtril) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n_edges) return;
  const int i = edges[2 * e], j = edges[2 * e + 1];
  if (i < 0 || i >= n || j < 0 || j >= n) return;
  const int si = system[i];
  if (si < 0 || si >= s) return;
  const Tril64 L = load_tril64(tril + 6 * (int64_t)si);
  const double sh[3] = {(double)shifts[3 * e], (double)shifts[3 * e + 1], (double)shifts[3 * e + 2]};
  double sL[3];
  row_times_tril64(sh, L, sL);
  const double d[3] = {pos[3 * j] - pos[3 * i] + sL[0], pos[3 * j + 1] - pos[3 * i + 1] + sL[1],
                       pos[3 * j + 2] - pos[3 * i + 2] + sL[2]};
  const double r2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
  double en = 0.0, dedr2 = 0.0;  // dE/d(r^2)
  if ((terms & 1) && lj_sigma) {
    const int ti = species[i], tj = species[j];
    const double sig = lj_sigma[ti * nsp + tj], eps = lj_eps[ti * nsp + tj];
    const double rc = rc_lj[si];
    if (r2 < rc * rc) {
      const double inv = 1.0 / r2, s2 = sig * sig * inv, c6 = s2 * s2 * s2;
      en += 4.0 * eps * (c6 * c6 - c6);
      dedr2 += -12.0 * eps * c6 * (2.0 * c6 - 1.0) * inv;
    }
  }
  if (terms & 6) {
    const double r = sqrt(r2), qq = q[i] * q[j] * ke;
    if (terms & 2) {
      const double a = alpha[si];
      if (r < rc_ew[si]) {
        const double er = erfc(a * r);
        en += qq * er / r;
        const double dedr = qq * (-er / r2 - 2.0 * a * 0.56418958354775628695 * exp(-a * a * r2) / r);
        dedr2 += dedr / (2.0 * r);
      }
    }
    if (terms & 4) {
      en -= qq / r;
      dedr2 -= -qq / (r2 * r) / 2.0;
    }
  }
  const double g[3] = {2.0 * dedr2 * d[0], 2.0 * dedr2 * d[1], 2.0 * dedr2 * d[2]};
  atomicAdd(&energy[si], 0.5 * en);
  for (int a = 0; a < 3; ++a) {
    atomicAdd(&grad[3 * (int64_t)j + a], 0.5 * g[a]);
    atomicAdd(&grad[3 * (int64_t)i + a], -0.5 * g[a]);
  }
  if (dtril) {
    atomicAdd(&dtril[6 * (int64_t)si + 0], 0.5 * sh[0] * g[0]);
    atomicAdd(&dtril[6 * (int64_t)si + 1], 0.5 * sh[1] * g[0]);
    atomicAdd(&dtril[6 * (int64_t)si + 2], 0.5 * sh[1] * g[1]);
    atomicAdd(&dtril[6 * (int64_t)si + 3], 0.5 * sh[2] * g[0]);
    atomicAdd(&dtril[6 * (int64_t)si + 4], 0.5 * sh[2] * g[1]);
    atomicAdd(&dtril[6 * (int64_t)si + 5], 0.5 * sh[2] * g[2]);
  }
}

// Real-space Lennard-Jones + Ewald forces of systems whose cell widths are all at
// least twice the larger cutoff, so that every pair within a cutoff is its minimum
// image and each ordered pair (i, j != i) is counted once: the edge set of
// neighbour_list at rc with the energies of lennard_jones_energy /
// ewald_short_range_energy (each pair term halved over the two directions), with no
// stored list.  A block owns 16 atoms; each half-warp holds all 16 (lane % 16 = atom)
// and the 32 half-warps split the partners j, so a half-warp reads one partner at a
// time (a broadcast from L1).  The difference is formed in float64, the minimum image
// and pair terms in float32, the 32 partial forces are summed in a fixed order through
// shared memory and the energy is float64.
constexpr int kRealAtoms = 16, kRealWarps = 16, kRealStreams = 2 * kRealWarps;

__global__ void __launch_bounds__(32 * kRealWarps) real_allpairs_kernel(
    const double *pos, const double *q, const int32_t *species, const int32_t *sys_offset, const double *tril,
    const double *lj_sigma, const double *lj_eps, int nsp, const double *rc_lj, const double *alpha,
    const double *rc_ew, double ke, int terms, double *energy, double *grad, kups_status *status) {
  __shared__ float2 ljt[64];
  __shared__ float part[kRealStreams][kRealAtoms][3];
  __shared__ double red[40];
  const int s = blockIdx.y;
  const int a0 = sys_offset[s], n = sys_offset[s + 1] - a0;
  if ((int)blockIdx.x * kRealAtoms >= n) return;  // uniform over the block
  // cell, inverse and widths once per block (float64 is scarce on this part)
  __shared__ float cellf[12];
  __shared__ int refused;
  if (threadIdx.x == 0) {
    const Tril64 L64 = load_tril64(tril + 6 * (int64_t)s);
    const Tril64 I64 = inverse_tril64(L64);
    double w[3];
    perpendicular_widths64(L64, w);
    const double rm = fmax((terms & 1) ? rc_lj[s] : 0.0, (terms & 2) ? rc_ew[s] : 0.0);
    refused = fmin(w[0], fmin(w[1], w[2])) < 2.0 * rm;
    if (refused) status_error(status, KUPS_ERR_UNSUPPORTED, s);
    for (int k = 0; k < 6; ++k) {
      cellf[k] = (float)L64.t[k];
      cellf[6 + k] = (float)I64.t[k];
    }
  }
  __syncthreads();
  if (refused) return;
  const double rlj = (terms & 1) ? rc_lj[s] : 0.0, rew = (terms & 2) ? rc_ew[s] : 0.0;
  const double rmax = fmax(rlj, rew);
  float L[6], I[6];
  for (int k = 0; k < 6; ++k) {
    L[k] = cellf[k];
    I[k] = cellf[6 + k];
  }
  if ((terms & 1) && nsp * nsp <= 64)
    for (int k = threadIdx.x; k < nsp * nsp; k += blockDim.x) {
      const double sg = lj_sigma[k];
      ljt[k] = make_float2((float)(sg * sg), (float)(4.0 * lj_eps[k]));
    }
  __syncthreads();
  const float rc2_lj = (float)(rlj * rlj), rc2_ew = (float)(rew * rew), rc2 = (float)(rmax * rmax);
  const float al = (terms & 2) ? (float)alpha[s] : 0.f;
  const float two_al_rsqrtpi = 2.0f * al * 0.56418958354775628695f;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int slot = lane & (kRealAtoms - 1), stream_id = warp * 2 + (lane >> 4);
  const int il = blockIdx.x * kRealAtoms + slot;
  const bool act = il < n;
  const int gi = a0 + (act ? il : 0);
  const double xi = pos[3 * (int64_t)gi], yi = pos[3 * (int64_t)gi + 1], zi = pos[3 * (int64_t)gi + 2];
  const float qi = (float)(q[gi] * ke);
  const int ti = (terms & 1) ? species[gi] : 0;
  float fx = 0.f, fy = 0.f, fz = 0.f;  // dE/dx_i, this warp's partners
  float ef = 0.f;
  const int per = (n + kRealStreams - 1) / kRealStreams;
  const int j0 = stream_id * per, j1 = min(n, j0 + per);
  for (int j = j0; j < j1; ++j) {
    const int gj = a0 + j;
    const float d0 = (float)(pos[3 * (int64_t)gj] - xi), d1 = (float)(pos[3 * (int64_t)gj + 1] - yi),
                d2 = (float)(pos[3 * (int64_t)gj + 2] - zi);
    float f0 = (d0 * I[0] + d1 * I[1]) + d2 * I[3], f1 = d1 * I[2] + d2 * I[4], f2 = d2 * I[5];
    f0 -= rintf(f0);
    f1 -= rintf(f1);
    f2 -= rintf(f2);
    const float dx = (f0 * L[0] + f1 * L[1]) + f2 * L[3], dy = f1 * L[2] + f2 * L[4], dz = f2 * L[5];
    const float r2 = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
    if (r2 >= rc2 || j == il || !act) continue;
    float dedr2 = 0.f;  // dE/d(r^2) of the pair
    const float ir = rsqrtf(r2);
    if ((terms & 1) && r2 < rc2_lj) {
      const float2 c = ljt[ti * nsp + species[gj]];
      const float inv = ir * ir, s2 = c.x * inv, c6 = s2 * s2 * s2;
      ef += c.y * (c6 * c6 - c6);
      dedr2 += -0.5f * c.y * c6 * (12.f * c6 - 6.f) * inv;
    }
    if ((terms & 2) && r2 < rc2_ew) {
      const float r = r2 * ir, qq = qi * (float)q[gj];
      const float er = erfc_cheb(al * r);
      ef += qq * er * ir;
      dedr2 += 0.5f * ir * qq * (-er * ir * ir - two_al_rsqrtpi * __expf(-al * al * r2) * ir);
    }
    // d = x_j - x_i: dE/dx_i = -2 dE/d(r^2) d for this ordered pair (both halves)
    fx = fmaf(-2.f * dedr2, dx, fx);
    fy = fmaf(-2.f * dedr2, dy, fy);
    fz = fmaf(-2.f * dedr2, dz, fz);
  }
  part[stream_id][slot][0] = fx;
  part[stream_id][slot][1] = fy;
  part[stream_id][slot][2] = fz;
  __syncthreads();
  if (threadIdx.x < kRealAtoms && act) {
    float gx = 0.f, gy = 0.f, gz = 0.f;
    for (int k = 0; k < kRealStreams; ++k) {
      gx += part[k][slot][0];
      gy += part[k][slot][1];
      gz += part[k][slot][2];
    }
    grad[3 * (int64_t)gi] = gx;
    grad[3 * (int64_t)gi + 1] = gy;
    grad[3 * (int64_t)gi + 2] = gz;
  }
  const double esum = block_sum(0.5 * (double)ef, red);
  if (threadIdx.x == 0) atomicAdd(&energy[s], esum);
}

// ---------------------------------------------------------------- packed real space
// The all-pairs kernel above forms every pair difference in float64 (three float64
// subtractions per pair test, slow on this part) and runs the LJ + erfc branch for a
// whole warp whenever any lane has a partner inside the cutoff (~11 % of pair tests
// in a dense melt, so ~98 % of warp iterations at ~11 % lane use).  The packed path:
//  * a pack kernel stores each coordinate as a float pair hi = fl(x), lo = fl(x - hi);
//    a difference (hj - hi) + (lj - li) then carries float32 relative error in d
//    itself (the rounding of hj - hi is relative to the result), with no float64;
//  * the force kernel tests 32 partners per pass into a per-lane hit mask and then
//    evaluates only the hits (loop count = the warp's largest hit count, not 32).
// Pair terms, the minimum image and the fixed-order reduction are those of the
// all-pairs kernel.
// Packed arrays are indexed by system * max_atoms + local index (inside the workspace
// for any sys_offset); a system above max_atoms is refused.
__global__ void real_pack_kernel(const double *pos, const double *q, const int32_t *species, const int32_t *sys_offset,
                                 int terms, int max_atoms, float4 *hi, float4 *lo, kups_status *status) {
  const int s = blockIdx.y;
  const int a0 = sys_offset[s], n = sys_offset[s + 1] - a0;
  if (n > max_atoms) {
    if (blockIdx.x == 0 && threadIdx.x == 0) status_error(status, KUPS_ERR_INVALID, s);
    return;
  }
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    const int64_t g = a0 + k, p = (int64_t)s * max_atoms + k;
    float h[3], l[3];
    for (int a = 0; a < 3; ++a) {
      const double x = pos[3 * g + a];
      h[a] = (float)x;
      l[a] = (float)(x - (double)h[a]);
    }
    hi[p] = make_float4(h[0], h[1], h[2], (float)q[g]);
    lo[p] = make_float4(l[0], l[1], l[2], __int_as_float((terms & 1) ? species[g] : 0));
  }
}

__global__ void __launch_bounds__(32 * kRealWarps) real_packed_kernel(
    const int32_t *sys_offset, const double *tril, const double *lj_sigma, const double *lj_eps, int nsp,
    const double *rc_lj, const double *alpha, const double *rc_ew, double ke, int terms, int max_atoms,
    const float4 *hi, const float4 *lo, double *energy, double *grad, kups_status *status) {
  // blockIdx.z of gridDim.z takes an equal share of every atom's partners; with more than one
  // share the blocks add their partial forces (terms & 8 is then required)
  __shared__ float2 ljt[64];
  __shared__ float part[kRealStreams][kRealAtoms][3];
  __shared__ double red[40];
  __shared__ uint16_t queue[kRealWarps][32 * 32];  // per warp: hits of one pass (half << 9 | slot << 5 | t)
  const int s = blockIdx.y;
  const int a0 = sys_offset[s], n = sys_offset[s + 1] - a0;
  if ((int)blockIdx.x * kRealAtoms >= n || n > max_atoms) return;  // uniform over the block
  const int64_t pb = (int64_t)s * max_atoms;  // this system's rows of the packed arrays
  // cell, inverse and widths once per block (float64 is scarce on this part)
  __shared__ float cellf[12];
  __shared__ int refused;
  if (threadIdx.x == 0) {
    const Tril64 L64 = load_tril64(tril + 6 * (int64_t)s);
    const Tril64 I64 = inverse_tril64(L64);
    double wd[3];
    perpendicular_widths64(L64, wd);
    const double rmax = fmax((terms & 1) ? rc_lj[s] : 0.0, (terms & 2) ? rc_ew[s] : 0.0);
    refused = fmin(wd[0], fmin(wd[1], wd[2])) < 2.0 * rmax;
    if (refused) status_error(status, KUPS_ERR_UNSUPPORTED, s);
    for (int k = 0; k < 6; ++k) {
      cellf[k] = (float)L64.t[k];
      cellf[6 + k] = (float)I64.t[k];
    }
  }
  __syncthreads();
  if (refused) return;
  float L[6], I[6];
  for (int k = 0; k < 6; ++k) {
    L[k] = cellf[k];
    I[k] = cellf[6 + k];
  }
  const double rlj = (terms & 1) ? rc_lj[s] : 0.0, rew = (terms & 2) ? rc_ew[s] : 0.0;
  const double rmax = fmax(rlj, rew);
  const float kef = (float)ke;
  if ((terms & 1) && nsp * nsp <= 64)
    for (int k = threadIdx.x; k < nsp * nsp; k += blockDim.x) {
      const double sg = lj_sigma[k];
      ljt[k] = make_float2((float)(sg * sg), (float)(4.0 * lj_eps[k]));
    }
  __syncthreads();
  const float rc2_lj = (float)(rlj * rlj), rc2_ew = (float)(rew * rew), rc2 = (float)(rmax * rmax);
  const float al = (terms & 2) ? (float)alpha[s] : 0.f;
  const float two_al_rsqrtpi = 2.0f * al * 0.56418958354775628695f;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int slot = lane & (kRealAtoms - 1), stream_id = warp * 2 + (lane >> 4);
  const int il = blockIdx.x * kRealAtoms + slot;
  const bool act = il < n;
  const int64_t gi = a0 + (act ? il : 0);
  const float4 hi_i = hi[pb + (act ? il : 0)], lo_i = lo[pb + (act ? il : 0)];
  // minimum-image difference x_j - x_i from the hi / lo pairs
  auto diff = [&](int64_t gj, float &dx, float &dy, float &dz, float &r2) {
    const float4 hj = hi[gj], lj = lo[gj];
    const float d0 = (hj.x - hi_i.x) + (lj.x - lo_i.x), d1 = (hj.y - hi_i.y) + (lj.y - lo_i.y),
                d2 = (hj.z - hi_i.z) + (lj.z - lo_i.z);
    float f0 = (d0 * I[0] + d1 * I[1]) + d2 * I[3], f1 = d1 * I[2] + d2 * I[4], f2 = d2 * I[5];
    f0 -= rintf(f0);
    f1 -= rintf(f1);
    f2 -= rintf(f2);
    dx = (f0 * L[0] + f1 * L[1]) + f2 * L[3];
    dy = f1 * L[2] + f2 * L[4];
    dz = f2 * L[5];
    r2 = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
  };
  for (int k = threadIdx.x; k < kRealStreams * kRealAtoms * 3; k += blockDim.x) (&part[0][0][0])[k] = 0.f;
  __syncthreads();
  float ef = 0.f;
  const int n_streams = kRealStreams * (int)gridDim.z;
  const int per = (n + n_streams - 1) / n_streams;
  const int sbase = (int)blockIdx.z * kRealStreams;
  const int j0 = (sbase + stream_id) * per, j1 = min(n, j0 + per);
  // chunk starts of the warp's two streams
  const int j0h[2] = {(sbase + warp * 2) * per, (sbase + warp * 2 + 1) * per};
  uint16_t *wq = queue[warp];
  const int passes = (per + 31) / 32;  // the same for both half-warps of a warp
  for (int pass = 0; pass < passes; ++pass) {
    const int c0 = j0 + pass * 32;
    const int cn = max(0, min(32, j1 - c0));
    uint32_t hits = 0;
#pragma unroll 4
    for (int t = 0; t < 32; ++t) {
      if (t < cn) {  // four independent partner loads in flight
        float dx, dy, dz, r2;
        diff(pb + c0 + t, dx, dy, dz, r2);
        hits |= (uint32_t)(r2 < rc2) << t;
      }
    }
    if (cn > 0 && c0 <= il && il < c0 + cn) hits &= ~(1u << (il - c0));  // not the atom itself
    if (!act) hits = 0;
    // append this lane's hits to the warp's queue (exclusive prefix of the counts)
    const int cnt = __popc(hits);
    int off = cnt;
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, off, o);
      if (lane >= o) off += y;
    }
    const int total = __shfl_sync(0xffffffffu, off, 31);
    off -= cnt;
    const uint16_t tag = (uint16_t)(((lane >> 4) << 9) | (slot << 5));
    while (hits) {
      const int t = __ffs(hits) - 1;
      hits &= hits - 1;
      wq[off++] = tag | (uint16_t)t;
    }
    __syncwarp();
    // every lane takes queued pairs until the queue is empty
    for (int e = lane; e < total; e += 32) {
      const int code = wq[e];
      const int h = code >> 9, sl = (code >> 5) & 15, t = code & 31;
      const int64_t ii = pb + blockIdx.x * kRealAtoms + sl;
      const int64_t gj = pb + j0h[h] + pass * 32 + t;
      const float4 hi_a = hi[ii], lo_a = lo[ii], hj = hi[gj], lj = lo[gj];
      const float d0 = (hj.x - hi_a.x) + (lj.x - lo_a.x), d1 = (hj.y - hi_a.y) + (lj.y - lo_a.y),
                  d2 = (hj.z - hi_a.z) + (lj.z - lo_a.z);
      float f0 = (d0 * I[0] + d1 * I[1]) + d2 * I[3], f1 = d1 * I[2] + d2 * I[4], f2 = d2 * I[5];
      f0 -= rintf(f0);
      f1 -= rintf(f1);
      f2 -= rintf(f2);
      const float dx = (f0 * L[0] + f1 * L[1]) + f2 * L[3], dy = f1 * L[2] + f2 * L[4], dz = f2 * L[5];
      const float r2 = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
      float dedr2 = 0.f;
      const float ir = rsqrtf(r2);  // a few ulp; one MUFU op instead of IEEE sqrt and divisions
      if ((terms & 1) && r2 < rc2_lj) {
        const float2 c = ljt[__float_as_int(lo_a.w) * nsp + __float_as_int(lj.w)];
        const float inv = ir * ir, s2 = c.x * inv, c6 = s2 * s2 * s2;
        ef += c.y * (c6 * c6 - c6);
        dedr2 += -0.5f * c.y * c6 * (12.f * c6 - 6.f) * inv;
      }
      if ((terms & 2) && r2 < rc2_ew) {
        const float r = r2 * ir, qq = (hi_a.w * kef) * hj.w;
        const float er = erfc_cheb(al * r);
        ef += qq * er * ir;
        dedr2 += 0.5f * ir * qq * (-er * ir * ir - two_al_rsqrtpi * __expf(-al * al * r2) * ir);
      }
      float *pp = part[warp * 2 + h][sl];
      atomicAdd(pp, -2.f * dedr2 * dx);
      atomicAdd(pp + 1, -2.f * dedr2 * dy);
      atomicAdd(pp + 2, -2.f * dedr2 * dz);
    }
    __syncwarp();
  }
  __syncthreads();
  if (threadIdx.x < kRealAtoms && act) {
    float gx = 0.f, gy = 0.f, gz = 0.f;
    for (int k = 0; k < kRealStreams; ++k) {
      gx += part[k][slot][0];
      gy += part[k][slot][1];
      gz += part[k][slot][2];
    }
    if (gridDim.z > 1) {  // several blocks share atom gi
      atomicAdd(&grad[3 * gi], (double)gx);
      atomicAdd(&grad[3 * gi + 1], (double)gy);
      atomicAdd(&grad[3 * gi + 2], (double)gz);
    } else if (terms & 8) {  // add onto the caller's gradient (this block owns atom gi)
      grad[3 * gi] += gx;
      grad[3 * gi + 1] += gy;
      grad[3 * gi + 2] += gz;
    } else {
      grad[3 * gi] = gx;
      grad[3 * gi + 1] = gy;
      grad[3 * gi + 2] = gz;
    }
  }
  const double esum = block_sum(0.5 * (double)ef, red);
  if (threadIdx.x == 0) atomicAdd(&energy[s], esum);
}

inline size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

// The reciprocal-space launch sequence of kups_ewald_recip and
// kups_ewald_recip_static: setup, structure factor, energy and forces.
// `base` is 256-byte aligned scratch of at least recip_scratch_bytes().
inline size_t recip_scratch_bytes(int32_t n_systems, int32_t n_kvecs) {
  return align256(sizeof(RecipSys) * (size_t)n_systems) +
         align256(sizeof(Coef) * (size_t)n_systems * (size_t)n_kvecs);
}

int32_t recip_launch(char *base, const double *positions, const double *charges, const int32_t *sys_offset,
                     int32_t n_systems, int32_t max_atoms_per_system, const double *tril, const int32_t *kvec_n,
                     int32_t n_kvecs, const double *alpha, double coulomb_k, double *energy, double *grad,
                     double *grad_tril, double *structure_factor, kups_status *status, cudaStream_t stream) {
  RecipSys *sysp = (RecipSys *)base;
  Coef *coef = (Coef *)(base + align256(sizeof(RecipSys) * (size_t)n_systems));
  recip_setup_kernel<<<n_systems, 256, 0, stream>>>(tril, kvec_n, n_systems, n_kvecs, sysp, status);
  KUPS_CUDA_TRY(cudaMemsetAsync(structure_factor, 0, sizeof(double) * 2 * (size_t)n_systems * n_kvecs, stream));
  const int chunks = (max_atoms_per_system + kAtomsPerChunk - 1) / kAtomsPerChunk;
  if (n_kvecs > 0 && chunks > 0) {
    dim3 g((n_kvecs + kKPerBlock - 1) / kKPerBlock, chunks, n_systems);
    structure_factor_kernel<<<g, kKPerBlock, 0, stream>>>(positions, charges, sys_offset, kvec_n,
                                                          n_kvecs, sysp, structure_factor, grad);
  }
  KUPS_CUDA_TRY(cudaMemsetAsync(energy, 0, sizeof(double) * (size_t)n_systems, stream));
  if (grad_tril) KUPS_CUDA_TRY(cudaMemsetAsync(grad_tril, 0, sizeof(double) * 6 * (size_t)n_systems, stream));
  // one warp per block: the per-k float64 exp and divisions spread over many SMs
  recip_energy_kernel<<<dim3((unsigned)std::max(1, (n_kvecs + 31) / 32), n_systems), 32, 0, stream>>>(
      kvec_n, n_kvecs, alpha, sysp, structure_factor, coulomb_k, coef, energy, grad_tril);
  if (chunks > 0 && n_kvecs > 0) {
    // enough k splits that the launch holds about 16 warps per SM
    const int kblocks = (n_kvecs + kKPerBlock - 1) / kKPerBlock;
    const int want = std::max(1, (16 * device_sm_count()) / std::max(1, 4 * chunks * n_systems));
    const int splits = std::min(kblocks, want);
    const int per = (kblocks + splits - 1) / splits;
    dim3 g(chunks, n_systems, (kblocks + per - 1) / per);
    recip_force_kernel<<<g, kAtomsPerChunk * 4, 0, stream>>>(positions, charges, sys_offset, kvec_n,
                                                             n_kvecs, sysp, coef, coulomb_k, grad,
                                                             grad_tril, per);
  } else if (chunks > 0) {
    dim3 g(chunks, n_systems, 1);
    recip_force_kernel<<<g, kAtomsPerChunk * 4, 0, stream>>>(positions, charges, sys_offset, kvec_n,
                                                             n_kvecs, sysp, coef, coulomb_k, grad,
                                                             grad_tril, 0);
  }
  return cudaGetLastError() == cudaSuccess ? KUPS_OK : KUPS_ERR_CUDA;
}

}  // namespace
}  // namespace kups

using namespace kups;

extern "C" size_t kups_ewald_recip_workspace_bytes(int32_t n_systems, int32_t n_kvecs) {
  return recip_scratch_bytes(n_systems, n_kvecs) + 512;
}

extern "C" int32_t kups_ewald_recip(const double *positions, const double *charges,
                                    const int32_t *sys_offset, int32_t n_systems,
                                    int32_t max_atoms_per_system, const double *tril,
                                    const int32_t *kvec_n, int32_t n_kvecs, const double *alpha,
                                    double coulomb_k, double *energy, double *grad,
                                    double *grad_tril, double *structure_factor,
                                    void *workspace, size_t workspace_bytes, kups_status *status,
                                    void *stream_) {
  if (n_systems < 0 || n_kvecs < 0 || max_atoms_per_system < 0) return KUPS_ERR_INVALID;
  if (workspace_bytes < kups_ewald_recip_workspace_bytes(n_systems, n_kvecs)) return KUPS_ERR_INVALID;
  if (n_systems == 0) return KUPS_OK;
  char *base = (char *)(((uintptr_t)workspace + 255) & ~uintptr_t(255));
  return recip_launch(base, positions, charges, sys_offset, n_systems, max_atoms_per_system, tril, kvec_n,
                      n_kvecs, alpha, coulomb_k, energy, grad, grad_tril, structure_factor, status,
                      (cudaStream_t)stream_);
}

// Reciprocal energy from given structure factors (the energy step of the launch
// sequence above; its scratch is the same workspace).
extern "C" int32_t kups_ewald_recip_energy(const double *tril, const int32_t *kvec_n, int32_t n_kvecs,
                                           const double *alpha, int32_t n_systems, double coulomb_k,
                                           const double *structure_factor, double *energy, void *workspace,
                                           size_t workspace_bytes, kups_status *status, void *stream_) {
  cudaStream_t stream = (cudaStream_t)stream_;
  if (n_systems < 0 || n_kvecs < 0) return KUPS_ERR_INVALID;
  if (workspace_bytes < kups_ewald_recip_workspace_bytes(n_systems, n_kvecs)) return KUPS_ERR_INVALID;
  if (n_systems == 0) return KUPS_OK;
  char *base = (char *)(((uintptr_t)workspace + 255) & ~uintptr_t(255));
  RecipSys *sysp = (RecipSys *)base;
  Coef *coef = (Coef *)(base + align256(sizeof(RecipSys) * (size_t)n_systems));
  recip_setup_kernel<<<n_systems, 256, 0, stream>>>(tril, kvec_n, n_systems, n_kvecs, sysp, status);
  KUPS_CUDA_TRY(cudaMemsetAsync(energy, 0, sizeof(double) * (size_t)n_systems, stream));
  recip_energy_kernel<<<dim3((unsigned)std::max(1, (n_kvecs + 31) / 32), n_systems), 32, 0, stream>>>(
      kvec_n, n_kvecs, alpha, sysp, structure_factor, coulomb_k, coef, energy, nullptr);
  return cudaGetLastError() == cudaSuccess ? KUPS_OK : KUPS_ERR_CUDA;
}

// ---------------------------------------------------------------------------
// kups_ewald_recip_static: the reciprocal-space computation above with its
// scratch (per-system cell data, then per-(system, k) coefficients) in one
// fixed device array instead of a caller-supplied workspace.  It serves
// callers that have no device allocator to draw a workspace from, e.g. an
// FFI handler that a host framework hands only its input and output buffers.
//
// The array is shared by every call on a device and keeps whatever the last
// call left in it; every byte a call reads is written earlier in the same
// call, so nothing in it has to start at zero.  Two calls whose launches
// overlap in time (different streams, or different host threads) race on it.
// The array lives in this file's module: every device on which any kernel of
// this file runs holds its KUPS_EWALD_RECIP_STATIC_SCRATCH_BYTES until the
// process exits (or the device is reset).
namespace kups {
namespace {
constexpr size_t kStaticScratchBytes = KUPS_EWALD_RECIP_STATIC_SCRATCH_BYTES;
constexpr int kStaticMaxDevices = 64;
std::mutex g_static_scratch_mutex;
void *g_static_scratch_ptr[kStaticMaxDevices] = {};
}  // namespace
static __device__ __align__(256) unsigned char g_recip_static_scratch[kStaticScratchBytes];
}  // namespace kups

extern "C" int32_t kups_ewald_recip_static(const double *positions, const double *charges,
                                           const int32_t *sys_offset, int32_t n_systems,
                                           int32_t max_atoms_per_system, const double *tril,
                                           const int32_t *kvec_n, int32_t n_kvecs,
                                           const double *alpha, double coulomb_k, double *energy,
                                           double *grad, double *grad_tril,
                                           double *structure_factor, kups_status *status,
                                           void *stream_) {
  if (n_systems < 0 || n_kvecs < 0 || max_atoms_per_system < 0) return KUPS_ERR_INVALID;
  // Sizes beyond the array are refused before anything is touched.
  if ((size_t)n_systems > kStaticScratchBytes / sizeof(RecipSys)) return KUPS_ERR_CAPACITY;
  if (n_kvecs > 0 && (size_t)n_systems > kStaticScratchBytes / sizeof(Coef) / (size_t)n_kvecs)
    return KUPS_ERR_CAPACITY;
  if (recip_scratch_bytes(n_systems, n_kvecs) > kStaticScratchBytes) return KUPS_ERR_CAPACITY;
  if (n_systems == 0) return KUPS_OK;
  // Once per device, with that device current: look up the array's address.
  int dev = 0;
  KUPS_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kStaticMaxDevices) return KUPS_ERR_UNSUPPORTED;
  char *base = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_static_scratch_mutex);
    if (g_static_scratch_ptr[dev] == nullptr) {
      void *p = nullptr;
      if (cudaGetSymbolAddress(&p, g_recip_static_scratch) != cudaSuccess || p == nullptr)
        return KUPS_ERR_CUDA;
      g_static_scratch_ptr[dev] = p;
    }
    base = (char *)g_static_scratch_ptr[dev];
  }
  return recip_launch(base, positions, charges, sys_offset, n_systems, max_atoms_per_system, tril, kvec_n,
                      n_kvecs, alpha, coulomb_k, energy, grad, grad_tril, structure_factor, status,
                      (cudaStream_t)stream_);
}

extern "C" int32_t kups_ewald_self(const double *charges, const int32_t *sys_offset,
                                   int32_t n_systems, const double *alpha, double coulomb_k,
                                   double *energy, void *stream) {
  if (n_systems < 0) return KUPS_ERR_INVALID;
  if (n_systems == 0) return KUPS_OK;
  self_energy_kernel<<<n_systems, 256, 0, (cudaStream_t)stream>>>(charges, sys_offset, alpha,
                                                                 coulomb_k, energy);
  return cudaGetLastError() == cudaSuccess ? KUPS_OK : KUPS_ERR_CUDA;
}

extern "C" int32_t kups_pair_edges(const double *positions, const int32_t *system,
                                   const int32_t *species, const double *charges, int64_t n,
                                   const double *tril, int32_t n_systems, const double *lj_sigma,
                                   const double *lj_epsilon, int32_t n_species,
                                   const double *lj_cutoff, const double *alpha,
                                   const double *ewald_cutoff, double coulomb_k, int32_t terms,
                                   const int32_t *edges, const int32_t *shifts, int64_t n_edges,
                                   double *energy, double *grad, double *grad_tril,
                                   kups_status *status, void *stream_) {
  cudaStream_t stream = (cudaStream_t)stream_;
  if (n < 0 || n_systems < 0 || n_edges < 0 || (terms & ~7) != 0) return KUPS_ERR_INVALID;
  if ((terms & 1) && (lj_sigma == nullptr || n_species <= 0)) return KUPS_ERR_INVALID;
  if (n_systems > 0) {
    KUPS_CUDA_TRY(cudaMemsetAsync(energy, 0, sizeof(double) * n_systems, stream));
    if (grad_tril) KUPS_CUDA_TRY(cudaMemsetAsync(grad_tril, 0, sizeof(double) * 6 * n_systems, stream));
  }
  if (n > 0) KUPS_CUDA_TRY(cudaMemsetAsync(grad, 0, sizeof(double) * 3 * n, stream));
  if (n_edges == 0) return KUPS_OK;
  pair_edges_kernel<<<(unsigned)((n_edges + 255) / 256), 256, 0, stream>>>(
      positions, system, species, charges, n, tril, n_systems, lj_sigma, lj_epsilon, n_species,
      lj_cutoff, alpha, ewald_cutoff, coulomb_k, terms, edges, shifts, n_edges, energy, grad,
      grad_tril);
  (void)status;
  return cudaGetLastError() == cudaSuccess ? KUPS_OK : KUPS_ERR_CUDA;
}

extern "C" int32_t kups_lj_ewald_real_forces(const double *positions, const double *charges,
                                             const int32_t *species, const int32_t *sys_offset,
                                             int32_t n_systems, int32_t max_atoms_per_system,
                                             const double *tril, const double *lj_sigma,
                                             const double *lj_epsilon, int32_t n_species,
                                             const double *lj_cutoff, const double *alpha,
                                             const double *ewald_cutoff, double coulomb_k, int32_t terms,
                                             double *energy, double *grad, kups_status *status,
                                             void *stream_) {
  cudaStream_t stream = (cudaStream_t)stream_;
  if (n_systems < 0 || max_atoms_per_system < 0 || terms < 1 || terms > 3) return KUPS_ERR_INVALID;
  if ((terms & 1) && (n_species < 1 || n_species > 8 || lj_sigma == nullptr || lj_epsilon == nullptr))
    return KUPS_ERR_INVALID;
  if (n_systems == 0) return KUPS_OK;
  KUPS_CUDA_TRY(cudaMemsetAsync(energy, 0, sizeof(double) * (size_t)n_systems, stream));
  if (max_atoms_per_system == 0) return KUPS_OK;
  dim3 g((max_atoms_per_system + kRealAtoms - 1) / kRealAtoms, n_systems);
  real_allpairs_kernel<<<g, 32 * kRealWarps, 0, stream>>>(positions, charges, species, sys_offset, tril, lj_sigma,
                                                    lj_epsilon, n_species, lj_cutoff, alpha, ewald_cutoff,
                                                    coulomb_k, terms, energy, grad, status);
  return cudaGetLastError() == cudaSuccess ? KUPS_OK : KUPS_ERR_CUDA;
}

extern "C" size_t kups_lj_ewald_real_forces_workspace_bytes(int32_t n_systems, int32_t max_atoms_per_system) {
  if (n_systems <= 0 || max_atoms_per_system <= 0) return 256;
  const size_t cap = (size_t)n_systems * (size_t)max_atoms_per_system;
  return 2 * align256(cap * sizeof(float4)) + 256;
}

extern "C" int32_t kups_lj_ewald_real_forces_packed(const double *positions, const double *charges,
                                                    const int32_t *species, const int32_t *sys_offset,
                                                    int32_t n_systems, int32_t max_atoms_per_system,
                                                    const double *tril, const double *lj_sigma,
                                                    const double *lj_epsilon, int32_t n_species,
                                                    const double *lj_cutoff, const double *alpha,
                                                    const double *ewald_cutoff, double coulomb_k, int32_t terms,
                                                    double *energy, double *grad, void *workspace,
                                                    size_t workspace_bytes, kups_status *status, void *stream_) {
  cudaStream_t stream = (cudaStream_t)stream_;
  const int splits_req = (terms >> 8) & 15;  // partner shares per atom block; 0: chosen here
  terms &= 255;
  if (n_systems < 0 || max_atoms_per_system < 0 || (terms & ~11) != 0 || (terms & 3) == 0) return KUPS_ERR_INVALID;
  if ((terms & 1) && (n_species < 1 || n_species > 8 || lj_sigma == nullptr || lj_epsilon == nullptr))
    return KUPS_ERR_INVALID;
  if (n_systems == 0) return KUPS_OK;
  if (!(terms & 8)) KUPS_CUDA_TRY(cudaMemsetAsync(energy, 0, sizeof(double) * (size_t)n_systems, stream));
  if (max_atoms_per_system == 0) return KUPS_OK;
  if (workspace == nullptr ||
      workspace_bytes < kups_lj_ewald_real_forces_workspace_bytes(n_systems, max_atoms_per_system))
    return KUPS_ERR_INVALID;
  const size_t cap = (size_t)n_systems * (size_t)max_atoms_per_system;
  char *base = reinterpret_cast<char *>(((uintptr_t)workspace + 255) & ~uintptr_t(255));
  float4 *hi = reinterpret_cast<float4 *>(base);
  float4 *lo = reinterpret_cast<float4 *>(base + align256(cap * sizeof(float4)));
  dim3 gp((max_atoms_per_system + 255) / 256, n_systems);
  real_pack_kernel<<<gp, 256, 0, stream>>>(positions, charges, species, sys_offset, terms, max_atoms_per_system, hi,
                                           lo, status);
  // partner shares: the caller's choice (a launch-shape tuner's), else one.  Shares add their
  // partial forces, so they need terms & 8 (the caller's gradient is the base).  One share
  // measured fastest on the 4000-ion melt (250 blocks on 152 SMs: 0.152 ms per force
  // evaluation against 0.164 / 0.166 / 0.171 for 2 / 3 / 4 shares).
  const int splits = (terms & 8) && splits_req > 0 ? splits_req : 1;
  dim3 g((max_atoms_per_system + kRealAtoms - 1) / kRealAtoms, n_systems, splits);
  real_packed_kernel<<<g, 32 * kRealWarps, 0, stream>>>(sys_offset, tril, lj_sigma, lj_epsilon, n_species, lj_cutoff,
                                                        alpha, ewald_cutoff, coulomb_k, terms, max_atoms_per_system,
                                                        hi, lo, energy, grad, status);
  return cudaGetLastError() == cudaSuccess ? KUPS_OK : KUPS_ERR_CUDA;
}

namespace kups {
namespace {
__global__ void erfc_eval_kernel(const float *x, int64_t n, float *out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = erfc_cheb(x[i]);
}
}  // namespace
}  // namespace kups

extern "C" int32_t kups_erfc_eval(const float *x, int64_t n, float *out, void *stream) {
  if (n < 0) return KUPS_ERR_INVALID;
  if (n == 0) return KUPS_OK;
  erfc_eval_kernel<<<(unsigned)((n + 255) / 256), 256, 0, (cudaStream_t)stream>>>(x, n, out);
  return cudaGetLastError() == cudaSuccess ? KUPS_OK : KUPS_ERR_CUDA;
}
