// Per-system virial observables from positions, dU/dx, dU/dtril and momenta:
// the atomic virial stress, the molecular virial stress of the RASPA convention,
// the lattice-gradient stress, the kinetic energy and the instantaneous pressure.
//
// Replaces src/kups/observables/stress.py:64-118 (_stress_via_lattice_vector_gradients,
// _stress_via_virial_theorem, _molecular_stress_via_virial_theorem),
// src/kups/md/observables.py:17-61 (particle_kinetic_energy summed per system,
// instantaneous_pressure with d = 3) and pressure.py:27-29 (_pressure_from_stress).
//
//   atomic     sigma_ab = -(sum_i r_ia g_ib + (L^T G)_ab) / V
//   molecular  sigma    = -(sym(sum_i w_i (x) g_i) + L^T G) / V,  sym(A) = (A + A^T) / 2,
//              w_i = r_i - wrap(r_i - R_g(i)), R_g = wrap(mean_j wrap(r_j - r_a) + r_a)
//              over the atoms j of group g, a the group's first atom
//   lattice    sigma    = -G / V
//   pressure   P = 2 K / (3 V) + Tr(sigma_atomic) / 3   (K = 0 without momenta)
// with g_i = dU/dr_i, G = dU/dL (lower triangular, from dU/dtril), V = |L00 L11 L22|,
// wrap() into the fractional cell [-0.5, 0.5).  Each system uses its own volume; the
// reference's molecular stress divides every system by the first system's volume
// (stress.py:114), the same number for one system or equal cells.
//
// Layout of the work: one warp walks 32 * kPerLane consecutive particles, each lane
// keeping float64 running sums while the warp's particles stay in one system (the
// usual layout: particles grouped by system), so a warp issues one shuffle reduction
// and one atomic per accumulator per run instead of per particle.  The molecular
// stress needs each group's centre first: an anchor pass (first atom of the group,
// atomicMin), a sum pass (minimum images relative to the anchor) and a per-group
// pass (mean, shift back, wrap).  Everything is float64: an observable evaluated
// when sampled, not in every step.
#include <algorithm>

#include "common.cuh"

namespace kups {
namespace {

constexpr int kAcc = 19;      // per system: K, sum r_a g_b (9), sum w_a g_b (9)
constexpr int kPerLane = 8;   // particles per lane in one warp's run
constexpr int kThreads = 256;

inline size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

// wrap(r) into the fractional cell [-0.5, 0.5): f = r @ L^-1, f = mod(f + 0.5, 1) - 0.5, f @ L
// (unitcell.py:139-171), with the rounding of the float64 restatement.
__device__ inline void wrap64(const double r[3], const Tril64 &L, const Tril64 &Li, double out[3]) {
  double f[3];
  row_times_tril64(r, Li, f);
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const double x = __dadd_rn(f[a], 0.5);
    f[a] = __dsub_rn(__dsub_rn(x, floor(x)), 0.5);
  }
  row_times_tril64(f, L, out);
}

// The image the wrap takes: n = floor(f + 0.5), f = d @ L^-1 (the same rounding as
// wrap64), so that wrap(d) = d - n @ L.  Returns false when n = 0 (wrap(d) = d up to the
// rounding of the round trip through fractional coordinates).
__device__ inline bool wrap_image64(const double d[3], const Tril64 &Li, double n[3]) {
  double f[3];
  row_times_tril64(d, Li, f);
#pragma unroll
  for (int a = 0; a < 3; ++a) n[a] = floor(__dadd_rn(f[a], 0.5));
  return n[0] != 0.0 || n[1] != 0.0 || n[2] != 0.0;
}

__device__ inline bool valid_index(int v, int n) { return v >= 0 && v < n; }

// 1 / m to float64 accuracy without a float64 division: the float32 reciprocal
// (relative error about 1e-7) refined by one Newton step y (2 - m y), which squares
// the relative error.
__device__ inline double recip64(double m) {
  const double y = (double)(1.0f / (float)m);
  return y * fma(-m, y, 2.0);
}

// inv[s] = L_s^-1 (tril order), once per system for the passes below.
__global__ void cell_inverse_kernel(const double *tril, int32_t n_sys, double *inv) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n_sys) return;
  const Tril64 Li = inverse_tril64(load_tril64(tril + 6 * (int64_t)s));
#pragma unroll
  for (int k = 0; k < 6; ++k) inv[6 * (int64_t)s + k] = Li.t[k];
}

__global__ void group_anchor_kernel(const int32_t *group, const int32_t *system, int64_t n, int32_t n_groups,
                                    int32_t n_sys, int32_t *anchor, kups_status *status) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int g = group[i], s = system[i];
  if (!valid_index(g, n_groups) || !valid_index(s, n_sys)) {
    status_error(status, KUPS_ERR_INVALID, i);
    return;
  }
  atomicMin(&anchor[g], (int32_t)i);
}

// gsum[g] += (wrap(r_i - r_anchor), 1)
__global__ void group_sum_kernel(const double *pos, const int32_t *group, const int32_t *system, int64_t n,
                                 int32_t n_groups, int32_t n_sys, const double *tril, const double *inv,
                                 const int32_t *anchor, double *gsum) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int g = group[i], s = system[i];
  if (!valid_index(g, n_groups) || !valid_index(s, n_sys)) return;
  const int a = anchor[g];
  const Tril64 L = load_tril64(tril + 6 * (int64_t)s);
  const Tril64 Li = load_tril64(inv + 6 * (int64_t)s);
  double d[3], img[3];
#pragma unroll
  for (int c = 0; c < 3; ++c) d[c] = __dsub_rn(pos[3 * i + c], pos[3 * (int64_t)a + c]);
  if (wrap_image64(d, Li, img)) {  // wrap(d) = d - img @ L
    double nL[3];
    row_times_tril64(img, L, nL);
#pragma unroll
    for (int c = 0; c < 3; ++c) d[c] = __dsub_rn(d[c], nL[c]);
  }
#pragma unroll
  for (int c = 0; c < 3; ++c) atomicAdd(&gsum[4 * (int64_t)g + c], d[c]);
  atomicAdd(&gsum[4 * (int64_t)g + 3], 1.0);
}

// gsum[g] <- (wrap(sum / max(count, 1) + r_anchor), count): the group's centre in place.
__global__ void group_centre_kernel(const double *pos, const int32_t *system, int64_t n, int32_t n_groups,
                                    const double *tril, const double *inv, const int32_t *anchor, double *gsum) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= n_groups) return;
  const int a = anchor[g];
  if (a < 0 || a >= n) return;  // empty group: no atom reads it
  const Tril64 L = load_tril64(tril + 6 * (int64_t)system[a]);
  const Tril64 Li = load_tril64(inv + 6 * (int64_t)system[a]);
  const double cnt = fmax(gsum[4 * (int64_t)g + 3], 1.0);
  double c[3], w[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) c[k] = __dadd_rn(__ddiv_rn(gsum[4 * (int64_t)g + k], cnt), pos[3 * (int64_t)a + k]);
  wrap64(c, L, Li, w);
#pragma unroll
  for (int k = 0; k < 3; ++k) gsum[4 * (int64_t)g + k] = w[k];
}

template <int NV>
__device__ inline void flush_run(double (&acc)[NV], int sys, double *out) {
#pragma unroll
  for (int k = 0; k < NV; ++k) {
    const double v = warp_sum(acc[k]);
    if ((threadIdx.x & 31) == 0 && sys >= 0 && v != 0.0) atomicAdd(&out[(int64_t)sys * kAcc + k], v);
    acc[k] = 0.0;
  }
}

template <bool MOL, bool KE>
__global__ void __launch_bounds__(kThreads) virial_accumulate_kernel(
    const double *pos, const double *grad, const int32_t *system, int64_t n, int32_t n_sys,
    const int32_t *group, int32_t n_groups, const double *gcentre, const double *tril, const double *inv,
    const double *mom,
    const double *mass, double *out, kups_status *status) {
  constexpr int NV = MOL ? kAcc : 10;
  const unsigned full = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const int64_t base = (((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5) * (32 * kPerLane);
  if (base >= n) return;  // the same for every lane of the warp
  double run[NV];
#pragma unroll
  for (int k = 0; k < NV; ++k) run[k] = 0.0;
  int cur = -1, lsys = -1;
  Tril64 L, Li;
  for (int j = 0; j < kPerLane; ++j) {
    const int64_t i = base + (int64_t)j * 32 + lane;
    int s = -1;
    double v[NV];
#pragma unroll
    for (int k = 0; k < NV; ++k) v[k] = 0.0;
    if (i < n) {
      s = system[i];
      if (!valid_index(s, n_sys)) {
        status_error(status, KUPS_ERR_INVALID, i);
        s = -1;
      }
    }
    if (s >= 0) {
      const double r[3] = {pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]};
      const double g[3] = {grad[3 * i], grad[3 * i + 1], grad[3 * i + 2]};
      if (KE) {
        const double p0 = mom[3 * i], p1 = mom[3 * i + 1], p2 = mom[3 * i + 2];
        v[0] = 0.5 * (p0 * p0 + p1 * p1 + p2 * p2) * recip64(mass[i]);
      }
#pragma unroll
      for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int b = 0; b < 3; ++b) v[1 + 3 * a + b] = r[a] * g[b];
      if (MOL) {
        const int gi = group[i];
        if (valid_index(gi, n_groups)) {
          if (s != lsys) {
            L = load_tril64(tril + 6 * (int64_t)s);
            Li = load_tril64(inv + 6 * (int64_t)s);
            lsys = s;
          }
          // w = r - wrap(r - R) = R + n @ L: the centre's image nearest the atom
          double w[3], d[3], n[3];
#pragma unroll
          for (int c = 0; c < 3; ++c) {
            w[c] = gcentre[4 * (int64_t)gi + c];
            d[c] = __dsub_rn(r[c], w[c]);
          }
          if (wrap_image64(d, Li, n)) {
            double nL[3];
            row_times_tril64(n, L, nL);
#pragma unroll
            for (int c = 0; c < 3; ++c) w[c] = __dadd_rn(w[c], nL[c]);
          }
#pragma unroll
          for (int a = 0; a < 3; ++a)
#pragma unroll
            for (int b = 0; b < 3; ++b) v[10 + 3 * a + b] = w[a] * g[b];
        } else {
          status_error(status, KUPS_ERR_INVALID, i);
        }
      }
    }
    if (j == 0) cur = __shfl_sync(full, s, 0);
    if (__all_sync(full, s == cur)) {
#pragma unroll
      for (int k = 0; k < NV; ++k) run[k] += v[k];
    } else {
      // the run ends inside these 32 particles: close it, add them one system at a time
      flush_run<NV>(run, cur, out);
#pragma unroll
      for (int k = 0; k < NV; ++k) add_system(out, kAcc, k, s, v[k]);
      cur = __shfl_sync(full, s, 31);
    }
  }
  flush_run<NV>(run, cur, out);
}

__global__ void virial_finish_kernel(const double *acc, const double *tril, const double *grad_tril, int32_t n_sys,
                                     bool have_ke, double *stress, double *mol_stress, double *lat_stress,
                                     double *kinetic, double *pressure) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n_sys) return;
  const double *t = tril + 6 * (int64_t)s;
  double L[3][3] = {{t[0], 0, 0}, {t[1], t[2], 0}, {t[3], t[4], t[5]}};
  double G[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
  if (grad_tril) {
    const double *q = grad_tril + 6 * (int64_t)s;
    G[0][0] = q[0];
    G[1][0] = q[1];
    G[1][1] = q[2];
    G[2][0] = q[3];
    G[2][1] = q[4];
    G[2][2] = q[5];
  }
  const double V = fabs(t[0] * t[2] * t[5]);
  const double *a = acc + (int64_t)s * kAcc;
  double LtG[3][3];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) LtG[i][j] = L[0][i] * G[0][j] + L[1][i] * G[1][j] + L[2][i] * G[2][j];
  double tr = 0.0;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      const double sa = -(a[1 + 3 * i + j] + LtG[i][j]) / V;
      if (i == j) tr += sa;
      if (stress) stress[9 * (int64_t)s + 3 * i + j] = sa;
      if (mol_stress)
        mol_stress[9 * (int64_t)s + 3 * i + j] = (-0.5 * (a[10 + 3 * i + j] + a[10 + 3 * j + i]) - LtG[i][j]) / V;
      if (lat_stress) lat_stress[9 * (int64_t)s + 3 * i + j] = -G[i][j] / V;
    }
  const double K = have_ke ? a[0] : 0.0;
  if (kinetic) kinetic[s] = K;
  if (pressure) pressure[s] = 2.0 * K / (3.0 * V) + tr / 3.0;
}

inline unsigned blocks_for(int64_t n, int threads) { return (unsigned)std::max<int64_t>(1, (n + threads - 1) / threads); }

}  // namespace
}  // namespace kups

using namespace kups;

extern "C" size_t kups_virial_stress_workspace_bytes(int32_t n_systems, int32_t n_groups) {
  if (n_systems < 0 || n_groups < 0) return 0;
  return align256(sizeof(double) * (kAcc + 6) * (size_t)n_systems) +
         align256(sizeof(double) * 4 * (size_t)n_groups) + align256(sizeof(int32_t) * (size_t)n_groups) + 256;
}

extern "C" int32_t kups_virial_stress(const double *positions, const double *grad, const int32_t *system,
                                      int64_t n_particles, const double *tril, const double *grad_tril,
                                      int32_t n_systems, const int32_t *group, int32_t n_groups,
                                      const double *momenta, const double *masses, double *stress,
                                      double *molecular_stress, double *lattice_stress, double *kinetic,
                                      double *pressure, void *workspace, size_t workspace_bytes,
                                      kups_status *status, void *stream_) {
  cudaStream_t stream = (cudaStream_t)stream_;
  const bool mol = molecular_stress != nullptr;
  const bool ke = momenta != nullptr;
  if (n_particles < 0 || n_systems < 0 || n_groups < 0) return KUPS_ERR_INVALID;
  if (n_systems > 0 && !tril) return KUPS_ERR_INVALID;
  if (n_particles > 0 && (!positions || !grad || !system || !status)) return KUPS_ERR_INVALID;
  if (ke && !masses) return KUPS_ERR_INVALID;
  if (kinetic && !ke) return KUPS_ERR_INVALID;
  if (mol && (!group || n_particles >= (int64_t)INT32_MAX)) return KUPS_ERR_INVALID;
  if (n_systems == 0) return KUPS_OK;
  if (workspace_bytes < kups_virial_stress_workspace_bytes(n_systems, mol ? n_groups : 0)) return KUPS_ERR_INVALID;
  char *base = (char *)(((uintptr_t)workspace + 255) & ~uintptr_t(255));
  double *acc = (double *)base;
  double *inv = acc + kAcc * (size_t)n_systems;
  double *gsum = (double *)(base + align256(sizeof(double) * (kAcc + 6) * (size_t)n_systems));
  int32_t *anchor = (int32_t *)((char *)gsum + align256(sizeof(double) * 4 * (size_t)(mol ? n_groups : 0)));
  KUPS_CUDA_TRY(cudaMemsetAsync(acc, 0, sizeof(double) * kAcc * (size_t)n_systems, stream));
  cell_inverse_kernel<<<blocks_for(n_systems, 128), 128, 0, stream>>>(tril, n_systems, inv);
  if (mol && n_groups > 0 && n_particles > 0) {
    KUPS_CUDA_TRY(cudaMemsetAsync(gsum, 0, sizeof(double) * 4 * (size_t)n_groups, stream));
    KUPS_CUDA_TRY(cudaMemsetAsync(anchor, 0x7f, sizeof(int32_t) * (size_t)n_groups, stream));  // 0x7f7f7f7f
    group_anchor_kernel<<<blocks_for(n_particles, kThreads), kThreads, 0, stream>>>(
        group, system, n_particles, n_groups, n_systems, anchor, status);
    group_sum_kernel<<<blocks_for(n_particles, kThreads), kThreads, 0, stream>>>(
        positions, group, system, n_particles, n_groups, n_systems, tril, inv, anchor, gsum);
    group_centre_kernel<<<blocks_for(n_groups, kThreads), kThreads, 0, stream>>>(positions, system, n_particles,
                                                                                 n_groups, tril, inv, anchor, gsum);
  }
  if (n_particles > 0) {
    const int64_t warps = (n_particles + 32 * kPerLane - 1) / (32 * kPerLane);
    const unsigned blocks = blocks_for(warps * 32, kThreads);
#define KUPS_VIRIAL_LAUNCH(M, K)                                                                              \
  virial_accumulate_kernel<M, K><<<blocks, kThreads, 0, stream>>>(positions, grad, system, n_particles,       \
                                                                  n_systems, group, n_groups, gsum, tril, inv,\
                                                                  momenta, masses, acc, status)
    if (mol && ke) KUPS_VIRIAL_LAUNCH(true, true);
    else if (mol) KUPS_VIRIAL_LAUNCH(true, false);
    else if (ke) KUPS_VIRIAL_LAUNCH(false, true);
    else KUPS_VIRIAL_LAUNCH(false, false);
#undef KUPS_VIRIAL_LAUNCH
  }
  virial_finish_kernel<<<blocks_for(n_systems, 128), 128, 0, stream>>>(acc, tril, grad_tril, n_systems, ke, stress,
                                                                       molecular_stress, lattice_stress, kinetic,
                                                                       pressure);
  return cudaGetLastError() == cudaSuccess ? KUPS_OK : KUPS_ERR_CUDA;
}
