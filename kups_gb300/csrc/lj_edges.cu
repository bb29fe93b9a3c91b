// Lennard-Jones energy, dE/dx and dE/dtril over a directed edge list.
//
// Replaces lennard_jones_energy (src/kups/potential/classical/lennard_jones.py:149-178)
// and the jax.vjp gradient of PotentialFromEnergy with respect to
// PositionAndUnitCell (src/kups/potential/common/energy.py:264-355,
// lennard_jones.py:481-488).  Per directed edge e = (i, j, s):
//   d = x_j - x_i + s @ L,  r2 = |d|^2,  c6 = (sigma^2 / r2)^3,
//   E_e = 4 eps (c6^2 - c6) [r2 < rc^2],  g = dE_e/dd = -24 eps c6 (2 c6 - 1) d / r2,
// and E_s = sum E_e / 2, dE/dx_j += g/2, dE/dx_i -= g/2, dE/dL_ab += s_a g_b / 2.
// The distance vector is formed in float64; the pair arithmetic runs in
// float32 (pair_fp32) or float64; every sum is float64.
#include "common.cuh"

namespace kups {
namespace {

template <typename R>
__device__ inline void lj_pair(R r2, R sig, R eps, R rc2, R &e, R &dedr2) {
  if (r2 < rc2) {
    const R inv = R(1) / r2;
    const R s2 = sig * sig * inv;
    const R c6 = s2 * s2 * s2;
    e = R(4) * eps * (c6 * c6 - c6);
    dedr2 = R(-12) * eps * c6 * (R(2) * c6 - R(1)) * inv;
  } else {
    e = R(0);
    dedr2 = R(0);
  }
}

__global__ void lj_edges_kernel(const double *pos, const int32_t *system, const int32_t *species,
                                int64_t n, const double *tril, const double *cutoffs, int32_t s,
                                const double *sigma, const double *epsilon, int32_t nsp,
                                const int32_t *edges, const int32_t *shifts, int64_t n_edges,
                                double *energy, double *grad, double *grad_tril, int pair_fp32,
                                kups_status *status) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  int sys = -1;
  double en = 0, g[3] = {0, 0, 0}, sh[3] = {0, 0, 0};
  if (e < n_edges) {
    const int i = edges[2 * e], j = edges[2 * e + 1];
    if (i >= 0 && i < n && j >= 0 && j < n) {
      const int si = system[i];
      if (si >= 0 && si < s) {
        sys = si;
        const Tril64 L = load_tril64(tril + 6 * (int64_t)si);
        sh[0] = shifts[3 * e];
        sh[1] = shifts[3 * e + 1];
        sh[2] = shifts[3 * e + 2];
        double sL[3];
        row_times_tril64(sh, L, sL);
        const double d[3] = {pos[3 * j] - pos[3 * i] + sL[0], pos[3 * j + 1] - pos[3 * i + 1] + sL[1],
                             pos[3 * j + 2] - pos[3 * i + 2] + sL[2]};
        const int ti = species[i], tj = species[j];
        const double sig = sigma[ti * nsp + tj], eps = epsilon[ti * nsp + tj];
        const double rc = cutoffs[si];
        const double r2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
        double dedr2;
        if (pair_fp32) {
          float ef, df;
          lj_pair<float>((float)r2, (float)sig, (float)eps, (float)(rc * rc), ef, df);
          en = ef;
          dedr2 = df;
        } else {
          lj_pair<double>(r2, sig, eps, rc * rc, en, dedr2);
        }
        if (!isfinite(en) || !isfinite(dedr2)) status_error(status, KUPS_ERR_NONFINITE, e);
        for (int a = 0; a < 3; ++a) g[a] = 2.0 * dedr2 * d[a];
        for (int a = 0; a < 3; ++a) {
          atomicAdd(&grad[3 * (int64_t)j + a], 0.5 * g[a]);
          atomicAdd(&grad[3 * (int64_t)i + a], -0.5 * g[a]);
        }
      }
    }
  }
  add_system(energy, 1, 0, sys, 0.5 * en);
  // dE/dL_ab for (a, b) in tril order
  add_system(grad_tril, 6, 0, sys, 0.5 * sh[0] * g[0]);
  add_system(grad_tril, 6, 1, sys, 0.5 * sh[1] * g[0]);
  add_system(grad_tril, 6, 2, sys, 0.5 * sh[1] * g[1]);
  add_system(grad_tril, 6, 3, sys, 0.5 * sh[2] * g[0]);
  add_system(grad_tril, 6, 4, sys, 0.5 * sh[2] * g[1]);
  add_system(grad_tril, 6, 5, sys, 0.5 * sh[2] * g[2]);
}

}  // namespace
}  // namespace kups

using namespace kups;

extern "C" int32_t kups_lj_edges(const double *positions, const int32_t *system,
                                 const int32_t *species, int64_t n, const double *tril,
                                 const double *cutoffs, int32_t s, const double *sigma,
                                 const double *epsilon, int32_t nsp, const int32_t *edges,
                                 const int32_t *shifts, int64_t n_edges, double *energy,
                                 double *grad, double *grad_tril, int32_t pair_fp32,
                                 kups_status *status, void *stream_) {
  cudaStream_t stream = (cudaStream_t)stream_;
  if (n < 0 || s < 0 || n_edges < 0 || nsp <= 0) return KUPS_ERR_INVALID;
  if (s > 0) {
    KUPS_CUDA_TRY(cudaMemsetAsync(energy, 0, sizeof(double) * s, stream));
    KUPS_CUDA_TRY(cudaMemsetAsync(grad_tril, 0, sizeof(double) * 6 * s, stream));
  }
  if (n > 0) KUPS_CUDA_TRY(cudaMemsetAsync(grad, 0, sizeof(double) * 3 * n, stream));
  if (n_edges == 0) return KUPS_OK;
  const unsigned grid = (unsigned)((n_edges + 255) / 256);
  lj_edges_kernel<<<grid, 256, 0, stream>>>(positions, system, species, n, tril, cutoffs, s, sigma,
                                            epsilon, nsp, edges, shifts, n_edges, energy, grad,
                                            grad_tril, pair_fp32, status);
  return cudaGetLastError() == cudaSuccess ? KUPS_OK : KUPS_ERR_CUDA;
}

// Global analytic LJ tail correction (lennard_jones.py:276-340): per system, species counts
// N_a, density N_a N_b / V, t1 = (sigma_ab / rc)^3, t2 = t1^3,
//   E = sum_ab (8/3) pi N_a N_b / V eps_ab sigma_ab^3 (t2 / 3 - t1) mask_ab,
//   P = sum_ab (16/3) pi N_a N_b / V^2 eps_ab sigma_ab^3 (2 t2 / 3 - t1) mask_ab.
// One block per system counts its species in shared memory (atoms grouped by sys_offset).
namespace kups {
namespace {
constexpr int kTailMaxSpecies = 64;
__global__ void lj_tail_kernel(const int32_t *species, const int32_t *sys_offset, const double *tril,
                               const double *sigma, const double *eps, const int32_t *mask, int nsp,
                               const double *cutoff, double *energy, double *pressure, kups_status *status) {
  __shared__ int cnt[kTailMaxSpecies];
  __shared__ int bad;
  const int s = blockIdx.x;
  for (int t = threadIdx.x; t < nsp; t += blockDim.x) cnt[t] = 0;
  if (threadIdx.x == 0) bad = 0;
  __syncthreads();
  const int a0 = sys_offset[s], a1 = sys_offset[s + 1];
  for (int i = a0 + threadIdx.x; i < a1; i += blockDim.x) {
    const int t = species[i];
    if (t < 0 || t >= nsp) bad = 1;
    else atomicAdd(&cnt[t], 1);
  }
  __syncthreads();
  if (threadIdx.x != 0) return;
  if (bad) {
    status_error(status, KUPS_ERR_INVALID, s);
    return;
  }
  const double *t6 = tril + 6 * (int64_t)s;
  const double v = fabs(t6[0] * t6[2] * t6[5]);
  const double rc = cutoff[s];
  const double pi = 3.14159265358979323846;
  double e = 0.0, p = 0.0;
  for (int a = 0; a < nsp; ++a)
    for (int b = 0; b < nsp; ++b) {
      const int k = a * nsp + b;
      if (mask != nullptr ? mask[k] == 0 : eps[k] <= 0.0) continue;
      const double sg = sigma[k], s3 = sg * sg * sg, t1 = s3 / (rc * rc * rc), t2 = t1 * t1 * t1;
      const double rho = (double)cnt[a] * (double)cnt[b] / v;
      e += (8.0 / 3.0) * pi * rho * eps[k] * s3 * (t2 / 3.0 - t1);
      p += (16.0 / 3.0) * pi * rho / v * eps[k] * s3 * (t2 / 3.0 * 2.0 - t1);
    }
  if (energy) energy[s] = e;
  if (pressure) pressure[s] = p;
}
}  // namespace
}  // namespace kups

extern "C" int32_t kups_lj_tail_correction(const int32_t *species, const int32_t *sys_offset, int32_t n_systems,
                                           const double *tril, const double *sigma, const double *epsilon,
                                           const int32_t *tail_mask, int32_t n_species, const double *cutoff,
                                           double *energy, double *pressure, kups_status *status, void *stream) {
  if (n_systems < 0 || n_species < 1 || n_species > kups::kTailMaxSpecies) return KUPS_ERR_INVALID;
  if (n_systems == 0) return KUPS_OK;
  kups::lj_tail_kernel<<<n_systems, 256, 0, (cudaStream_t)stream>>>(species, sys_offset, tril, sigma, epsilon,
                                                                    tail_mask, n_species, cutoff, energy, pressure,
                                                                    status);
  return cudaGetLastError() == cudaSuccess ? KUPS_OK : KUPS_ERR_CUDA;
}
