// Velocity-Verlet / BAOAB building blocks on the reference's float64 particle
// table, for systems too large for the fused shared-memory kernel.
//
// kups_md_kick:  p += F dt_s * scale            (MomentumStep, src/kups/md/integrators.py:217-263)
// kups_md_drift: r += p / m dt_s * scale, then wrap into fractional
//                [-0.5, 0.5)                     (PositionStep + MinimumImageConventionFlow, :104-211)
// kups_md_thermostat: p = c1 p + sqrt(kT (1 - c1^2)) sqrt(m) eta,
//                c1 = exp(-gamma dt)            (StochasticStep, :330-401); eta from
//                Philox4x32-10 keyed by (seed, particle), counter = step.
// Forces are F = -grad (the potential's dE/dx).
#include <algorithm>

#include "common.cuh"

namespace kups {
namespace {

__global__ void kick_kernel(double *mom, const double *grad, const int32_t *system, const double *dt,
                            double scale, int64_t n) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double h = dt[system[i]] * scale;
  for (int a = 0; a < 3; ++a) mom[3 * i + a] -= grad[3 * i + a] * h;
}

__global__ void drift_kernel(double *pos, const double *mom, const double *mass, const int32_t *system,
                             const double *dt, const double *tril, double scale, int64_t n) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int s = system[i];
  const double h = dt[s] * scale / mass[i];
  double r[3];
  for (int a = 0; a < 3; ++a) r[a] = pos[3 * i + a] + mom[3 * i + a] * h;
  const Tril64 L = load_tril64(tril + 6 * (int64_t)s);
  const Tril64 inv = inverse_tril64(L);
  double f[3];
  row_times_tril64(r, inv, f);
  for (int a = 0; a < 3; ++a) f[a] = (f[a] + 0.5) - floor(f[a] + 0.5) - 0.5;
  row_times_tril64(f, L, r);
  for (int a = 0; a < 3; ++a) pos[3 * i + a] = r[a];
}

__global__ void thermostat_kernel(double *mom, const double *mass, const int32_t *system,
                                  const double *dt, const double *kT, const double *friction,
                                  uint64_t seed, uint64_t step, const uint64_t *step_ptr, int64_t n) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  if (step_ptr != nullptr) step = *step_ptr;
  const int s = system[i];
  const double c1 = exp(-friction[s] * dt[s]);
  const double amp = sqrt(kT[s] * (1.0 - c1 * c1)) * sqrt(mass[i]);
  float eta[4];
  normal4(seed, (uint64_t)i, step, eta);
  for (int a = 0; a < 3; ++a) mom[3 * i + a] = c1 * mom[3 * i + a] + amp * (double)eta[a];
}

}  // namespace
// Threads per block for a per-atom float64 kernel: 256 once there are enough atoms to
// fill every SM, fewer (down to one warp) below that, so that a small system's atoms
// spread over all SMs instead of queueing on the float64 units of a few.
inline unsigned atom_block(int64_t n) {
  const int sms = device_sm_count();
  const int64_t per = (n + sms - 1) / sms;
  return (unsigned)std::min<int64_t>(256, std::max<int64_t>(32, (per + 31) / 32 * 32));
}

}  // namespace kups

using namespace kups;

extern "C" int32_t kups_md_kick(double *momenta, const double *grad, const int32_t *system,
                                const double *dt, double scale, int64_t n, void *stream) {
  if (n < 0) return KUPS_ERR_INVALID;
  if (n == 0) return KUPS_OK;
  kick_kernel<<<(unsigned)((n + atom_block(n) - 1) / atom_block(n)), atom_block(n), 0, (cudaStream_t)stream>>>(momenta, grad, system, dt,
                                                                             scale, n);
  return cudaGetLastError() == cudaSuccess ? KUPS_OK : KUPS_ERR_CUDA;
}

extern "C" int32_t kups_md_drift(double *positions, const double *momenta, const double *masses,
                                 const int32_t *system, const double *dt, const double *tril,
                                 double scale, int64_t n, void *stream) {
  if (n < 0) return KUPS_ERR_INVALID;
  if (n == 0) return KUPS_OK;
  drift_kernel<<<(unsigned)((n + atom_block(n) - 1) / atom_block(n)), atom_block(n), 0, (cudaStream_t)stream>>>(positions, momenta, masses,
                                                                              system, dt, tril, scale, n);
  return cudaGetLastError() == cudaSuccess ? KUPS_OK : KUPS_ERR_CUDA;
}

extern "C" int32_t kups_md_thermostat(double *momenta, const double *masses, const int32_t *system,
                                      const double *dt, const double *kT, const double *friction,
                                      uint64_t seed, uint64_t step, int64_t n, void *stream) {
  if (n < 0) return KUPS_ERR_INVALID;
  if (n == 0) return KUPS_OK;
  thermostat_kernel<<<(unsigned)((n + atom_block(n) - 1) / atom_block(n)), atom_block(n), 0, (cudaStream_t)stream>>>(
      momenta, masses, system, dt, kT, friction, seed, step, nullptr, n);
  return cudaGetLastError() == cudaSuccess ? KUPS_OK : KUPS_ERR_CUDA;
}

// The same with the step read from device memory when the kernel runs, so a captured CUDA
// graph that also advances the counter replays successive steps.
extern "C" int32_t kups_md_thermostat_counted(double *momenta, const double *masses, const int32_t *system,
                                              const double *dt, const double *kT, const double *friction,
                                              uint64_t seed, const uint64_t *step, int64_t n, void *stream) {
  if (n < 0 || step == nullptr) return KUPS_ERR_INVALID;
  if (n == 0) return KUPS_OK;
  thermostat_kernel<<<(unsigned)((n + atom_block(n) - 1) / atom_block(n)), atom_block(n), 0, (cudaStream_t)stream>>>(
      momenta, masses, system, dt, kT, friction, seed, 0, step, n);
  return cudaGetLastError() == cudaSuccess ? KUPS_OK : KUPS_ERR_CUDA;
}
