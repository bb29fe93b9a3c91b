// Edge-set kernels of the local machine-learned potential (message passing over the
// neighbour list): the geometry of every directed edge, the sum of per-edge messages
// onto the edge's first atom, and the forces and cell gradient from the gradient of the
// energy with respect to the edge vectors.
//
// Replaces the gather / segment-sum / vjp steps of local_mliap_energy_full
// (src/kups/potential/mliap/local.py:310-356): d_ij = x_j - x_i + s @ L
// (Edges.difference_vectors, src/kups/core/neighborlist.py:164-184), msg_i = sum_j m_ij
// (jax.ops.segment_sum over the first index) and, through the chain rule of
// PotentialFromEnergy (src/kups/potential/common/energy.py:264-355) with Cartesian
// positions held fixed, dE/dx_i = -sum_{e: i_e = i} g_e + sum_{e: j_e = i} g_e and
// dE/dL_ab = sum_e s_e,a g_e,b, g_e = dE/dd_e.  The model functions themselves are the
// caller's.  Rows past n_edges, or with an index outside [0, n), are padding.
#include "common.cuh"

namespace kups {
namespace {

__global__ void edge_vectors_kernel(const double *pos, const int32_t *system, int64_t n, const double *tril,
                                    int32_t s, const int32_t *edges, const int32_t *shifts, int64_t ne, double *d) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= ne) return;
  const int i = edges[2 * e], j = edges[2 * e + 1];
  double v[3] = {0.0, 0.0, 0.0};
  if (i >= 0 && i < n && j >= 0 && j < n) {
    const int si = system[i];
    if (si >= 0 && si < s) {
      const Tril64 L = load_tril64(tril + 6 * (int64_t)si);
      const double sh[3] = {(double)shifts[3 * e], (double)shifts[3 * e + 1], (double)shifts[3 * e + 2]};
      double sL[3];
      row_times_tril64(sh, L, sL);
      for (int a = 0; a < 3; ++a) v[a] = pos[3 * (int64_t)j + a] - pos[3 * (int64_t)i + a] + sL[a];
    }
  }
  for (int a = 0; a < 3; ++a) d[3 * e + a] = v[a];
}

// One thread per (edge, feature); consecutive threads walk the features of an edge.
__global__ void edge_segment_sum_kernel(const double *values, int32_t width, const int32_t *edges, int64_t ne,
                                        int64_t n, double *out) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ne * width) return;
  const int64_t e = t / width;
  const int f = (int)(t - e * width);
  const int i = edges[2 * e];
  if (i < 0 || i >= n || edges[2 * e + 1] < 0 || edges[2 * e + 1] >= n) return;
  atomicAdd(&out[(int64_t)i * width + f], values[t]);
}

__global__ void edge_gradients_kernel(const double *g, const int32_t *system, int64_t n, int32_t s,
                                      const int32_t *edges, const int32_t *shifts, int64_t ne, double *grad,
                                      double *grad_tril) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  int sys = -1;
  double ge[3] = {0, 0, 0}, sh[3] = {0, 0, 0};
  if (e < ne) {
    const int i = edges[2 * e], j = edges[2 * e + 1];
    if (i >= 0 && i < n && j >= 0 && j < n && system[i] >= 0 && system[i] < s) {
      sys = system[i];
      for (int a = 0; a < 3; ++a) {
        ge[a] = g[3 * e + a];
        sh[a] = (double)shifts[3 * e + a];
        atomicAdd(&grad[3 * (int64_t)j + a], ge[a]);
        atomicAdd(&grad[3 * (int64_t)i + a], -ge[a]);
      }
    }
  }
  if (grad_tril != nullptr) {
    add_system(grad_tril, 6, 0, sys, sh[0] * ge[0]);
    add_system(grad_tril, 6, 1, sys, sh[1] * ge[0]);
    add_system(grad_tril, 6, 2, sys, sh[1] * ge[1]);
    add_system(grad_tril, 6, 3, sys, sh[2] * ge[0]);
    add_system(grad_tril, 6, 4, sys, sh[2] * ge[1]);
    add_system(grad_tril, 6, 5, sys, sh[2] * ge[2]);
  }
}

}  // namespace
}  // namespace kups

using namespace kups;

extern "C" int32_t kups_edge_vectors(const double *positions, const int32_t *system, int64_t n, const double *tril,
                                     int32_t n_systems, const int32_t *edges, const int32_t *shifts, int64_t n_edges,
                                     double *d, void *stream) {
  if (n < 0 || n_systems < 0 || n_edges < 0) return KUPS_ERR_INVALID;
  if (n_edges == 0) return KUPS_OK;
  edge_vectors_kernel<<<(unsigned)((n_edges + 255) / 256), 256, 0, (cudaStream_t)stream>>>(
      positions, system, n, tril, n_systems, edges, shifts, n_edges, d);
  return cudaGetLastError() == cudaSuccess ? KUPS_OK : KUPS_ERR_CUDA;
}

extern "C" int32_t kups_edge_segment_sum(const double *values, int32_t width, const int32_t *edges, int64_t n_edges,
                                         int64_t n, double *out, void *stream_) {
  cudaStream_t stream = (cudaStream_t)stream_;
  if (width < 0 || n_edges < 0 || n < 0) return KUPS_ERR_INVALID;
  if (n > 0 && width > 0) KUPS_CUDA_TRY(cudaMemsetAsync(out, 0, sizeof(double) * (size_t)n * width, stream));
  const int64_t total = n_edges * (int64_t)width;
  if (total == 0) return KUPS_OK;
  edge_segment_sum_kernel<<<(unsigned)((total + 255) / 256), 256, 0, stream>>>(values, width, edges, n_edges, n, out);
  return cudaGetLastError() == cudaSuccess ? KUPS_OK : KUPS_ERR_CUDA;
}

extern "C" int32_t kups_edge_gradients(const double *dE_dd, const int32_t *system, int64_t n, int32_t n_systems,
                                       const int32_t *edges, const int32_t *shifts, int64_t n_edges, double *grad,
                                       double *grad_tril, void *stream_) {
  cudaStream_t stream = (cudaStream_t)stream_;
  if (n < 0 || n_systems < 0 || n_edges < 0) return KUPS_ERR_INVALID;
  if (n > 0) KUPS_CUDA_TRY(cudaMemsetAsync(grad, 0, sizeof(double) * 3 * (size_t)n, stream));
  if (grad_tril != nullptr && n_systems > 0)
    KUPS_CUDA_TRY(cudaMemsetAsync(grad_tril, 0, sizeof(double) * 6 * (size_t)n_systems, stream));
  if (n_edges == 0) return KUPS_OK;
  edge_gradients_kernel<<<(unsigned)((n_edges + 255) / 256), 256, 0, stream>>>(dE_dd, system, n, n_systems, edges,
                                                                              shifts, n_edges, grad, grad_tril);
  return cudaGetLastError() == cudaSuccess ? KUPS_OK : KUPS_ERR_CUDA;
}
