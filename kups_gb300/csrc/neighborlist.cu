// Reference-exact periodic neighbour list (float64 membership test).
//
// Replaces CellListNeighborList / DenseNearestNeighborList.__call__
// (src/kups/core/neighborlist.py:902-1077) for rh = None.  The edge set is the
// one basic_neighborlist (:743-786) produces; the cell grid here is this
// library's own (any grid whose cells are at least rc wide yields the same
// set, which is why the reference's Dense and CellList variants share a test
// suite).  Pipeline, all stream-ordered:
//   count atoms per system -> per-system setup (inverse cell, widths, image
//   counts, cell grid) -> bin atoms -> scan -> scatter -> sort each cell by
//   particle index (deterministic order) -> count edges per lh particle ->
//   scan -> write edges (never past capacity) -> pad the tail.
#include <algorithm>

#include "common.cuh"
#include "scan.cuh"

namespace kups {
namespace {

struct SysNL {
  Tril64 L;
  Tril64 inv;
  double rc2;
  int nc[3];
  int nimg[3];
  int image_mode;  // prod(nimg) > 1: explicit image offsets, all system pairs are candidates
  int n_atoms;
  int64_t cell_base;
};

struct NLWork {
  SysNL *sys;
  double *frac;         // [N, 3] unwrapped fractional coordinates
  int *cell_of;         // [N] global cell id or -1
  int *cell_start;      // [n_cells_cap + 1]
  int *cell_fill;       // [n_cells_cap]
  int *cell_items;      // [N]
  int64_t *edge_off;    // [N + 1]
  int64_t *scan_tmp;    // scan block sums (int64)
  int *scan_tmp32;      // scan block sums (int32)
  int64_t *n_cells;     // [1]
  int64_t n_cells_cap;
};

inline size_t align_up(size_t x) { return (x + 255) & ~size_t(255); }

// Cells allotted: never more than max(1, 2 * atoms) per system, so the total
// is bounded by n_systems + 2 * n_particles.
inline int64_t cells_capacity(int64_t n, int32_t s) { return (int64_t)s + 2 * n + 1; }

size_t layout(NLWork *w, char *base, int64_t n, int32_t s) {
  size_t off = 0;
  auto take = [&](size_t bytes) {
    char *p = base ? base + off : nullptr;
    off += align_up(bytes);
    return p;
  };
  const int64_t cc = cells_capacity(n, s);
  NLWork t;
  t.sys = (SysNL *)take(sizeof(SysNL) * (size_t)s);
  t.frac = (double *)take(sizeof(double) * 3 * (size_t)n);
  t.cell_of = (int *)take(sizeof(int) * (size_t)n);
  t.cell_start = (int *)take(sizeof(int) * (size_t)(cc + 1));
  t.cell_fill = (int *)take(sizeof(int) * (size_t)cc);
  t.cell_items = (int *)take(sizeof(int) * (size_t)n);
  t.edge_off = (int64_t *)take(sizeof(int64_t) * (size_t)(n + 1));
  const int64_t nb = scan_blocks_needed(std::max<int64_t>(n + 1, cc + 1));
  t.scan_tmp = (int64_t *)take(sizeof(int64_t) * (size_t)nb);
  t.scan_tmp32 = (int *)take(sizeof(int) * (size_t)nb);
  t.n_cells = (int64_t *)take(sizeof(int64_t));
  t.n_cells_cap = cc;
  if (w) *w = t;
  return off;
}

__global__ void count_atoms_kernel(const int32_t *system, int64_t n, int32_t s, SysNL *sys) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int32_t si = system[i];
  if (si >= 0 && si < s) atomicAdd(&sys[si].n_atoms, 1);
}

// One block: per-system parameters and the exclusive scan of cells per system.
__global__ void setup_systems_kernel(const double *tril, const double *cutoffs, int32_t s,
                                     SysNL *sys, int64_t *n_cells) {
  __shared__ int64_t scratch[32];
  int64_t carry = 0;
  for (int base = 0; base < s; base += blockDim.x) {
    const int k = base + threadIdx.x;
    int64_t cells = 0;
    if (k < s) {
      SysNL p = sys[k];
      p.L = load_tril64(tril + 6 * (int64_t)k);
      p.inv = inverse_tril64(p.L);
      const double rc = cutoffs[k];
      p.rc2 = rc * rc;
      double w[3];
      perpendicular_widths64(p.L, w);
      const bool finite = isfinite(rc);
      int prod = 1;
      for (int a = 0; a < 3; ++a) {
        int n = 1;
        if (finite) {
          const double x = ceil(2.0 * rc / w[a]);
          n = x > 1e6 ? 1000001 : (int)x;
          if (n < 1) n = 1;
          if (n % 2 == 0) n += 1;
        }
        p.nimg[a] = n;
        prod *= (n > 1 ? n : 1);
      }
      p.image_mode = prod > 1;
      int64_t budget = 2 * (int64_t)p.n_atoms;
      if (budget < 1) budget = 1;
      for (int a = 0; a < 3; ++a) {
        int c = 1;
        if (finite && !p.image_mode) {
          const double x = floor(w[a] / rc);
          c = x < 1.0 ? 1 : (x > 1024.0 ? 1024 : (int)x);
        }
        p.nc[a] = c;
      }
      while ((int64_t)p.nc[0] * p.nc[1] * p.nc[2] > budget) {
        int am = 0;
        for (int a = 1; a < 3; ++a)
          if (p.nc[a] > p.nc[am]) am = a;
        p.nc[am] = (p.nc[am] + 1) / 2;
      }
      cells = (int64_t)p.nc[0] * p.nc[1] * p.nc[2];
      sys[k] = p;
    }
    int64_t chunk;
    const int64_t ex = block_exclusive_scan<int64_t>(cells, scratch, &chunk);
    if (k < s) sys[k].cell_base = carry + ex;
    carry += chunk;
    __syncthreads();
  }
  if (threadIdx.x == 0) *n_cells = carry;
}

__device__ inline int wrap_cell(double f, int nc) {
  double w = f - floor(f);  // [0, 1)
  int c = (int)(w * nc);
  return c >= nc ? nc - 1 : (c < 0 ? 0 : c);
}

__global__ void bin_kernel(const double *positions, const int32_t *system, int64_t n, int32_t s,
                           const SysNL *sys, double *frac, int *cell_of, int *cell_count) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int32_t si = system[i];
  if (si < 0 || si >= s) {
    cell_of[i] = -1;
    return;
  }
  const SysNL &p = sys[si];
  const double r[3] = {positions[3 * i], positions[3 * i + 1], positions[3 * i + 2]};
  double f[3];
  row_times_tril64(r, p.inv, f);
  frac[3 * i] = f[0];
  frac[3 * i + 1] = f[1];
  frac[3 * i + 2] = f[2];
  const int cx = wrap_cell(f[0], p.nc[0]), cy = wrap_cell(f[1], p.nc[1]),
            cz = wrap_cell(f[2], p.nc[2]);
  const int c = (int)p.cell_base + (cz * p.nc[1] + cy) * p.nc[0] + cx;
  cell_of[i] = c;
  atomicAdd(&cell_count[c], 1);
}

__global__ void scatter_kernel(const int *cell_of, int64_t n, const int *cell_start,
                               int *cell_fill, int *cell_items) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int c = cell_of[i];
  if (c < 0) return;
  const int slot = atomicAdd(&cell_fill[c], 1);
  cell_items[cell_start[c] + slot] = (int)i;
}

__global__ void sort_cells_kernel(const int *cell_start, const int64_t *n_cells, int *items) {
  const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= *n_cells) return;
  const int b = cell_start[c], e = cell_start[c + 1];
  for (int k = b + 1; k < e; ++k) {
    const int v = items[k];
    int m = k - 1;
    while (m >= b && items[m] > v) {
      items[m + 1] = items[m];
      --m;
    }
    items[m + 1] = v;
  }
}

// Candidate test of the reference for the pair (i, j) and offset o.
// Returns true if (i, j, shift) is an edge; writes the shift.
__device__ inline bool edge_test(const SysNL &p, const double fi[3], const double fj[3],
                                 const int o[3], bool use_image, int shift[3], bool same_excl) {
  double d0[3] = {__dadd_rn(fi[0], -fj[0]), __dadd_rn(fi[1], -fj[1]), __dadd_rn(fi[2], -fj[2])};
  double ms[3] = {rint(d0[0]), rint(d0[1]), rint(d0[2])};
  double sh[3];
  bool is_min = true;
  if (use_image) {
    for (int a = 0; a < 3; ++a) {
      sh[a] = (double)o[a];
      is_min = is_min && (ms[a] == sh[a]);
    }
  } else {
    sh[0] = ms[0];
    sh[1] = ms[1];
    sh[2] = ms[2];
  }
  double d[3] = {__dadd_rn(d0[0], -sh[0]), __dadd_rn(d0[1], -sh[1]), __dadd_rn(d0[2], -sh[2])};
  double real[3];
  row_times_tril64(d, p.L, real);
  const double d2 = norm2_64(real);
  if (!(d2 < p.rc2)) return false;
  if (same_excl && is_min) return false;
  shift[0] = (int)sh[0];
  shift[1] = (int)sh[1];
  shift[2] = (int)sh[2];
  return true;
}

template <bool WRITE>
__global__ void pairs_kernel(const int32_t *system, const int32_t *inclusion,
                             const int32_t *exclusion, int64_t n, int32_t n_incl, int32_t s,
                             const SysNL *sys, const double *frac, const int *cell_of,
                             const int *cell_start, const int *cell_items, int64_t *edge_off,
                             int32_t *edges, int32_t *shifts, int64_t cap) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int32_t si = system[i];
  const int32_t inc = inclusion[i];
  int64_t count = 0;
  int64_t out = WRITE ? edge_off[i] : 0;
  if (si >= 0 && si < s && inc >= 0 && inc < n_incl) {
    const SysNL p = sys[si];
    const double fi[3] = {frac[3 * i], frac[3 * i + 1], frac[3 * i + 2]};
    const int32_t exi = exclusion[i];
    const int ci = cell_of[i] - (int)p.cell_base;
    const int cx = ci % p.nc[0], cy = (ci / p.nc[0]) % p.nc[1], cz = ci / (p.nc[0] * p.nc[1]);
    // Distinct neighbour cells per axis (1, 2 or 3 of them).
    int lx[3], ly[3], lz[3], nx, ny, nz;
    auto axis = [](int c, int nc, int *l, int &m) {
      if (nc == 1) {
        l[0] = 0;
        m = 1;
      } else if (nc == 2) {
        l[0] = 0;
        l[1] = 1;
        m = 2;
      } else {
        l[0] = (c + nc - 1) % nc;
        l[1] = c;
        l[2] = (c + 1) % nc;
        m = 3;
      }
    };
    axis(cx, p.nc[0], lx, nx);
    axis(cy, p.nc[1], ly, ny);
    axis(cz, p.nc[2], lz, nz);
    const int hx = (p.nimg[0] - 1) / 2, hy = (p.nimg[1] - 1) / 2, hz = (p.nimg[2] - 1) / 2;
    for (int az = 0; az < nz; ++az)
      for (int ay = 0; ay < ny; ++ay)
        for (int ax = 0; ax < nx; ++ax) {
          const int c = (int)p.cell_base + (lz[az] * p.nc[1] + ly[ay]) * p.nc[0] + lx[ax];
          const int b = cell_start[c], e = cell_start[c + 1];
          for (int k = b; k < e; ++k) {
            const int j = cell_items[k];
            if (inclusion[j] != inc) continue;
            const double fj[3] = {frac[3 * j], frac[3 * j + 1], frac[3 * j + 2]};
            const bool same_ex = exclusion[j] == exi;
            int sh[3];
            if (!p.image_mode) {
              const int o[3] = {0, 0, 0};
              if (edge_test(p, fi, fj, o, false, sh, same_ex)) {
                if (WRITE && out < cap) {
                  edges[2 * out] = (int32_t)i;
                  edges[2 * out + 1] = j;
                  shifts[3 * out] = sh[0];
                  shifts[3 * out + 1] = sh[1];
                  shifts[3 * out + 2] = sh[2];
                }
                ++out;
                ++count;
              }
            } else {
              for (int ox = -hx; ox <= hx; ++ox)
                for (int oy = -hy; oy <= hy; ++oy)
                  for (int oz = -hz; oz <= hz; ++oz) {
                    const int o[3] = {ox, oy, oz};
                    if (edge_test(p, fi, fj, o, true, sh, same_ex)) {
                      if (WRITE && out < cap) {
                        edges[2 * out] = (int32_t)i;
                        edges[2 * out + 1] = j;
                        shifts[3 * out] = sh[0];
                        shifts[3 * out + 1] = sh[1];
                        shifts[3 * out + 2] = sh[2];
                      }
                      ++out;
                      ++count;
                    }
                  }
            }
          }
        }
  }
  if (!WRITE) edge_off[i] = count;
}

__global__ void check_capacity_kernel(const int64_t *n_edges, int64_t cap, kups_status *st) {
  if (*n_edges > cap) status_capacity(st, KUPS_CAP_EDGES, *n_edges, -1);
}

__global__ void pad_kernel(const int64_t *n_edges, int64_t cap, int64_t n, int32_t *edges,
                           int32_t *shifts) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= cap || e < *n_edges) return;
  edges[2 * e] = (int32_t)n;
  edges[2 * e + 1] = (int32_t)n;
  shifts[3 * e] = shifts[3 * e + 1] = shifts[3 * e + 2] = 0;
}

}  // namespace
}  // namespace kups

using namespace kups;

extern "C" size_t kups_neighborlist_workspace_bytes(int64_t n_particles, int32_t n_systems) {
  return layout(nullptr, nullptr, n_particles, n_systems) + 256;
}

extern "C" int32_t kups_neighborlist_build(const double *positions, const int32_t *system,
                                           const int32_t *inclusion, const int32_t *exclusion,
                                           int64_t n, int32_t n_incl, const double *tril,
                                           const double *cutoffs, int32_t s, int32_t *edges,
                                           int32_t *shifts, int64_t cap, int64_t *n_edges,
                                           void *workspace, size_t ws_bytes,
                                           kups_status *status, void *stream_) {
  cudaStream_t stream = (cudaStream_t)stream_;
  if (n < 0 || s < 0 || cap < 0 || n >= (int64_t)INT32_MAX) return KUPS_ERR_INVALID;
  if (ws_bytes < kups_neighborlist_workspace_bytes(n, s)) return KUPS_ERR_INVALID;
  char *base = (char *)(((uintptr_t)workspace + 255) & ~uintptr_t(255));
  NLWork w;
  layout(&w, base, n, s);
  KUPS_CUDA_TRY(cudaMemsetAsync(n_edges, 0, sizeof(int64_t), stream));
  if (s == 0 || n == 0) {
    if (cap > 0)
      pad_kernel<<<(unsigned)((cap + 255) / 256), 256, 0, stream>>>(n_edges, cap, n, edges, shifts);
    return cudaGetLastError() == cudaSuccess ? KUPS_OK : KUPS_ERR_CUDA;
  }
  const unsigned gb = (unsigned)((n + 255) / 256);
  KUPS_CUDA_TRY(cudaMemsetAsync(w.sys, 0, sizeof(SysNL) * s, stream));
  KUPS_CUDA_TRY(cudaMemsetAsync(w.cell_start, 0, sizeof(int) * (w.n_cells_cap + 1), stream));
  KUPS_CUDA_TRY(cudaMemsetAsync(w.cell_fill, 0, sizeof(int) * w.n_cells_cap, stream));
  count_atoms_kernel<<<gb, 256, 0, stream>>>(system, n, s, w.sys);
  setup_systems_kernel<<<1, 1024, 0, stream>>>(tril, cutoffs, s, w.sys, w.n_cells);
  bin_kernel<<<gb, 256, 0, stream>>>(positions, system, n, s, w.sys, w.frac, w.cell_of,
                                     w.cell_start);
  KUPS_CUDA_TRY(exclusive_scan<int>(w.cell_start, w.n_cells_cap + 1, w.scan_tmp32, nullptr, stream));
  scatter_kernel<<<gb, 256, 0, stream>>>(w.cell_of, n, w.cell_start, w.cell_fill, w.cell_items);
  sort_cells_kernel<<<(unsigned)((w.n_cells_cap + 255) / 256), 256, 0, stream>>>(
      w.cell_start, w.n_cells, w.cell_items);
  pairs_kernel<false><<<(unsigned)((n + 127) / 128), 128, 0, stream>>>(system, inclusion, exclusion, n, n_incl, s, w.sys,
                                              w.frac, w.cell_of, w.cell_start, w.cell_items,
                                              w.edge_off, edges, shifts, cap);
  KUPS_CUDA_TRY(exclusive_scan<int64_t>(w.edge_off, n, w.scan_tmp, n_edges, stream));
  pairs_kernel<true><<<(unsigned)((n + 127) / 128), 128, 0, stream>>>(system, inclusion, exclusion, n, n_incl, s, w.sys,
                                             w.frac, w.cell_of, w.cell_start, w.cell_items,
                                             w.edge_off, edges, shifts, cap);
  check_capacity_kernel<<<1, 1, 0, stream>>>(n_edges, cap, status);
  if (cap > 0)
    pad_kernel<<<(unsigned)((cap + 255) / 256), 256, 0, stream>>>(n_edges, cap, n, edges, shifts);
  return cudaGetLastError() == cudaSuccess ? KUPS_OK : KUPS_ERR_CUDA;
}
