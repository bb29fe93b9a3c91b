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
  int refused;     // more than kMaxNLImages image offsets: no edges, KUPS_ERR_UNSUPPORTED recorded
};

// Image offsets per candidate pair beyond which a system is refused instead of searched (a
// cutoff of many cell widths: 11^3 offsets is a cutoff of about five widths; the
// reference's own image replication would materialise that many copies of every pair).
constexpr double kMaxNLImages = 1331.0;

struct NLWork {
  SysNL *sys;
  double *frac;         // [N, 3] unwrapped fractional coordinates
  int *cell_of;         // [N] global cell id or -1
  int *cell_start;      // [n_cells_cap + 1]
  int *cell_fill;       // [n_cells_cap]
  int *cell_items;      // [N]
  int64_t *edge_off;    // [N + 1], or [27 N + 1] for the split pair search
  bool split;           // one thread per (particle, neighbour cell): N <= kNLSplitMax
  int64_t *scan_tmp;    // scan block sums (int64)
  int *scan_tmp32;      // scan block sums (int32)
  int64_t *n_cells;     // [1]
  int64_t n_cells_cap;
};

inline size_t align_up(size_t x) { return (x + 255) & ~size_t(255); }

// Neighbour cells per particle, and the batch size up to which the pair search runs one
// thread per (particle, neighbour cell) instead of one per particle (a single system of a
// few thousand particles otherwise occupies a few SMs).
constexpr int kNLCells = 27;
constexpr int64_t kNLSplitMax = 32768;

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
  t.split = n <= kNLSplitMax;
  const int64_t n_off = t.split ? kNLCells * n : n;
  t.edge_off = (int64_t *)take(sizeof(int64_t) * (size_t)(n_off + 1));
  const int64_t nb = scan_blocks_needed(std::max<int64_t>(n_off + 1, cc + 1));
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
__global__ void __launch_bounds__(1024) setup_systems_kernel(const double *tril, const double *cutoffs, int32_t s,
                                     SysNL *sys, int64_t *n_cells, kups_status *status) {
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
      double prod = 1.0;
      for (int a = 0; a < 3; ++a) {
        int n = 1;
        if (finite) {
          const double x = ceil(2.0 * rc / w[a]);
          n = x > 1e6 ? 1000001 : (int)x;
          if (n < 1) n = 1;
          if (n % 2 == 0) n += 1;
        }
        p.nimg[a] = n;
        prod *= (double)n;
      }
      p.refused = prod > kMaxNLImages;
      if (p.refused) {
        status_error(status, KUPS_ERR_UNSUPPORTED, k);
        p.nimg[0] = p.nimg[1] = p.nimg[2] = 1;
        prod = 1.0;
      }
      p.image_mode = prod > 1.0;
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

// One thread per particle, or with SPLIT one thread per (particle, neighbour cell): thread
// a n + i scans cell a = (az * 3 + ay) * 3 + ax of particle i's (up to) 3 x 3 x 3 cells, so
// that a batch of few particles still fills the GPU, and the lanes of a warp (consecutive,
// cell-sorted particles) scan the same relative cell in step.  Offsets are kept at 27 i + a,
// the (particle, az, ay, ax) order of the per-particle form's loops, so both forms write the
// same edges in the same order.
template <bool WRITE, bool SPLIT>
__global__ void pairs_kernel(const int32_t *system, const int32_t *inclusion,
                             const int32_t *exclusion, int64_t n, int32_t n_incl, int32_t s,
                             const SysNL *sys, const double *frac, const int *cell_of,
                             const int *cell_start, const int *cell_items, int64_t *edge_off,
                             int32_t *edges, int32_t *shifts, int64_t cap) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (SPLIT ? kNLCells * n : n)) return;
  const int a_only = SPLIT ? (int)(t / n) : -1;
  const int64_t i = SPLIT ? t - (int64_t)a_only * n : t;
  const int64_t slot = SPLIT ? i * kNLCells + a_only : i;  // this thread's offset entry
  const int32_t si = system[i];
  const int32_t inc = inclusion[i];
  int64_t count = 0;
  int64_t out = WRITE ? edge_off[slot] : 0;
  if (si >= 0 && si < s && inc >= 0 && inc < n_incl && !sys[si].refused) {
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
          if (SPLIT && (az * 3 + ay) * 3 + ax != a_only) continue;
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
  if (!WRITE) edge_off[slot] = count;
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
  setup_systems_kernel<<<1, 1024, 0, stream>>>(tril, cutoffs, s, w.sys, w.n_cells, status);
  bin_kernel<<<gb, 256, 0, stream>>>(positions, system, n, s, w.sys, w.frac, w.cell_of,
                                     w.cell_start);
  KUPS_CUDA_TRY(exclusive_scan<int>(w.cell_start, w.n_cells_cap + 1, w.scan_tmp32, nullptr, stream));
  scatter_kernel<<<gb, 256, 0, stream>>>(w.cell_of, n, w.cell_start, w.cell_fill, w.cell_items);
  sort_cells_kernel<<<(unsigned)((w.n_cells_cap + 255) / 256), 256, 0, stream>>>(
      w.cell_start, w.n_cells, w.cell_items);
  const int64_t n_thr = w.split ? kNLCells * n : n;
  const unsigned gp = (unsigned)((n_thr + 127) / 128);
  if (w.split)
    pairs_kernel<false, true><<<gp, 128, 0, stream>>>(system, inclusion, exclusion, n, n_incl, s, w.sys, w.frac,
                                                      w.cell_of, w.cell_start, w.cell_items, w.edge_off, edges,
                                                      shifts, cap);
  else
    pairs_kernel<false, false><<<gp, 128, 0, stream>>>(system, inclusion, exclusion, n, n_incl, s, w.sys, w.frac,
                                                       w.cell_of, w.cell_start, w.cell_items, w.edge_off, edges,
                                                       shifts, cap);
  KUPS_CUDA_TRY(exclusive_scan<int64_t>(w.edge_off, n_thr, w.scan_tmp, n_edges, stream));
  if (w.split)
    pairs_kernel<true, true><<<gp, 128, 0, stream>>>(system, inclusion, exclusion, n, n_incl, s, w.sys, w.frac,
                                                     w.cell_of, w.cell_start, w.cell_items, w.edge_off, edges,
                                                     shifts, cap);
  else
    pairs_kernel<true, false><<<gp, 128, 0, stream>>>(system, inclusion, exclusion, n, n_incl, s, w.sys, w.frac,
                                                      w.cell_of, w.cell_start, w.cell_items, w.edge_off, edges,
                                                      shifts, cap);
  check_capacity_kernel<<<1, 1, 0, stream>>>(n_edges, cap, status);
  if (cap > 0)
    pad_kernel<<<(unsigned)((cap + 255) / 256), 256, 0, stream>>>(n_edges, cap, n, edges, shifts);
  return cudaGetLastError() == cudaSuccess ? KUPS_OK : KUPS_ERR_CUDA;
}

// ---------------------------------------------------------------------------
// rh subset: edges (i in lh, j in rh) within the cutoff of the pair's system,
// the rh particles given separately (NearestNeighborList.__call__ with rh,
// src/kups/core/neighborlist.py:226-255; basic_neighborlist :743-786).  The lh
// particles are binned into the cell grid of the full mode; each rh particle
// scans the lh cells around its own cell.  Candidate rules as the reference's
// _build_segmentation_mask (:505-539), _filter_candidates (:692-740) and
// _compact_edges (:651-689):
//   * same system, same valid inclusion label (lh and rh labels);
//   * the image rule and strict d^2 < rc^2 of the full mode, difference lh - rh;
//   * exclusion labels equal (lh vs rh) drop the minimum image only;
//   * with rh_index_remap (rh particle j stands for lh particle remap[j]):
//     a pair whose lh particle is itself one of the remapped ones is kept only
//     for i >= remap[j], and every edge (i, remap[j], s) is written together
//     with its reverse (remap[j], i, -s);
//   * without remap, edges are (i, j) with j indexing rh.
// Padding rows hold max(n_lh, n_rh).
namespace kups {
namespace {

struct RhWork {
  NLWork lh;
  uint8_t *in_remap;  // [n_lh]: lh particle i is some remap[j]
  int64_t *rh_off;    // [n_rh + 1]
  int64_t *rh_scan;   // scan block sums
};

size_t rh_layout(RhWork *w, char *base, int64_t n_lh, int64_t n_rh, int32_t s) {
  size_t off = layout(w ? &w->lh : nullptr, base, n_lh, s);
  auto take = [&](size_t bytes) {
    char *p = base ? base + off : nullptr;
    off += align_up(bytes);
    return p;
  };
  uint8_t *flags = (uint8_t *)take((size_t)std::max<int64_t>(n_lh, 1));
  int64_t *roff = (int64_t *)take(sizeof(int64_t) * (size_t)(n_rh + 1));
  int64_t *rscan = (int64_t *)take(sizeof(int64_t) * (size_t)scan_blocks_needed(n_rh + 1));
  if (w) {
    w->in_remap = flags;
    w->rh_off = roff;
    w->rh_scan = rscan;
  }
  return off;
}

__global__ void mark_remap_kernel(const int32_t *remap, int64_t n_rh, int64_t n_lh, uint8_t *flags) {
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n_rh) return;
  const int32_t r = remap[j];
  if (r >= 0 && r < n_lh) flags[r] = 1;
}

template <bool WRITE>
__global__ void pairs_rh_kernel(const int32_t *lh_incl, const int32_t *lh_excl, int64_t n_lh,
                                const double *rh_pos, const int32_t *rh_system, const int32_t *rh_incl,
                                const int32_t *rh_excl, int64_t n_rh, const int32_t *remap,
                                const uint8_t *in_remap, int32_t n_incl, int32_t s, const SysNL *sys,
                                const double *frac, const int *cell_start, const int *cell_items,
                                int64_t *rh_off, int64_t oob, int32_t *edges, int32_t *shifts, int64_t cap) {
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n_rh) return;
  const int32_t sj = rh_system[j];
  const int32_t inc = rh_incl[j];
  int64_t count = 0;
  int64_t out = WRITE ? rh_off[j] : 0;
  if (sj >= 0 && sj < s && inc >= 0 && inc < n_incl && !sys[sj].refused) {
    const SysNL p = sys[sj];
    const double r[3] = {rh_pos[3 * j], rh_pos[3 * j + 1], rh_pos[3 * j + 2]};
    double fj[3];
    row_times_tril64(r, p.inv, fj);
    const int cx = wrap_cell(fj[0], p.nc[0]), cy = wrap_cell(fj[1], p.nc[1]), cz = wrap_cell(fj[2], p.nc[2]);
    const int32_t exj = rh_excl[j];
    const int64_t ro = remap != nullptr ? (int64_t)remap[j] : j;
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
    auto emit = [&](int i, const int sh[3]) {
      if (WRITE) {
        if (out < cap) {
          edges[2 * out] = i;
          edges[2 * out + 1] = (int32_t)ro;
          shifts[3 * out] = sh[0];
          shifts[3 * out + 1] = sh[1];
          shifts[3 * out + 2] = sh[2];
        }
        ++out;
        if (remap != nullptr) {
          if (out < cap) {
            edges[2 * out] = (int32_t)ro;
            edges[2 * out + 1] = i;
            shifts[3 * out] = -sh[0];
            shifts[3 * out + 1] = -sh[1];
            shifts[3 * out + 2] = -sh[2];
          }
          ++out;
        }
      }
      count += remap != nullptr ? 2 : 1;
    };
    for (int az = 0; az < nz; ++az)
      for (int ay = 0; ay < ny; ++ay)
        for (int ax = 0; ax < nx; ++ax) {
          const int c = (int)p.cell_base + (lz[az] * p.nc[1] + ly[ay]) * p.nc[0] + lx[ax];
          const int b = cell_start[c], e = cell_start[c + 1];
          for (int k = b; k < e; ++k) {
            const int i = cell_items[k];
            if (lh_incl[i] != inc) continue;
            if (remap != nullptr && in_remap[i] && !((int64_t)i >= ro)) continue;
            const double fi[3] = {frac[3 * i], frac[3 * i + 1], frac[3 * i + 2]};
            const bool same_ex = lh_excl[i] == exj;
            int sh[3];
            if (!p.image_mode) {
              const int o[3] = {0, 0, 0};
              if (edge_test(p, fi, fj, o, false, sh, same_ex)) emit(i, sh);
            } else {
              for (int ox = -hx; ox <= hx; ++ox)
                for (int oy = -hy; oy <= hy; ++oy)
                  for (int oz = -hz; oz <= hz; ++oz) {
                    const int o[3] = {ox, oy, oz};
                    if (edge_test(p, fi, fj, o, true, sh, same_ex)) emit(i, sh);
                  }
            }
          }
        }
  }
  (void)oob;
  if (!WRITE) rh_off[j] = count;
}

// neighborlist_changes' split of the combined call (src/kups/core/neighborlist.py:1425-1515):
// removed = both ends < n (old positions), added = an end >= n (a new position) and no end
// that is the old copy of a changed particle; appended indices n + m become p_idx[m].
__global__ void split_flags_kernel(const int32_t *edges, const int64_t *n_edges, int64_t n, int64_t k,
                                   const uint8_t *is_changed, int64_t *add_flag, int64_t *rem_flag, int64_t total) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= total) return;
  int64_t a = 0, r = 0;
  if (e < *n_edges && e < total - 1) {  // entry total - 1 only closes the scan
    const int64_t c0 = edges[2 * e], c1 = edges[2 * e + 1];
    r = (c0 < n) && (c1 < n);
    const bool stale = ((c0 < n) && is_changed[c0]) || ((c1 < n) && is_changed[c1]);
    a = (c0 < n + k) && (c1 < n + k) && ((c0 >= n) || (c1 >= n)) && !stale;
  }
  add_flag[e] = a;
  rem_flag[e] = r;
}

__global__ void split_write_kernel(const int32_t *edges, const int32_t *shifts, const int64_t *n_edges, int64_t n,
                                   const int32_t *p_idx, const int64_t *add_off, const int64_t *rem_off,
                                   int64_t total, int32_t *add_e, int32_t *add_s, int64_t add_cap, int32_t *rem_e,
                                   int32_t *rem_s, int64_t rem_cap) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= total || e >= *n_edges) return;
  const bool a = add_off[e + 1] > add_off[e], r = rem_off[e + 1] > rem_off[e];
  if (!a && !r) return;
  int64_t c[2] = {edges[2 * e], edges[2 * e + 1]};
  for (int t = 0; t < 2; ++t)
    if (c[t] >= n) c[t] = p_idx[c[t] - n];
  int32_t *oe = a ? add_e : rem_e;
  int32_t *os = a ? add_s : rem_s;
  const int64_t slot = a ? add_off[e] : rem_off[e];
  if (slot >= (a ? add_cap : rem_cap)) return;
  oe[2 * slot] = (int32_t)c[0];
  oe[2 * slot + 1] = (int32_t)c[1];
  for (int t = 0; t < 3; ++t) os[3 * slot + t] = shifts[3 * e + t];
}

__global__ void pad_from_kernel(const int64_t *count, int64_t cap, int64_t fill, int32_t *edges, int32_t *shifts) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= cap || e < *count) return;
  edges[2 * e] = (int32_t)fill;
  edges[2 * e + 1] = (int32_t)fill;
  shifts[3 * e] = shifts[3 * e + 1] = shifts[3 * e + 2] = 0;
}

__global__ void split_check_kernel(const int64_t *n_add, int64_t add_cap, const int64_t *n_rem, int64_t rem_cap,
                                   kups_status *st) {
  if (*n_add > add_cap) status_capacity(st, KUPS_CAP_EDGES, *n_add, -1);
  if (*n_rem > rem_cap) status_capacity(st, KUPS_CAP_EDGES, *n_rem, -1);
}

__global__ void mark_changed_kernel(const int32_t *p_idx, int64_t k, int64_t n, uint8_t *is_changed) {
  const int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (m < k && p_idx[m] >= 0 && p_idx[m] < n) is_changed[p_idx[m]] = 1;
}

}  // namespace
}  // namespace kups

extern "C" size_t kups_neighborlist_rh_workspace_bytes(int64_t n_lh, int64_t n_rh, int32_t n_systems) {
  return rh_layout(nullptr, nullptr, n_lh, n_rh, n_systems) + 256;
}

extern "C" int32_t kups_neighborlist_build_rh(
    const double *lh_positions, const int32_t *lh_system, const int32_t *lh_inclusion, const int32_t *lh_exclusion,
    int64_t n_lh, const double *rh_positions, const int32_t *rh_system, const int32_t *rh_inclusion,
    const int32_t *rh_exclusion, int64_t n_rh, const int32_t *rh_index_remap, int32_t n_incl, const double *tril,
    const double *cutoffs, int32_t s, int32_t *edges, int32_t *shifts, int64_t cap, int64_t *n_edges,
    void *workspace, size_t ws_bytes, kups_status *status, void *stream_) {
  cudaStream_t stream = (cudaStream_t)stream_;
  if (n_lh < 0 || n_rh < 0 || s < 0 || cap < 0 || n_lh >= (int64_t)INT32_MAX || n_rh >= (int64_t)INT32_MAX)
    return KUPS_ERR_INVALID;
  if (ws_bytes < kups_neighborlist_rh_workspace_bytes(n_lh, n_rh, s)) return KUPS_ERR_INVALID;
  const int64_t oob = std::max(n_lh, n_rh);
  char *base = (char *)(((uintptr_t)workspace + 255) & ~uintptr_t(255));
  RhWork w;
  rh_layout(&w, base, n_lh, n_rh, s);
  KUPS_CUDA_TRY(cudaMemsetAsync(n_edges, 0, sizeof(int64_t), stream));
  if (s == 0 || n_lh == 0 || n_rh == 0) {
    if (cap > 0) pad_kernel<<<(unsigned)((cap + 255) / 256), 256, 0, stream>>>(n_edges, cap, oob, edges, shifts);
    return cudaGetLastError() == cudaSuccess ? KUPS_OK : KUPS_ERR_CUDA;
  }
  const int64_t n = n_lh;
  const unsigned gb = (unsigned)((n + 255) / 256);
  NLWork &l = w.lh;
  KUPS_CUDA_TRY(cudaMemsetAsync(l.sys, 0, sizeof(SysNL) * s, stream));
  KUPS_CUDA_TRY(cudaMemsetAsync(l.cell_start, 0, sizeof(int) * (l.n_cells_cap + 1), stream));
  KUPS_CUDA_TRY(cudaMemsetAsync(l.cell_fill, 0, sizeof(int) * l.n_cells_cap, stream));
  KUPS_CUDA_TRY(cudaMemsetAsync(w.in_remap, 0, (size_t)std::max<int64_t>(n, 1), stream));
  count_atoms_kernel<<<gb, 256, 0, stream>>>(lh_system, n, s, l.sys);
  setup_systems_kernel<<<1, 1024, 0, stream>>>(tril, cutoffs, s, l.sys, l.n_cells, status);
  bin_kernel<<<gb, 256, 0, stream>>>(lh_positions, lh_system, n, s, l.sys, l.frac, l.cell_of, l.cell_start);
  KUPS_CUDA_TRY(exclusive_scan<int>(l.cell_start, l.n_cells_cap + 1, l.scan_tmp32, nullptr, stream));
  scatter_kernel<<<gb, 256, 0, stream>>>(l.cell_of, n, l.cell_start, l.cell_fill, l.cell_items);
  sort_cells_kernel<<<(unsigned)((l.n_cells_cap + 255) / 256), 256, 0, stream>>>(l.cell_start, l.n_cells,
                                                                                 l.cell_items);
  if (rh_index_remap != nullptr)
    mark_remap_kernel<<<(unsigned)((n_rh + 255) / 256), 256, 0, stream>>>(rh_index_remap, n_rh, n, w.in_remap);
  const unsigned gr = (unsigned)((n_rh + 127) / 128);
  pairs_rh_kernel<false><<<gr, 128, 0, stream>>>(lh_inclusion, lh_exclusion, n, rh_positions, rh_system,
                                                 rh_inclusion, rh_exclusion, n_rh, rh_index_remap, w.in_remap,
                                                 n_incl, s, l.sys, l.frac, l.cell_start, l.cell_items, w.rh_off, oob,
                                                 edges, shifts, cap);
  KUPS_CUDA_TRY(exclusive_scan<int64_t>(w.rh_off, n_rh, w.rh_scan, n_edges, stream));
  pairs_rh_kernel<true><<<gr, 128, 0, stream>>>(lh_inclusion, lh_exclusion, n, rh_positions, rh_system,
                                                rh_inclusion, rh_exclusion, n_rh, rh_index_remap, w.in_remap, n_incl,
                                                s, l.sys, l.frac, l.cell_start, l.cell_items, w.rh_off, oob, edges,
                                                shifts, cap);
  check_capacity_kernel<<<1, 1, 0, stream>>>(n_edges, cap, status);
  if (cap > 0) pad_kernel<<<(unsigned)((cap + 255) / 256), 256, 0, stream>>>(n_edges, cap, oob, edges, shifts);
  return cudaGetLastError() == cudaSuccess ? KUPS_OK : KUPS_ERR_CUDA;
}

extern "C" size_t kups_neighborlist_split_workspace_bytes(int64_t n_edges_total, int64_t n) {
  const int64_t m = n_edges_total + 1;
  return 2 * align_up(sizeof(int64_t) * (size_t)m) + 2 * align_up(sizeof(int64_t) * (size_t)scan_blocks_needed(m)) +
         align_up((size_t)std::max<int64_t>(n, 1)) + 256;
}

extern "C" int32_t kups_neighborlist_split_changes(const int32_t *edges, const int32_t *shifts,
                                                   const int64_t *n_edges, int64_t edge_rows, int64_t n,
                                                   const int32_t *p_idx, int64_t k, int32_t *added_edges,
                                                   int32_t *added_shifts, int64_t added_cap, int64_t *n_added,
                                                   int32_t *removed_edges, int32_t *removed_shifts,
                                                   int64_t removed_cap, int64_t *n_removed, void *workspace,
                                                   size_t ws_bytes, kups_status *status, void *stream_) {
  cudaStream_t stream = (cudaStream_t)stream_;
  if (edge_rows < 0 || n < 0 || k < 0 || added_cap < 0 || removed_cap < 0) return KUPS_ERR_INVALID;
  if (ws_bytes < kups_neighborlist_split_workspace_bytes(edge_rows, n)) return KUPS_ERR_INVALID;
  const int64_t m = edge_rows + 1;
  char *base = (char *)(((uintptr_t)workspace + 255) & ~uintptr_t(255));
  int64_t *add_off = (int64_t *)base;
  int64_t *rem_off = (int64_t *)(base + align_up(sizeof(int64_t) * (size_t)m));
  int64_t *scan_a = (int64_t *)(base + 2 * align_up(sizeof(int64_t) * (size_t)m));
  int64_t *scan_r = (int64_t *)((char *)scan_a + align_up(sizeof(int64_t) * (size_t)scan_blocks_needed(m)));
  uint8_t *changed = (uint8_t *)((char *)scan_r + align_up(sizeof(int64_t) * (size_t)scan_blocks_needed(m)));
  KUPS_CUDA_TRY(cudaMemsetAsync(changed, 0, (size_t)std::max<int64_t>(n, 1), stream));
  if (k > 0) mark_changed_kernel<<<(unsigned)((k + 255) / 256), 256, 0, stream>>>(p_idx, k, n, changed);
  const unsigned g = (unsigned)((m + 255) / 256);
  split_flags_kernel<<<g, 256, 0, stream>>>(edges, n_edges, n, k, changed, add_off, rem_off, m);
  KUPS_CUDA_TRY(exclusive_scan<int64_t>(add_off, m, scan_a, n_added, stream));
  KUPS_CUDA_TRY(exclusive_scan<int64_t>(rem_off, m, scan_r, n_removed, stream));
  split_write_kernel<<<g, 256, 0, stream>>>(edges, shifts, n_edges, n, p_idx, add_off, rem_off, edge_rows,
                                            added_edges, added_shifts, added_cap, removed_edges, removed_shifts,
                                            removed_cap);
  split_check_kernel<<<1, 1, 0, stream>>>(n_added, added_cap, n_removed, removed_cap, status);
  if (added_cap > 0)
    pad_from_kernel<<<(unsigned)((added_cap + 255) / 256), 256, 0, stream>>>(n_added, added_cap, n, added_edges,
                                                                            added_shifts);
  if (removed_cap > 0)
    pad_from_kernel<<<(unsigned)((removed_cap + 255) / 256), 256, 0, stream>>>(n_removed, removed_cap, n,
                                                                              removed_edges, removed_shifts);
  return cudaGetLastError() == cudaSuccess ? KUPS_OK : KUPS_ERR_CUDA;
}
