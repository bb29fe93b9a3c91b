// Fused Lennard-Jones molecular dynamics: a persistent kernel that runs many
// MD steps for thousands of independent periodic systems.
//
// Replaces, per step, the propagator assembled by make_md_propagator
// (src/kups/application/md/simulation.py:74-119): velocity Verlet
// (src/kups/md/integrators.py:273-318) or BAOAB Langevin (:405-455) with the
// Lennard-Jones potential (src/kups/potential/classical/lennard_jones.py:149-178)
// and a periodic neighbour list (src/kups/core/neighborlist.py:743-786) as
// derivative_computation.
//
// Design (GB300):
//  * one CTA owns one system at a time (work queue, largest systems first) and
//    keeps, for all of that system's steps, in shared memory: the atoms'
//    float4 positions followed by their periodic-image copies ("ghosts": every
//    image within cutoff + skin of the cell), momenta (+mass), forces
//    (+distance travelled since the last list build) and a cell grid over the
//    extended region;
//  * the Verlet list (cutoff + skin) holds uint16 indices into
//    [atoms | ghosts] and lives in this CTA's slice of the workspace, laid out
//    so that the `tpa` lanes serving one atom read consecutive words; it is
//    rebuilt in-kernel when any atom has travelled more than skin / 2;
//  * per pair: one shared-memory float4 load, three subtractions (image
//    shifts are baked into the ghost copies), the exact r^2 < rc^2 test of
//    lennard_jones_edge_energy, float32 arithmetic; per-system energies,
//    kinetic energies and virials are reduced in float64;
//  * positions are re-wrapped into fractional [-0.5, 0.5) at every list
//    build and on exit (the reference wraps every step with
//    MinimumImageConventionFlow, integrators.py:104-141; wrapping between
//    builds only changes the representation, never a distance).
#include <algorithm>

#include "common.cuh"

namespace kups {
namespace {

constexpr int kMaxAtoms = 2048;
constexpr int kMaxGhosts = 4096;
constexpr int kMaxItems = kMaxAtoms + kMaxGhosts;
constexpr int kMaxCells = 1024;
constexpr int kMaxSpecies = 8;
constexpr int kShiftSide = 5;  // image offsets in [-2, 2]^3
constexpr int kShiftCount = kShiftSide * kShiftSide * kShiftSide;
constexpr int kThreads = 1024;
constexpr int kScratchPerCta = 3 * kMaxAtoms > 2 * kMaxGhosts ? 3 * kMaxAtoms : 2 * kMaxGhosts;  // float4s

// Per-system record kept in the workspace between calls: with it a call resumes a
// system exactly where the previous call on the same workspace left it (same
// cell-sorted order, internal unwrapped positions, image copies, travelled
// distances and Verlet list) instead of rebuilding.  The record is trusted only
// if every field below equals this call's input bit for bit and every atom's
// internal position, wrapped as the write-back wraps it, equals the input.
struct SysRecord {
  int32_t valid, n, tpa, cap;
  int32_t n_ghosts, pad0;
  uint32_t rc, skin;
  uint32_t tril[6];
  uint32_t pad1[2];
};
static_assert(sizeof(SysRecord) == 64, "system record is 64 bytes");

// Pointers into the caller's workspace (layout of md_layout below).
struct MdWork {
  float4 *scratch;   // [ctas][kScratchPerCta] staging of the list builds
  SysRecord *rec;    // [S]
  float4 *apos;      // [N] internal positions in cell-sorted slot order
  uint32_t *ameta;   // [N] input index of the slot | neighbour count << 16
  float *atrav;      // [N] distance travelled since the last list build
  uint32_t *gmeta;   // [S][kMaxGhosts] image copies: source slot | shift code << 16
  uint2 *lists;      // [N * md_units_per_atom] Verlet lists, system s from sys_offset[s] * md_units_per_atom
};

inline size_t md_align(size_t x) { return (x + 255) & ~size_t(255); }

// 8-byte list units reserved per atom: capacity / 4 rounded up to a multiple of the
// largest lane count (16), so the unit index ((u / tpa) * n + i) * tpa + u % tpa of
// every u < capacity / 4 stays below n times this for any tpa <= 16.
__host__ __device__ inline size_t md_units_per_atom(int capacity) {
  return ((size_t)(capacity / 4) + 15) & ~size_t(15);
}

struct MdLayout {
  size_t scratch, rec, apos, ameta, atrav, gmeta, lists, total;
};

// Byte offsets from the 256-byte aligned workspace base (the queue word sits at 0).
inline MdLayout md_layout(int ctas, int64_t n_atoms, int n_systems, int capacity) {
  MdLayout l;
  size_t o = 256;
  l.scratch = o;
  o += md_align((size_t)ctas * kScratchPerCta * sizeof(float4));
  l.rec = o;
  o += md_align((size_t)n_systems * sizeof(SysRecord));
  l.apos = o;
  o += md_align((size_t)n_atoms * sizeof(float4));
  l.ameta = o;
  o += md_align((size_t)n_atoms * sizeof(uint32_t));
  l.atrav = o;
  o += md_align((size_t)n_atoms * sizeof(float));
  l.gmeta = o;
  o += md_align((size_t)n_systems * kMaxGhosts * sizeof(uint32_t));
  l.lists = o;
  o += md_align((size_t)n_atoms * md_units_per_atom(capacity) * sizeof(uint2));
  l.total = o;
  return l;
}

struct SysParams {
  float L[6];     // L00 L10 L11 L20 L21 L22
  float inv[6];
  float rc2, rl2, half_skin;
  float m[3];     // margins in fractional units
  int K[3];       // image layers per side
  int nc[3];
  float ext[3];   // 1 + 2 m
  float coff[3];  // 0.5 + m
  float cscale[3];  // cells per fractional unit
  float dt, c1, c2;
  float rc, rl;
  double Ld[6];   // the cell in float64 (the barostat scales it)
  double Lid[9];  // its inverse, row-major 3 x 3, formed by set_inverse64 when Ld changes
  // CSVR (integrators 2, 3) and stochastic cell rescaling (integrator 3), set
  // up in float64 once per system and used in float32 per step
  float csvr_c1, csvr_omc1;  // exp(-dt / tau_T), 1 - exp(-dt / tau_T)
  float kTf;
  float scr_a, scr_b, p0f;   // dt / tau_P beta, 2 kT beta dt / tau_P, P0
  double mumin, mumax;
  int dof;
};

struct Smem {
  SysParams p;
  float4 pos[kMaxItems];
  float4 mom[kMaxAtoms];
  float4 frc[kMaxAtoms];
  uint32_t ghost_meta[kMaxGhosts];  // source atom | shift code << 16
  uint16_t bin_a[kMaxItems];  // scratch of the counting sorts (cell, then new slot, of an item)
  uint16_t bin_b[kMaxItems];  // scratch of the counting sorts (items grouped by cell)
  int cell_start[kMaxCells + 1];   // atoms of cell c: [cell_start[c], cell_start[c + 1])
  int ghost_start[kMaxCells + 1];  // ghosts of cell c: n + [ghost_start[c], ghost_start[c + 1])
  int cell_fill[kMaxCells];
  uint16_t gid[kMaxAtoms];  // index of each (cell-sorted) atom inside its system's input order
  uint16_t nbr_count[kMaxAtoms];
  float4 shift_vec[kShiftCount];
  float2 lj[kMaxSpecies * kMaxSpecies];  // (sigma^2, 4 eps)
  double red[72];
  int iscan[40];
  int n_ghosts;
  int flag;
  int next_sys;
  int work;
  float alpha;  // CSVR momentum scale of the coming step
  float mu;     // barostat scale of this step
  float red_f[12 * 32];  // per-warp partials of block_sums
  double red_d[12];
};


// Explicit fused multiply-adds: every inlined copy rounds the same way (the compiler would
// otherwise contract each copy as its context suggests), so wraps, cell indices and the virial
// sums agree bit for bit wherever they are formed.
__device__ inline void frac_of(const SysParams &p, float x, float y, float z, float f[3]) {
  f[0] = __fmaf_rn(z, p.inv[3], __fmaf_rn(y, p.inv[1], __fmul_rn(x, p.inv[0])));
  f[1] = __fmaf_rn(z, p.inv[4], __fmul_rn(y, p.inv[2]));
  f[2] = __fmul_rn(z, p.inv[5]);
}

__device__ inline void cart_of(const SysParams &p, const float f[3], float &x, float &y, float &z) {
  x = __fmaf_rn(f[2], p.L[3], __fmaf_rn(f[1], p.L[1], __fmul_rn(f[0], p.L[0])));
  y = __fmaf_rn(f[2], p.L[4], __fmul_rn(f[1], p.L[2]));
  z = __fmul_rn(f[2], p.L[5]);
}

// Wrap into fractional [-0.5, 0.5) by subtracting whole lattice vectors; an
// atom already inside the cell is left bit-for-bit unchanged.
__device__ inline void wrap_position(const SysParams &p, float4 &q, float f[3]) {
  frac_of(p, q.x, q.y, q.z, f);
  const float n0 = floorf(f[0] + 0.5f), n1 = floorf(f[1] + 0.5f), n2 = floorf(f[2] + 0.5f);
  if (n0 != 0.f || n1 != 0.f || n2 != 0.f) {
    const float nn[3] = {n0, n1, n2};
    float sx, sy, sz;
    cart_of(p, nn, sx, sy, sz);
    q.x -= sx;
    q.y -= sy;
    q.z -= sz;
    f[0] -= n0;
    f[1] -= n1;
    f[2] -= n2;
  }
}

__device__ inline int shift_code(int ox, int oy, int oz) {
  return ((ox + 2) * kShiftSide + (oy + 2)) * kShiftSide + (oz + 2);
}

__device__ inline int cell_coord(float pf, float off, float scale, int nc) {
  int c = (int)floorf((pf + off) * scale);
  return c < 0 ? 0 : (c >= nc ? nc - 1 : c);
}

__device__ inline int cell_of_point(const SysParams &p, float x, float y, float z, int &cx, int &cy,
                                    int &cz) {
  float f[3];
  frac_of(p, x, y, z, f);
  cx = cell_coord(f[0], p.coff[0], p.cscale[0], p.nc[0]);
  cy = cell_coord(f[1], p.coff[1], p.cscale[1], p.nc[1]);
  cz = cell_coord(f[2], p.coff[2], p.cscale[2], p.nc[2]);
  return (cz * p.nc[1] + cy) * p.nc[0] + cx;
}

// Cell-dependent parameters from p.L and p.rl (one thread): inverse, image
// margins m = rl / width per axis, image layers K = ceil(m) and the cell grid
// over the extended region [-0.5 - m, 0.5 + m).
__device__ void set_cell(SysParams &p) {
  const float A = p.L[0], B = p.L[1], C = p.L[2], D = p.L[3], E = p.L[4], F = p.L[5];
  p.inv[0] = 1.0f / A;
  p.inv[2] = 1.0f / C;
  p.inv[5] = 1.0f / F;
  p.inv[1] = -(B * p.inv[0]) / C;
  p.inv[4] = -(E * p.inv[2]) / F;
  p.inv[3] = -((D * p.inv[0]) + (E * p.inv[1])) / F;
  const float rl = p.rl;
  const float vol = fabsf(A * C * F);
  const float c0 = C * F, c1 = B * F, c2 = B * E - C * D;
  const float w[3] = {vol / sqrtf(c0 * c0 + c1 * c1 + c2 * c2),
                      vol / sqrtf((A * F) * (A * F) + (A * E) * (A * E)), vol / fabsf(A * C)};
  int ncell = 1;
  for (int d = 0; d < 3; ++d) {
    p.m[d] = rl / w[d];
    p.K[d] = (int)ceilf(p.m[d]);
    p.ext[d] = 1.0f + 2.0f * p.m[d];
    p.nc[d] = max(1, (int)floorf(p.ext[d] * w[d] / rl));
    ncell *= p.nc[d];
  }
  while (ncell > kMaxCells) {
    int am = 0;
    for (int d = 1; d < 3; ++d)
      if (p.nc[d] > p.nc[am]) am = d;
    p.nc[am] = (p.nc[am] + 1) / 2;
    ncell = p.nc[0] * p.nc[1] * p.nc[2];
  }
  for (int d = 0; d < 3; ++d) {
    p.coff[d] = 0.5f + p.m[d];
    p.cscale[d] = (float)p.nc[d] / p.ext[d];
  }
}

__device__ inline void set_shift_vectors(Smem &sm) {
  for (int c = threadIdx.x; c < kShiftCount; c += blockDim.x) {
    const int ox = c / 25 - 2, oy = (c / 5) % 5 - 2, oz = c % 5 - 2;
    const float f[3] = {(float)ox, (float)oy, (float)oz};
    float x, y, z;
    cart_of(sm.p, f, x, y, z);
    sm.shift_vec[c] = make_float4(x, y, z, 0.f);
  }
}

// Lanes serving one atom: the smallest power of two (<= 16) that still gives
// every thread of the block an atom-lane to work on.
__device__ inline int choose_tpa(int n, int threads, int min_lanes) {
  int t = min_lanes;
  while (t < 16 && n * t < threads) t <<= 1;
  return t;
}

__device__ __forceinline__ void prof_add(unsigned long long *prof, int k, long long &t0) {
  if (prof != nullptr && threadIdx.x == 0) {
    const long long t = clock64();
    atomicAdd(&prof[k], (unsigned long long)(t - t0));
    t0 = t;
  }
}

// Counting sort of `count` items by cell into cell-contiguous order: on entry
// sm.bin_a[k] holds the cell of item k; on exit sm.bin_a[k] holds the item's
// new slot and `start` the exclusive prefix of the per-cell counts.  The order
// inside a cell follows the item index, so the result is deterministic.
__device__ void sort_by_cell(Smem &sm, int count, int ncell, int *start) {
  const int tid = threadIdx.x, nt = blockDim.x;
  for (int c = tid; c <= ncell; c += nt) start[c] = 0;
  __syncthreads();
  for (int k = tid; k < count; k += nt) atomicAdd(&start[sm.bin_a[k]], 1);
  __syncthreads();
  int carry = 0;
  for (int b0 = 0; b0 < ncell; b0 += nt) {
    const int c = b0 + tid;
    const int v = c < ncell ? start[c] : 0;
    int tot;
    const int ex = block_exclusive_scan<int>(v, sm.iscan, &tot);
    __syncthreads();
    if (c < ncell) {
      start[c] = carry + ex;
      sm.cell_fill[c] = carry + ex;
    }
    carry += tot;
  }
  if (tid == 0) start[ncell] = carry;
  __syncthreads();
  for (int k = tid; k < count; k += nt) {
    const int slot = atomicAdd(&sm.cell_fill[sm.bin_a[k]], 1);
    sm.bin_b[slot] = (uint16_t)k;
  }
  __syncthreads();
  for (int k = tid; k < count; k += nt) {
    int lo = 0, hi = ncell - 1;  // cell with start[c] <= k < start[c + 1]
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (start[mid] <= k) lo = mid; else hi = mid - 1;
    }
    const int b = start[lo], e = start[lo + 1];
    const uint16_t v = sm.bin_b[k];
    int r = 0;
    for (int m = b; m < e; ++m) r += sm.bin_b[m] < v;
    sm.bin_a[v] = (uint16_t)(b + r);
  }
  __syncthreads();
}

// Wrap and cell-sort the atoms, build the cell-sorted ghost copies and the
// Verlet list.  Returns false (and records the requirement) if a capacity is
// exceeded.  `scratch` is this CTA's slice of global workspace (permutation
// staging, 48 bytes per atom).
// Verlet-list layout: 8-byte units of four uint16 item indices; unit u of atom i
// sits at ((u / tpa) * n + i) * tpa + u % tpa, so the tpa lanes serving atom i, and
// the atoms of a warp, read consecutive units.  Entry e of atom i is slot (e / tpa) % 4
// of unit (e / (4 tpa)) * tpa + e % tpa: at each slot the atom's lanes hold consecutive
// entries.  The last row of 4 tpa entries is padded with the far-away sentinel item.
__device__ __noinline__ bool rebuild(Smem &sm, const SysParams &p, int n, int tpa, uint2 *nl,
                                     int nb_cap, kups_status *status, int sys_index,
                                     unsigned long long *prof, float4 *scratch) {
  const int tid = threadIdx.x, nt = blockDim.x;
  long long tp = clock64();
  const int ncell = p.nc[0] * p.nc[1] * p.nc[2];
  // 1. wrap atoms into [-0.5, 0.5), reset travelled distance, sort atoms by cell
  for (int i = tid; i < n; i += nt) {
    float4 q = sm.pos[i];
    float f[3];
    wrap_position(p, q, f);
    sm.pos[i] = q;
    sm.frc[i].w = 0.0f;
    int cx, cy, cz;
    sm.bin_a[i] = (uint16_t)cell_of_point(p, q.x, q.y, q.z, cx, cy, cz);
  }
  __syncthreads();
  sort_by_cell(sm, n, ncell, sm.cell_start);
  for (int i = tid; i < n; i += nt) {
    const int d = sm.bin_a[i];
    float4 m = sm.mom[i];
    scratch[3 * d] = sm.pos[i];
    scratch[3 * d + 1] = m;
    scratch[3 * d + 2] = make_float4(sm.frc[i].x, sm.frc[i].y, sm.frc[i].z, __int_as_float((int)sm.gid[i]));
  }
  __syncthreads();
  for (int i = tid; i < n; i += nt) {
    sm.pos[i] = scratch[3 * i];
    sm.mom[i] = scratch[3 * i + 1];
    const float4 f = scratch[3 * i + 2];
    sm.frc[i] = make_float4(f.x, f.y, f.z, 0.0f);
    sm.gid[i] = (uint16_t)__float_as_int(f.w);
  }
  __syncthreads();
  prof_add(prof, 6, tp);
  // 2. ghosts: count, write in atom-major order, then sort by cell
  int my_total = 0;
  for (int i = tid; i < n; i += nt) {
    const float4 q = sm.pos[i];
    float f[3];
    frac_of(p, q.x, q.y, q.z, f);
    int c = 0;
    for (int ox = -p.K[0]; ox <= p.K[0]; ++ox)
      for (int oy = -p.K[1]; oy <= p.K[1]; ++oy)
        for (int oz = -p.K[2]; oz <= p.K[2]; ++oz) {
          if (ox == 0 && oy == 0 && oz == 0) continue;
          const float g0 = f[0] + ox, g1 = f[1] + oy, g2 = f[2] + oz;
          c += (g0 >= -0.5f - p.m[0]) & (g0 < 0.5f + p.m[0]) & (g1 >= -0.5f - p.m[1]) &
               (g1 < 0.5f + p.m[1]) & (g2 >= -0.5f - p.m[2]) & (g2 < 0.5f + p.m[2]);
        }
    my_total += c;
  }
  int total;
  int base = block_exclusive_scan<int>(my_total, sm.iscan, &total);
  __syncthreads();
  if (total > kMaxGhosts - 1) {  // one slot stays free for the sentinel item
    if (tid == 0) status_capacity(status, KUPS_CAP_GHOSTS, total + 1, sys_index);
    return false;
  }
  for (int i = tid; i < n; i += nt) {
    const float4 q = sm.pos[i];
    float f[3];
    frac_of(p, q.x, q.y, q.z, f);
    for (int ox = -p.K[0]; ox <= p.K[0]; ++ox)
      for (int oy = -p.K[1]; oy <= p.K[1]; ++oy)
        for (int oz = -p.K[2]; oz <= p.K[2]; ++oz) {
          if (ox == 0 && oy == 0 && oz == 0) continue;
          const float g0 = f[0] + ox, g1 = f[1] + oy, g2 = f[2] + oz;
          if ((g0 >= -0.5f - p.m[0]) & (g0 < 0.5f + p.m[0]) & (g1 >= -0.5f - p.m[1]) &
              (g1 < 0.5f + p.m[1]) & (g2 >= -0.5f - p.m[2]) & (g2 < 0.5f + p.m[2])) {
            const int code = shift_code(ox, oy, oz);
            const float4 sv = sm.shift_vec[code];
            const float4 gq = make_float4(q.x + sv.x, q.y + sv.y, q.z + sv.z, q.w);
            int cx, cy, cz;
            sm.bin_a[base] = (uint16_t)cell_of_point(p, gq.x, gq.y, gq.z, cx, cy, cz);
            scratch[2 * base] = gq;
            scratch[2 * base + 1] = make_float4(__int_as_float((int)((uint32_t)i | ((uint32_t)code << 16))), 0.f, 0.f, 0.f);
            ++base;
          }
        }
  }
  __syncthreads();
  sort_by_cell(sm, total, ncell, sm.ghost_start);
  for (int g = tid; g < total; g += nt) {
    const int d = sm.bin_a[g];
    sm.pos[n + d] = scratch[2 * g];
    sm.ghost_meta[d] = (uint32_t)__float_as_int(scratch[2 * g + 1].x);
  }
  const int n_items = n + total;
  if (tid == 0) {
    sm.pos[n_items] = make_float4(1e15f, 1e15f, 1e15f, __int_as_float(0));  // sentinel item
    sm.flag = 0;
    sm.work = 0;
  }
  __syncthreads();
  prof_add(prof, 7, tp);
  // 3. Verlet list.  Work unit: a chunk of up to 32 consecutive (cell-sorted)
  //    atoms of one x-row of cells, one lane per atom (a system's atoms fill
  //    only the central rows of the extended grid, so whole rows as units left
  //    warps idle); sm.bin_b[r] holds the exclusive prefix of the rows' chunk
  //    counts.  The candidates of a chunk are the contiguous atom and ghost
  //    ranges of the 3 x 3 neighbour rows over the x-range of the chunk's cells
  //    plus one cell either side, read once per warp (shared-memory broadcast).
  //    Hits of 32 candidates are gathered in a per-lane bit mask, then appended
  //    in candidate order (deterministic), four per 8-byte store.
  const int lane = threadIdx.x & 31;
  const int ltpa = __ffs(tpa) - 1;
  const uint32_t sent = (uint32_t)n_items;
  const int n_rows = p.nc[1] * p.nc[2];
  uint16_t *rowp = sm.bin_b;
  {
    int carry = 0;
    for (int r0 = 0; r0 < n_rows; r0 += nt) {
      const int r = r0 + tid;
      const int v = r < n_rows ? (sm.cell_start[(r + 1) * p.nc[0]] - sm.cell_start[r * p.nc[0]] + 31) >> 5 : 0;
      int tot;
      const int ex = block_exclusive_scan<int>(v, sm.iscan, &tot);
      __syncthreads();
      if (r < n_rows) rowp[r] = (uint16_t)(carry + ex);
      carry += tot;
    }
    if (tid == 0) rowp[n_rows] = (uint16_t)carry;
    __syncthreads();
  }
  const int n_chunks = rowp[n_rows];
  int my_max = 0;
  while (true) {
    int unit = 0;
    if (lane == 0) unit = atomicAdd(&sm.work, 1);
    unit = __shfl_sync(0xffffffffu, unit, 0);
    if (unit >= n_chunks) break;
    int row = 0, hi = n_rows - 1;  // the last row with rowp[row] <= unit (empty rows share it)
    while (row < hi) {
      const int mid = (row + hi + 1) >> 1;
      if (rowp[mid] <= unit) row = mid; else hi = mid - 1;
    }
    const int cy = row % p.nc[1], cz = row / p.nc[1];
    const int rowc = row * p.nc[0];
    const int ab = sm.cell_start[rowc], ae = sm.cell_start[rowc + p.nc[0]];
    const int z0 = max(cz - 1, 0), z1 = min(cz + 1, p.nc[2] - 1);
    const int y0 = max(cy - 1, 0), y1 = min(cy + 1, p.nc[1] - 1);
    const float rl2 = p.rl2;
    {
      const int a0 = ab + (unit - rowp[row]) * 32;
      // x-range of the chunk's cells (cells of a row are consecutive)
      const int last = min(a0 + 32, ae) - 1;
      int cfirst = 0, clast = 0;
      for (int c = 0; c < p.nc[0]; ++c) {
        if (sm.cell_start[rowc + c] <= a0) cfirst = c;
        if (sm.cell_start[rowc + c] <= last) clast = c;
      }
      const int x0 = max(cfirst - 1, 0), x1 = min(clast + 1, p.nc[0] - 1);
      const bool mine = a0 + lane < ae;
      const int i = mine ? a0 + lane : ab;
      const float4 q = sm.pos[i];
      int cnt = 0;
      // entry e of atom i: row t = e / (4 tpa) of its list, lane g = e % tpa, slot k of
      // the lane's 4-entry unit = (e / tpa) % 4, so at each slot the atom's tpa lanes read
      // tpa consecutive entries (consecutive candidates in cell order: mostly distinct banks)
      uint16_t *nl16 = reinterpret_cast<uint16_t *>(nl);
      auto put = [&](int e, uint32_t j) {
        const int t = e >> (ltpa + 2), g = e & (tpa - 1), k = (e >> ltpa) & 3;
        nl16[((((size_t)t * n + i) << ltpa) + g) * 4 + k] = (uint16_t)j;
      };
      auto push = [&](uint32_t j) {
        if (cnt < nb_cap) put(cnt, j);
        ++cnt;
      };
      auto scan_range = [&](int kb, int ke) {
        for (int k0 = kb; k0 < ke; k0 += 32) {
          const int kn = min(32, ke - k0);
          uint32_t hits = 0;
#pragma unroll 4
          for (int t = 0; t < kn; ++t) {
            const float4 o = sm.pos[k0 + t];
            const float dx = o.x - q.x, dy = o.y - q.y, dz = o.z - q.z;
            const bool h = fmaf(dz, dz, fmaf(dy, dy, dx * dx)) < rl2;
            hits |= (uint32_t)h << t;
          }
          if (k0 <= i && i < k0 + kn) hits &= ~(1u << (i - k0));  // not the atom itself
          if (!mine) hits = 0;
          while (hits) {
            const int t = __ffs(hits) - 1;
            hits &= hits - 1;
            push((uint32_t)(k0 + t));
          }
        }
      };
      for (int z = z0; z <= z1; ++z)
        for (int y = y0; y <= y1; ++y) {
          const int row = (z * p.nc[1] + y) * p.nc[0];
          scan_range(sm.cell_start[row + x0], sm.cell_start[row + x1 + 1]);
          scan_range(n + sm.ghost_start[row + x0], n + sm.ghost_start[row + x1 + 1]);
        }
      if (mine) {
        const int total_cnt = cnt;
        // pad the last row with the sentinel item (whole rows of at most nb_cap entries stay
        // below n * md_units_per_atom units, which rounds nb_cap / 4 up to 16 units)
        if (cnt <= nb_cap)
          for (; cnt & (4 * tpa - 1); ++cnt) put(cnt, sent);
        sm.nbr_count[i] = (uint16_t)min(total_cnt, nb_cap);
        my_max = max(my_max, total_cnt);
      }
    }
  }
  if (my_max > nb_cap) atomicMax(&sm.flag, my_max);
  __syncthreads();
  prof_add(prof, 9, tp);
  const int need = sm.flag;
  if (need > nb_cap) {
    if (tid == 0) status_capacity(status, KUPS_CAP_NEIGHBORS, need, sys_index);
    return false;
  }
  if (tid == 0) sm.n_ghosts = total;
  __syncthreads();
  return true;
}

__device__ __forceinline__ void update_ghosts(Smem &sm, int n) {
  const int ng = sm.n_ghosts;
  for (int g = threadIdx.x; g < ng; g += blockDim.x) {
    const uint32_t m = sm.ghost_meta[g];
    const float4 q = sm.pos[m & 0xffffu];
    const float4 sv = sm.shift_vec[m >> 16];
    sm.pos[n + g] = make_float4(q.x + sv.x, q.y + sv.y, q.z + sv.z, q.w);
  }
}

__device__ __forceinline__ float rcp_approx(float x) {
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

// Per-atom pair energies of the last force evaluation with ENERGY, kept in the counting-sort
// scratch: no phase between a force evaluation and the sum of its energies sorts anything.
__device__ inline float *atom_energy(Smem &sm) { return reinterpret_cast<float *>(sm.bin_a); }

// 1.0f where a < b, else 0.0f, in one instruction.
__device__ __forceinline__ float lt_mask(float a, float b) {
  float m;
  asm("set.lt.f32.f32 %0, %1, %2;" : "=f"(m) : "f"(a), "f"(b));
  return m;
}

// Accumulators of one lane for one atom: forces and energy as pairs (the two list entries a
// lane evaluates together, added at the end), the virial scalar.
struct PairAcc {
  float2 fx, fy, fz, e;
  float w[6];
};

// Pair constants of one species pair, each held twice for the packed float32x2 arithmetic:
// sigma^2, -12 (4 eps), 6 (4 eps) and 4 eps.
struct PairConst {
  float2 s2, a12n, a6, a;
};

// Two neighbours j0, j1 of atom i at once with packed float32x2 operations (each lane of a
// packed operation rounds exactly as the scalar operation).  Per pair: d = x_j - x_i,
// r2 = |d|^2, c6 = (sigma^2 / r2)^3, and with nfs = c6 (6 a - 12 a c6) / r2 (a = 4 eps):
// F_i += nfs d, e_i += a (c6^2 - c6) (half of it is the atom's share), W += -(1/2) fs d d.
// Pairs at r2 >= rc2 contribute exactly zero (their 1 / r2 is masked to zero).
template <bool ENERGY, bool VIRIAL, bool SINGLE>
__device__ __forceinline__ void lj_pair2(const Smem &sm, const float4 &xi, int ti, int nsp, uint32_t j0,
                                         uint32_t j1, float rc2, const PairConst &pc, PairAcc &acc) {
  const float4 p0 = sm.pos[j0], p1 = sm.pos[j1];
  const float2 dx = make_float2(p0.x - xi.x, p1.x - xi.x);
  const float2 dy = make_float2(p0.y - xi.y, p1.y - xi.y);
  const float2 dz = make_float2(p0.z - xi.z, p1.z - xi.z);
  const float2 r2 = __ffma2_rn(dz, dz, __ffma2_rn(dy, dy, __fmul2_rn(dx, dx)));
  PairConst c = pc;
  if (!SINGLE) {
    const float2 c0 = sm.lj[ti * nsp + __float_as_int(p0.w)];
    const float2 c1 = sm.lj[ti * nsp + __float_as_int(p1.w)];
    c.s2 = make_float2(c0.x, c1.x);
    c.a12n = make_float2(-12.0f * c0.y, -12.0f * c1.y);
    c.a6 = make_float2(6.0f * c0.y, 6.0f * c1.y);
    c.a = make_float2(c0.y, c1.y);
  }
  const float2 inv = __fmul2_rn(make_float2(rcp_approx(r2.x), rcp_approx(r2.y)),
                                make_float2(lt_mask(r2.x, rc2), lt_mask(r2.y, rc2)));
  const float2 s2 = __fmul2_rn(c.s2, inv);
  const float2 c6 = __fmul2_rn(__fmul2_rn(s2, s2), s2);
  const float2 nfs = __fmul2_rn(__fmul2_rn(c6, __ffma2_rn(c.a12n, c6, c.a6)), inv);
  acc.fx = __ffma2_rn(nfs, dx, acc.fx);
  acc.fy = __ffma2_rn(nfs, dy, acc.fy);
  acc.fz = __ffma2_rn(nfs, dz, acc.fz);
  if (ENERGY) acc.e = __fadd2_rn(acc.e, __fmul2_rn(c.a, __ffma2_rn(c6, c6, make_float2(-c6.x, -c6.y))));
  if (VIRIAL) {
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      const float h = 0.5f * (q ? nfs.y : nfs.x);  // (1/2) d_c g_b = -(1/2) fs d_c d_b
      const float ex = q ? dx.y : dx.x, ey = q ? dy.y : dy.x, ez = q ? dz.y : dz.x;
      acc.w[0] = fmaf(h * ex, ex, acc.w[0]);
      acc.w[1] = fmaf(h * ey, ex, acc.w[1]);
      acc.w[2] = fmaf(h * ey, ey, acc.w[2]);
      acc.w[3] = fmaf(h * ez, ex, acc.w[3]);
      acc.w[4] = fmaf(h * ez, ey, acc.w[4]);
      acc.w[5] = fmaf(h * ez, ez, acc.w[5]);
    }
  }
}

// Forces into sm.frc[i].xyz.  With ENERGY, each atom's potential energy (sum over its
// pairs / 2) into atom_energy(sm)[i]; with VIRIAL, adds the
// Cartesian pair virial W_cb = 1/2 sum d_c g_b ([xx, yx, yy, zx, zy, zz]) to wv.
// Warps take 32 / tpa atoms at a time from a shared counter (sm.work, zeroed
// by the caller before the preceding barrier), so uneven neighbour counts do
// not leave warps idle at the barrier; with VIRIAL, warp w takes groups w, w + warps, ... in
// order instead, so that each thread's virial partial sums (and hence the block's sum) are the
// same on every run.  Each lane loads a 4-entry list unit (8 bytes) per iteration, fetched
// one iteration ahead, and evaluates its entries two at a time.
template <bool ENERGY, bool VIRIAL, bool SINGLE>
__device__ __forceinline__ void compute_forces(Smem &sm, int n, int nsp, int tpa, const uint2 *nl,
                                               float rc2, float sig2, float a4, float wv[6]) {
  const int lane = threadIdx.x & 31;
  const int lane_g = lane & (tpa - 1);
  const int per_warp = 32 / tpa;
  const size_t stride = (size_t)n * tpa;
  PairConst pc;
  pc.s2 = make_float2(sig2, sig2);
  pc.a12n = make_float2(-12.0f * a4, -12.0f * a4);
  pc.a6 = make_float2(6.0f * a4, 6.0f * a4);
  pc.a = make_float2(a4, a4);
  const int n_warps = blockDim.x >> 5;
  int next = threadIdx.x >> 5;  // static schedule (VIRIAL)
  while (true) {
    int wb = 0;
    if (VIRIAL) {
      wb = next * per_warp;
      next += n_warps;
    } else {
      if (lane == 0) wb = atomicAdd(&sm.work, per_warp);
      wb = __shfl_sync(0xffffffffu, wb, 0);
    }
    if (wb >= n) break;
    const int i = wb + lane / tpa;
    const bool active = i < n;
    PairAcc acc;
    acc.fx = acc.fy = acc.fz = acc.e = make_float2(0.f, 0.f);
#pragma unroll
    for (int k = 0; k < 6; ++k) acc.w[k] = 0.f;
    if (active) {
      const float4 xi = sm.pos[i];
      const int ti = __float_as_int(xi.w);
      const int nu = ((sm.nbr_count[i] + 4 * tpa - 1) >> (2 + __ffs(tpa) - 1)) * tpa;  // whole rows of units
      const uint2 *row = nl + (size_t)i * tpa + lane_g;
      int u = lane_g;
      uint2 v0 = make_uint2(0u, 0u), v1 = make_uint2(0u, 0u);
      if (u < nu) v0 = row[0];
      if (u + tpa < nu) v1 = row[stride];
      while (u < nu) {
        const uint2 cur = v0;
        v0 = v1;
        row += stride;
        u += tpa;
        if (u + tpa < nu) v1 = row[stride];
        lj_pair2<ENERGY, VIRIAL, SINGLE>(sm, xi, ti, nsp, cur.x & 0xffffu, cur.x >> 16, rc2, pc, acc);
        lj_pair2<ENERGY, VIRIAL, SINGLE>(sm, xi, ti, nsp, cur.y & 0xffffu, cur.y >> 16, rc2, pc, acc);
      }
    }
    float fx = acc.fx.x + acc.fx.y, fy = acc.fy.x + acc.fy.y, fz = acc.fz.x + acc.fz.y;
    for (int o = tpa >> 1; o > 0; o >>= 1) {
      fx += __shfl_xor_sync(0xffffffffu, fx, o);
      fy += __shfl_xor_sync(0xffffffffu, fy, o);
      fz += __shfl_xor_sync(0xffffffffu, fz, o);
    }
    if (active && lane_g == 0) {
      float4 f = sm.frc[i];
      f.x = fx;
      f.y = fy;
      f.z = fz;
      sm.frc[i] = f;
    }
    if (ENERGY) {  // the atom's pair energy / 2, lanes summed in a fixed order
      float e = acc.e.x + acc.e.y;
      for (int o = tpa >> 1; o > 0; o >>= 1) e += __shfl_xor_sync(0xffffffffu, e, o);
      if (active && lane_g == 0) atom_energy(sm)[i] = 0.5f * e;
    }
    if (VIRIAL) {
#pragma unroll
      for (int k = 0; k < 6; ++k) wv[k] += acc.w[k];
    }
  }
}

template <bool ENERGY, bool VIRIAL>
__device__ __forceinline__ void forces_dispatch(Smem &sm, int n, int nsp, int tpa, const uint2 *nl,
                                                float rc2, float sig2, float a4, float wv[6]) {
  if (nsp == 1)
    compute_forces<ENERGY, VIRIAL, true>(sm, n, nsp, tpa, nl, rc2, sig2, a4, wv);
  else
    compute_forces<ENERGY, VIRIAL, false>(sm, n, nsp, tpa, nl, rc2, sig2, a4, wv);
}

static_assert(sizeof(Smem) <= 227 * 1024, "fused MD shared memory above the per-CTA limit");
static_assert(sizeof(Smem::bin_a) >= kMaxAtoms * sizeof(float), "per-atom energies fit the sort scratch");

// Key offsets that separate the system-level draws (CSVR R1, the barostat's R)
// and the chi-squared normals from the per-atom Langevin noise.
constexpr uint64_t kSysSeed = 0x6a09e667f3bcc909ull;
constexpr uint64_t kChiSeed = 0xbb67ae8584caa73bull;

// Block-wide sums of N floats, returned to every thread in float64: each warp
// adds in float, then warp k adds the warp partials of value k in float64 (FP64
// issue is scarce on this part, so only 32 x N double additions are made, the N
// sums side by side).  Contains two __syncthreads().
template <int N>
__device__ inline void block_sums(const float (&v)[N], Smem &sm, double (&out)[N]) {
  static_assert(N <= 12, "block_sums scratch holds 12 values");
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int nw = (blockDim.x + 31) >> 5;
#pragma unroll
  for (int k = 0; k < N; ++k) {
    float x = v[k];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    if (lane == 0) sm.red_f[k * 32 + wid] = x;
  }
  __syncthreads();
  // warp k adds the warp partials of value k in float64 (the N sums run side by side)
  for (int k = wid; k < N; k += nw) {
    const double x = warp_sum(lane < nw ? (double)sm.red_f[k * 32 + lane] : 0.0);
    if (lane == 0) sm.red_d[k] = x;
  }
  __syncthreads();
#pragma unroll
  for (int k = 0; k < N; ++k) out[k] = sm.red_d[k];
}

// Sum of the per-atom energies of the last ENERGY force evaluation (thread k takes atoms
// k, k + blockDim.x, ...: a fixed order, so the result does not depend on which warp took
// which atom in the force phase), returned to every thread.
__device__ inline double atom_energy_sum(Smem &sm, int n) {
  float e = 0.f;
  for (int i = threadIdx.x; i < n; i += blockDim.x) e += atom_energy(sm)[i];
  const float v[1] = {e};
  double r[1];
  block_sums<1>(v, sm, r);
  return r[0];
}

// One standard normal (Box-Muller on two words) and one uniform in (0, 1] from
// one Philox block.
__device__ inline void normal_uniform(uint64_t seed, uint64_t stream, uint64_t counter, float &z, float &u) {
  U4 c{(uint32_t)counter, (uint32_t)(counter >> 32), (uint32_t)stream, (uint32_t)(stream >> 32)};
  const U4 r = philox4x32_10(c, (uint32_t)seed, (uint32_t)(seed >> 32));
  z = sqrtf(-2.0f * logf(u01_open0(r.x))) * cospif(2.0f * u01_open0(r.y));
  u = u01_open0(r.z);
}

// Gamma(a, 1) for a >= 1 by Marsaglia and Tsang's squeeze-and-reject method
// ("A simple method for generating gamma variables", ACM TOMS 26, 2000):
// d = a - 1/3, c = 1 / sqrt(9 d); for x ~ N(0, 1), y = c x > -1, v = (1 + y)^3
// and u ~ U(0, 1), accept d v when u < 1 - 0.0331 x^4 or
// ln u < x^2 / 2 + d (1 - v + ln v).  With d c^2 = 1/9 the right-hand side is
// 3 d (ln(1 + y) - y + y^2 / 2 - y^3 / 3) = 3 d sum_{k >= 4} (-1)^(k+1) y^k / k,
// summed as a series for |y| <= 1/4 (no cancellation in float32) and directly
// above.  Each trial takes its own Philox block (stream | trial); acceptance is
// above 95 % per trial, and after 64 rejected trials (probability below 1e-80)
// the mean a is returned.  One thread, float32 (FP64 is scarce on this part).
__device__ float gamma_mt(float a, uint64_t seed, uint64_t stream, uint64_t counter) {
  const float d = a - (1.0f / 3.0f), c = rsqrtf(9.0f * d);
  for (int t = 0; t < 64; ++t) {
    float x, u;
    normal_uniform(seed, (stream << 6) | (uint64_t)t, counter, x, u);
    const float y = c * x;
    if (y <= -1.0f) continue;
    const float v = (1.0f + y) * (1.0f + y) * (1.0f + y);
    const float x2 = x * x;
    if (u < 1.0f - 0.0331f * x2 * x2) return d * v;
    float h;
    if (fabsf(y) <= 0.25f) {
      // sum_{k=4}^{19} (-1)^(k+1) y^k / k, Horner in y from the top term
      float acc = 0.0f;
#pragma unroll
      for (int k = 19; k >= 4; --k) acc = fmaf(acc, y, ((k & 1) ? 1.0f : -1.0f) / (float)k);
      const float y2 = y * y;
      h = acc * (y2 * y2);
    } else {
      h = log1pf(y) - y + 0.5f * y * y - y * y * y * (1.0f / 3.0f);
    }
    if (logf(u) < 3.0f * d * h) return d * v;
  }
  return a;
}

// CSVR scale of the coming step (CSVRStep, integrators.py:519-596); all threads
// call it, thread 0 works: R1 ~ N(0, 1), R2 ~ chi^2(N_dof - 1) = 2 Gamma((N_dof - 1) / 2)
// and alpha^2 = c1 + c2 (R1^2 + R2) + 2 R1 sqrt(c1 c2), c1 = exp(-dt / tau_T),
// c2 = (1 - c1) K_target / (K N_dof), in float64.  N_dof = 3 N - 3, so
// N_dof - 1 >= 2 whenever N >= 2; a single atom (no thermal degrees of freedom)
// or a system at rest keeps alpha = 1 (the reference's formula divides by zero
// there).
__device__ void csvr_alpha(Smem &sm, double ke, uint64_t seed, int sys, uint64_t counter) {
  if (threadIdx.x == 0) {
    const SysParams &p = sm.p;
    float alpha = 1.0f;
    if (p.dof > 0 && ke > 0.0) {
      float z[4];
      normal4(seed ^ kSysSeed, (uint64_t)sys, counter, z);
      const float r1 = z[0];
      const float r2 = 2.0f * gamma_mt(0.5f * (float)(p.dof - 1), seed ^ kChiSeed, (uint64_t)sys, counter);
      const float c1 = p.csvr_c1;
      // c2 = (1 - c1) K_target / (K N_dof) with K_target = N_dof kT / 2
      const float c2 = p.csvr_omc1 * (0.5f * p.kTf) / (float)ke;
      const float a2 = c1 + c2 * (r1 * r1 + r2) + 2.0f * r1 * sqrtf(c1 * c2);
      alpha = sqrtf(fmaxf(a2, 0.0f));
    }
    sm.alpha = alpha;
  }
  __syncthreads();
}

// Resume system s from its record (all threads call; returns the same value in
// every thread).  On success the shared state (cell-sorted atoms, momenta,
// forces with travelled distances, image copies, neighbour counts) is exactly
// what the previous call held at its last step, and the Verlet list in the
// workspace is the one it built.  On failure nothing of the shared state is
// relied upon: the caller loads the input and rebuilds.
__device__ __noinline__ bool try_resume(Smem &sm, const SysParams &p, const kups_md_args &a, const MdWork &w,
                                        int s, int a0, int n, int tpa, const float4 *gpos, const float4 *gmom,
                                        const float4 *gfrc) {
  const int tid = threadIdx.x, nt = blockDim.x;
  const int cap = a.neighbor_capacity;
  if (tid == 0) {
    const SysRecord r = w.rec[s];
    bool ok = r.valid == 1 && r.n == n && r.tpa == tpa && r.cap == cap && r.n_ghosts >= 0 &&
              r.n_ghosts <= kMaxGhosts - 1 && r.rc == __float_as_uint(a.cutoff[s]) &&
              r.skin == __float_as_uint(a.skin[s]);
    for (int k = 0; k < 6; ++k) ok = ok && r.tril[k] == __float_as_uint(a.tril[6 * (int64_t)s + k]);
    sm.flag = ok ? 1 : 0;
    sm.n_ghosts = ok ? r.n_ghosts : 0;
  }
  for (int k = tid; k < kMaxAtoms / 32; k += nt) sm.cell_fill[k] = 0;  // bitmap of input indices seen
  __syncthreads();
  if (sm.flag == 0) return false;
  int bad = 0;
  for (int i = tid; i < n; i += nt) {
    const uint32_t m = w.ameta[a0 + i];
    const int g = (int)(m & 0xffffu), c = (int)(m >> 16);
    if (g >= n || c > cap) {
      bad = 1;
      continue;
    }
    const uint32_t bit = 1u << (g & 31);
    if (atomicOr(reinterpret_cast<unsigned *>(&sm.cell_fill[g >> 5]), bit) & bit) {
      bad = 1;  // an input index claimed twice
      continue;
    }
    float4 q = w.apos[a0 + i];
    float f[3];
    wrap_position(p, q, f);
    const float4 in = gpos[a0 + g];
    bad |= (__float_as_uint(q.x) != __float_as_uint(in.x)) | (__float_as_uint(q.y) != __float_as_uint(in.y)) |
           (__float_as_uint(q.z) != __float_as_uint(in.z)) | (__float_as_uint(q.w) != __float_as_uint(in.w));
  }
  if (__syncthreads_or(bad)) return false;
  const int ng = sm.n_ghosts;
  int badg = 0;
  for (int k = tid; k < ng; k += nt) {
    const uint32_t m = w.gmeta[(size_t)s * kMaxGhosts + k];
    badg |= ((int)(m & 0xffffu) >= n) | ((int)(m >> 16) >= kShiftCount);
    sm.ghost_meta[k] = m;
  }
  for (int i = tid; i < n; i += nt) {
    const uint32_t m = w.ameta[a0 + i];
    const int g = (int)(m & 0xffffu);
    sm.pos[i] = w.apos[a0 + i];
    sm.gid[i] = (uint16_t)g;
    sm.nbr_count[i] = (uint16_t)(m >> 16);
    sm.mom[i] = gmom[a0 + g];
    float4 F = gfrc[a0 + g];
    F.w = w.atrav[a0 + i];
    sm.frc[i] = F;
  }
  if (__syncthreads_or(badg)) return false;
  update_ghosts(sm, n);
  if (tid == 0) {
    sm.pos[n + ng] = make_float4(1e15f, 1e15f, 1e15f, __int_as_float(0));  // sentinel item
    sm.work = 0;
  }
  __syncthreads();
  return true;
}

// Record of system s for the next call (all threads call).
__device__ void save_record(const Smem &sm, const kups_md_args &a, const MdWork &w, int s, int a0, int n, int tpa,
                            bool valid) {
  const int tid = threadIdx.x, nt = blockDim.x;
  for (int i = tid; i < n; i += nt) {
    w.apos[a0 + i] = sm.pos[i];
    w.ameta[a0 + i] = (uint32_t)sm.gid[i] | ((uint32_t)sm.nbr_count[i] << 16);
    w.atrav[a0 + i] = sm.frc[i].w;
  }
  const int ng = sm.n_ghosts;
  for (int k = tid; k < ng; k += nt) w.gmeta[(size_t)s * kMaxGhosts + k] = sm.ghost_meta[k];
  if (tid == 0) {
    SysRecord r;
    r.valid = valid ? 1 : 0;
    r.n = n;
    r.tpa = tpa;
    r.cap = a.neighbor_capacity;
    r.n_ghosts = ng;
    r.pad0 = 0;
    r.rc = __float_as_uint(a.cutoff[s]);
    r.skin = __float_as_uint(a.skin[s]);
    for (int k = 0; k < 6; ++k) r.tril[k] = __float_as_uint(a.tril[6 * (int64_t)s + k]);
    r.pad1[0] = r.pad1[1] = 0;
    w.rec[s] = r;
  }
}

// fw += f (x) F in tril order [xx, yx, yy, zx, zy, zz] (f fractional, F a force), with explicit
// fused multiply-adds so the per-step record and the launch's final virial round identically
__device__ __forceinline__ void add_fw(float fw[6], const float f[3], const float4 &F) {
  fw[0] = __fmaf_rn(f[0], F.x, fw[0]);
  fw[1] = __fmaf_rn(f[1], F.x, fw[1]);
  fw[2] = __fmaf_rn(f[1], F.y, fw[2]);
  fw[3] = __fmaf_rn(f[2], F.x, fw[3]);
  fw[4] = __fmaf_rn(f[2], F.y, fw[4]);
  fw[5] = __fmaf_rn(f[2], F.z, fw[5]);
}

// The float64 inverse of the lower-triangular cell p.Ld (one thread; float64 divisions are slow
// on this part, so it is formed once per cell, not per step).
__device__ inline void set_inverse64(SysParams &p) {
  const double A = p.Ld[0], B = p.Ld[1], C = p.Ld[2], D = p.Ld[3], E = p.Ld[4], F = p.Ld[5];
  const double i00 = 1.0 / A, i11 = 1.0 / C, i22 = 1.0 / F;
  const double i10 = -(B * i00) / C, i21 = -(E * i11) / F, i20 = -((D * i00) + (E * i10)) / F;
  const double Li[9] = {i00, 0.0, 0.0, i10, i11, 0.0, i20, i21, i22};
  for (int k = 0; k < 9; ++k) p.Lid[k] = Li[k];
}

// dE/dtril [xx, yx, yy, zx, zy, zz] of a system from block sums r[0..5] of the pair virial
// W_cb = 1/2 sum d_c g_b (Cartesian, [xx, yx, yy, zx, zy, zz]) and r[6..11] of
// sum_i f_i,a F_i,b over atoms (f fractional, wrapped; F the force), written by thread 0:
// X_ab = sum_c (L^-1)_ca W_cb + sum_i f_i,a F_i,b.  Returns Tr W (every thread).
__device__ double virial_from_sums(const SysParams &p, const double r[12], double *out) {
  // only thread 0 forms the cell inverse (float64 divisions: a handful of FP64 operations per
  // thread of a 1024-thread block would cost the whole block tens of microseconds per call)
  if (threadIdx.x == 0) {
    double W[3][3];
    W[0][0] = r[0];
    W[1][0] = W[0][1] = r[1];
    W[1][1] = r[2];
    W[2][0] = W[0][2] = r[3];
    W[2][1] = W[1][2] = r[4];
    W[2][2] = r[5];
    const int ia[6] = {0, 1, 1, 2, 2, 2}, ib[6] = {0, 0, 1, 0, 1, 2};
    for (int k = 0; k < 6; ++k) {
      double x = 0.0;
      for (int c = 0; c < 3; ++c) x += p.Lid[3 * c + ia[k]] * W[c][ib[k]];
      out[k] = x + r[6 + k];
    }
  }
  return r[0] + r[2] + r[5];
}

template <int INTEGRATOR>
__global__ void __launch_bounds__(kThreads, 1)
md_lj_kernel(kups_md_args a, MdWork w, int *queue, kups_status *status) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  Smem &sm = *reinterpret_cast<Smem *>(smem_raw);
  const int tid = threadIdx.x, nt = blockDim.x;
  float4 *gpos = reinterpret_cast<float4 *>(a.pos);
  float4 *gmom = reinterpret_cast<float4 *>(a.mom);
  float4 *gfrc = reinterpret_cast<float4 *>(a.force);
  float4 *scratch = w.scratch + (size_t)blockIdx.x * kScratchPerCta;
  unsigned long long *prof = reinterpret_cast<unsigned long long *>(a.profile);
  const int nsp = a.n_species;
  for (int k = tid; k < nsp * nsp; k += nt)
    sm.lj[k] = make_float2(a.lj_table[2 * k], a.lj_table[2 * k + 1]);
  const float sig2_0 = a.lj_table[0], a4_0 = a.lj_table[1];

  while (true) {
    if (tid == 0) sm.next_sys = atomicAdd(queue, 1);
    __syncthreads();
    const int q = sm.next_sys;
    __syncthreads();
    if (q >= a.n_systems) break;
    const int s = a.order[q];
    const int a0 = a.sys_offset[s];
    const int n = a.sys_offset[s + 1] - a0;
    if (n <= 0) continue;
    if (n > kMaxAtoms) {
      if (tid == 0) status_capacity(status, KUPS_CAP_ATOMS, n, s);
      continue;
    }
    if ((int64_t)a0 + n > a.n_atoms || a0 < 0) {  // the workspace regions are sized by n_atoms
      if (tid == 0) status_error(status, KUPS_ERR_INVALID, s);
      continue;
    }
    uint2 *nl = w.lists + (size_t)a0 * md_units_per_atom(a.neighbor_capacity);
    long long t0 = clock64();
    // ---- per-system parameters, computed once into shared memory
    SysParams &p = sm.p;
    if (tid == 0) {
      if (INTEGRATOR == 3) {
        for (int k = 0; k < 6; ++k) p.Ld[k] = a.cell[6 * (int64_t)s + k];
      } else {
        for (int k = 0; k < 6; ++k) p.Ld[k] = (double)a.tril[6 * (int64_t)s + k];
      }
      for (int k = 0; k < 6; ++k) p.L[k] = (float)p.Ld[k];
      set_inverse64(p);
      const float rc = a.cutoff[s], skin = a.skin[s], rl = rc + skin;
      p.rc = rc;
      p.rl = rl;
      p.rc2 = rc * rc;
      p.rl2 = rl * rl;
      p.half_skin = 0.5f * skin;
      set_cell(p);
      p.dt = a.dt[s];
      p.c1 = expf(-a.friction[s] * p.dt);
      p.c2 = sqrtf(a.kT[s] * (1.0f - p.c1 * p.c1));
      if (INTEGRATOR >= 2) {
        const double x = -(double)p.dt / a.thermostat_tau[s];
        p.csvr_c1 = (float)exp(x);
        p.csvr_omc1 = (float)-expm1(x);
        p.kTf = a.kT[s];
        p.dof = 3 * n - 3;
      }
      if (INTEGRATOR == 3) {
        const double ratio = (double)p.dt / a.barostat_tau[s] * a.compressibility[s];
        p.scr_a = (float)ratio;
        p.scr_b = (float)(2.0 * (double)a.kT[s] * ratio);
        p.p0f = (float)a.target_pressure[s];
        p.mumin = a.min_scale[s];
        p.mumax = 1.0 / a.min_scale[s];
      }
    }
    __syncthreads();
    if (p.K[0] > 2 || p.K[1] > 2 || p.K[2] > 2) {
      if (tid == 0) status_error(status, KUPS_ERR_UNSUPPORTED, s);
      continue;
    }
    set_shift_vectors(sm);
    const int tpa = choose_tpa(n, nt, a.min_lanes_per_atom);
    bool ok = true;
    const bool resumed = INTEGRATOR != 3 && a.reuse_lists != 0 &&
                         try_resume(sm, p, a, w, s, a0, n, tpa, gpos, gmom, gfrc);
    if (tid == 0) w.rec[s].valid = 0;  // set again when this call has written the record
    if (!resumed) {
      int bad_species = 0;
      for (int i = tid; i < n; i += nt) {
        const float4 qv = gpos[a0 + i];
        const int t = __float_as_int(qv.w);
        bad_species |= (t < 0) | (t >= nsp);
        sm.pos[i] = qv;
        sm.mom[i] = gmom[a0 + i];
        sm.frc[i] = gfrc[a0 + i];
        sm.gid[i] = (uint16_t)i;
      }
      if (__syncthreads_or(bad_species)) {
        if (tid == 0) status_error(status, KUPS_ERR_INVALID, s);
        continue;
      }
      ok = rebuild(sm, p, n, tpa, nl, a.neighbor_capacity, status, s, prof, scratch);
      if (tid == 0) sm.work = 0;
      __syncthreads();
      if (!ok) continue;
      if (tid == 0 && a.rebuilds != nullptr) a.rebuilds[s] += 1;
    }
    prof_add(prof, 0, t0);
    // hot scalars in registers
    const float rc2 = p.rc2, dt = p.dt, hdt = 0.5f * p.dt, c1 = p.c1, c2 = p.c2;
    const float half_skin = p.half_skin;
    // list-validity threshold on the distance travelled (in the frame of the last
    // build): with the cell scaled by m since that build, a pair missing from the
    // list is at least m (rc + skin - 2 d) apart, so the list holds while
    // d <= (rc + skin - rc / m) / 2 (skin / 2 at m = 1)
    float thr = half_skin, inv_mcum = 1.0f;
    double mcum = 1.0;
    float wv[6] = {0, 0, 0, 0, 0, 0};
    bool energy_valid = false;  // atom_energy holds the current forces' energies
    if (!a.forces_valid) {
      if (a.n_steps == 0 && a.virial != nullptr)
        forces_dispatch<true, true>(sm, n, nsp, tpa, nl, rc2, sig2_0, a4_0, wv);
      else
        forces_dispatch<true, false>(sm, n, nsp, tpa, nl, rc2, sig2_0, a4_0, wv);
      __syncthreads();
      energy_valid = true;
    }
    if (INTEGRATOR >= 2 && a.n_steps > 0) {
      float ke = 0.f;
      for (int i = tid; i < n; i += nt) {
        const float4 m = sm.mom[i];
        ke += 0.5f * fmaf(m.z, m.z, fmaf(m.y, m.y, m.x * m.x)) / m.w;
      }
      const float kv[1] = {ke};
      double kt[1];
      block_sums<1>(kv, sm, kt);
      csvr_alpha(sm, kt[0], a.seed, a.system_base + s, a.step0);
    }
    const bool trace_v = INTEGRATOR != 3 && a.trace_virial != nullptr;
    for (int step = 0; step < a.n_steps && ok; ++step) {
      const bool last = step == a.n_steps - 1;
      const bool want_e = last || a.trace_pe != nullptr || a.trace_ke != nullptr || trace_v;
      // ---- (CSVR) B A (O A)
      const float alpha = INTEGRATOR >= 2 ? sm.alpha : 1.0f;
      if (tid == 0) sm.work = 0;
      int moved_far = 0;
      for (int i = tid; i < n; i += nt) {
        float4 x = sm.pos[i], m = sm.mom[i], f = sm.frc[i];
        const float inv_m = 1.0f / m.w;
        if (INTEGRATOR >= 2) {
          m.x = __fmul_rn(m.x, alpha);
          m.y = __fmul_rn(m.y, alpha);
          m.z = __fmul_rn(m.z, alpha);
        }
        m.x = fmaf(f.x, hdt, m.x);
        m.y = fmaf(f.y, hdt, m.y);
        m.z = fmaf(f.z, hdt, m.z);
        float dx, dy, dz;
        if (INTEGRATOR != 1) {
          const float sc = inv_m * dt;
          dx = m.x * sc;
          dy = m.y * sc;
          dz = m.z * sc;
        } else {
          const float sc = inv_m * hdt;
          dx = m.x * sc;
          dy = m.y * sc;
          dz = m.z * sc;
          float eta[4];
          normal4(a.seed, (uint64_t)(a.atom_base + a0 + sm.gid[i]), a.step0 + (uint64_t)step, eta);
          const float amp = c2 * sqrtf(m.w);
          m.x = fmaf(c1, m.x, amp * eta[0]);
          m.y = fmaf(c1, m.y, amp * eta[1]);
          m.z = fmaf(c1, m.z, amp * eta[2]);
          dx = fmaf(m.x, sc, dx);
          dy = fmaf(m.y, sc, dy);
          dz = fmaf(m.z, sc, dz);
        }
        x.x += dx;
        x.y += dy;
        x.z += dz;
        const float len = sqrtf(fmaf(dz, dz, fmaf(dy, dy, dx * dx)));
        if (INTEGRATOR == 3)
          f.w = fmaf(len, inv_mcum, f.w);
        else
          f.w += len;
        moved_far |= f.w > thr;
        sm.pos[i] = x;
        sm.mom[i] = m;
        sm.frc[i] = f;
      }
      const int need = __syncthreads_or(moved_far);
      prof_add(prof, 1, t0);
      if (need) {
        if (tid == 0 && a.rebuilds != nullptr) a.rebuilds[s] += 1;
        ok = rebuild(sm, p, n, tpa, nl, a.neighbor_capacity, status, s, prof, scratch);
        if (!ok) break;
        mcum = 1.0;
        thr = half_skin;
        inv_mcum = 1.0f;
        if (tid == 0) sm.work = 0;
        __syncthreads();
      } else {
        update_ghosts(sm, n);
        __syncthreads();
      }
      prof_add(prof, 2, t0);
      // ---- forces
      if (INTEGRATOR == 3) {
        // the barostat needs the pair virial at every step
#pragma unroll
        for (int k = 0; k < 6; ++k) wv[k] = 0.f;
        forces_dispatch<false, true>(sm, n, nsp, tpa, nl, rc2, sig2_0, a4_0, wv);
      } else if ((last && a.virial != nullptr) || trace_v) {
        if (trace_v) {
#pragma unroll
          for (int k = 0; k < 6; ++k) wv[k] = 0.f;
        }
        forces_dispatch<true, true>(sm, n, nsp, tpa, nl, rc2, sig2_0, a4_0, wv);
      } else if (want_e) {
        forces_dispatch<true, false>(sm, n, nsp, tpa, nl, rc2, sig2_0, a4_0, wv);
      } else {
        forces_dispatch<false, false>(sm, n, nsp, tpa, nl, rc2, sig2_0, a4_0, wv);
      }
      __syncthreads();
      prof_add(prof, 3, t0);
      // ---- B (and kinetic energy when recorded or needed by the thermostat)
      const bool need_ke = want_e || INTEGRATOR >= 2;
      float ke = 0.f;
      float fwt[6] = {0, 0, 0, 0, 0, 0};  // sum_i f_i,a F_i,b (per-step virial record)
      for (int i = tid; i < n; i += nt) {
        float4 m = sm.mom[i];
        const float4 f = sm.frc[i];
        m.x = fmaf(f.x, hdt, m.x);
        m.y = fmaf(f.y, hdt, m.y);
        m.z = fmaf(f.z, hdt, m.z);
        sm.mom[i] = m;
        if (need_ke) ke += 0.5f * fmaf(m.z, m.z, fmaf(m.y, m.y, m.x * m.x)) / m.w;
        if (INTEGRATOR != 3 && trace_v) {
          float4 x = sm.pos[i];
          float fr[3];
          wrap_position(p, x, fr);
          add_fw(fwt, fr, f);
        }
      }
      if (INTEGRATOR != 3 && trace_v) {
        const float v[12] = {wv[0], wv[1], wv[2], wv[3], wv[4], wv[5], fwt[0], fwt[1], fwt[2], fwt[3], fwt[4], fwt[5]};
        double r[12];
        block_sums<12>(v, sm, r);
        virial_from_sums(p, r, a.trace_virial + ((int64_t)step * a.n_systems + s) * 6);
      }
      double ke_tot = 0.0;
      double w6[6];
      if (INTEGRATOR == 3) {
        const float v[7] = {ke, wv[0], wv[1], wv[2], wv[3], wv[4], wv[5]};
        double r[7];
        block_sums<7>(v, sm, r);
        ke_tot = r[0];
        for (int k = 0; k < 6; ++k) w6[k] = r[k + 1];
      } else if (need_ke) {
        const float v[1] = {ke};
        double r[1];
        block_sums<1>(v, sm, r);
        ke_tot = r[0];
      }
      prof_add(prof, 4, t0);
      if (INTEGRATOR == 3) {
        // ---- stochastic cell rescaling (integrators.py:710-789): pressure from the
        // kinetic energy and the pair virial, P = (2 K - Tr W) / 3V, then
        // d eps = dt / tau_P beta (P - P0) + sqrt(2 kT beta dt / (tau_P V)) R and
        // mu = exp(d eps / 3) clipped to [mu_min, 1 / mu_min] scale cell and positions
        if (tid == 0) {
          // float32 on the one thread (FP64 is scarce); mu = 1 + expm1(d eps / 3)
          // keeps mu - 1 to float32 relative precision, the cell stays float64
          const float vol = fabsf(p.L[0] * p.L[2] * p.L[5]);
          const float prs = (float)(2.0 * ke_tot - (w6[0] + w6[2] + w6[5])) / (3.0f * vol);
          float z[4];
          normal4(a.seed ^ kSysSeed, (uint64_t)(a.system_base + s), a.step0 + (uint64_t)step, z);
          const float deps = p.scr_a * (prs - p.p0f) + sqrtf(p.scr_b / vol) * z[1];
          const double mu = fmin(fmax(1.0 + (double)expm1f(deps * (1.0f / 3.0f)), p.mumin), p.mumax);
          for (int k = 0; k < 6; ++k) {
            p.Ld[k] *= mu;
            p.L[k] = (float)p.Ld[k];
          }
          set_inverse64(p);
          set_cell(p);
          sm.mu = (float)mu;
          sm.work = 0;
        }
        __syncthreads();
        prof_add(prof, 8, t0);
        if (p.K[0] > 2 || p.K[1] > 2 || p.K[2] > 2) {
          if (tid == 0) status_error(status, KUPS_ERR_UNSUPPORTED, s);
          ok = false;
          break;
        }
        set_shift_vectors(sm);
        const float mu = sm.mu;
        mcum *= (double)mu;
        inv_mcum = (float)(1.0 / mcum);
        thr = mcum == 1.0 ? half_skin : 0.5f * (p.rl - p.rc * inv_mcum);
        int far = 0;
        for (int i = tid; i < n; i += nt) {
          float4 x = sm.pos[i];
          x.x = __fmul_rn(x.x, mu);
          x.y = __fmul_rn(x.y, mu);
          x.z = __fmul_rn(x.z, mu);
          sm.pos[i] = x;
          far |= sm.frc[i].w > thr;
        }
        if (__syncthreads_or(far)) {
          if (tid == 0 && a.rebuilds != nullptr) a.rebuilds[s] += 1;
          ok = rebuild(sm, p, n, tpa, nl, a.neighbor_capacity, status, s, prof, scratch);
          if (!ok) break;
          mcum = 1.0;
          thr = half_skin;
          inv_mcum = 1.0f;
          if (tid == 0) sm.work = 0;
          __syncthreads();
        } else {
          update_ghosts(sm, n);
          __syncthreads();
        }
        prof_add(prof, 2, t0);
        // ---- forces at the rescaled positions (the next step's first kick)
        if (last && a.virial != nullptr) {
#pragma unroll
          for (int k = 0; k < 6; ++k) wv[k] = 0.f;
          forces_dispatch<true, true>(sm, n, nsp, tpa, nl, rc2, sig2_0, a4_0, wv);
        } else if (want_e) {
          forces_dispatch<true, false>(sm, n, nsp, tpa, nl, rc2, sig2_0, a4_0, wv);
        } else {
          forces_dispatch<false, false>(sm, n, nsp, tpa, nl, rc2, sig2_0, a4_0, wv);
        }
        __syncthreads();
        prof_add(prof, 3, t0);
      }
      if (want_e) {
        const double pe_tot = atom_energy_sum(sm, n);
        if (tid == 0) {
          if (a.trace_pe) a.trace_pe[(int64_t)step * a.n_systems + s] = pe_tot;
          if (a.trace_ke) a.trace_ke[(int64_t)step * a.n_systems + s] = ke_tot;
          if (last) {
            a.energy[s] = pe_tot;
            a.kinetic[s] = ke_tot;
          }
        }
      }
      prof_add(prof, 4, t0);
      if (INTEGRATOR >= 2 && !last) {
        csvr_alpha(sm, ke_tot, a.seed, a.system_base + s, a.step0 + (uint64_t)step + 1);
        prof_add(prof, 8, t0);
      }
    }
    if (!ok) continue;
    if (a.n_steps == 0) {
      float ke = 0.f;
      for (int i = tid; i < n; i += nt) {
        const float4 m = sm.mom[i];
        ke += 0.5f * fmaf(m.z, m.z, fmaf(m.y, m.y, m.x * m.x)) / m.w;
      }
      const double pe_tot = energy_valid ? atom_energy_sum(sm, n) : 0.0;
      const double ke_tot = block_sum((double)ke, sm.red + 36);
      if (tid == 0) {
        a.energy[s] = pe_tot;
        a.kinetic[s] = ke_tot;
      }
    }
    // ---- write back (wrapped positions), virial dE/dtril
    float fw[6] = {0, 0, 0, 0, 0, 0};  // sum_i f_i,a F_i,b for (a, b) in tril order
    __syncthreads();
    for (int i = tid; i < n; i += nt) {
      float4 x = sm.pos[i];
      float f[3];
      wrap_position(p, x, f);
      const int o = a0 + sm.gid[i];
      gpos[o] = x;
      gmom[o] = sm.mom[i];
      float4 F = sm.frc[i];
      F.w = 0.f;
      gfrc[o] = F;
      add_fw(fw, f, F);
    }
    if (a.virial != nullptr) {
      const float v[12] = {wv[0], wv[1], wv[2], wv[3], wv[4], wv[5], fw[0], fw[1], fw[2], fw[3], fw[4], fw[5]};
      double r[12];
      block_sums<12>(v, sm, r);
      const double trw = virial_from_sums(p, r, a.virial + 6 * (int64_t)s);
      if (tid == 0 && a.pressure != nullptr) {
        // sum_i dU/dr_i (x) r_i + h^T dU/dh = sum over pairs of d (x) dU/dd = W for a pair
        // potential: P = (2 K - Tr W) / 3V
        const double vol = fabs(p.Ld[0] * p.Ld[2] * p.Ld[5]);
        a.pressure[s] = (2.0 * a.kinetic[s] - trw) / (3.0 * vol);
      }
    }
    if (INTEGRATOR == 3 && tid == 0)
      for (int k = 0; k < 6; ++k) a.cell[6 * (int64_t)s + k] = p.Ld[k];
    save_record(sm, a, w, s, a0, n, tpa, INTEGRATOR != 3);
    prof_add(prof, 5, t0);
    __syncthreads();
  }
}

}  // namespace
}  // namespace kups

using namespace kups;

template <int INTEGRATOR>
static cudaError_t launch_md(const kups_md_args &a, int ctas, int threads, size_t smem, const MdWork &w,
                             int *queue, kups_status *status, cudaStream_t stream) {
  cudaError_t e = cudaFuncSetAttribute(md_lj_kernel<INTEGRATOR>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)smem);
  if (e != cudaSuccess) return e;
  md_lj_kernel<INTEGRATOR><<<ctas, threads, smem, stream>>>(a, w, queue, status);
  return cudaSuccess;
}

extern "C" int32_t kups_lj_md_max_atoms(void) { return kMaxAtoms; }

extern "C" size_t kups_lj_md_workspace_bytes(const kups_md_args *a) {
  const int ctas = a->n_ctas > 0 ? a->n_ctas : device_sm_count();
  return md_layout(ctas, a->n_atoms < 0 ? 0 : a->n_atoms, a->n_systems < 0 ? 0 : a->n_systems,
                   a->neighbor_capacity).total + 256;
}

extern "C" int32_t kups_lj_md_run(const kups_md_args *a, void *workspace, size_t ws_bytes,
                                  kups_status *status, void *stream_) {
  cudaStream_t stream = (cudaStream_t)stream_;
  if (a == nullptr || a->n_systems < 0 || a->n_steps < 0 || a->n_species <= 0 ||
      a->n_species > kMaxSpecies || a->neighbor_capacity <= 0 || a->neighbor_capacity > 4096 ||
      a->neighbor_capacity % 16 != 0 ||
      a->integrator < 0 || a->integrator > 3)
    return KUPS_ERR_INVALID;
  if (a->integrator >= 2 && a->thermostat_tau == nullptr) return KUPS_ERR_INVALID;
  if (a->integrator == 3 && (a->target_pressure == nullptr || a->barostat_tau == nullptr ||
                             a->compressibility == nullptr || a->min_scale == nullptr ||
                             a->cell == nullptr))
    return KUPS_ERR_INVALID;
  if (a->integrator == 3 && a->trace_virial != nullptr) return KUPS_ERR_INVALID;
  if (ws_bytes < kups_lj_md_workspace_bytes(a)) return KUPS_ERR_INVALID;
  if (a->n_systems == 0) return KUPS_OK;
  const int ctas = a->n_ctas > 0 ? a->n_ctas : device_sm_count();
  const int threads = a->block_threads > 0 ? a->block_threads : kThreads;
  if (threads % 32 != 0 || threads > kThreads || threads < 64) return KUPS_ERR_INVALID;
  const int lanes = a->min_lanes_per_atom;
  // a power of two up to 16: md_units_per_atom keeps whole rows of tpa units inside the lists
  if (lanes != 0 && lanes != 1 && lanes != 2 && lanes != 4 && lanes != 8 && lanes != 16)
    return KUPS_ERR_INVALID;
  kups_md_args args = *a;
  if (args.min_lanes_per_atom == 0) args.min_lanes_per_atom = 2;
  if (a->n_atoms < 0 || a->atom_base < 0 || a->system_base < 0) return KUPS_ERR_INVALID;
  char *base = reinterpret_cast<char *>(((uintptr_t)workspace + 255) & ~uintptr_t(255));
  int *queue = reinterpret_cast<int *>(base);
  const MdLayout l = md_layout(ctas, a->n_atoms, a->n_systems, a->neighbor_capacity);
  MdWork w;
  w.scratch = reinterpret_cast<float4 *>(base + l.scratch);
  w.rec = reinterpret_cast<SysRecord *>(base + l.rec);
  w.apos = reinterpret_cast<float4 *>(base + l.apos);
  w.ameta = reinterpret_cast<uint32_t *>(base + l.ameta);
  w.atrav = reinterpret_cast<float *>(base + l.atrav);
  w.gmeta = reinterpret_cast<uint32_t *>(base + l.gmeta);
  w.lists = reinterpret_cast<uint2 *>(base + l.lists);
  KUPS_CUDA_TRY(cudaMemsetAsync(queue, 0, sizeof(int), stream));
  const size_t smem = sizeof(Smem);
  switch (a->integrator) {
    case 0: KUPS_CUDA_TRY(launch_md<0>(args, ctas, threads, smem, w, queue, status, stream)); break;
    case 1: KUPS_CUDA_TRY(launch_md<1>(args, ctas, threads, smem, w, queue, status, stream)); break;
    case 2: KUPS_CUDA_TRY(launch_md<2>(args, ctas, threads, smem, w, queue, status, stream)); break;
    default: KUPS_CUDA_TRY(launch_md<3>(args, ctas, threads, smem, w, queue, status, stream)); break;
  }
  return cudaGetLastError() == cudaSuccess ? KUPS_OK : KUPS_ERR_CUDA;
}

// ---------------------------------------------------------------- layout conversion
// Reference layout (float64 [N, 3] arrays + masses + species, any particle
// order) <-> packed float4 arrays grouped by system.  perm[k] is the
// reference index of packed atom k (identity if perm is null).
namespace kups {
namespace {
__global__ void md_pack_kernel(const double *pos, const double *mom, const double *frc,
                               const double *mass, const int32_t *species, const int32_t *perm,
                               int64_t n, float4 *pos4, float4 *mom4, float4 *frc4) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const int64_t i = perm ? perm[k] : k;
  pos4[k] = make_float4((float)pos[3 * i], (float)pos[3 * i + 1], (float)pos[3 * i + 2],
                        __int_as_float(species[i]));
  mom4[k] = make_float4((float)mom[3 * i], (float)mom[3 * i + 1], (float)mom[3 * i + 2],
                        (float)mass[i]);
  if (frc)
    frc4[k] = make_float4((float)frc[3 * i], (float)frc[3 * i + 1], (float)frc[3 * i + 2], 0.f);
  else
    frc4[k] = make_float4(0.f, 0.f, 0.f, 0.f);
}

__global__ void md_unpack_kernel(const float4 *pos4, const float4 *mom4, const float4 *frc4,
                                 const int32_t *perm, int64_t n, double *pos, double *mom,
                                 double *frc) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const int64_t i = perm ? perm[k] : k;
  const float4 p = pos4[k], m = mom4[k];
  pos[3 * i] = p.x; pos[3 * i + 1] = p.y; pos[3 * i + 2] = p.z;
  mom[3 * i] = m.x; mom[3 * i + 1] = m.y; mom[3 * i + 2] = m.z;
  if (frc) {
    const float4 f = frc4[k];
    frc[3 * i] = f.x; frc[3 * i + 1] = f.y; frc[3 * i + 2] = f.z;
  }
}
}  // namespace
}  // namespace kups

extern "C" int32_t kups_md_pack(const double *pos, const double *mom, const double *force,
                                const double *mass, const int32_t *species, const int32_t *perm,
                                int64_t n, void *pos4, void *mom4, void *force4, void *stream) {
  if (n < 0) return KUPS_ERR_INVALID;
  if (n == 0) return KUPS_OK;
  kups::md_pack_kernel<<<(unsigned)((n + 255) / 256), 256, 0, (cudaStream_t)stream>>>(
      pos, mom, force, mass, species, perm, n, (float4 *)pos4, (float4 *)mom4, (float4 *)force4);
  return cudaGetLastError() == cudaSuccess ? KUPS_OK : KUPS_ERR_CUDA;
}

extern "C" int32_t kups_md_unpack(const void *pos4, const void *mom4, const void *force4,
                                  const int32_t *perm, int64_t n, double *pos, double *mom,
                                  double *force, void *stream) {
  if (n < 0) return KUPS_ERR_INVALID;
  if (n == 0) return KUPS_OK;
  kups::md_unpack_kernel<<<(unsigned)((n + 255) / 256), 256, 0, (cudaStream_t)stream>>>(
      (const float4 *)pos4, (const float4 *)mom4, (const float4 *)force4, perm, n, pos, mom, force);
  return cudaGetLastError() == cudaSuccess ? KUPS_OK : KUPS_ERR_CUDA;
}
