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

struct Smem {
  float4 pos[kMaxItems];
  float4 mom[kMaxAtoms];
  float4 frc[kMaxAtoms];
  uint32_t ghost_meta[kMaxGhosts];  // source atom | shift code << 16
  uint16_t cell_of[kMaxItems];
  uint16_t cell_items[kMaxItems];
  int cell_start[kMaxCells + 1];
  int cell_fill[kMaxCells];
  uint16_t nbr_count[kMaxAtoms];
  float4 shift_vec[kShiftCount];
  float2 lj[kMaxSpecies * kMaxSpecies];  // (sigma^2, 4 eps)
  double red[72];
  int iscan[40];
  int n_ghosts;
  int flag;
  int next_sys;
};

struct SysParams {
  float L[6];     // L00 L10 L11 L20 L21 L22
  float inv[6];
  float rc2, rl2, half_skin;
  float m[3];     // margins in fractional units
  int K[3];       // image layers per side
  int nc[3];
  float ext[3];   // 1 + 2 m
  float dt, c1, c2;
};

__device__ inline void frac_of(const SysParams &p, float x, float y, float z, float f[3]) {
  f[0] = (x * p.inv[0] + y * p.inv[1]) + z * p.inv[3];
  f[1] = y * p.inv[2] + z * p.inv[4];
  f[2] = z * p.inv[5];
}

__device__ inline void cart_of(const SysParams &p, const float f[3], float &x, float &y, float &z) {
  x = (f[0] * p.L[0] + f[1] * p.L[1]) + f[2] * p.L[3];
  y = f[1] * p.L[2] + f[2] * p.L[4];
  z = f[2] * p.L[5];
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

__device__ inline int cell_coord(float pf, float m, float ext, int nc) {
  int c = (int)floorf((pf + 0.5f + m) / ext * (float)nc);
  return c < 0 ? 0 : (c >= nc ? nc - 1 : c);
}

// Cost model for the number of lanes serving one atom in the force loop.
__device__ inline int choose_tpa(int n, int threads) {
  int best = 1;
  float best_cost = 1e30f;
  for (int t = 1; t <= 16; t <<= 1) {
    const int rounds = (n * t + threads - 1) / threads;
    const float cost = rounds * (72.0f / t + 6.0f * __log2f((float)t) + 4.0f);
    if (cost < best_cost) {
      best_cost = cost;
      best = t;
    }
  }
  return best;
}

// Wrap atoms, build the ghost copies, the cell grid and the Verlet list.
// Returns false (and records the requirement) if a capacity is exceeded.
__device__ bool rebuild(Smem &sm, const SysParams &p, int n, int tpa, uint16_t *nl, int nb_cap,
                        kups_status *status, int sys_index) {
  const int tid = threadIdx.x, nt = blockDim.x;
  // 1. wrap atoms into [-0.5, 0.5), reset travelled distance, count ghosts
  int my_total = 0;
  {
    for (int i = tid; i < n; i += nt) {
      float4 q = sm.pos[i];
      float f[3];
      wrap_position(p, q, f);
      sm.pos[i] = q;
      sm.frc[i].w = 0.0f;
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
  }
  int total;
  int base = block_exclusive_scan<int>(my_total, sm.iscan, &total);
  __syncthreads();
  if (total > kMaxGhosts) {
    if (tid == 0) status_capacity(status, KUPS_CAP_GHOSTS, total, sys_index);
    return false;
  }
  // 2. write ghosts (deterministic order: atom-major, offset order)
  {
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
              sm.pos[n + base] = make_float4(q.x + sv.x, q.y + sv.y, q.z + sv.z, q.w);
              sm.ghost_meta[base] = (uint32_t)i | ((uint32_t)code << 16);
              ++base;
            }
          }
    }
  }
  const int n_items = n + total;
  const int ncell = p.nc[0] * p.nc[1] * p.nc[2];
  for (int c = tid; c < ncell; c += nt) {
    sm.cell_start[c] = 0;
    sm.cell_fill[c] = 0;
  }
  __syncthreads();
  // 3. bin items into the extended grid
  for (int it = tid; it < n_items; it += nt) {
    const float4 q = sm.pos[it];
    float f[3];
    frac_of(p, q.x, q.y, q.z, f);
    const int cx = cell_coord(f[0], p.m[0], p.ext[0], p.nc[0]);
    const int cy = cell_coord(f[1], p.m[1], p.ext[1], p.nc[1]);
    const int cz = cell_coord(f[2], p.m[2], p.ext[2], p.nc[2]);
    const int c = (cz * p.nc[1] + cy) * p.nc[0] + cx;
    sm.cell_of[it] = (uint16_t)c;
    atomicAdd(&sm.cell_start[c], 1);
  }
  __syncthreads();
  {
    int carry = 0;
    for (int b0 = 0; b0 < ncell; b0 += nt) {
      const int c = b0 + tid;
      const int v = c < ncell ? sm.cell_start[c] : 0;
      int tot;
      const int ex = block_exclusive_scan<int>(v, sm.iscan, &tot);
      __syncthreads();
      if (c < ncell) sm.cell_start[c] = carry + ex;
      carry += tot;
    }
    if (tid == 0) sm.cell_start[ncell] = carry;
  }
  __syncthreads();
  for (int it = tid; it < n_items; it += nt) {
    const int c = sm.cell_of[it];
    const int slot = atomicAdd(&sm.cell_fill[c], 1);
    sm.cell_items[sm.cell_start[c] + slot] = (uint16_t)it;
  }
  __syncthreads();
  for (int c = tid; c < ncell; c += nt) {  // deterministic order inside each cell
    const int b = sm.cell_start[c], e = sm.cell_start[c + 1];
    for (int k = b + 1; k < e; ++k) {
      const uint16_t v = sm.cell_items[k];
      int m = k - 1;
      while (m >= b && sm.cell_items[m] > v) {
        sm.cell_items[m + 1] = sm.cell_items[m];
        --m;
      }
      sm.cell_items[m + 1] = v;
    }
  }
  if (tid == 0) sm.flag = 0;
  __syncthreads();
  // 4. Verlet list: entry k of atom i at ((k / tpa) * n + i) * tpa + k % tpa
  int my_max = 0;
  for (int i = tid; i < n; i += nt) {
    const float4 q = sm.pos[i];
    const int c = sm.cell_of[i];
    const int cx = c % p.nc[0], cy = (c / p.nc[0]) % p.nc[1], cz = c / (p.nc[0] * p.nc[1]);
    int cnt = 0;
    for (int z = max(cz - 1, 0); z <= min(cz + 1, p.nc[2] - 1); ++z)
      for (int y = max(cy - 1, 0); y <= min(cy + 1, p.nc[1] - 1); ++y)
        for (int x = max(cx - 1, 0); x <= min(cx + 1, p.nc[0] - 1); ++x) {
          const int cc = (z * p.nc[1] + y) * p.nc[0] + x;
          const int b = sm.cell_start[cc], e = sm.cell_start[cc + 1];
          for (int k = b; k < e; ++k) {
            const int j = sm.cell_items[k];
            if (j == i) continue;
            const float4 o = sm.pos[j];
            const float dx = o.x - q.x, dy = o.y - q.y, dz = o.z - q.z;
            const float r2 = dx * dx + dy * dy + dz * dz;
            if (r2 < p.rl2) {
              if (cnt < nb_cap) nl[((size_t)(cnt / tpa) * n + i) * tpa + (cnt % tpa)] = (uint16_t)j;
              ++cnt;
            }
          }
        }
    sm.nbr_count[i] = (uint16_t)min(cnt, nb_cap);
    my_max = max(my_max, cnt);
  }
  if (my_max > nb_cap) {
    atomicMax(&sm.flag, my_max);
  }
  __syncthreads();
  const int need = sm.flag;
  if (need > nb_cap) {
    if (tid == 0) status_capacity(status, KUPS_CAP_NEIGHBORS, need, sys_index);
    return false;
  }
  if (tid == 0) sm.n_ghosts = total;
  __syncthreads();
  return true;
}

__device__ inline void update_ghosts(Smem &sm, int n) {
  const int ng = sm.n_ghosts;
  for (int g = threadIdx.x; g < ng; g += blockDim.x) {
    const uint32_t m = sm.ghost_meta[g];
    const float4 q = sm.pos[m & 0xffffu];
    const float4 sv = sm.shift_vec[m >> 16];
    sm.pos[n + g] = make_float4(q.x + sv.x, q.y + sv.y, q.z + sv.z, q.w);
  }
}

// Forces into sm.frc[i].xyz; returns this thread's share of the potential
// energy (float64) and adds the Cartesian pair virial W_cb = 1/2 sum d_c g_b
// (symmetric, [xx, yx, yy, zx, zy, zz]) into wv when VIRIAL.
template <bool VIRIAL>
__device__ double compute_forces(Smem &sm, const SysParams &p, int n, int nsp, int tpa,
                                 const uint16_t *nl, float wv[6]) {
  const int lane_g = threadIdx.x & (tpa - 1);
  const int grp = threadIdx.x / tpa;
  const int ngrp = blockDim.x / tpa;
  double e_acc = 0.0;
  for (int base = 0; base < n; base += ngrp) {
    const int i = base + grp;
    const bool active = i < n;
    float fx = 0.f, fy = 0.f, fz = 0.f, e = 0.f;
    float w0 = 0.f, w1 = 0.f, w2 = 0.f, w3 = 0.f, w4 = 0.f, w5 = 0.f;
    if (active) {
      const float4 xi = sm.pos[i];
      const int ti = __float_as_int(xi.w);
      const int cnt = sm.nbr_count[i];
      const uint16_t *row = nl + (size_t)i * tpa + lane_g;
      const size_t stride = (size_t)n * tpa;
      int r = 0;
      for (int k = lane_g; k < cnt; k += tpa, ++r) {
        const int j = row[(size_t)r * stride];
        const float4 xj = sm.pos[j];
        const float dx = xj.x - xi.x, dy = xj.y - xi.y, dz = xj.z - xi.z;
        const float r2 = dx * dx + dy * dy + dz * dz;
        if (r2 < p.rc2) {
          const float2 c = sm.lj[ti * nsp + __float_as_int(xj.w)];
          const float inv = __fdividef(1.0f, r2);
          const float s2 = c.x * inv;
          const float c6 = s2 * s2 * s2;
          // g = dE/dd = -6 (4 eps) c6 (2 c6 - 1) / r2 * d ; F_i = sum_j g
          const float fs = 6.0f * c.y * c6 * (2.0f * c6 - 1.0f) * inv;
          fx -= fs * dx;
          fy -= fs * dy;
          fz -= fs * dz;
          e += c.y * (c6 * c6 - c6);
          if (VIRIAL) {
            const float h = -0.5f * fs;  // (1/2) d_c g_b = -(1/2) fs d_c d_b
            w0 += h * dx * dx;
            w1 += h * dy * dx;
            w2 += h * dy * dy;
            w3 += h * dz * dx;
            w4 += h * dz * dy;
            w5 += h * dz * dz;
          }
        }
      }
    }
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
    e_acc += 0.5 * (double)e;
    if (VIRIAL) {
      wv[0] += w0; wv[1] += w1; wv[2] += w2; wv[3] += w3; wv[4] += w4; wv[5] += w5;
    }
  }
  return e_acc;
}

template <int INTEGRATOR>
__global__ void __launch_bounds__(kThreads, 1)
md_lj_kernel(kups_md_args a, uint16_t *nl_ws, int *queue, kups_status *status) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  Smem &sm = *reinterpret_cast<Smem *>(smem_raw);
  const int tid = threadIdx.x, nt = blockDim.x;
  float4 *gpos = reinterpret_cast<float4 *>(a.pos);
  float4 *gmom = reinterpret_cast<float4 *>(a.mom);
  float4 *gfrc = reinterpret_cast<float4 *>(a.force);
  uint16_t *nl = nl_ws + (size_t)blockIdx.x * kMaxAtoms * a.neighbor_capacity;
  const int nsp = a.n_species;
  for (int k = tid; k < nsp * nsp; k += nt)
    sm.lj[k] = make_float2(a.lj_table[2 * k], a.lj_table[2 * k + 1]);

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
    // ---- per-system parameters (uniform across the block)
    SysParams p;
    {
      for (int k = 0; k < 6; ++k) p.L[k] = a.tril[6 * (int64_t)s + k];
      const float A = p.L[0], B = p.L[1], C = p.L[2], D = p.L[3], E = p.L[4], F = p.L[5];
      p.inv[0] = 1.0f / A;
      p.inv[2] = 1.0f / C;
      p.inv[5] = 1.0f / F;
      p.inv[1] = -(B * p.inv[0]) / C;
      p.inv[4] = -(E * p.inv[2]) / F;
      p.inv[3] = -((D * p.inv[0]) + (E * p.inv[1])) / F;
      const float rc = a.cutoff[s], skin = a.skin[s], rl = rc + skin;
      p.rc2 = rc * rc;
      p.rl2 = rl * rl;
      p.half_skin = 0.5f * skin;
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
      p.dt = a.dt[s];
      p.c1 = expf(-a.friction[s] * p.dt);
      p.c2 = sqrtf(a.kT[s] * (1.0f - p.c1 * p.c1));
    }
    if (p.K[0] > 2 || p.K[1] > 2 || p.K[2] > 2) {
      if (tid == 0) status_error(status, KUPS_ERR_UNSUPPORTED, s);
      continue;
    }
    for (int c = tid; c < kShiftCount; c += nt) {
      const int ox = c / 25 - 2, oy = (c / 5) % 5 - 2, oz = c % 5 - 2;
      const float f[3] = {(float)ox, (float)oy, (float)oz};
      float x, y, z;
      cart_of(p, f, x, y, z);
      sm.shift_vec[c] = make_float4(x, y, z, 0.f);
    }
    int bad_species = 0;
    for (int i = tid; i < n; i += nt) {
      const float4 q = gpos[a0 + i];
      const int t = __float_as_int(q.w);
      bad_species |= (t < 0) | (t >= nsp);
      sm.pos[i] = q;
      sm.mom[i] = gmom[a0 + i];
      sm.frc[i] = gfrc[a0 + i];
    }
    if (__syncthreads_or(bad_species)) {
      if (tid == 0) status_error(status, KUPS_ERR_INVALID, s);
      continue;
    }
    const int tpa = choose_tpa(n, nt);
    bool ok = rebuild(sm, p, n, tpa, nl, a.neighbor_capacity, status, s);
    if (!ok) continue;
    float wv[6] = {0, 0, 0, 0, 0, 0};
    double pe = 0.0;
    if (!a.forces_valid) {
      if (a.n_steps == 0 && a.virial != nullptr)
        pe = compute_forces<true>(sm, p, n, nsp, tpa, nl, wv);
      else
        pe = compute_forces<false>(sm, p, n, nsp, tpa, nl, wv);
      __syncthreads();
    }
    const float hdt = 0.5f * p.dt;
    for (int step = 0; step < a.n_steps && ok; ++step) {
      const bool last = step == a.n_steps - 1;
      // ---- B A (O A)
      int moved_far = 0;
      for (int i = tid; i < n; i += nt) {
        float4 x = sm.pos[i], m = sm.mom[i], f = sm.frc[i];
        const float inv_m = 1.0f / m.w;
        m.x += f.x * hdt;
        m.y += f.y * hdt;
        m.z += f.z * hdt;
        float dx, dy, dz;
        if (INTEGRATOR == 0) {
          dx = m.x * inv_m * p.dt;
          dy = m.y * inv_m * p.dt;
          dz = m.z * inv_m * p.dt;
        } else {
          dx = m.x * inv_m * hdt;
          dy = m.y * inv_m * hdt;
          dz = m.z * inv_m * hdt;
          float eta[4];
          normal4(a.seed, (uint64_t)(a0 + i), a.step0 + (uint64_t)step, eta);
          const float amp = p.c2 * sqrtf(m.w);
          m.x = p.c1 * m.x + amp * eta[0];
          m.y = p.c1 * m.y + amp * eta[1];
          m.z = p.c1 * m.z + amp * eta[2];
          dx += m.x * inv_m * hdt;
          dy += m.y * inv_m * hdt;
          dz += m.z * inv_m * hdt;
        }
        x.x += dx;
        x.y += dy;
        x.z += dz;
        f.w += sqrtf(dx * dx + dy * dy + dz * dz);
        moved_far |= f.w > p.half_skin;
        sm.pos[i] = x;
        sm.mom[i] = m;
        sm.frc[i] = f;
      }
      const int need = __syncthreads_or(moved_far);
      if (need) {
        if (tid == 0 && a.rebuilds != nullptr) a.rebuilds[s] += 1;
        ok = rebuild(sm, p, n, tpa, nl, a.neighbor_capacity, status, s);
        if (!ok) break;
      } else {
        update_ghosts(sm, n);
        __syncthreads();
      }
      // ---- forces
      const bool want_e = last || a.trace_pe != nullptr;
      if (last && a.virial != nullptr)
        pe = compute_forces<true>(sm, p, n, nsp, tpa, nl, wv);
      else
        pe = compute_forces<false>(sm, p, n, nsp, tpa, nl, wv);
      __syncthreads();
      // ---- B, kinetic energy
      double ke = 0.0;
      for (int i = tid; i < n; i += nt) {
        float4 m = sm.mom[i];
        const float4 f = sm.frc[i];
        m.x += f.x * hdt;
        m.y += f.y * hdt;
        m.z += f.z * hdt;
        sm.mom[i] = m;
        ke += 0.5 * ((double)m.x * m.x + (double)m.y * m.y + (double)m.z * m.z) / (double)m.w;
      }
      if (want_e || a.trace_ke != nullptr) {
        const double pe_tot = block_sum(pe, sm.red);
        const double ke_tot = block_sum(ke, sm.red + 36);
        if (tid == 0) {
          if (a.trace_pe) a.trace_pe[(int64_t)step * a.n_systems + s] = pe_tot;
          if (a.trace_ke) a.trace_ke[(int64_t)step * a.n_systems + s] = ke_tot;
          if (last) {
            a.energy[s] = pe_tot;
            a.kinetic[s] = ke_tot;
          }
        }
      } else {
        __syncthreads();
      }
    }
    if (!ok) continue;
    if (a.n_steps == 0) {
      double ke = 0.0;
      for (int i = tid; i < n; i += nt) {
        const float4 m = sm.mom[i];
        ke += 0.5 * ((double)m.x * m.x + (double)m.y * m.y + (double)m.z * m.z) / (double)m.w;
      }
      const double pe_tot = block_sum(pe, sm.red);
      const double ke_tot = block_sum(ke, sm.red + 36);
      if (tid == 0) {
        a.energy[s] = pe_tot;
        a.kinetic[s] = ke_tot;
      }
    }
    // ---- write back (wrapped positions), virial dE/dtril
    float fw[6] = {0, 0, 0, 0, 0, 0};  // sum_i f_i,a F_i,b for (a, b) in tril order
    for (int i = tid; i < n; i += nt) {
      float4 x = sm.pos[i];
      float f[3];
      wrap_position(p, x, f);
      gpos[a0 + i] = x;
      gmom[a0 + i] = sm.mom[i];
      float4 F = sm.frc[i];
      F.w = 0.f;
      gfrc[a0 + i] = F;
      fw[0] += f[0] * F.x;
      fw[1] += f[1] * F.x;
      fw[2] += f[1] * F.y;
      fw[3] += f[2] * F.x;
      fw[4] += f[2] * F.y;
      fw[5] += f[2] * F.z;
    }
    if (a.virial != nullptr) {
      // X_ab = sum_c (L^-1)_{ca} W_cb ; W symmetric from wv = [xx, yx, yy, zx, zy, zz]
      double W[3][3];
      double acc[6];
      for (int k = 0; k < 6; ++k) acc[k] = block_sum((double)wv[k], sm.red + 0), __syncthreads();
      W[0][0] = acc[0];
      W[1][0] = W[0][1] = acc[1];
      W[1][1] = acc[2];
      W[2][0] = W[0][2] = acc[3];
      W[2][1] = W[1][2] = acc[4];
      W[2][2] = acc[5];
      double fwt[6];
      for (int k = 0; k < 6; ++k) fwt[k] = block_sum((double)fw[k], sm.red + 36), __syncthreads();
      // inverse (float64 from the float32 cell)
      const double A = p.L[0], B = p.L[1], C = p.L[2], D = p.L[3], E = p.L[4], F = p.L[5];
      double Li[3][3] = {{1.0 / A, 0, 0}, {0, 1.0 / C, 0}, {0, 0, 1.0 / F}};
      Li[1][0] = -(B * Li[0][0]) / C;
      Li[2][1] = -(E * Li[1][1]) / F;
      Li[2][0] = -((D * Li[0][0]) + (E * Li[1][0])) / F;
      const int ia[6] = {0, 1, 1, 2, 2, 2}, ib[6] = {0, 0, 1, 0, 1, 2};
      if (tid == 0) {
        for (int k = 0; k < 6; ++k) {
          double x = 0.0;
          for (int c = 0; c < 3; ++c) x += Li[c][ia[k]] * W[c][ib[k]];
          a.virial[6 * (int64_t)s + k] = x + fwt[k];
        }
      }
    }
    __syncthreads();
  }
}

}  // namespace
}  // namespace kups

using namespace kups;

extern "C" int32_t kups_lj_md_max_atoms(void) { return kMaxAtoms; }

extern "C" size_t kups_lj_md_workspace_bytes(const kups_md_args *a) {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int ctas = a->n_ctas > 0 ? a->n_ctas : (sms > 0 ? sms : 1);
  return 256 + (size_t)ctas * kMaxAtoms * (size_t)a->neighbor_capacity * sizeof(uint16_t) + 256;
}

extern "C" int32_t kups_lj_md_run(const kups_md_args *a, void *workspace, size_t ws_bytes,
                                  kups_status *status, void *stream_) {
  cudaStream_t stream = (cudaStream_t)stream_;
  if (a == nullptr || a->n_systems < 0 || a->n_steps < 0 || a->n_species <= 0 ||
      a->n_species > kMaxSpecies || a->neighbor_capacity <= 0 || a->neighbor_capacity > 4096 ||
      a->neighbor_capacity % 16 != 0 ||
      (a->integrator != 0 && a->integrator != 1))
    return KUPS_ERR_INVALID;
  if (ws_bytes < kups_lj_md_workspace_bytes(a)) return KUPS_ERR_INVALID;
  if (a->n_systems == 0) return KUPS_OK;
  int dev = 0, sms = 0;
  KUPS_CUDA_TRY(cudaGetDevice(&dev));
  KUPS_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const int ctas = a->n_ctas > 0 ? a->n_ctas : sms;
  const int threads = a->block_threads > 0 ? a->block_threads : kThreads;
  if (threads % 32 != 0 || threads > kThreads || threads < 64) return KUPS_ERR_INVALID;
  int *queue = reinterpret_cast<int *>(((uintptr_t)workspace + 255) & ~uintptr_t(255));
  uint16_t *nl = reinterpret_cast<uint16_t *>(reinterpret_cast<char *>(queue) + 256);
  KUPS_CUDA_TRY(cudaMemsetAsync(queue, 0, sizeof(int), stream));
  const size_t smem = sizeof(Smem);
  if (a->integrator == 0) {
    KUPS_CUDA_TRY(cudaFuncSetAttribute(md_lj_kernel<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    md_lj_kernel<0><<<ctas, threads, smem, stream>>>(*a, nl, queue, status);
  } else {
    KUPS_CUDA_TRY(cudaFuncSetAttribute(md_lj_kernel<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    md_lj_kernel<1><<<ctas, threads, smem, stream>>>(*a, nl, queue, status);
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
