// Batched grand-canonical Monte Carlo of rigid molecules in rigid frameworks.
//
// Replaces, per MC step and for every system at once, MCMCPropagator.__call__
// (src/kups/core/propagator.py:312-345) with the moves of
// make_gcmc_mcmc_propagator (src/kups/mcmc/moves.py:1078-1230: translation
// :222-244, rotation about the centre of mass :247-265 with :158-197,
// reinsertion :268-295, insertion :573-675, deletion :678-773), the
// incremental energy of LocalGraphSumComposer (src/kups/potential/common/graph.py:419-453)
// over the changed pairs of neighborlist_changes (src/kups/core/neighborlist.py:1425-1515),
// the incremental structure factor (src/kups/potential/classical/ewald.py:442-486,
// 604-657), the global LJ tail correction (lennard_jones.py:276-315), the
// muVT acceptance (src/kups/mcmc/probability.py:98-225) and
// acceptance_target_schedule (src/kups/core/parameter_scheduler.py:161-208).
//
// One CTA owns one system for all n_steps (systems are independent); the
// move kind of a step is drawn from a counter that every CTA evaluates alike,
// so all systems make the same kind of move in a step, as propose_mixed does
// (propagator.py:244-273), and so is the insert/delete coin (moves.py:1217).
// Randomness: Philox4x32-10 keyed by the seed, stream = system, counter = step.
//
// Pair enumeration follows the reference neighbour list exactly
// (neighborlist.py:453-624): with n_a = odd ceil(2 rc / w_a) images per axis,
// if prod(n_a) == 1 the shift is round(f_i - f_j); otherwise every offset of
// the centred n_x x n_y x n_z grid is tried (no minimum image on axes with
// n_a == 1), and intramolecular pairs are excluded on the minimum image only.
// Pair arithmetic float32, energy differences and the log acceptance float64.
#include "common.cuh"
#include "proposal.cuh"

namespace kups {
namespace {

constexpr int kDefaultThreads = 128;  // threads per CTA unless kups_gcmc_args.block_threads says otherwise
constexpr int kMaxApm = 8;       // atoms per molecule
constexpr int kMaxSpeciesMC = 8;
constexpr int kMaxKVec = 4096;
constexpr int kMaxImg = 5;       // odd image count per axis
constexpr int kMaxM = 16;        // |n_a| of a k vector
constexpr int kTab = 2 * kMaxM + 1;
constexpr int kMaxNearGroups = 512;  // host groups of 32 atoms a system's near lists can hold

struct ImgCfg {
  int n[3];
  int image_mode;
  float rc2;
};

struct StepShared {
  float4 old_pos[kMaxApm];  // (x, y, z, species bits)
  float4 new_pos[kMaxApm];
  float q[kMaxApm];
  int kind;      // 0 translate, 1 rotate, 2 reinsert, 3 insert, 4 delete
  int mol;       // molecule slot
  int has_old, has_new;
  double de_real;
  double de_recip;
  int accept;
  double log_p;
  double de_total;
  double ln_ratio;  // log proposal ratio of the learned insertion density (0 when uniform)
  // host energy cache (kups_gcmc_args.host_cache): keys of the old and new positions, whether
  // the old molecule's entry matched, and its energy
  unsigned long long old_key, new_key;
  int cache_hit;
  double e_host_old;
};

// 64-bit key of a molecule's atom positions (FNV-1a over the float bits; never 0, which marks
// an empty cache entry).
__device__ inline unsigned long long position_key(const float4 *p, int apm) {
  unsigned long long h = 0xcbf29ce484222325ull;
  for (int i = 0; i < apm; ++i) {
    const uint32_t w[3] = {__float_as_uint(p[i].x), __float_as_uint(p[i].y), __float_as_uint(p[i].z)};
    for (int k = 0; k < 3; ++k) h = (h ^ w[k]) * 0x100000001b3ull;
  }
  return h | 1ull;
}

__device__ inline void frac32(const float inv[6], float x, float y, float z, float f[3]) {
  f[0] = (x * inv[0] + y * inv[1]) + z * inv[3];
  f[1] = y * inv[2] + z * inv[4];
  f[2] = z * inv[5];
}

__device__ inline void cart32(const float L[6], const float f[3], float c[3]) {
  c[0] = (f[0] * L[0] + f[1] * L[1]) + f[2] * L[3];
  c[1] = f[1] * L[2] + f[2] * L[4];
  c[2] = f[2] * L[5];
}

__device__ inline void wrap32(const float L[6], const float inv[6], float c[3]) {
  float f[3];
  frac32(inv, c[0], c[1], c[2], f);
  for (int a = 0; a < 3; ++a) f[a] = (f[a] + 0.5f) - floorf(f[a] + 0.5f) - 0.5f;
  cart32(L, f, c);
}

struct F3 {
  double v[3];
};

// Fractional coordinates of a molecule's atom mean (atoms unwrapped against atom 0).
__device__ inline F3 anchor_frac(const float4 *p, int apm, const float L[6], const float inv[6]) {
  float m[3] = {0.f, 0.f, 0.f};
  for (int i = 0; i < apm; ++i) {
    float d[3] = {p[i].x - p[0].x, p[i].y - p[0].y, p[i].z - p[0].z};
    wrap32(L, inv, d);
    for (int c = 0; c < 3; ++c) m[c] += d[c];
  }
  float f[3];
  frac32(inv, p[0].x + m[0] / apm, p[0].y + m[1] / apm, p[0].z + m[2] / apm, f);
  return F3{{(double)f[0], (double)f[1], (double)f[2]}};
}

__device__ inline U4 rng4(uint64_t seed, uint64_t stream, uint64_t ctr) {
  U4 c{(uint32_t)ctr, (uint32_t)(ctr >> 32), (uint32_t)stream, (uint32_t)(stream >> 32)};
  return philox4x32_10(c, (uint32_t)seed, (uint32_t)(seed >> 32));
}

__device__ inline float u01(uint32_t v) { return (float)(v >> 8) * (1.0f / 16777216.0f); }  // [0, 1)

// Shoemake uniform rotation (quaternion.py:71-98): w, x, y, z
__device__ inline void shoemake(float u1, float u2, float u3, float q[4]) {
  float s2, c2, s3, c3;
  sincospif(2.0f * u2, &s2, &c2);
  sincospif(2.0f * u3, &s3, &c3);
  const float a = sqrtf(1.0f - u1), b = sqrtf(u1);
  q[0] = a * s2;
  q[1] = a * c2;
  q[2] = b * s3;
  q[3] = b * c3;
}

// q ** e (quaternion.py:241-263): scale the rotation angle by e
__device__ inline void qpow(const float qin[4], float e, float q[4]) {
  float w = qin[0], x = qin[1], y = qin[2], z = qin[3];
  if (w < 0.f) {
    w = -w; x = -x; y = -y; z = -z;
  }
  const float angle = 2.0f * acosf(fminf(fmaxf(w, -1.0f), 1.0f));
  const float sh = sqrtf(x * x + y * y + z * z);
  const float inv = sh > 1e-10f ? 1.0f / sh : 1.0f;
  const float ax = x * inv, ay = y * inv, az = z * inv;
  float s, c;
  sincosf(0.5f * angle * e, &s, &c);
  q[0] = c;
  q[1] = ax * s;
  q[2] = ay * s;
  q[3] = az * s;
}

// rotate v by the matrix of q (quaternion.py:266-285), v' = R v
__device__ inline void qrot(const float q[4], const float v[3], float o[3]) {
  const float w = q[0], x = q[1], y = q[2], z = q[3];
  const float x2 = x * x, y2 = y * y, z2 = z * z, w2 = w * w;
  const float xy = x * y, zw = z * w, xz = x * z, yw = y * w, yz = y * z, xw = x * w;
  o[0] = (x2 - y2 - z2 + w2) * v[0] + 2.f * (xy - zw) * v[1] + 2.f * (xz + yw) * v[2];
  o[1] = 2.f * (xy + zw) * v[0] + (-x2 + y2 - z2 + w2) * v[1] + 2.f * (yz - xw) * v[2];
  o[2] = 2.f * (xz - yw) * v[0] + 2.f * (yz + xw) * v[1] + (-x2 - y2 + z2 + w2) * v[2];
}

__device__ inline float pair_u(float r2, int ti, int tj, float qq, const float2 *lj, int nsp,
                               const ImgCfg &lj_img, const ImgCfg &ew_img, float alpha, float ke,
                               bool in_lj, bool in_ew) {
  // one reciprocal square root serves both terms (a few ulp; IEEE division and square
  // root would each cost a multi-instruction sequence per pair)
  const float ir = rsqrtf(r2);
  float e = 0.f;
  if (in_lj && r2 < lj_img.rc2) {
    const float2 c = lj[ti * nsp + tj];
    const float s2 = c.x * (ir * ir);
    const float c6 = s2 * s2 * s2;
    e += c.y * (c6 * c6 - c6);
  }
  if (in_ew && r2 < ew_img.rc2 && qq != 0.f) {
    const float r = r2 * ir;
    e += ke * qq * erfc_cheb(alpha * r) * ir;
  }
  return e;
}

// Sum over the reference's image set of the pair (a at fa, j at fj) for one
// term configuration; `excl` drops the minimum image (same molecule).
__device__ inline float pair_images(const float L[6], const float fa[3], const float fj[3], int ti,
                                    int tj, float qq, const float2 *lj, int nsp, const ImgCfg &li,
                                    const ImgCfg &ei, float alpha, float ke, bool excl) {
  float d0[3] = {fa[0] - fj[0], fa[1] - fj[1], fa[2] - fj[2]};
  const float ms[3] = {rintf(d0[0]), rintf(d0[1]), rintf(d0[2])};
  float e = 0.f;
  // LJ and Ewald may use different image sets; enumerate the union
  const bool any_img = li.image_mode || ei.image_mode;
  const bool same = li.image_mode == ei.image_mode && li.n[0] == ei.n[0] && li.n[1] == ei.n[1] &&
                    li.n[2] == ei.n[2];
  if (any_img && same) {
    const int hx = li.n[0] / 2, hy = li.n[1] / 2, hz = li.n[2] / 2;
    for (int ox = -hx; ox <= hx; ++ox)
      for (int oy = -hy; oy <= hy; ++oy)
        for (int oz = -hz; oz <= hz; ++oz) {
          if (excl && ms[0] == (float)ox && ms[1] == (float)oy && ms[2] == (float)oz) continue;
          float d[3] = {d0[0] - ox, d0[1] - oy, d0[2] - oz}, c[3];
          cart32(L, d, c);
          e += pair_u(c[0] * c[0] + c[1] * c[1] + c[2] * c[2], ti, tj, qq, lj, nsp, li, ei, alpha, ke, true, true);
        }
    return e;
  }
  if (!any_img) {
    if (excl) return 0.f;
    float d[3] = {d0[0] - ms[0], d0[1] - ms[1], d0[2] - ms[2]}, c[3];
    cart32(L, d, c);
    const float r2 = c[0] * c[0] + c[1] * c[1] + c[2] * c[2];
    return pair_u(r2, ti, tj, qq, lj, nsp, li, ei, alpha, ke, true, true);
  }
  const int hx = max(li.n[0], ei.n[0]) / 2, hy = max(li.n[1], ei.n[1]) / 2, hz = max(li.n[2], ei.n[2]) / 2;
  for (int ox = -hx; ox <= hx; ++ox)
    for (int oy = -hy; oy <= hy; ++oy)
      for (int oz = -hz; oz <= hz; ++oz) {
        const float o[3] = {(float)ox, (float)oy, (float)oz};
        // per term: is this offset in its set, and what shift does it imply
        bool in_l, in_e;
        float sl[3], se[3];
        in_l = true;
        in_e = true;
        if (li.image_mode) {
          in_l = abs(ox) <= li.n[0] / 2 && abs(oy) <= li.n[1] / 2 && abs(oz) <= li.n[2] / 2;
          sl[0] = o[0]; sl[1] = o[1]; sl[2] = o[2];
        } else {
          in_l = ox == 0 && oy == 0 && oz == 0;
          sl[0] = ms[0]; sl[1] = ms[1]; sl[2] = ms[2];
        }
        if (ei.image_mode) {
          in_e = abs(ox) <= ei.n[0] / 2 && abs(oy) <= ei.n[1] / 2 && abs(oz) <= ei.n[2] / 2;
          se[0] = o[0]; se[1] = o[1]; se[2] = o[2];
        } else {
          in_e = ox == 0 && oy == 0 && oz == 0;
          se[0] = ms[0]; se[1] = ms[1]; se[2] = ms[2];
        }
        if (in_l) {
          const bool is_min = (sl[0] == ms[0]) && (sl[1] == ms[1]) && (sl[2] == ms[2]);
          if (!(excl && is_min)) {
            float d[3] = {d0[0] - sl[0], d0[1] - sl[1], d0[2] - sl[2]}, c[3];
            cart32(L, d, c);
            e += pair_u(c[0] * c[0] + c[1] * c[1] + c[2] * c[2], ti, tj, qq, lj, nsp, li, ei, alpha, ke,
                        true, false);
          }
        }
        if (in_e) {
          const bool is_min = (se[0] == ms[0]) && (se[1] == ms[1]) && (se[2] == ms[2]);
          if (!(excl && is_min)) {
            float d[3] = {d0[0] - se[0], d0[1] - se[1], d0[2] - se[2]}, c[3];
            cart32(L, d, c);
            e += pair_u(c[0] * c[0] + c[1] * c[1] + c[2] * c[2], ti, tj, qq, lj, nsp, li, ei, alpha, ke,
                        false, true);
          }
        }
      }
  return e;
}

// Optional phase timing (kups_gcmc_args::profile): thread 0 adds the clock cycles since the
// last mark to counter k; with profiling on, a barrier closes the phase first so a span covers
// every thread's share of it.
__device__ __forceinline__ void gcmc_mark(unsigned long long *prof, int k, long long &t0) {
  if (prof == nullptr) return;
  __syncthreads();
  if (threadIdx.x == 0) {
    const long long t = clock64();
    atomicAdd(&prof[k], (unsigned long long)(t - t0));
    t0 = t;
  }
}

// kThreads per CTA, 896 / kThreads resident CTAs per SM (at most 73 registers a thread): at 128
// threads 1024 replicas run in one wave on 152 SMs, each CTA keeping its system for all n_steps.
template <int kThreads>
__global__ void __launch_bounds__(kThreads, 896 / kThreads) gcmc_kernel(kups_gcmc_args a, kups_status *status) {
  __shared__ StepShared sh;
  __shared__ float2 lj[kMaxSpeciesMC * kMaxSpeciesMC];
  // per-axis phase tables of the step's moved atoms: e^{2 pi i n f_a}, |n| <= kMaxM
  extern __shared__ float2 ph[];  // [2 apm][3][kTab]
  __shared__ double red[40];
  __shared__ float Lf[6], If[6];
  __shared__ float4 mfa[2 * kMaxApm];  // moved atoms (old, then new): fractional xyz, species bits
  __shared__ float mq[2 * kMaxApm];
  __shared__ int mon[2 * kMaxApm];
  // near-group lists of the step (minimum-image path with group bounds): for the new end and
  // for the old end of the move, the host groups within reach of any of its atoms and, per
  // group, which moved atoms reach it
  __shared__ uint16_t near_g[2][kMaxNearGroups], near_m[2][kMaxNearGroups];
  __shared__ float gsum[2][kMaxNearGroups];  // per end and host group: its pair energy (0 if skipped)
  __shared__ int near_n[2], iscan[32];
  const int s = blockIdx.x;
  const int tid = threadIdx.x;
  const int apm = a.atoms_per_mol;
  const int nsp = a.n_species;
  const int nk = a.n_kvecs;
  // the system's mutable scalars live in shared memory for the launch (read once, written back
  // at the end), so no step waits on a global round trip for them; ss.tail_b / ss.tail_c give
  // the tail correction as a function of the molecule count N (coef_ab = (8/3) pi eps sigma^3
  // [(sigma/rc)^9 / 3 - (sigma/rc)^3] / V, masked):
  //   E_tail(N) = sum_ab coef_ab c_a c_b, c = fw + N motif  =>  E_tail(N) - E_tail(0) = b N + c N^2
  __shared__ struct {
    double energy, tail_b, tail_c, self_excl;
    int n_mol;
    float width[4], width_max[4];
    uint32_t hist[4][4];
    int hist_idx[4];
    int attempted[5], accepted[5];  // this launch's counts
  } ss;
  for (int k = tid; k < nsp * nsp; k += kThreads)
    lj[k] = make_float2(a.lj_table[2 * k], a.lj_table[2 * k + 1]);
  if (tid == 0) {
    const Tril64 L = load_tril64(a.tril + 6 * (int64_t)s);
    const Tril64 inv = inverse_tril64(L);
    for (int k = 0; k < 6; ++k) {
      Lf[k] = (float)L.t[k];
      If[k] = (float)inv.t[k];
    }
    ss.energy = a.energy[s];
    ss.n_mol = a.n_mol[s];
    for (int k = 0; k < 4; ++k) {
      ss.width[k] = a.width[s * 4 + k];
      ss.width_max[k] = a.width_max[s * 4 + k];
      ss.hist_idx[k] = a.history_index[s * 4 + k];
      for (int w = 0; w < 4; ++w) ss.hist[k][w] = a.history[((int64_t)s * 4 + k) * 4 + w];
    }
    for (int k = 0; k < 5; ++k) ss.attempted[k] = ss.accepted[k] = 0;
    ss.self_excl = a.self_energy_mol[s] + a.exclusion_energy_mol[s];
    double tb = 0.0, tcq = 0.0;
    if (a.tail_coef != nullptr) {
      const double *tc = a.tail_coef + (int64_t)s * nsp * nsp;
      for (int p = 0; p < nsp; ++p)
        for (int q = 0; q < nsp; ++q) {
          const double fp = a.fw_species_count[s * nsp + p], fq = a.fw_species_count[s * nsp + q];
          const double mp = a.motif_species_count[p], mq_ = a.motif_species_count[q];
          tb += tc[p * nsp + q] * (fp * mq_ + mp * fq);
          tcq += tc[p * nsp + q] * (mp * mq_);
        }
    }
    ss.tail_b = tb;
    ss.tail_c = tcq;
  }
  __syncthreads();
  // image configurations of the two terms (neighborlist.py:461-466)
  ImgCfg li, ei;
  float wdt[3];  // perpendicular widths
  {
    const Tril64 L = load_tril64(a.tril + 6 * (int64_t)s);
    double w[3];
    perpendicular_widths64(L, w);
    for (int d = 0; d < 3; ++d) wdt[d] = (float)w[d];
    const double rcs[2] = {a.rc_lj[s], a.rc_ew[s]};
    for (int t = 0; t < 2; ++t) {
      ImgCfg &c = t == 0 ? li : ei;
      int prod = 1;
      for (int d = 0; d < 3; ++d) {
        int n = (int)ceil(2.0 * rcs[t] / w[d]);
        n = n < 1 ? 1 : n;
        if (n % 2 == 0) n += 1;
        if (n > kMaxImg) {
          n = kMaxImg;
          if (tid == 0) status_error(status, KUPS_ERR_UNSUPPORTED, s);
        }
        c.n[d] = n;
        prod *= n;
      }
      c.image_mode = prod > 1;
      c.rc2 = (float)(rcs[t] * rcs[t]);
    }
  }
  const bool min_image = !li.image_mode && !ei.image_mode;
  const float rc2_any = fmaxf(li.rc2, ei.rc2), rc_any = sqrtf(rc2_any);
  const float4 *grp = reinterpret_cast<const float4 *>(a.fw_group);
  const int lane = tid & 31;
  const float alpha = (float)a.alpha[s];
  const float ke = (float)a.coulomb_k;
  const double kT = a.kT[s];
  const double volume = fabs(a.tril[6 * (int64_t)s] * a.tril[6 * (int64_t)s + 2] * a.tril[6 * (int64_t)s + 5]);
  const double inv_kT = 1.0 / kT;
  const double lnfv = a.log_activity[s] + log(volume);  // ln(f V / kT), once per launch
  const int fw0 = a.fw_start[s], fwn = a.fw_count[s];
  float4 *gpos = reinterpret_cast<float4 *>(a.guest_pos) + (int64_t)s * a.max_mol * apm;
  const float4 *motif = reinterpret_cast<const float4 *>(a.motif_pos);
  const float4 *fwp = reinterpret_cast<const float4 *>(a.fw_pos);
  double *sk = a.structure_factor + (int64_t)s * nk * 2;
  const double *pk = a.prefactor + (int64_t)s * nk;
  const int32_t *kn = a.kvec_n + (int64_t)s * nk * 3;
  // scratch per system (arrays of S x n_k after a reserved first one): float32 mirrors of
  // S(k) (re-derived from the float64 value at every commit) and of P(k) with the packed
  // table offsets of the k vectors.  Reading the mirrors keeps float64<->float32
  // conversions (float64-pipe work) off the per-step path.
  const int64_t snk = (int64_t)a.n_systems * nk;
  float2 *sk32 = reinterpret_cast<float2 *>(a.workspace) + snk + (int64_t)s * nk;
  // (P, packed k); one table for all systems with k_shared (every CTA writes the same values)
  float2 *pk32 = reinterpret_cast<float2 *>(a.workspace) + 2 * snk + (a.k_shared ? 0 : (int64_t)s * nk);
  // the phase tables hold |n_a| <= kMaxM: a system with a larger k vector is refused
  {
    int bad = 0;
    for (int k = tid; k < nk; k += kThreads) {
      const int n0 = kn[3 * k], n1 = kn[3 * k + 1], n2 = kn[3 * k + 2];
      bad |= (abs(n0) > kMaxM) | (abs(n1) > kMaxM) | (abs(n2) > kMaxM);
      const uint32_t packed = (uint32_t)(n0 + kMaxM) | ((uint32_t)(n1 + kMaxM) << 8) | ((uint32_t)(n2 + kMaxM) << 16);
      pk32[k] = make_float2((float)pk[k], __uint_as_float(packed));
      sk32[k] = make_float2((float)sk[2 * k], (float)sk[2 * k + 1]);
    }
    if (__syncthreads_or(bad)) {
      if (tid == 0) status_error(status, KUPS_ERR_UNSUPPORTED, s);
      return;
    }
  }
  const bool learned = a.proposal_node != nullptr;
  // the host energy cache serves the minimum-image path, where a molecule's host energy is a
  // function of its positions alone
  const bool use_cache = a.host_cache != nullptr && min_image;
  double ob[5] = {0.0, 0.0, 0.0, 0.0, 0.0};  // thread 0: this launch's U, N, U N, N^2, U^2 sums
  unsigned long long *prof = a.profile;
  long long t0 = clock64();
  for (int step = 0; step < a.n_steps; ++step) {
    const uint64_t ctr = a.step0 + (uint64_t)step;
    // ---------------------------------------------------------------- proposal (thread 0)
    if (tid == 0) {
      const int nmol = ss.n_mol;
      int kind;
      if (a.proposals != nullptr) {
        kind = a.proposals[s].kind;
      } else {
        const U4 g = rng4(a.seed, 0, ctr);  // shared by all systems
        const float u = u01(g.x);
        kind = 0;
        while (kind < 3 && u >= a.move_cum[kind]) ++kind;  // 0..3 (3 = exchange)
        if (kind == 3) kind = (g.y & 1u) ? 4 : 3;          // shared insert / delete coin
      }
      // per-system draws of this step: counters 8 ctr + 0 .. 4 (selection, rotation,
      // offset, translation normals, acceptance)
      const U4 r1 = rng4(a.seed, 1 + (uint64_t)s, 8 * ctr);
      const U4 r2 = rng4(a.seed, 1 + (uint64_t)s, 8 * ctr + 1);
      const U4 r3 = rng4(a.seed, 1 + (uint64_t)s, 8 * ctr + 2);
      sh.kind = kind;
      sh.has_old = 0;
      sh.has_new = 0;
      sh.ln_ratio = 0.0;
      int mol = -1;
      if (kind == 3) {
        mol = nmol;  // next free slot
        if (nmol < a.max_mol) sh.has_new = 1;
        else status_capacity(status, KUPS_CAP_ATOMS, (int64_t)(nmol + 1) * apm, s);
      } else if (nmol > 0) {
        mol = a.proposals != nullptr ? a.proposals[s].mol : (int)(r1.x % (uint32_t)nmol);
        if (mol >= 0 && mol < nmol) {
          sh.has_old = 1;
          sh.has_new = kind != 4;
        } else {
          mol = -1;  // an out-of-range replayed proposal changes nothing
        }
      }
      sh.mol = mol;
      for (int i = 0; i < apm; ++i) sh.q[i] = a.motif_charge[i];
      if (sh.has_old)
        for (int i = 0; i < apm; ++i) sh.old_pos[i] = gpos[mol * apm + i];
      if (sh.has_new) {
        if (a.proposals != nullptr) {
          for (int i = 0; i < apm; ++i) sh.new_pos[i] = reinterpret_cast<const float4 *>(a.proposals[s].pos)[i];
        } else if (kind == 0) {  // translation: N(0, 1) * width per axis, wrap
          float eta[4];
          normal4(a.seed, 1 + (uint64_t)s, 8 * ctr + 3, eta);
          const float w = ss.width[0];
          for (int i = 0; i < apm; ++i) {
            const float4 p = sh.old_pos[i];
            float c[3] = {p.x + eta[0] * w, p.y + eta[1] * w, p.z + eta[2] * w};
            wrap32(Lf, If, c);
            sh.new_pos[i] = make_float4(c[0], c[1], c[2], p.w);
          }
        } else if (kind == 1 || kind == 2) {  // rotation about the COM (q ** w), reinsertion
          float com[3] = {0.f, 0.f, 0.f};
          const float4 r0 = sh.old_pos[0];
          float rel[kMaxApm][3];
          for (int i = 0; i < apm; ++i) {
            const float4 p = sh.old_pos[i];
            float d[3] = {p.x - r0.x, p.y - r0.y, p.z - r0.z};
            wrap32(Lf, If, d);
            for (int c = 0; c < 3; ++c) com[c] += d[c];
          }
          for (int c = 0; c < 3; ++c) com[c] = com[c] / apm;
          float cm[3] = {com[0] + r0.x, com[1] + r0.y, com[2] + r0.z};
          wrap32(Lf, If, cm);
          for (int i = 0; i < apm; ++i) {
            const float4 p = sh.old_pos[i];
            float d[3] = {p.x - cm[0], p.y - cm[1], p.z - cm[2]};
            wrap32(Lf, If, d);
            for (int c = 0; c < 3; ++c) rel[i][c] = d[c];
          }
          float q0[4], q[4];
          shoemake(u01(r2.x), u01(r2.y), u01(r2.z), q0);
          if (kind == 1) qpow(q0, ss.width[1], q);
          else for (int c = 0; c < 4; ++c) q[c] = q0[c];
          float shift[3] = {0.f, 0.f, 0.f};
          if (kind == 2) {
            const float fo[3] = {u01(r3.x), u01(r3.y), u01(r3.z)};
            cart32(Lf, fo, shift);
          }
          for (int i = 0; i < apm; ++i) {
            float o[3];
            qrot(q, rel[i], o);
            float c[3] = {o[0] + cm[0], o[1] + cm[1], o[2] + cm[2]};
            wrap32(Lf, If, c);
            if (kind == 2) {
              c[0] += shift[0];
              c[1] += shift[1];
              c[2] += shift[2];
              wrap32(Lf, If, c);
            }
            sh.new_pos[i] = make_float4(c[0], c[1], c[2], sh.old_pos[i].w);
          }
        } else if (kind == 3) {  // insertion: template @ R + uniform offset, wrap
          float q[4];
          shoemake(u01(r2.x), u01(r2.y), u01(r2.z), q);
          float fo[3] = {u01(r3.x), u01(r3.y), u01(r3.z)};
          float centre[3] = {0.f, 0.f, 0.f};
          if (learned) {
            // the template's atom mean goes to a point drawn from the grid density
            const double ua[3] = {u32_open0(r3.x), u32_open0(r3.y), u32_open0(r3.z)};
            double fd[3];
            sh.ln_ratio = -grid_sample(a.proposal_node, a.proposal_cdf, a.proposal_grid, u53(r1.x, r1.y),
                                       u53(r1.z, r1.w), ua, fd);
            for (int c = 0; c < 3; ++c) fo[c] = (float)fd[c];
            for (int i = 0; i < apm; ++i) {
              centre[0] += motif[i].x / apm;
              centre[1] += motif[i].y / apm;
              centre[2] += motif[i].z / apm;
            }
          }
          float shift[3];
          cart32(Lf, fo, shift);
          for (int i = 0; i < apm; ++i) {
            const float4 m = motif[i];
            const float v[3] = {m.x - centre[0], m.y - centre[1], m.z - centre[2]};
            float o[3];
            qrot(q, v, o);
            float c[3] = {o[0] + shift[0], o[1] + shift[1], o[2] + shift[2]};
            wrap32(Lf, If, c);
            sh.new_pos[i] = make_float4(c[0], c[1], c[2], m.w);
          }
        }
      }
      if (learned && a.proposals != nullptr && kind == 3 && sh.has_new)
        sh.ln_ratio = -grid_log_q(a.proposal_node, a.proposal_cdf, a.proposal_grid,
                                  anchor_frac(sh.new_pos, apm, Lf, If).v);
      if (learned && kind == 4 && sh.has_old)
        sh.ln_ratio = grid_log_q(a.proposal_node, a.proposal_cdf, a.proposal_grid,
                                 anchor_frac(sh.old_pos, apm, Lf, If).v);
      sh.cache_hit = 0;
      sh.e_host_old = 0.0;
      if (use_cache) {
        sh.old_key = sh.has_old ? position_key(sh.old_pos, apm) : 0ull;
        sh.new_key = sh.has_new ? position_key(sh.new_pos, apm) : 0ull;
        if (sh.has_old) {
          const double *ent = a.host_cache + ((int64_t)s * a.max_mol + mol) * 2;
          if (__double_as_longlong(ent[1]) == (long long)sh.old_key) {
            sh.cache_hit = 1;
            sh.e_host_old = ent[0];
          }
        }
      }
    }
    __syncthreads();
    const int has_old = sh.has_old, has_new = sh.has_new, mol = sh.mol, kind = sh.kind;
    // ---------------------------------------------------------------- real space: moved vs others
    float e_acc = 0.f;
    const int nmol = ss.n_mol;
    const int n_other = fwn + nmol * apm;
    // moved atoms (old state, then new) in fractional coordinates, staged once per step
    if (tid < 2 * apm) {
      const int st = tid / apm, i = tid % apm;
      const float4 p = st == 0 ? sh.old_pos[i] : sh.new_pos[i];
      float f[3];
      frac32(If, p.x, p.y, p.z, f);
      mfa[tid] = make_float4(f[0], f[1], f[2], p.w);
      mq[tid] = sh.q[i];
      mon[tid] = st == 0 ? has_old : has_new;
    }
    __syncthreads();
    gcmc_mark(prof, 0, t0);
    const int nm = 2 * apm;
    float e_host_new = 0.f, e_host_old = 0.f;  // minimum-image path: host terms, by end
    const int cache_hit = sh.cache_hit;
    if (min_image) {
      // every axis has one image: the pair is taken at its minimum image, one rounding
      // per moved atom and partner.  Host atoms go by warp in aligned groups of 32; a
      // group is skipped for a moved atom when, along some axis a, the circular distance
      // of the atom's fractional coordinate to the group's centre minus the group's half
      // extent, times the width w_a, reaches the cutoff (|cart(d)| >= |d_a| w_a, and the
      // rounded image's d_a is the circular distance, so no pair within it is dropped).
      unsigned on_mask = 0u;  // moved atoms to take against the host (old ones unless cached)
      for (int m = 0; m < nm; ++m) on_mask |= (mon[m] && !(m < apm && cache_hit)) ? (1u << m) : 0u;
      const int n_groups = (fwn + 31) >> 5;
      if (n_groups <= kMaxNearGroups) {
        // 1. every (group, moved atom) bound at once (without group bounds every group is near),
        //    then the near groups of each end compacted in a fixed order (a thread's groups t,
        //    t + threads, ... after those of lower threads)
        unsigned gm[kMaxNearGroups / 64 + 1];
        int cnt_new = 0, cnt_old = 0, slot = 0;
        for (int g = tid; g < n_groups; g += kThreads, ++slot) {
          gsum[0][g] = 0.f;
          gsum[1][g] = 0.f;
          if (grp == nullptr) {
            gm[slot] = on_mask;
            const unsigned old_bits = (1u << apm) - 1u;
            cnt_old += (on_mask & old_bits) != 0u;
            cnt_new += (on_mask & ~old_bits) != 0u;
            continue;
          }
          const int gi = (fw0 >> 5) + g;
          const float4 c = grp[2 * gi], h = grp[2 * gi + 1];
          unsigned mk = 0u;
          for (unsigned mm = on_mask; mm != 0u; mm &= mm - 1u) {
            const int m = __ffs(mm) - 1;
            const float4 fa = mfa[m];
            float dx = fa.x - c.x, dy = fa.y - c.y, dz = fa.z - c.z;
            dx = fabsf(dx - rintf(dx));
            dy = fabsf(dy - rintf(dy));
            dz = fabsf(dz - rintf(dz));
            const float sep = fmaxf(fmaxf(fmaxf(dx - h.x, 0.f) * wdt[0], fmaxf(dy - h.y, 0.f) * wdt[1]),
                                    fmaxf(dz - h.z, 0.f) * wdt[2]);
            if (sep < rc_any) mk |= 1u << m;
          }
          gm[slot] = mk;
          const unsigned old_bits = (1u << apm) - 1u;
          cnt_old += (mk & old_bits) != 0u;
          cnt_new += (mk & ~old_bits) != 0u;
        }
        int tot;
        const int off = block_exclusive_scan<int>(cnt_new | (cnt_old << 16), iscan, &tot);
        int on = off & 0xffff, oo = off >> 16;
        slot = 0;
        for (int g = tid; g < n_groups; g += kThreads, ++slot) {
          const unsigned mk = gm[slot], old_bits = (1u << apm) - 1u;
          if (mk & ~old_bits) {
            near_g[0][on] = (uint16_t)g;
            near_m[0][on++] = (uint16_t)(mk & ~old_bits);
          }
          if (mk & old_bits) {
            near_g[1][oo] = (uint16_t)g;
            near_m[1][oo++] = (uint16_t)(mk & old_bits);
          }
        }
        if (tid == 0) {
          near_n[0] = tot & 0xffff;
          near_n[1] = tot >> 16;
        }
        __syncthreads();
        // 2. the near groups of each end dealt to the warps in turn (balanced), lanes on atoms;
        //    each group's energy is reduced in the warp and kept per group, so the end's total
        //    (summed over groups in group order) depends neither on which warp took a group nor
        //    on which groups were skipped: the same positions give the same bits
        const int warp = tid >> 5, n_warps = kThreads >> 5;
        for (int end = 0; end < 2; ++end) {
          for (int q = warp; q < near_n[end]; q += n_warps) {
            const int g = near_g[end][q], j = g * 32 + lane;
            float v = 0.f;
            if (j < fwn) {
              const float4 pj = fwp[fw0 + j];
              const float qj = a.fw_charge[fw0 + j];
              float fj[3];
              frac32(If, pj.x, pj.y, pj.z, fj);
              const int tj = __float_as_int(pj.w);
              for (unsigned mm = near_m[end][q]; mm != 0u; mm &= mm - 1u) {
                const int m = __ffs(mm) - 1;
                const float4 fa = mfa[m];
                float d[3] = {fa.x - fj[0], fa.y - fj[1], fa.z - fj[2]}, c[3];
                d[0] -= rintf(d[0]);
                d[1] -= rintf(d[1]);
                d[2] -= rintf(d[2]);
                cart32(Lf, d, c);
                const float r2 = c[0] * c[0] + c[1] * c[1] + c[2] * c[2];
                if (r2 >= rc2_any) continue;
                v += pair_u(r2, __float_as_int(fa.w), tj, mq[m] * qj, lj, nsp, li, ei, alpha, ke, true, true);
              }
            }
            v = warp_sum(v);
            if (lane == 0) gsum[end][g] = v;
          }
        }
        __syncthreads();
        if (tid < 32) {  // group order: lane l sums groups l, l + 32, ...; block_sum_f adds the lanes
          for (int g = tid; g < n_groups; g += 32) {
            e_host_new += gsum[0][g];
            e_host_old += gsum[1][g];
          }
        }
      } else
      for (int base = (tid & ~31); base < fwn; base += kThreads) {
        unsigned near = on_mask;
        if (grp != nullptr) {
          bool close = false;
          if (lane < nm && ((on_mask >> lane) & 1u)) {
            const int gi = (fw0 + base) >> 5;
            const float4 c = grp[2 * gi], h = grp[2 * gi + 1], fa = mfa[lane];
            float dx = fa.x - c.x, dy = fa.y - c.y, dz = fa.z - c.z;
            dx = fabsf(dx - rintf(dx));
            dy = fabsf(dy - rintf(dy));
            dz = fabsf(dz - rintf(dz));
            const float sep = fmaxf(fmaxf(fmaxf(dx - h.x, 0.f) * wdt[0], fmaxf(dy - h.y, 0.f) * wdt[1]),
                                    fmaxf(dz - h.z, 0.f) * wdt[2]);
            close = sep < rc_any;
          }
          near = __ballot_sync(0xffffffffu, close);
        }
        const int j = base + lane;
        if (j >= fwn || near == 0u) continue;
        const float4 pj = fwp[fw0 + j];
        const float qj = a.fw_charge[fw0 + j];
        float fj[3];
        frac32(If, pj.x, pj.y, pj.z, fj);
        const int tj = __float_as_int(pj.w);
        for (unsigned mm = near; mm != 0u; mm &= mm - 1u) {
          const int m = __ffs(mm) - 1;
          const float4 fa = mfa[m];
          float d[3] = {fa.x - fj[0], fa.y - fj[1], fa.z - fj[2]}, c[3];
          d[0] -= rintf(d[0]);
          d[1] -= rintf(d[1]);
          d[2] -= rintf(d[2]);
          cart32(Lf, d, c);
          const float r2 = c[0] * c[0] + c[1] * c[1] + c[2] * c[2];
          if (r2 >= rc2_any) continue;
          const float u = pair_u(r2, __float_as_int(fa.w), tj, mq[m] * qj, lj, nsp, li, ei, alpha, ke, true, true);
          if (m < apm) e_host_old += u;
          else e_host_new += u;
        }
      }
      gcmc_mark(prof, 1, t0);
      // guest atoms (not grouped)
      for (int j = fwn + tid; j < n_other; j += kThreads) {
        float4 pj;
        float qj;
        {
          const int g = j - fwn;
          if (has_old && g / apm == mol) continue;  // the moved molecule itself
          pj = gpos[g];
          qj = a.motif_charge[g % apm];
        }
        float fj[3];
        frac32(If, pj.x, pj.y, pj.z, fj);
        const int tj = __float_as_int(pj.w);
        for (int m = 0; m < nm; ++m) {
          if (!mon[m]) continue;
          const float4 fa = mfa[m];
          float d[3] = {fa.x - fj[0], fa.y - fj[1], fa.z - fj[2]}, c[3];
          d[0] -= rintf(d[0]);
          d[1] -= rintf(d[1]);
          d[2] -= rintf(d[2]);
          cart32(Lf, d, c);
          const float r2 = c[0] * c[0] + c[1] * c[1] + c[2] * c[2];
          if (r2 >= rc2_any) continue;
          const float sg = m < apm ? -1.f : 1.f;
          e_acc += sg * pair_u(r2, __float_as_int(fa.w), tj, mq[m] * qj, lj, nsp, li, ei, alpha, ke, true, true);
        }
      }
    } else
    for (int j = tid; j < n_other; j += kThreads) {
      float4 pj;
      float qj;
      if (j < fwn) {
        pj = fwp[fw0 + j];
        qj = a.fw_charge[fw0 + j];
      } else {
        const int g = j - fwn;
        if (has_old && g / apm == mol) continue;  // the moved molecule itself
        pj = gpos[g];
        qj = a.motif_charge[g % apm];
      }
      float fj[3];
      frac32(If, pj.x, pj.y, pj.z, fj);
      const int tj = __float_as_int(pj.w);
      for (int st = 0; st < 2; ++st) {
        if ((st == 0 && !has_old) || (st == 1 && !has_new)) continue;
        const float sign = st == 0 ? -1.f : 1.f;
        for (int i = 0; i < apm; ++i) {
          const float4 pa = st == 0 ? sh.old_pos[i] : sh.new_pos[i];
          float fa[3];
          frac32(If, pa.x, pa.y, pa.z, fa);
          e_acc += sign * pair_images(Lf, fa, fj, __float_as_int(pa.w), tj, sh.q[i] * qj, lj, nsp, li, ei,
                                      alpha, ke, false);
        }
      }
    }
    // moved vs moved (same molecule): 1/2 sum over ordered pairs incl. self images
    for (int t = tid; t < 2 * apm * apm; t += kThreads) {
      const int st = t / (apm * apm), ab = t % (apm * apm), ia = ab / apm, ib = ab % apm;
      if ((st == 0 && !has_old) || (st == 1 && !has_new)) continue;
      const float4 pa = st == 0 ? sh.old_pos[ia] : sh.new_pos[ia];
      const float4 pb = st == 0 ? sh.old_pos[ib] : sh.new_pos[ib];
      float fa[3], fb[3];
      frac32(If, pa.x, pa.y, pa.z, fa);
      frac32(If, pb.x, pb.y, pb.z, fb);
      const float sign = st == 0 ? -0.5f : 0.5f;
      e_acc += sign * pair_images(Lf, fa, fb, __float_as_int(pa.w), __float_as_int(pb.w), sh.q[ia] * sh.q[ib], lj,
                                  nsp, li, ei, alpha, ke, true);
    }
    double de_real = block_sum_f(e_acc, red);
    double e_host_new_tot = 0.0, e_host_old_tot = 0.0;
    if (min_image) {  // host terms: new minus old end, the old one from the cache on a hit
      e_host_new_tot = block_sum_f(e_host_new, red);
      e_host_old_tot = cache_hit ? sh.e_host_old : block_sum_f(e_host_old, red);
      de_real += e_host_new_tot - e_host_old_tot;
    }
    gcmc_mark(prof, 2, t0);
    // ---------------------------------------------------------------- reciprocal space
    // per-k terms in float32 (|term| <~ 15 eV: ~1e-6 eV rounding each), the k sum of a
    // thread in float32, the block sum and S(k) itself in float64
    float de_rec_f = 0.f;
    // e^{2 pi i n . f} = prod_a e^{2 pi i n_a f_a}: each table entry from sincospif of the
    // reduced phase, each k from two complex products of three entries
    for (int e = tid; e < nm * 3 * kTab; e += kThreads) {
      const int m = e / (3 * kTab), ax = (e / kTab) % 3, nn = e % kTab - kMaxM;
      const float4 f = mfa[m];
      float t = nn * (ax == 0 ? f.x : ax == 1 ? f.y : f.z);
      t -= rintf(t);
      float sn, cs;
      sincospif(2.0f * t, &sn, &cs);
      ph[e] = make_float2(cs, sn);
    }
    __syncthreads();
    gcmc_mark(prof, 3, t0);
    // the step's change of S(k) (cos and sin parts) at the k vector of table entry pkk, from the
    // phase tables; the commit forms it again on acceptance instead of storing it every step
    auto delta_sk = [&](float2 pkk, float &dc, float &ds) {
      const uint32_t packed = __float_as_uint(pkk.y);
      const int n0 = packed & 0xffu, n1 = (packed >> 8) & 0xffu, n2 = (packed >> 16) & 0xffu;
      dc = 0.f;
      ds = 0.f;
      for (int m = 0; m < nm; ++m) {
        if (!mon[m]) continue;
        const float2 *t = ph + m * 3 * kTab;
        const float2 a = t[n0], b = t[kTab + n1], c = t[2 * kTab + n2];
        const float abr = a.x * b.x - a.y * b.y, abi = a.x * b.y + a.y * b.x;
        const float cs = abr * c.x - abi * c.y, sn = abr * c.y + abi * c.x;
        const float w = m < apm ? -mq[m] : mq[m];
        dc += w * cs;
        ds += w * sn;
      }
    };
    for (int k = tid; k < nk; k += kThreads) {
      const float2 pkk = pk32[k];
      float dc, ds;
      delta_sk(pkk, dc, ds);
      const float2 sck = sk32[k];
      de_rec_f = fmaf(pkk.x, fmaf(2.f, fmaf(sck.x, dc, sck.y * ds), fmaf(dc, dc, ds * ds)), de_rec_f);
    }
    __syncthreads();
    const double de_rec = block_sum_f(de_rec_f, red) * a.coulomb_k;
    gcmc_mark(prof, 4, t0);
    // ---------------------------------------------------------------- acceptance (thread 0)
    if (tid == 0) {
      double de = de_real + de_rec;
      const int n_old = nmol;
      int n_new = n_old;
      if (kind == 3 && has_new) n_new = n_old + 1;
      if (kind == 4 && has_old) n_new = n_old - 1;
      if (n_new != n_old) {
        const double sgn = n_new > n_old ? 1.0 : -1.0;
        de += sgn * ss.self_excl;
        // tail correction with the molecule counts before / after
        const double dn = (double)(n_new - n_old), dn2 = (double)n_new * n_new - (double)n_old * n_old;
        de += ss.tail_b * dn + ss.tail_c * dn2;
      }
      double logp = -de * inv_kT + sh.ln_ratio;
      if (n_new != n_old) {
        // ln n_old! - ln n_new! for n_new = n_old +- 1 is -ln n_new (insert) or +ln n_old (delete)
        logp += (n_new - n_old) * lnfv + (n_new > n_old ? -log((double)n_new) : log((double)n_old));
      }
      const U4 r4 = rng4(a.seed, 1 + (uint64_t)s, 8 * ctr + 4);
      const double u = ((double)(r4.w >> 8) + 1.0) * (1.0 / 16777216.0);  // (0, 1]
      int accept = logp > log(u);
      if (a.proposals != nullptr && a.proposals[s].force_reject) accept = 0;
      if (kind == 3 && !has_new) accept = 0;  // no free slot: capacity recorded, nothing changes
      sh.accept = accept;
      sh.log_p = logp;
      sh.de_total = de;
      if (a.trace != nullptr) {
        kups_gcmc_trace &t = a.trace[(int64_t)step * a.n_systems + s];
        t.kind = kind;
        t.mol = mol;
        t.accept = accept;
        t.n_mol = n_old;
        t.has_old = has_old;
        t.has_new = has_new;
        t.width = ss.width[kind >= 3 ? 3 : kind];
        t.pad = 0;
        t.de = de;
        t.log_p = logp;
        t.log_u = log(u);
        t.ln_ratio = sh.ln_ratio;
        for (int i = 0; i < kMaxApm; ++i) {
          const float4 p = i < apm && has_new ? sh.new_pos[i] : make_float4(0.f, 0.f, 0.f, 0.f);
          t.new_pos[i][0] = p.x;
          t.new_pos[i][1] = p.y;
          t.new_pos[i][2] = p.z;
          t.new_pos[i][3] = p.w;
        }
      }
      sh.de_real = de_real;
      sh.de_recip = de_rec;
      if (a.out_delta != nullptr) {
        a.out_delta[4 * (int64_t)s] = de;
        a.out_delta[4 * (int64_t)s + 1] = de_real;
        a.out_delta[4 * (int64_t)s + 2] = de_rec;
        a.out_delta[4 * (int64_t)s + 3] = logp;
      }
    }
    __syncthreads();
    const int accept = sh.accept;
    // ---------------------------------------------------------------- commit
    if (accept) {
      for (int k = tid; k < nk; k += kThreads) {
        float2 d;
        delta_sk(pk32[k], d.x, d.y);
        const double c = sk[2 * k] + (double)d.x, sn = sk[2 * k + 1] + (double)d.y;
        sk[2 * k] = c;
        sk[2 * k + 1] = sn;
        sk32[k] = make_float2((float)c, (float)sn);
      }
      if (tid == 0) {
        ss.energy += sh.de_total;
        double *cache = use_cache ? a.host_cache + (int64_t)s * a.max_mol * 2 : nullptr;
        if (kind == 3 && has_new) {
          for (int i = 0; i < apm; ++i) gpos[mol * apm + i] = sh.new_pos[i];
          ss.n_mol = nmol + 1;
        } else if (kind == 4 && has_old) {
          const int last = nmol - 1;
          for (int i = 0; i < apm; ++i) gpos[mol * apm + i] = gpos[last * apm + i];
          ss.n_mol = last;
          if (cache != nullptr) {  // the entry follows the molecule moved into the slot
            cache[2 * mol] = cache[2 * last];
            cache[2 * mol + 1] = cache[2 * last + 1];
          }
        } else if (has_new) {
          for (int i = 0; i < apm; ++i) gpos[mol * apm + i] = sh.new_pos[i];
        }
        if (cache != nullptr && has_new) {
          cache[2 * mol] = e_host_new_tot;
          cache[2 * mol + 1] = __longlong_as_double((long long)sh.new_key);
        }
      }
    } else if (tid == 0 && use_cache && has_old && !cache_hit) {  // rejected: keep what the miss computed
      double *ent = a.host_cache + ((int64_t)s * a.max_mol + mol) * 2;
      ent[0] = e_host_old_tot;
      ent[1] = __longlong_as_double((long long)sh.old_key);
    }
    // ---------------------------------------------------------------- statistics and step widths
    if (tid == 0) {
      ss.attempted[kind] += 1;
      ss.accepted[kind] += accept;
      const int sched = kind >= 3 ? 3 : kind;  // insert / delete share the exchange scheduler
      const int hs = a.history_len;
      uint32_t *hist = ss.hist[sched];
      int idx = ss.hist_idx[sched];
      const uint32_t bit = 1u << (idx & 31);
      hist[idx >> 5] = accept ? (hist[idx >> 5] | bit) : (hist[idx >> 5] & ~bit);
      idx = (idx + 1) % hs;
      ss.hist_idx[sched] = idx;
      if (idx == 0) {
        int acc = 0;
        for (int w = 0; w < 4; ++w) {
          const uint32_t m = w * 32 >= hs ? 0u : (w * 32 + 32 <= hs ? 0xffffffffu : ((1u << (hs - w * 32)) - 1u));
          acc += __popc(hist[w] & m);
        }
        const float avg = (float)acc / hs;
        const float target = 0.5f, tol = 0.05f, mult = 1.1f;
        float v = ss.width[sched];
        float nv = avg < target ? v / mult : v * mult;  // step widths correlate negatively
        nv = fmaxf(nv, 0.0f);
        const float ub = ss.width_max[sched];
        if (ub > 0.f) nv = fminf(nv, ub);
        if (fabsf(avg - target) > tol) ss.width[sched] = nv;
      }
      if (a.obs_sums != nullptr) {
        const double u = ss.energy, nm = (double)ss.n_mol;
        ob[0] += u;
        ob[1] += nm;
        ob[2] += __dmul_rn(u, nm);  // rounded products, as the reference's float64 series hold them
        ob[3] += __dmul_rn(nm, nm);
        ob[4] += __dmul_rn(u, u);
      }
    }
    __syncthreads();
    gcmc_mark(prof, 5, t0);
  }
  if (tid == 0) {  // the launch's state back to the caller's arrays
    if (a.obs_sums != nullptr)
      for (int k = 0; k < 5; ++k) a.obs_sums[5 * (int64_t)s + k] += ob[k];
    a.energy[s] = ss.energy;
    a.n_mol[s] = ss.n_mol;
    for (int k = 0; k < 4; ++k) {
      a.width[s * 4 + k] = ss.width[k];
      a.history_index[s * 4 + k] = ss.hist_idx[k];
      for (int w = 0; w < 4; ++w) a.history[((int64_t)s * 4 + k) * 4 + w] = ss.hist[k][w];
    }
    for (int k = 0; k < 5; ++k) {
      a.attempted[5 * (int64_t)s + k] += ss.attempted[k];
      a.accepted[5 * (int64_t)s + k] += ss.accepted[k];
    }
  }
}

}  // namespace
}  // namespace kups

using namespace kups;

extern "C" int32_t kups_gcmc_run(const kups_gcmc_args *a, kups_status *status, void *stream) {
  if (a == nullptr || a->n_systems < 0 || a->n_steps < 0 || a->atoms_per_mol <= 0 ||
      a->atoms_per_mol > kMaxApm || a->n_species <= 0 || a->n_species > kMaxSpeciesMC ||
      a->n_kvecs < 0 || a->n_kvecs > kMaxKVec || a->history_len <= 0 || a->history_len > 128 ||
      a->max_mol < 0)
    return KUPS_ERR_INVALID;
  if (a->proposal_node != nullptr && (a->proposal_cdf == nullptr || a->proposal_grid < 2 || a->proposal_grid > 256))
    return KUPS_ERR_INVALID;
  if (a->n_systems == 0 || a->n_steps == 0) return KUPS_OK;
  if (a->n_kvecs > 0 && a->workspace == nullptr) return KUPS_ERR_INVALID;
  const size_t smem = sizeof(float2) * 2 * (size_t)a->atoms_per_mol * 3 * kTab;
  const int threads = a->block_threads > 0 ? a->block_threads : kDefaultThreads;
  cudaStream_t st = (cudaStream_t)stream;
  switch (threads) {
    case 64: gcmc_kernel<64><<<a->n_systems, 64, smem, st>>>(*a, status); break;
    case 128: gcmc_kernel<128><<<a->n_systems, 128, smem, st>>>(*a, status); break;
    case 256: gcmc_kernel<256><<<a->n_systems, 256, smem, st>>>(*a, status); break;
    default: return KUPS_ERR_INVALID;
  }
  return cudaGetLastError() == cudaSuccess ? KUPS_OK : KUPS_ERR_CUDA;
}
