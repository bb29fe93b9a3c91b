// Bonded edge-set potentials: energy, dE/dx and dE/dtril over an edge list of
// order D (bonds 2, angles 3, dihedrals and inversions 4).
//
// Replaces the energies of src/kups/potential/classical/ harmonic.py:83-163
// (harmonic bond, harmonic angle), morse.py:142-171, cosine_angle.py:152-221,
// dihedral.py:214-273 and inversion.py:136-209 evaluated on the HyperGraph of an
// EdgeSetGraphConstructor (src/kups/potential/common/graph.py:289-361), with the
// gradient PotentialFromEnergy takes by jax.vjp with respect to
// PositionAndUnitCell (src/kups/potential/common/energy.py:264-355).
//
// One thread per edge (i_0, ..., i_{D-1}) with integer image shifts s_m:
//   v_m = x_{i_m} - x_{i_0} + s_m @ L  (Edges.difference_vectors,
//   src/kups/core/neighborlist.py:164-204), E_e(v_1 .. v_{D-1}) with the
//   parameter row of the edge's species tuple, g_m = dE_e/dv_m analytic, then
//   dE/dx_{i_m} += g_m, dE/dx_{i_0} -= sum_m g_m, dE/dL_ab += sum_m s_ma g_mb,
//   E_s += E_e for the system of i_0.  Difference vectors in float64; the
//   edge's arithmetic in float64, or in float32 with fp32 (this part issues
//   about 2 float64 FMA per cycle per SM, so the float64 angles, square roots
//   and trigonometry bound the float64 mode); per-system sums are warp sums (in
//   float in the float32 mode) added by one float64 atomic per warp, per-atom
//   gradients float64 atomics (atom 0's summed over the edge first), and the
//   image term s @ L is formed only for non-zero shifts.  The float32
//   mode takes angles as atan2 of cross and dot products and the cosine-angle and
//   inversion energies in factored forms, equal to the reference's in exact
//   arithmetic but without its cancellations, which float32 would amplify.
// Angle derivatives: d cos t / dv1 = v2 / (r1 r2) - cos t v1 / r1^2 (and 1 <-> 2).
// Dihedral: phi = atan2(|b2| b1 . (b2 x b3), (b1 x b2) . (b2 x b3)) with
// b1 = x_j - x_i, b2 = x_k - x_j, b3 = x_l - x_k, m = b1 x b2, n = b2 x b3; its
// position derivatives are the closed forms of Blondel and Karplus (J. Comput.
// Chem. 17, 1132, 1996): dphi/dx_i = -|b2| m / |m|^2, dphi/dx_l = |b2| n / |n|^2,
// dphi/dx_j = -(1 + p) dphi/dx_i + q dphi/dx_l, dphi/dx_k = p dphi/dx_i - (1 + q) dphi/dx_l,
// p = b1.b2 / |b2|^2, q = b3.b2 / |b2|^2.  Inversion: derivatives of
// sin w = (v1 . n / (|n| + eps)) / (|v1| + eps), n = v2 x v3, with the
// reference's 1e-10 regularisers kept.
#include <cmath>

#include "common.cuh"

namespace kups {
namespace {

constexpr double kEps = 1e-10;

template <typename R>
__device__ inline void cross3(const R a[3], const R b[3], R c[3]) {
  c[0] = a[1] * b[2] - a[2] * b[1];
  c[1] = a[2] * b[0] - a[0] * b[2];
  c[2] = a[0] * b[1] - a[1] * b[0];
}
template <typename R>
__device__ inline R dot3(const R a[3], const R b[3]) {
  return a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
}

template <int KIND>
struct Kind;
template <>
struct Kind<0> { static constexpr int order = 2, params = 2; };  // harmonic bond: x0, k
template <>
struct Kind<1> { static constexpr int order = 2, params = 3; };  // Morse: r0, D, alpha
template <>
struct Kind<2> { static constexpr int order = 3, params = 2; };  // harmonic angle: theta0 (deg), k
template <>
struct Kind<3> { static constexpr int order = 3, params = 3; };  // cosine angle: theta0 (rad), k, linear_tol
template <>
struct Kind<4> { static constexpr int order = 4, params = 3; };  // dihedral: V, n, phi0
template <>
struct Kind<5> { static constexpr int order = 4, params = 2; };  // inversion: omega0, k

// Energy of one edge and g[m] = dE/dv_{m+1}.
template <int KIND, typename R>
__device__ R edge_energy_grad(const R (*v)[3], const R *p, R (*g)[3]) {
  if (KIND == 0 || KIND == 1) {
    const R r = sqrt(dot3(v[0], v[0]));
    R e, dedr;
    if (KIND == 0) {
      e = (r - p[0]) * (r - p[0]) * p[1];
      dedr = R(2.0) * p[1] * (r - p[0]);
    } else {
      const R x = exp(-p[2] * (r - p[0]));
      e = p[1] * (R(1.0) - x) * (R(1.0) - x);
      dedr = R(2.0) * p[1] * (R(1.0) - x) * p[2] * x;
    }
    const R f = r > R(0.0) ? dedr / r : R(0.0);
    for (int a = 0; a < 3; ++a) g[0][a] = f * v[0][a];
    return e;
  } else if ((KIND == 2 || KIND == 3) && sizeof(R) == 4) {
    // float32: theta = atan2(|v1 x v2|, v1 . v2) and the derivatives through
    // v1 x (v1 x v2), which keep float32 digits near 0 and pi where acos and
    // 1 / sqrt(1 - cos^2) lose them
    R cr[3], t1[3], t2[3];
    cross3(v[0], v[1], cr);
    cross3(v[0], cr, t1);
    cross3(v[1], cr, t2);
    const R sn = sqrt(dot3(cr, cr)), cs = dot3(v[0], v[1]);
    const R r1s = dot3(v[0], v[0]), r2s = dot3(v[1], v[1]);
    R e, f1, f2;  // g[0] = f1 * v1 x (v1 x v2), g[1] = f2 * v2 x (v1 x v2)
    if (KIND == 2) {
      const R th = atan2(sn, cs) * (R(180.0) / R(M_PI));
      e = (th - p[0]) * (th - p[0]) * p[1];
      const R f = sn > R(0.0) ? R(2.0) * p[1] * (th - p[0]) * (R(180.0) / R(M_PI)) / sn : R(0.0);
      f1 = f / r1s;
      f2 = -f / r2s;
    } else {
      // k (c0 + c1 c + c2 (2c^2 - 1)) = 2 k c2 (c - cos theta0)^2
      const R r12 = sqrt(r1s * r2s), c = cs / r12;
      const R cc = fmin(fmax(c, -R(1.0)), R(1.0));
      const R th0 = p[0], k = p[1];
      R dedc;
      if (fabs(th0 - R(M_PI)) < p[2]) {
        e = k * (R(1.0) + cc);
        dedc = k;
      } else {
        const R c2 = R(1.0) / (R(4.0) * fmax(sin(th0) * sin(th0), R(1e-10))), d = cc - cos(th0);
        e = R(2.0) * k * c2 * d * d;
        dedc = R(4.0) * k * c2 * d;
      }
      if (fabs(c) > R(1.0)) dedc = R(0.0);
      f1 = -dedc / (r1s * r12);
      f2 = dedc / (r2s * r12);
    }
    for (int a = 0; a < 3; ++a) {
      g[0][a] = f1 * t1[a];
      g[1][a] = f2 * t2[a];
    }
    return e;
  } else if (KIND == 2 || KIND == 3) {
    const R r1 = sqrt(dot3(v[0], v[0])), r2 = sqrt(dot3(v[1], v[1]));
    const R c = dot3(v[0], v[1]) / (r1 * r2);
    R e, dedc;
    if (KIND == 2) {
      // the reference takes arccos of the unclipped cosine; clamping keeps
      // round-off above 1 from turning a straight angle into NaN
      const R cc = fmin(fmax(c, -R(1.0)), R(1.0));
      const R th = acos(cc) * (R(180.0) / R(M_PI));
      e = (th - p[0]) * (th - p[0]) * p[1];
      dedc = -R(2.0) * p[1] * (th - p[0]) * (R(180.0) / R(M_PI)) / sqrt(fmax(R(1.0) - cc * cc, R(1e-30)));
    } else {
      const R cc = fmin(fmax(c, -R(1.0)), R(1.0));
      const R th0 = p[0], k = p[1];
      if (fabs(th0 - R(M_PI)) < p[2]) {
        e = k * (R(1.0) + cc);
        dedc = k;
      } else {
        const R s2 = sin(th0) * sin(th0), ct0 = cos(th0);
        const R c2 = R(1.0) / (R(4.0) * fmax(s2, R(1e-10)));
        const R c1 = -R(4.0) * c2 * ct0, c0 = c2 * (R(2.0) * ct0 * ct0 + R(1.0));
        e = k * (c0 + c1 * cc + c2 * (R(2.0) * cc * cc - R(1.0)));
        dedc = k * (c1 + R(4.0) * c2 * cc);
      }
      if (fabs(c) > R(1.0)) dedc = R(0.0);  // clipped: no gradient
    }
    const R i12 = R(1.0) / (r1 * r2);
    for (int a = 0; a < 3; ++a) {
      g[0][a] = dedc * (v[1][a] * i12 - c * v[0][a] / (r1 * r1));
      g[1][a] = dedc * (v[0][a] * i12 - c * v[1][a] / (r2 * r2));
    }
    return e;
  } else if (KIND == 4) {
    R b1[3], b2[3], b3[3];
    for (int a = 0; a < 3; ++a) {
      b1[a] = v[0][a];
      b2[a] = v[1][a] - v[0][a];
      b3[a] = v[2][a] - v[1][a];
    }
    R m[3], n[3];
    cross3(b1, b2, m);
    cross3(b2, b3, n);
    const R mm = dot3(m, m), nn = dot3(n, n), lb = sqrt(dot3(b2, b2));
    const R lm = sqrt(mm), ln = sqrt(nn);
    R n1[3], n2[3], bn[3], x[3];
    for (int a = 0; a < 3; ++a) {
      n1[a] = m[a] / (lm + R(kEps));
      n2[a] = n[a] / (ln + R(kEps));
      bn[a] = b2[a] / (lb + R(kEps));
    }
    cross3(n1, n2, x);
    const R phi = atan2(dot3(x, bn), dot3(n1, n2));
    const R V = p[0], per = p[1], phi0 = p[2];
    const R e = R(0.5) * V * (R(1.0) - cos(per * phi0) * cos(per * phi));
    const R dedphi = R(0.5) * V * cos(per * phi0) * per * sin(per * phi);
    if (mm > R(0.0) && nn > R(0.0) && lb > R(0.0)) {
      const R pp = dot3(b1, b2) / (lb * lb), qq = dot3(b3, b2) / (lb * lb);
      for (int a = 0; a < 3; ++a) {
        const R di = -lb / mm * m[a], dl = lb / nn * n[a];
        g[0][a] = dedphi * (-(R(1.0) + pp) * di + qq * dl);
        g[1][a] = dedphi * (pp * di - (R(1.0) + qq) * dl);
        g[2][a] = dedphi * dl;
      }
    } else {
      for (int k = 0; k < 3; ++k)
        for (int a = 0; a < 3; ++a) g[k][a] = R(0.0);
    }
    return e;
  } else if (sizeof(R) == 4) {
    // float32 inversion: w = atan2(v1 . n, |v1 x n|), n = v2 x v3, and the
    // energy in the cancellation-free form
    //   ks (c0 + c1 cos w + c2 cos 2w) = 8 ks c2 X^2, X = sin((w + w0)/2) sin((w - w0)/2),
    //   c0 + c1 + c2 = 8 c2 sin^4(w0 / 2)
    // dw/dv1 = (|u1| n - (v1 . n) n x u1 / |u1|) / (|n| |v1|)^2,
    // dw/dn = (|u1| v1 + (v1 . n) v1 x u1 / |u1|) / (|n| |v1|)^2, u1 = v1 x n
    R n[3], u[3], nu[3], vu[3];
    cross3(v[1], v[2], n);
    cross3(v[0], n, u);
    cross3(n, u, nu);
    cross3(v[0], u, vu);
    const R nn = dot3(n, n), la2 = dot3(v[0], v[0]), an = dot3(v[0], n), lu = sqrt(dot3(u, u));
    const R w = atan2(an, lu);
    const R om0 = p[0], k = p[1];
    const R den = nn * la2;
    const R sw = den > R(0.0) ? an * rsqrt(den) : R(0.0);
    R e, dedw;
    if (fabs(om0) < R(1e-6)) {
      const R h = sin(R(0.5) * w);
      e = R(2.0) * k * h * h;  // k (1 - cos w)
      dedw = k * sw;
    } else {
      const R s2 = sin(om0) * sin(om0), h0 = sin(R(0.5) * om0);
      const R c2 = R(1.0) / (R(4.0) * (s2 > R(1e-10) ? s2 : R(1.0)));
      const R ks = k / fmax(R(8.0) * c2 * h0 * h0 * h0 * h0, R(1e-10));
      const R X = sin(R(0.5) * (w + om0)) * sin(R(0.5) * (w - om0));
      e = R(8.0) * ks * c2 * X * X;
      dedw = R(8.0) * ks * c2 * X * sw;
    }
    const R f = den > R(0.0) ? dedw / den : R(0.0);
    const R q = lu > R(0.0) ? an / lu : R(0.0);
    R G[3], t[3];
    for (int a = 0; a < 3; ++a) {
      g[0][a] = f * (lu * n[a] - q * nu[a]);
      G[a] = f * (lu * v[0][a] + q * vu[a]);
    }
    cross3(v[2], G, t);
    for (int a = 0; a < 3; ++a) g[1][a] = t[a];
    cross3(G, v[1], t);
    for (int a = 0; a < 3; ++a) g[2][a] = t[a];
    return e;
  } else {
    R n[3];
    cross3(v[1], v[2], n);
    const R ln = sqrt(dot3(n, n)), la = sqrt(dot3(v[0], v[0]));
    const R an = dot3(v[0], n);
    const R s_raw = an / (ln + R(kEps)) / (la + R(kEps));
    const R s = fmin(fmax(s_raw, -R(1.0)), R(1.0));
    const R w = asin(s);
    const R om0 = p[0], k = p[1];
    const bool sp2 = fabs(om0) < R(1e-6);
    const R s2 = sin(om0) * sin(om0), cw0 = cos(om0);
    const R c2 = sp2 ? R(0.0) : R(1.0) / (R(4.0) * (s2 > R(1e-10) ? s2 : R(1.0)));
    const R c1 = sp2 ? -R(1.0) : -R(4.0) * c2 * cw0;
    const R c0 = sp2 ? R(1.0) : c2 * (R(2.0) * cw0 * cw0 + R(1.0));
    const R ks = sp2 ? k : k / fmax(c0 + c1 + c2, R(1e-10));
    const R e = ks * (c0 + c1 * cos(w) + c2 * cos(R(2.0) * w));
    const R dedw = ks * (-c1 * sin(w) - R(2.0) * c2 * sin(R(2.0) * w));
    const R deds = fabs(s_raw) <= R(1.0) ? dedw / sqrt(fmax(R(1.0) - s * s, R(1e-30))) : R(0.0);
    // ds/dv1 and ds/dn; dn/dv2 (x) and dn/dv3 (x) through the cross product
    R wv[3], t[3];
    const R inv_la = R(1.0) / (la + R(kEps)), inv_ln = R(1.0) / (ln + R(kEps));
    for (int a = 0; a < 3; ++a) {
      const R nu = n[a] * inv_ln;
      g[0][a] = deds * (nu * inv_la - (an * inv_ln) * inv_la * inv_la / (la > R(0.0) ? la : R(1.0)) * v[0][a]);
      wv[a] = (v[0][a] * inv_ln - an * inv_ln * inv_ln / (ln > R(0.0) ? ln : R(1.0)) * n[a]) * inv_la;
    }
    cross3(v[2], wv, t);
    for (int a = 0; a < 3; ++a) g[1][a] = deds * t[a];
    cross3(wv, v[1], t);
    for (int a = 0; a < 3; ++a) g[2][a] = deds * t[a];
    return e;
  }
}

// add_system for a float or double value: the warp's sum in R, added to the float64 array.
template <typename R>
__device__ inline void add_system_r(double *arr, int stride, int comp, int sys, R v) {
  const unsigned full = 0xffffffffu;
  const int s0 = __shfl_sync(full, sys, 0);
  if (__all_sync(full, sys == s0)) {
    v = warp_sum(v);
    if ((threadIdx.x & 31) == 0 && sys >= 0) atomicAdd(&arr[(int64_t)sys * stride + comp], (double)v);
  } else if (sys >= 0) {
    atomicAdd(&arr[(int64_t)sys * stride + comp], (double)v);
  }
}

template <int KIND, typename R>
__global__ void bonded_kernel(const double *pos, const int32_t *system, const int32_t *species, int64_t n,
                              const double *tril, int32_t n_sys, const int32_t *edges, const int32_t *shifts,
                              int64_t n_edges, const double *params, int32_t nsp, double *energy, double *grad,
                              double *grad_tril, kups_status *status) {
  constexpr int D = Kind<KIND>::order, P = Kind<KIND>::params;
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  int sys = -1;
  R en = R(0.0), dl[6] = {R(0.0), R(0.0), R(0.0), R(0.0), R(0.0), R(0.0)};
  if (e < n_edges) {
    int idx[D];
    bool ok = true;
    int64_t row = 0;
    for (int d = 0; d < D; ++d) {
      idx[d] = edges[(int64_t)D * e + d];
      ok &= idx[d] >= 0 && idx[d] < n;
    }
    if (ok) {
      for (int d = 0; d < D; ++d) {
        const int t = species[idx[d]];
        ok &= t >= 0 && t < nsp;
        row = row * nsp + t;
      }
    }
    const int s0 = ok ? system[idx[0]] : -1;
    if (!ok || s0 < 0 || s0 >= n_sys) {
      status_error(status, KUPS_ERR_INVALID, e);
    } else {
      sys = s0;
      const Tril64 L = load_tril64(tril + 6 * (int64_t)s0);
      // difference vectors in float64 (positions are float64), then the edge's arithmetic in R
      R v[D - 1][3], g[D - 1][3], pr[P];
      int sh[D - 1][3];
      const double *x0 = pos + 3 * (int64_t)idx[0];
      for (int m = 0; m < D - 1; ++m) {
        for (int a = 0; a < 3; ++a) sh[m][a] = shifts[((int64_t)(D - 1) * e + m) * 3 + a];
        // s @ L only for a non-zero shift (zero adds nothing: same result)
        double sL[3] = {0.0, 0.0, 0.0};
        if (sh[m][0] | sh[m][1] | sh[m][2]) {
          const double shd[3] = {(double)sh[m][0], (double)sh[m][1], (double)sh[m][2]};
          row_times_tril64(shd, L, sL);
        }
        for (int a = 0; a < 3; ++a) v[m][a] = (R)(pos[3 * (int64_t)idx[m + 1] + a] - x0[a] + sL[a]);
      }
      for (int k = 0; k < P; ++k) pr[k] = (R)params[row * P + k];
      en = edge_energy_grad<KIND, R>(v, pr, g);
      bool finite = isfinite(en);
      for (int m = 0; m < D - 1; ++m)
        for (int a = 0; a < 3; ++a) finite &= isfinite(g[m][a]);
      if (!finite) status_error(status, KUPS_ERR_NONFINITE, e);
      R g0[3] = {R(0.0), R(0.0), R(0.0)};  // atom 0 takes -sum_m g_m in one atomic per axis
      for (int m = 0; m < D - 1; ++m) {
        for (int a = 0; a < 3; ++a) {
          atomicAdd(&grad[3 * (int64_t)idx[m + 1] + a], (double)g[m][a]);
          g0[a] -= g[m][a];
        }
        dl[0] += R(sh[m][0]) * g[m][0];
        dl[1] += R(sh[m][1]) * g[m][0];
        dl[2] += R(sh[m][1]) * g[m][1];
        dl[3] += R(sh[m][2]) * g[m][0];
        dl[4] += R(sh[m][2]) * g[m][1];
        dl[5] += R(sh[m][2]) * g[m][2];
      }
      for (int a = 0; a < 3; ++a) atomicAdd(&grad[3 * (int64_t)idx[0] + a], (double)g0[a]);
    }
  }
  // warp sums in R (float32 mode: float, the warp total added in float64), one atomic per warp
  add_system_r<R>(energy, 1, 0, sys, en);
  if (grad_tril != nullptr)
    for (int k = 0; k < 6; ++k) add_system_r<R>(grad_tril, 6, k, sys, dl[k]);
}

// slot[i] = k for the k-th changed particle, -1 for every other particle (slot preset to -1).
__global__ void changed_slot_kernel(const int32_t *changed, int64_t n_changed, int64_t n, int32_t *slot,
                                    kups_status *status) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n_changed) return;
  const int32_t i = changed[k];
  if (i < 0 || i >= n) {
    status_error(status, KUPS_ERR_INVALID, k);
    return;
  }
  slot[i] = (int32_t)k;
}

// delta[s] += E_e(new) - E_e(old) over the edges with at least one changed atom: the
// old graph (weight -1) and new graph (weight +1) of LocalGraphSumComposer
// (src/kups/potential/common/graph.py:412-450) restricted, as EdgeSetGraphConstructor's
// probe path restricts them (:336-361), to the affected edges.  A changed atom d takes
// new_pos[slot[d]]; its wrap image n_d (new position = unwrapped - n_d @ L) moves the
// edge's shifts to s_m + n_{m+1} - n_0, which keeps each difference vector on the same
// image (the edge data the reference's probe updates).
// E_e(new) - E_e(old) of edge e whose atoms idx[] have slots sl[] (-1: not moved);
// returns the edge's system, or -1 (status recorded) for an invalid species or system.
template <int KIND, typename R>
__device__ int edge_delta(int64_t e, const int *idx, const int *sl, const double *pos, const int32_t *system,
                          const int32_t *species, const double *tril, int32_t n_sys, const int32_t *shifts,
                          const double *params, int32_t nsp, const double *new_pos, const int32_t *new_image,
                          double &de, kups_status *status) {
  constexpr int D = Kind<KIND>::order, P = Kind<KIND>::params;
  bool ok = true;
  int64_t row = 0;
  for (int d = 0; d < D; ++d) {
    const int t = species[idx[d]];
    ok &= t >= 0 && t < nsp;
    row = row * nsp + t;
  }
  const int s0 = system[idx[0]];
  if (!ok || s0 < 0 || s0 >= n_sys) {
    status_error(status, KUPS_ERR_INVALID, e);
    return -1;
  }
  const Tril64 L = load_tril64(tril + 6 * (int64_t)s0);
  double x_old[D][3], x_new[D][3], img[D][3];
  for (int d = 0; d < D; ++d)
    for (int a = 0; a < 3; ++a) {
      x_old[d][a] = pos[3 * (int64_t)idx[d] + a];
      x_new[d][a] = sl[d] >= 0 ? new_pos[3 * (int64_t)sl[d] + a] : x_old[d][a];
      img[d][a] = (sl[d] >= 0 && new_image) ? (double)new_image[3 * (int64_t)sl[d] + a] : 0.0;
    }
  R v_old[D - 1][3], v_new[D - 1][3], g[D - 1][3], pr[P];
  for (int m = 0; m < D - 1; ++m) {
    double sh[3], sh_new[3], sL[3], sL_new[3];
    for (int a = 0; a < 3; ++a) {
      sh[a] = shifts[((int64_t)(D - 1) * e + m) * 3 + a];
      sh_new[a] = sh[a] + img[m + 1][a] - img[0][a];
    }
    row_times_tril64(sh, L, sL);
    row_times_tril64(sh_new, L, sL_new);
    for (int a = 0; a < 3; ++a) {
      v_old[m][a] = (R)(x_old[m + 1][a] - x_old[0][a] + sL[a]);
      v_new[m][a] = (R)(x_new[m + 1][a] - x_new[0][a] + sL_new[a]);
    }
  }
  for (int k = 0; k < P; ++k) pr[k] = (R)params[row * P + k];
  const double e_new = (double)edge_energy_grad<KIND, R>(v_new, pr, g);
  const double e_old = (double)edge_energy_grad<KIND, R>(v_old, pr, g);
  de = e_new - e_old;
  if (!isfinite(de)) status_error(status, KUPS_ERR_NONFINITE, e);
  return s0;
}

// delta[s] += E_e(new) - E_e(old) over the edges with at least one changed atom: the
// old graph (weight -1) and new graph (weight +1) of LocalGraphSumComposer
// (src/kups/potential/common/graph.py:412-450) restricted, as EdgeSetGraphConstructor's
// probe path restricts them (:336-361), to the affected edges.  A changed atom d takes
// new_pos[slot[d]]; its wrap image n_d (new position = unwrapped - n_d @ L) moves the
// edge's shifts to s_m + n_{m+1} - n_0, which keeps each difference vector on the same
// image (the edge data the reference's probe updates).  This form scans every edge.
template <int KIND, typename R>
__global__ void bonded_delta_kernel(const double *pos, const int32_t *system, const int32_t *species, int64_t n,
                                    const double *tril, int32_t n_sys, const int32_t *edges, const int32_t *shifts,
                                    int64_t n_edges, const double *params, int32_t nsp, const int32_t *slot,
                                    const double *new_pos, const int32_t *new_image, double *delta,
                                    kups_status *status) {
  constexpr int D = Kind<KIND>::order;
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  int sys = -1;
  double de = 0.0;
  if (e < n_edges) {
    int idx[D], sl[D];
    bool ok = true, touched = false;
    for (int d = 0; d < D; ++d) {
      idx[d] = edges[(int64_t)D * e + d];
      ok &= idx[d] >= 0 && idx[d] < n;
    }
    if (ok)
      for (int d = 0; d < D; ++d) {
        sl[d] = slot[idx[d]];
        touched |= sl[d] >= 0;
      }
    if (!ok)
      status_error(status, KUPS_ERR_INVALID, e);
    else if (touched)
      sys = edge_delta<KIND, R>(e, idx, sl, pos, system, species, tril, n_sys, shifts, params, nsp, new_pos,
                                new_image, de, status);
  }
  add_system(delta, 1, 0, sys, de);
}

// The same sum through the atom -> edge incidence lists: changed atom k's edges are
// split over kDeltaSplit consecutive threads (edge j to thread j mod kDeltaSplit), so
// that a batch of a few thousand moved atoms spreads over every SM; an edge with
// several changed atoms belongs to the one earliest in `changed`.
constexpr int kDeltaSplit = 4;
template <int KIND, typename R>
__global__ void bonded_delta_incident_kernel(const double *pos, const int32_t *system, const int32_t *species,
                                             int64_t n, const double *tril, int32_t n_sys, const int32_t *edges,
                                             const int32_t *shifts, int64_t n_edges, const double *params,
                                             int32_t nsp, const int32_t *changed, int64_t n_changed,
                                             const int64_t *inc_offsets, const int32_t *inc_edges,
                                             const int32_t *slot, const double *new_pos, const int32_t *new_image,
                                             double *delta, kups_status *status) {
  constexpr int D = Kind<KIND>::order;
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t k = t / kDeltaSplit;
  if (k >= n_changed) return;
  const int32_t i = changed[k];
  if (i < 0 || i >= n) return;  // recorded by changed_slot_kernel
  for (int64_t q = inc_offsets[i] + t % kDeltaSplit; q < inc_offsets[i + 1]; q += kDeltaSplit) {
    const int64_t e = inc_edges[q];
    if (e < 0 || e >= n_edges) {
      status_error(status, KUPS_ERR_INVALID, e);
      continue;
    }
    int idx[D], sl[D];
    bool ok = true, mine = true;
    for (int d = 0; d < D; ++d) {
      idx[d] = edges[(int64_t)D * e + d];
      ok &= idx[d] >= 0 && idx[d] < n;
    }
    if (!ok) {
      status_error(status, KUPS_ERR_INVALID, e);
      continue;
    }
    for (int d = 0; d < D; ++d) {
      sl[d] = slot[idx[d]];
      mine &= sl[d] < 0 || sl[d] >= k;
    }
    if (!mine) continue;
    double de = 0.0;
    const int s = edge_delta<KIND, R>(e, idx, sl, pos, system, species, tril, n_sys, shifts, params, nsp, new_pos,
                                      new_image, de, status);
    if (s >= 0) atomicAdd(&delta[s], de);
  }
}

template <int KIND, typename R>
cudaError_t launch_bonded(const double *pos, const int32_t *system, const int32_t *species, int64_t n,
                          const double *tril, int32_t s, const int32_t *edges, const int32_t *shifts,
                          int64_t n_edges, const double *params, int32_t nsp, double *energy, double *grad,
                          double *grad_tril, kups_status *status, cudaStream_t stream) {
  const unsigned grid = (unsigned)((n_edges + 127) / 128);
  bonded_kernel<KIND, R><<<grid, 128, 0, stream>>>(pos, system, species, n, tril, s, edges, shifts, n_edges, params,
                                                nsp, energy, grad, grad_tril, status);
  return cudaGetLastError();
}

}  // namespace
}  // namespace kups

using namespace kups;

extern "C" int32_t kups_bonded_order(int32_t kind) {
  switch (kind) {
    case 0: return Kind<0>::order;
    case 1: return Kind<1>::order;
    case 2: return Kind<2>::order;
    case 3: return Kind<3>::order;
    case 4: return Kind<4>::order;
    case 5: return Kind<5>::order;
    default: return -1;
  }
}

extern "C" int32_t kups_bonded_param_count(int32_t kind) {
  switch (kind) {
    case 0: return Kind<0>::params;
    case 1: return Kind<1>::params;
    case 2: return Kind<2>::params;
    case 3: return Kind<3>::params;
    case 4: return Kind<4>::params;
    case 5: return Kind<5>::params;
    default: return -1;
  }
}

extern "C" int32_t kups_bonded_edges(int32_t kind, const double *positions, const int32_t *system,
                                     const int32_t *species, int64_t n_particles, const double *tril,
                                     int32_t n_systems, const int32_t *edges, const int32_t *shifts, int64_t n_edges,
                                     const double *params, int32_t n_species, double *energy, double *grad,
                                     double *grad_tril, int32_t fp32, kups_status *status, void *stream_) {
  cudaStream_t stream = (cudaStream_t)stream_;
  if (kind < 0 || kind > 5 || n_particles < 0 || n_systems < 0 || n_edges < 0 || n_species <= 0 ||
      n_species > 1024)
    return KUPS_ERR_INVALID;
  if (n_edges == 0) return KUPS_OK;
  if (positions == nullptr || system == nullptr || species == nullptr || tril == nullptr || edges == nullptr ||
      shifts == nullptr || params == nullptr || energy == nullptr || grad == nullptr || status == nullptr)
    return KUPS_ERR_INVALID;
  cudaError_t err;
  switch (kind * 2 + (fp32 ? 1 : 0)) {
#define KUPS_BONDED_CASE(K, R)                                                                                   \
  case 2 * K + (sizeof(R) == 4 ? 1 : 0):                                                                         \
    err = launch_bonded<K, R>(positions, system, species, n_particles, tril, n_systems, edges, shifts, n_edges,  \
                              params, n_species, energy, grad, grad_tril, status, stream);                       \
    break;
    KUPS_BONDED_CASE(0, double)
    KUPS_BONDED_CASE(0, float)
    KUPS_BONDED_CASE(1, double)
    KUPS_BONDED_CASE(1, float)
    KUPS_BONDED_CASE(2, double)
    KUPS_BONDED_CASE(2, float)
    KUPS_BONDED_CASE(3, double)
    KUPS_BONDED_CASE(3, float)
    KUPS_BONDED_CASE(4, double)
    KUPS_BONDED_CASE(4, float)
    KUPS_BONDED_CASE(5, double)
    KUPS_BONDED_CASE(5, float)
#undef KUPS_BONDED_CASE
    default:
      return KUPS_ERR_INVALID;
  }
  return err == cudaSuccess ? KUPS_OK : KUPS_ERR_CUDA;
}

extern "C" size_t kups_bonded_delta_workspace_bytes(int64_t n_particles) {
  return n_particles < 0 ? 0 : sizeof(int32_t) * (size_t)n_particles + 256;
}

extern "C" int32_t kups_bonded_delta(int32_t kind, const double *positions, const int32_t *system,
                                     const int32_t *species, int64_t n_particles, const double *tril,
                                     int32_t n_systems, const int32_t *edges, const int32_t *shifts, int64_t n_edges,
                                     const double *params, int32_t n_species, const int64_t *incidence_offsets,
                                     const int32_t *incidence_edges, const int32_t *changed,
                                     const double *new_positions, const int32_t *new_image, int64_t n_changed,
                                     double *delta, int32_t fp32, void *workspace, size_t workspace_bytes,
                                     kups_status *status, void *stream_) {
  cudaStream_t stream = (cudaStream_t)stream_;
  // slots hold positions in `changed` as int32
  if (kind < 0 || kind > 5 || n_particles < 0 || n_systems < 0 || n_edges < 0 || n_changed < 0 ||
      n_changed >= (int64_t)INT32_MAX || n_species <= 0 || n_species > 1024)
    return KUPS_ERR_INVALID;
  if (n_edges == 0 || n_changed == 0) return KUPS_OK;
  if (positions == nullptr || system == nullptr || species == nullptr || tril == nullptr || edges == nullptr ||
      shifts == nullptr || params == nullptr || changed == nullptr || new_positions == nullptr ||
      delta == nullptr || status == nullptr || workspace == nullptr)
    return KUPS_ERR_INVALID;
  if (n_particles >= (int64_t)INT32_MAX || workspace_bytes < kups_bonded_delta_workspace_bytes(n_particles))
    return KUPS_ERR_INVALID;
  int32_t *slot = (int32_t *)(((uintptr_t)workspace + 255) & ~uintptr_t(255));
  KUPS_CUDA_TRY(cudaMemsetAsync(slot, 0xff, sizeof(int32_t) * (size_t)n_particles, stream));  // -1
  changed_slot_kernel<<<(unsigned)((n_changed + 127) / 128), 128, 0, stream>>>(changed, n_changed, n_particles, slot,
                                                                              status);
  if ((incidence_offsets == nullptr) != (incidence_edges == nullptr)) return KUPS_ERR_INVALID;
  const bool incident = incidence_offsets != nullptr;
  const unsigned grid = (unsigned)((n_edges + 127) / 128);
  const unsigned grid_k = (unsigned)((n_changed * kDeltaSplit + 63) / 64);
  switch (kind * 2 + (fp32 ? 1 : 0)) {
#define KUPS_DELTA_CASE(K, R)                                                                                     \
  case 2 * K + (sizeof(R) == 4 ? 1 : 0):                                                                          \
    if (incident)                                                                                                 \
      bonded_delta_incident_kernel<K, R><<<grid_k, 64, 0, stream>>>(                                              \
          positions, system, species, n_particles, tril, n_systems, edges, shifts, n_edges, params, n_species,    \
          changed, n_changed, incidence_offsets, incidence_edges, slot, new_positions, new_image, delta, status); \
    else                                                                                                          \
      bonded_delta_kernel<K, R><<<grid, 128, 0, stream>>>(positions, system, species, n_particles, tril,          \
                                                          n_systems, edges, shifts, n_edges, params, n_species,   \
                                                          slot, new_positions, new_image, delta, status);         \
    break;
    KUPS_DELTA_CASE(0, double)
    KUPS_DELTA_CASE(0, float)
    KUPS_DELTA_CASE(1, double)
    KUPS_DELTA_CASE(1, float)
    KUPS_DELTA_CASE(2, double)
    KUPS_DELTA_CASE(2, float)
    KUPS_DELTA_CASE(3, double)
    KUPS_DELTA_CASE(3, float)
    KUPS_DELTA_CASE(4, double)
    KUPS_DELTA_CASE(4, float)
    KUPS_DELTA_CASE(5, double)
    KUPS_DELTA_CASE(5, float)
#undef KUPS_DELTA_CASE
    default:
      return KUPS_ERR_INVALID;
  }
  return cudaGetLastError() == cudaSuccess ? KUPS_OK : KUPS_ERR_CUDA;
}
