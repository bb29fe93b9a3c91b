// Piecewise-trilinear insertion density on a periodic G x G x G grid of
// fractional coordinates (the learned proposal; no counterpart in the
// reference, whose insertion draws the offset uniformly,
// src/kups/mcmc/moves.py:573-675).
//
// node[(i * G + j) * G + k] > 0 is the density's value at the grid node
// f = (i, j, k) / G.  Inside cell (i, j, k) the density is the trilinear
// interpolation of its eight corner values, so the cell's mass is the mean
// of its corners, and cdf[c] (float64, G^3 + 1 entries, cdf[0] = 0) is the
// running sum of those masses in cell order c = (i * G + j) * G + k.
//
// Sampling is exact:
//   1. cell c with probability P_c = (cdf[c + 1] - cdf[c]) / cdf[G^3];
//   2. corner b with probability d_b / sum_b d_b (d_b its value); the
//      trilinear density is the mixture of the eight product densities
//      prod_a l_a(t_a), l = 2t or 2(1 - t), weighted this way;
//   3. per axis t = sqrt(u) if the corner's bit is 1, else 1 - sqrt(u).
// The density in fractional measure is therefore
//   q_f(f) = P_c * G^3 * 8 * tri(t) / sum_b d_b,
// and the Cartesian density is q_f / V, so the insertion's log proposal
// ratio -ln(V q(x)) is -ln q_f(f) (and +ln q_f(f) for a deletion).
#pragma once

#include <math.h>
#include <stdint.h>

namespace kups {

// Uniform draws for the sampler from Philox words.
__device__ inline double u53(uint32_t hi, uint32_t lo) {  // [0, 1)
  return (double)((((uint64_t)(hi >> 11)) << 32) | lo) * (1.0 / 9007199254740992.0);
}
__device__ inline double u32_open0(uint32_t v) { return ((double)v + 1.0) * (1.0 / 4294967296.0); }  // (0, 1]

__device__ inline void grid_corners(const float *node, int g, int i, int j, int k, double d[8]) {
  const int i1 = i + 1 == g ? 0 : i + 1, j1 = j + 1 == g ? 0 : j + 1, k1 = k + 1 == g ? 0 : k + 1;
  for (int b = 0; b < 8; ++b) {
    const int ii = (b & 4) ? i1 : i, jj = (b & 2) ? j1 : j, kk = (b & 1) ? k1 : k;
    d[b] = (double)node[((int64_t)ii * g + jj) * g + kk];
  }
}

// ln q_f inside cell c = (i, j, k) at local coordinates t in [0, 1]^3.
__device__ inline double grid_cell_log_q(const double *cdf, int g, int64_t c, const double d[8], const double t[3]) {
  double tri = 0.0, sum = 0.0;
  for (int b = 0; b < 8; ++b) {
    const double w = ((b & 4) ? t[0] : 1.0 - t[0]) * ((b & 2) ? t[1] : 1.0 - t[1]) * ((b & 1) ? t[2] : 1.0 - t[2]);
    tri += d[b] * w;
    sum += d[b];
  }
  const double total = cdf[(int64_t)g * g * g];
  const double pc = (cdf[c + 1] - cdf[c]) / total;
  return log(pc) + 3.0 * log((double)g) + log(8.0 * tri / sum);
}

// ln q_f at fractional coordinates f (any periodic image).
__device__ inline double grid_log_q(const float *node, const double *cdf, int g, const double f_in[3]) {
  int ci[3];
  double t[3];
  for (int a = 0; a < 3; ++a) {
    const double f = f_in[a] - floor(f_in[a]);  // [0, 1]
    const double s = f * g;
    int c = (int)s;
    if (c >= g) c = g - 1;
    if (c < 0) c = 0;
    ci[a] = c;
    t[a] = fmin(fmax(s - c, 0.0), 1.0);
  }
  double d[8];
  grid_corners(node, g, ci[0], ci[1], ci[2], d);
  const int64_t c = ((int64_t)ci[0] * g + ci[1]) * g + ci[2];
  return grid_cell_log_q(cdf, g, c, d, t);
}

// Draws f (fractional, in [0, 1]^3) from the grid density and returns ln q_f(f).
//   u_cell, u_corner in [0, 1); u_axis in (0, 1].
__device__ inline double grid_sample(const float *node, const double *cdf, int g, double u_cell, double u_corner,
                                     const double u_axis[3], double f[3]) {
  const int64_t n = (int64_t)g * g * g;
  const double target = u_cell * cdf[n];
  int64_t lo = 0, hi = n;  // cdf[lo] <= target < cdf[hi]
  while (hi - lo > 1) {
    const int64_t mid = (lo + hi) >> 1;
    if (cdf[mid] <= target) lo = mid;
    else hi = mid;
  }
  const int i = (int)(lo / ((int64_t)g * g)), j = (int)((lo / g) % g), k = (int)(lo % g);
  double d[8];
  grid_corners(node, g, i, j, k, d);
  double sum = 0.0;
  for (int b = 0; b < 8; ++b) sum += d[b];
  const double pick = u_corner * sum;
  int corner = 7;
  double acc = 0.0;
  for (int b = 0; b < 8; ++b) {
    acc += d[b];
    if (pick < acc) {
      corner = b;
      break;
    }
  }
  double t[3];
  for (int a = 0; a < 3; ++a) {
    const double r = sqrt(u_axis[a]);
    t[a] = ((corner >> (2 - a)) & 1) ? r : 1.0 - r;
  }
  f[0] = (i + t[0]) / g;
  f[1] = (j + t[1]) / g;
  f[2] = (k + t[2]) / g;
  return grid_cell_log_q(cdf, g, lo, d, t);
}

}  // namespace kups
