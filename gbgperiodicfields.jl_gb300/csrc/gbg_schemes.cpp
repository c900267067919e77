// Spline scheme construction on the host (C ABI: gbg_scheme_*).
//
// The weights are the reference's: LalescuSpline's two-point Hermite interpolant whose
// derivatives come from centred finite differences (Fornberg weights), and
// LagrangeSpline's cardinal polynomials (GBGPeriodicFields.jl src/Interpolation.jl
// 227-424).  Both solve a small dense system, here by LU with partial pivoting -- the
// factorization Julia's `\` applies to a general square matrix.
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "gbg_common.cuh"

namespace {

using Mat = std::vector<double>;  // column-major

// Fornberg (1988) weights of the order-0..max_order derivatives at x0 for the given
// nodes; w[i + n*k].  Interpolation.jl:326-354.
Mat fornberg(double x0, const std::vector<double> &nodes, int max_order) {
  const int n = (int)nodes.size();
  const int cols = max_order + 1;
  Mat w((size_t)n * cols, 0.0);
  auto W = [&](int i, int k) -> double & { return w[(size_t)i + (size_t)n * k]; };
  double c1 = 1.0;
  double c4 = nodes[0] - x0;
  W(0, 0) = 1.0;
  for (int i = 1; i < n; ++i) {
    const int mn = std::min(i + 1, cols);
    double c2 = 1.0;
    const double c5 = c4;
    c4 = nodes[i] - x0;
    for (int j = 0; j < i; ++j) {
      const double c3 = nodes[i] - nodes[j];
      c2 *= c3;
      if (j == i - 1) {
        for (int k = mn - 1; k >= 1; --k)
          W(i, k) = c1 * ((double)k * W(i - 1, k - 1) - c5 * W(i - 1, k)) / c2;
        W(i, 0) = -c1 * c5 * W(i - 1, 0) / c2;
      }
      for (int k = mn - 1; k >= 1; --k) W(j, k) = (c4 * W(j, k) - (double)k * W(j, k - 1)) / c3;
      W(j, 0) = c4 * W(j, 0) / c3;
    }
    c1 = c2;
  }
  return w;
}

// Solves A X = B (A: n x n, B: n x r, column-major) by LU with partial pivoting.
bool solve(Mat a, int n, Mat &b, int r) {
  std::vector<int> piv(n);
  auto A = [&](int i, int j) -> double & { return a[(size_t)i + (size_t)n * j]; };
  auto B = [&](int i, int j) -> double & { return b[(size_t)i + (size_t)n * j]; };
  for (int k = 0; k < n; ++k) {
    int p = k;
    for (int i = k + 1; i < n; ++i)
      if (std::fabs(A(i, k)) > std::fabs(A(p, k))) p = i;
    if (A(p, k) == 0.0) return false;
    piv[k] = p;
    if (p != k)
      for (int j = 0; j < n; ++j) std::swap(A(k, j), A(p, j));
    for (int i = k + 1; i < n; ++i) {
      A(i, k) /= A(k, k);
      for (int j = k + 1; j < n; ++j) A(i, j) -= A(i, k) * A(k, j);
    }
  }
  for (int c = 0; c < r; ++c) {
    for (int k = 0; k < n; ++k)
      if (piv[k] != k) std::swap(B(k, c), B(piv[k], c));
    for (int i = 1; i < n; ++i)
      for (int j = 0; j < i; ++j) B(i, c) -= A(i, j) * B(j, c);
    for (int i = n - 1; i >= 0; --i) {
      for (int j = i + 1; j < n; ++j) B(i, c) -= A(i, j) * B(j, c);
      B(i, c) /= A(i, i);
    }
  }
  return true;
}

// Interpolation.jl:367-392: rows are the value and the derivatives 1..m at the two
// bracketing nodes (offsets 0 and 1), each derivative a centred finite difference over
// the 2n+1 stencil nodes around that node.
bool hermite(int n, int m, gbg_scheme &out) {
  const int nodes = 2 * n + 2, degree = 2 * m + 1, rows = degree + 1;
  Mat cond((size_t)rows * rows, 0.0), rhs((size_t)rows * nodes, 0.0);
  int row = 0;
  for (int node = 0; node <= 1; ++node) {
    std::vector<double> stencil;
    for (int s = -n; s <= n; ++s) stencil.push_back((double)(node + s));
    const Mat fd = fornberg((double)node, stencil, m);
    const int sn = (int)stencil.size();
    for (int d = 0; d <= m; ++d) {
      for (int power = d; power <= degree; ++power) {
        double falling = 1.0;
        for (int f = power - d + 1; f <= power; ++f) falling *= (double)f;
        cond[(size_t)row + (size_t)rows * power] = falling * std::pow((double)node, (double)(power - d));
      }
      for (int s = 0; s < sn; ++s) {
        const int column = (node - n + s) + n;  // position of the offset in -n..n+1
        rhs[(size_t)row + (size_t)rows * column] = fd[(size_t)s + (size_t)sn * d];
      }
      ++row;
    }
  }
  if (!solve(cond, rows, rhs, nodes)) return false;
  for (int q = 0; q < nodes; ++q)
    for (int r = 0; r < rows; ++r) out.coefficients[q + nodes * r] = rhs[(size_t)r + (size_t)rows * q];
  return true;
}

// Interpolation.jl:403-415: the inverse of the offsets' Vandermonde matrix.
bool lagrange(int n, gbg_scheme &out) {
  const int nodes = 2 * n + 2;
  Mat v((size_t)nodes * nodes), id((size_t)nodes * nodes, 0.0);
  for (int row = 0; row < nodes; ++row)
    for (int p = 0; p < nodes; ++p)
      v[(size_t)row + (size_t)nodes * p] = std::pow((double)(row - n), (double)p);
  for (int i = 0; i < nodes; ++i) id[(size_t)i + (size_t)nodes * i] = 1.0;
  if (!solve(v, nodes, id, nodes)) return false;
  for (int q = 0; q < nodes; ++q)
    for (int r = 0; r < nodes; ++r) out.coefficients[q + nodes * r] = id[(size_t)r + (size_t)nodes * q];
  return true;
}

}  // namespace

namespace gbg {

// An upper bound of max over q and t in [0, 1] of |w_q(t)| for w_q(t) = sum_r c[q, r] t^r.
// The power basis is converted to the Bernstein basis of the same degree; on [0, 1] a
// polynomial lies in the convex hull of its Bernstein coefficients, so the largest
// |b_k| bounds it.  For the spline schemes this is 1 (attained at the nodes), where the
// sum of |c[q, r]| over-estimates by up to 10^5.  `horner_slack` times sum_r |c[q, r]|
// is added for the rounding of the Horner evaluation in the working precision.
double weight_bound(const gbg_scheme &sch, double horner_slack) {
  const int n2 = sch.stencil_width, m = sch.num_powers, d = m - 1;
  double best = 0.0;
  for (int q = 0; q < n2; ++q) {
    double abs_sum = 0.0;
    for (int r = 0; r < m; ++r) abs_sum += std::fabs(sch.coefficients[q + n2 * r]);
    double hull = 0.0;
    for (int k = 0; k <= d; ++k) {
      // b_k = sum_{i <= k} C(k, i) / C(d, i) a_i; the ratio is built as a running product
      double b = 0.0, ratio = 1.0;  // ratio = C(k, i) / C(d, i)
      for (int i = 0; i <= k; ++i) {
        b += ratio * sch.coefficients[q + n2 * i];
        if (i < k) ratio *= (double)(k - i) / (double)(d - i);
      }
      hull = std::fmax(hull, std::fabs(b));
    }
    // the conversion's own rounding is far below this slack
    best = std::fmax(best, std::fmin(hull * (1.0 + 1e-12) + horner_slack * abs_sum, abs_sum));
  }
  return best;
}

}  // namespace gbg

extern "C" {

// Interpolation.jl:236-241 (_stencil_neighbours) + 244-258 (LalescuSpline).
gbg_status gbg_scheme_lalescu(int32_t stencil_width, int32_t smoothness, gbg_scheme *out) {
  gbg::clear_error();
  if (!out) return gbg::set_error(GBG_EARG, "LalescuSpline: null output");
  if (stencil_width < 2 || stencil_width % 2 != 0)
    return gbg::set_error(GBG_EARG, "LalescuSpline: stencil_width must be an even integer of at least 2, got " +
                                        std::to_string(stencil_width));
  const int n = stencil_width / 2 - 1;
  const int m = smoothness < 0 ? n : smoothness;
  if (m > 2 * n)
    return gbg::set_error(GBG_EARG, "LalescuSpline: smoothness must satisfy 0 <= smoothness <= stencil_width - 2");
  if (stencil_width > GBG_MAX_NODES || 2 * m + 2 > GBG_MAX_POWERS)
    return gbg::set_error(GBG_EUNSUPPORTED, "LalescuSpline: stencil wider than GBG_MAX_NODES");
  std::memset(out, 0, sizeof(*out));
  out->kind = GBG_SCHEME_LALESCU;
  out->stencil_width = stencil_width;
  out->smoothness = m;
  out->num_powers = 2 * m + 2;
  if (!hermite(n, m, *out)) return gbg::set_error(GBG_EARG, "LalescuSpline: singular system");
  return GBG_OK;
}

// Interpolation.jl:293-306 (LagrangeSpline).
gbg_status gbg_scheme_lagrange(int32_t stencil_width, gbg_scheme *out) {
  gbg::clear_error();
  if (!out) return gbg::set_error(GBG_EARG, "LagrangeSpline: null output");
  if (stencil_width < 2 || stencil_width % 2 != 0)
    return gbg::set_error(GBG_EARG, "LagrangeSpline: stencil_width must be an even integer of at least 2, got " +
                                        std::to_string(stencil_width));
  if (stencil_width > GBG_MAX_NODES)
    return gbg::set_error(GBG_EUNSUPPORTED, "LagrangeSpline: stencil wider than GBG_MAX_NODES");
  std::memset(out, 0, sizeof(*out));
  out->kind = GBG_SCHEME_LAGRANGE;
  out->stencil_width = stencil_width;
  out->smoothness = -1;
  out->num_powers = stencil_width;
  if (!lagrange(stencil_width / 2 - 1, *out)) return gbg::set_error(GBG_EARG, "LagrangeSpline: singular system");
  return GBG_OK;
}

gbg_status gbg_scheme_custom(int32_t stencil_width, int32_t num_powers, const double *coeffs,
                             gbg_scheme *out) {
  gbg::clear_error();
  if (!out || !coeffs) return gbg::set_error(GBG_EARG, "custom scheme: null pointer");
  if (stencil_width < 2 || stencil_width % 2 != 0 || num_powers < 1)
    return gbg::set_error(GBG_EARG, "custom scheme: stencil_width must be even and >= 2, num_powers >= 1");
  if (stencil_width > GBG_MAX_NODES || num_powers > GBG_MAX_POWERS)
    return gbg::set_error(GBG_EUNSUPPORTED, "custom scheme: larger than GBG_MAX_NODES x GBG_MAX_POWERS");
  std::memset(out, 0, sizeof(*out));
  out->kind = GBG_SCHEME_CUSTOM;
  out->stencil_width = stencil_width;
  out->smoothness = -1;
  out->num_powers = num_powers;
  std::memcpy(out->coefficients, coeffs, sizeof(double) * stencil_width * num_powers);
  return GBG_OK;
}

// Interpolation.jl:440-446, on the host in Float64.
gbg_status gbg_axis_weights(const gbg_scheme *s, double t, double *w) {
  gbg::clear_error();
  if (!s || !w) return gbg::set_error(GBG_EARG, "axis weights: null pointer");
  const int n2 = s->stencil_width, m2 = s->num_powers;
  for (int q = 0; q < n2; ++q) w[q] = s->coefficients[q + n2 * (m2 - 1)];
  for (int p = m2 - 2; p >= 0; --p)
    for (int q = 0; q < n2; ++q) {
      const double prod = w[q] * t;  // kept apart: the reference does not fuse
      w[q] = prod + s->coefficients[q + n2 * p];
    }
  return GBG_OK;
}

}  // extern "C"
