/*
 * gbg_oracle.c -- CPU oracle (test infrastructure only; see gbg_oracle.h).
 *
 * A plain-C restatement of the reference's spline gather/scatter, kept to the
 * reference's formulas, operation order and loop order so that, compiled with
 * -ffp-contract=off (Julia never contracts a*b+c into an FMA), each function
 * computes what the reference's CPU path computes.  Each function cites the
 * reference lines it follows (paths are relative to the GBGPeriodicFields.jl
 * project root).
 */
#include "gbg_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* Julia's integer mod: result carries the sign of the divisor, i.e. lies in [0, n). */
static inline int64_t imod(int64_t a, int64_t n) {
  int64_t r = a % n;
  return r < 0 ? r + n : r;
}

/* ---------------------------------------------------------------- weights */

/* Interpolation.jl:326-354 (Fornberg 1988), 0-based: w[i + n*k]. */
int gbgo_fornberg(double x0, const double *nodes, int n, int max_order, double *w) {
  if (n < 1 || max_order < 0) return GBGO_EARG;
  const int cols = max_order + 1;
#define W(i, k) w[(i) + n * (k)]
  memset(w, 0, sizeof(double) * (size_t)n * (size_t)cols);
  double product_left = 1.0;
  double difference_last = nodes[0] - x0;
  W(0, 0) = 1.0;
  for (int i = 1; i < n; ++i) {
    const int highest = (i + 1 < cols) ? i + 1 : cols; /* min(i, max_order+1), 1-based */
    double product_current = 1.0;
    const double difference_previous = difference_last;
    difference_last = nodes[i] - x0;
    for (int j = 0; j < i; ++j) {
      const double difference_nodes = nodes[i] - nodes[j];
      product_current *= difference_nodes;
      if (j == i - 1) {
        for (int k = highest - 1; k >= 1; --k)
          W(i, k) = product_left * ((double)k * W(i - 1, k - 1) - difference_previous * W(i - 1, k)) /
                    product_current;
        W(i, 0) = -product_left * difference_previous * W(i - 1, 0) / product_current;
      }
      for (int k = highest - 1; k >= 1; --k)
        W(j, k) = (difference_last * W(j, k) - (double)k * W(j, k - 1)) / difference_nodes;
      W(j, 0) = difference_last * W(j, 0) / difference_nodes;
    }
    product_left = product_current;
  }
#undef W
  return GBGO_OK;
}

/* Dense solve A X = B by LU with partial pivoting (what Julia's `\` does for a
 * general square matrix, through LAPACK getrf/getrs).  A: n x n, B: n x r, both
 * column-major; X overwrites B.  A is destroyed. */
static int lu_solve(double *a, int n, double *b, int r) {
  int piv[GBGO_MAX_POWERS];
  if (n > GBGO_MAX_POWERS) return GBGO_EARG;
#define A(i, j) a[(i) + n * (j)]
#define B(i, j) b[(i) + n * (j)]
  for (int k = 0; k < n; ++k) {
    int p = k;
    double best = fabs(A(k, k));
    for (int i = k + 1; i < n; ++i)
      if (fabs(A(i, k)) > best) { best = fabs(A(i, k)); p = i; }
    if (best == 0.0) return GBGO_EARG; /* singular */
    piv[k] = p;
    if (p != k)
      for (int j = 0; j < n; ++j) { double t = A(k, j); A(k, j) = A(p, j); A(p, j) = t; }
    for (int i = k + 1; i < n; ++i) {
      A(i, k) /= A(k, k);
      for (int j = k + 1; j < n; ++j) A(i, j) -= A(i, k) * A(k, j);
    }
  }
  for (int c = 0; c < r; ++c) {
    for (int k = 0; k < n; ++k)
      if (piv[k] != k) { double t = B(k, c); B(k, c) = B(piv[k], c); B(piv[k], c) = t; }
    for (int i = 1; i < n; ++i)
      for (int j = 0; j < i; ++j) B(i, c) -= A(i, j) * B(j, c);
    for (int i = n - 1; i >= 0; --i) {
      for (int j = i + 1; j < n; ++j) B(i, c) -= A(i, j) * B(j, c);
      B(i, c) /= A(i, i);
    }
  }
#undef A
#undef B
  return GBGO_OK;
}

/* Interpolation.jl:367-392.  coeffs: (2n+2) x (2m+2), column-major, [node q, power r]. */
int gbgo_hermite_weight_matrix(int n, int m, double *coeffs) {
  if (n < 0 || m < 0 || m > 2 * n) return GBGO_EARG;
  const int nodes = 2 * n + 2;
  const int degree = 2 * m + 1;
  const int rows = degree + 1;
  if (nodes > GBGO_MAX_NODES || rows > GBGO_MAX_POWERS) return GBGO_EARG;
  double conditions[GBGO_MAX_POWERS * GBGO_MAX_POWERS];
  double nodal[GBGO_MAX_POWERS * GBGO_MAX_NODES]; /* rows x nodes */
  memset(conditions, 0, sizeof conditions);
  memset(nodal, 0, sizeof nodal);
  int row = 0;
  for (int node = 0; node <= 1; ++node) {
    /* the centred stencil about this bracketing node: node-n .. node+n */
    double stencil[GBGO_MAX_NODES];
    const int sn = 2 * n + 1;
    for (int s = 0; s < sn; ++s) stencil[s] = (double)(node - n + s);
    double fd[GBGO_MAX_NODES * GBGO_MAX_POWERS];
    int st = gbgo_fornberg((double)node, stencil, sn, m, fd);
    if (st) return st;
    for (int d = 0; d <= m; ++d) {
      for (int power = d; power <= degree; ++power) {
        long long falling = 1; /* prod((power - d + 1):power) */
        for (int f = power - d + 1; f <= power; ++f) falling *= f;
        conditions[row + rows * power] = (double)falling * pow((double)node, (double)(power - d));
      }
      for (int s = 0; s < sn; ++s) {
        const int offset = node - n + s;       /* stencil offset */
        const int column = offset + n;         /* findfirst(==(offset), -n:n+1) */
        nodal[row + rows * column] = fd[s + sn * d];
      }
      ++row;
    }
  }
  int st = lu_solve(conditions, rows, nodal, nodes);
  if (st) return st;
  /* permutedims: coeffs[q, r] = solution[r, q] */
  for (int q = 0; q < nodes; ++q)
    for (int r = 0; r < rows; ++r) coeffs[q + nodes * r] = nodal[r + rows * q];
  return GBGO_OK;
}

/* Interpolation.jl:403-415. */
int gbgo_lagrange_weight_matrix(int n, double *coeffs) {
  if (n < 0) return GBGO_EARG;
  const int nodes = 2 * n + 2;
  if (nodes > GBGO_MAX_NODES) return GBGO_EARG;
  double v[GBGO_MAX_NODES * GBGO_MAX_NODES];
  double id[GBGO_MAX_NODES * GBGO_MAX_NODES];
  for (int row = 0; row < nodes; ++row) {
    const double offset = (double)(row - n);
    for (int power = 0; power < nodes; ++power) v[row + nodes * power] = pow(offset, (double)power);
  }
  for (int i = 0; i < nodes * nodes; ++i) id[i] = 0.0;
  for (int i = 0; i < nodes; ++i) id[i + nodes * i] = 1.0;
  int st = lu_solve(v, nodes, id, nodes);
  if (st) return st;
  for (int q = 0; q < nodes; ++q)
    for (int r = 0; r < nodes; ++r) coeffs[q + nodes * r] = id[r + nodes * q];
  return GBGO_OK;
}

/* Interpolation.jl:236-241 (_stencil_neighbours) + 244-258 (LalescuSpline). */
int gbgo_lalescu(int stencil_width, int smoothness, double *coeffs, int *n2, int *m2) {
  if (stencil_width < 2 || stencil_width % 2 != 0) return GBGO_EARG;
  const int n = stencil_width / 2 - 1;
  if (smoothness < 0 || smoothness > 2 * n) return GBGO_EARG;
  *n2 = 2 * n + 2;
  *m2 = 2 * smoothness + 2;
  return gbgo_hermite_weight_matrix(n, smoothness, coeffs);
}

/* Interpolation.jl:293-306 (LagrangeSpline). */
int gbgo_lagrange(int stencil_width, double *coeffs, int *n2, int *m2) {
  if (stencil_width < 2 || stencil_width % 2 != 0) return GBGO_EARG;
  const int n = stencil_width / 2 - 1;
  *n2 = 2 * n + 2;
  *m2 = 2 * n + 2;
  return gbgo_lagrange_weight_matrix(n, coeffs);
}

/* Interpolation.jl:440-446: w = c[:, M2]; for p = M2-1:-1:1, w = w .* t .+ c[:, p]. */
void gbgo_axis_weights_f64(const double *c, int n2, int m2, double t, double *w) {
  for (int q = 0; q < n2; ++q) w[q] = c[q + n2 * (m2 - 1)];
  for (int p = m2 - 2; p >= 0; --p)
    for (int q = 0; q < n2; ++q) w[q] = w[q] * t + c[q + n2 * p];
}
void gbgo_axis_weights_f32(const float *c, int n2, int m2, float t, float *w) {
  for (int q = 0; q < n2; ++q) w[q] = c[q + n2 * (m2 - 1)];
  for (int p = m2 - 2; p >= 0; --p)
    for (int q = 0; q < n2; ++q) w[q] = w[q] * t + c[q + n2 * p];
}

/* Interpolation.jl:456-460: ci = (x - o)/dx; base = floor(Int, ci); t = ci - base. */
int gbgo_locate_f64(double x, double origin, double spacing, int64_t *base, double *t) {
  const double ci = (x - origin) / spacing;
  const double fl = floor(ci);
  if (!isfinite(ci) || fl < -9.2e18 || fl > 9.2e18) return GBGO_ENONFINITE;
  *base = (int64_t)fl;
  *t = ci - fl;
  return GBGO_OK;
}
int gbgo_locate_f32(float x, float origin, float spacing, int64_t *base, float *t) {
  const float ci = (x - origin) / spacing;
  const float fl = floorf(ci);
  if (!isfinite(ci) || fl < -9.2e18f || fl > 9.2e18f) return GBGO_ENONFINITE;
  *base = (int64_t)fl;
  *t = ci - fl;
  return GBGO_OK;
}

/* Interpolation.jl:1000 + 1025-1027. */
void gbgo_walk(int64_t base, int64_t neighbourhood, int64_t extent, int width, int64_t *idx) {
  int64_t node = imod(base - neighbourhood, extent);
  for (int s = 0; s < width; ++s) {
    idx[s] = node;
    node = (node + 1 == extent) ? 0 : node + 1;
  }
}

/* ------------------------------------------------------- gather / scatter */

/* One generic body per element type.  T is the element type, SUF the suffix. */
#define GBGO_TRANSFER(T, SUF, FLOOR_LOCATE)                                                        \
  static int point_stencil_##SUF(const int64_t *gn, const T *o, const T *dx, const T *cT, int n2, \
                                 int m2, const T *pos, int64_t m, int64_t p, T *w1, T *w2, T *w3,  \
                                 int64_t *first) {                                                 \
    int64_t b[3];                                                                                  \
    T t[3];                                                                                        \
    for (int d = 0; d < 3; ++d) {                                                                  \
      int st = FLOOR_LOCATE(pos[p + m * d], o[d], dx[d], &b[d], &t[d]);                            \
      if (st) return st;                                                                           \
    }                                                                                              \
    gbgo_axis_weights_##SUF(cT, n2, m2, t[0], w1);                                                 \
    gbgo_axis_weights_##SUF(cT, n2, m2, t[1], w2);                                                 \
    gbgo_axis_weights_##SUF(cT, n2, m2, t[2], w3);                                                 \
    const int64_t nb = (n2 - 2) / 2;                                                               \
    for (int d = 0; d < 3; ++d) first[d] = imod(b[d] - nb, gn[d]);                                 \
    return GBGO_OK;                                                                                \
  }                                                                                                \
                                                                                                   \
  static int gather_body_##SUF(const int64_t *gn, const double *origin, const double *spacing,    \
                               int ncomp, const T *field, const T *pos, int64_t m,                 \
                               const int32_t *trav, const double *coeffs, int n2, int m2, T *out,  \
                               int nthreads) {                                                     \
    if (n2 < 1 || n2 > GBGO_MAX_NODES || m2 < 1 || m2 > GBGO_MAX_POWERS) return GBGO_EARG;        \
    T cT[GBGO_MAX_NODES * GBGO_MAX_POWERS];                                                        \
    for (int i = 0; i < n2 * m2; ++i) cT[i] = (T)coeffs[i]; /* _coefficients_as, 1360 */           \
    const T o[3] = {(T)origin[0], (T)origin[1], (T)origin[2]};                                     \
    const T dx[3] = {(T)spacing[0], (T)spacing[1], (T)spacing[2]};                                 \
    const int64_t nx = gn[0], ny = gn[1], nz = gn[2], npf = nx * ny * nz;                          \
    int status = GBGO_OK;                                                                          \
    _Pragma("omp parallel for schedule(static) num_threads(nthreads) if(nthreads > 1)")           \
    for (int64_t wi = 0; wi < m; ++wi) {                                                           \
      const int64_t p = trav ? (int64_t)trav[wi] - 1 : wi; /* _visit, 618-619 */                  \
      T w1[GBGO_MAX_NODES], w2[GBGO_MAX_NODES], w3[GBGO_MAX_NODES];                                \
      int64_t first[3];                                                                            \
      int st = point_stencil_##SUF(gn, o, dx, cT, n2, m2, pos, m, p, w1, w2, w3, first);           \
      if (st) { status = st; continue; }                                                           \
      for (int c = 0; c < ncomp; ++c) { /* Interpolation.jl:1028-1049 */                          \
        T acc = (T)0;                                                                              \
        int64_t node_z = first[2];                                                                 \
        for (int k = 0; k < n2; ++k) {                                                             \
          int64_t node_y = first[1];                                                               \
          for (int j = 0; j < n2; ++j) {                                                           \
            const T wyz = w2[j] * w3[k];                                                           \
            const int64_t plane = nx * node_y + nx * ny * node_z + npf * c;                        \
            int64_t node_x = first[0];                                                             \
            for (int i = 0; i < n2; ++i) {                                                         \
              acc += wyz * w1[i] * field[node_x + plane];                                          \
              node_x = (node_x + 1 == nx) ? 0 : node_x + 1;                                        \
            }                                                                                      \
            node_y = (node_y + 1 == ny) ? 0 : node_y + 1;                                          \
          }                                                                                        \
          node_z = (node_z + 1 == nz) ? 0 : node_z + 1;                                            \
        }                                                                                          \
        out[p + m * c] = acc;                                                                      \
      }                                                                                            \
    }                                                                                              \
    return status;                                                                                 \
  }                                                                                                \
                                                                                                   \
  static int scatter_body_##SUF(const int64_t *gn, const double *origin, const double *spacing,   \
                                int ncomp, T *field, const T *pos, int64_t m, const T *q,          \
                                const int32_t *trav, const double *coeffs, int n2, int m2,         \
                                double alpha, double beta, int nthreads) {                         \
    if (n2 < 1 || n2 > GBGO_MAX_NODES || m2 < 1 || m2 > GBGO_MAX_POWERS) return GBGO_EARG;        \
    const int64_t nx = gn[0], ny = gn[1], nz = gn[2], npf = nx * ny * nz;                          \
    /* Interpolation.jl:1309-1313: beta == 0 overwrites (NaN-safe fill), else data .*= T(beta) */ \
    const int64_t total = npf * ncomp;                                                             \
    if (beta == 0.0) {                                                                             \
      _Pragma("omp parallel for schedule(static) num_threads(nthreads) if(nthreads > 1)")         \
      for (int64_t i = 0; i < total; ++i) field[i] = (T)0;                                         \
    } else {                                                                                       \
      const T tb = (T)beta;                                                                        \
      _Pragma("omp parallel for schedule(static) num_threads(nthreads) if(nthreads > 1)")         \
      for (int64_t i = 0; i < total; ++i) field[i] *= tb;                                          \
    }                                                                                              \
    T cT[GBGO_MAX_NODES * GBGO_MAX_POWERS];                                                        \
    for (int i = 0; i < n2 * m2; ++i) cT[i] = (T)coeffs[i];                                        \
    const T o[3] = {(T)origin[0], (T)origin[1], (T)origin[2]};                                     \
    const T dx[3] = {(T)spacing[0], (T)spacing[1], (T)spacing[2]};                                 \
    const T factor = (T)alpha;                                                                     \
    int status = GBGO_OK;                                                                          \
    _Pragma("omp parallel for schedule(static) num_threads(nthreads) if(nthreads > 1)")           \
    for (int64_t wi = 0; wi < m; ++wi) {                                                           \
      const int64_t p = trav ? (int64_t)trav[wi] - 1 : wi;                                         \
      T w1[GBGO_MAX_NODES], w2[GBGO_MAX_NODES], w3[GBGO_MAX_NODES];                                \
      int64_t first[3];                                                                            \
      int st = point_stencil_##SUF(gn, o, dx, cT, n2, m2, pos, m, p, w1, w2, w3, first);           \
      if (st) { status = st; continue; }                                                           \
      for (int c = 0; c < ncomp; ++c) { /* Interpolation.jl:1084-1103 */                          \
        const T quantity = factor * q[p + m * c];                                                  \
        int64_t node_z = first[2];                                                                 \
        for (int k = 0; k < n2; ++k) {                                                             \
          int64_t node_y = first[1];                                                               \
          for (int j = 0; j < n2; ++j) {                                                           \
            const T wyz = w2[j] * w3[k];                                                           \
            const int64_t plane = nx * node_y + nx * ny * node_z + npf * c;                        \
            int64_t node_x = first[0];                                                             \
            for (int i = 0; i < n2; ++i) {                                                         \
              const T add = wyz * w1[i] * quantity;                                                \
              if (nthreads > 1) {                                                                  \
                _Pragma("omp atomic update") field[node_x + plane] += add;                         \
              } else {                                                                             \
                field[node_x + plane] += add;                                                      \
              }                                                                                    \
              node_x = (node_x + 1 == nx) ? 0 : node_x + 1;                                        \
            }                                                                                      \
            node_y = (node_y + 1 == ny) ? 0 : node_y + 1;                                          \
          }                                                                                        \
          node_z = (node_z + 1 == nz) ? 0 : node_z + 1;                                            \
        }                                                                                          \
      }                                                                                            \
    }                                                                                              \
    return status;                                                                                 \
  }

GBGO_TRANSFER(double, f64, gbgo_locate_f64)

static int locate_f32_adapter(float x, float o, float dx, int64_t *b, float *t) {
  return gbgo_locate_f32(x, o, dx, b, t);
}
GBGO_TRANSFER(float, f32, locate_f32_adapter)

static int resolve_threads(int nthreads) {
#ifdef _OPENMP
  return nthreads > 0 ? nthreads : omp_get_max_threads();
#else
  (void)nthreads;
  return 1;
#endif
}

int gbgo_gather_f64(const int64_t *gn, const double *origin, const double *spacing, int ncomp,
                    const double *field, const double *pos, int64_t m, const int32_t *trav,
                    const double *coeffs, int n2, int m2, double *out) {
  return gather_body_f64(gn, origin, spacing, ncomp, field, pos, m, trav, coeffs, n2, m2, out, 1);
}
int gbgo_gather_f32(const int64_t *gn, const double *origin, const double *spacing, int ncomp,
                    const float *field, const float *pos, int64_t m, const int32_t *trav,
                    const double *coeffs, int n2, int m2, float *out) {
  return gather_body_f32(gn, origin, spacing, ncomp, field, pos, m, trav, coeffs, n2, m2, out, 1);
}
int gbgo_scatter_f64(const int64_t *gn, const double *origin, const double *spacing, int ncomp,
                     double *field, const double *pos, int64_t m, const double *q,
                     const int32_t *trav, const double *coeffs, int n2, int m2, double alpha,
                     double beta) {
  return scatter_body_f64(gn, origin, spacing, ncomp, field, pos, m, q, trav, coeffs, n2, m2,
                          alpha, beta, 1);
}
int gbgo_scatter_f32(const int64_t *gn, const double *origin, const double *spacing, int ncomp,
                     float *field, const float *pos, int64_t m, const float *q,
                     const int32_t *trav, const double *coeffs, int n2, int m2, double alpha,
                     double beta) {
  return scatter_body_f32(gn, origin, spacing, ncomp, field, pos, m, q, trav, coeffs, n2, m2,
                          alpha, beta, 1);
}
int gbgo_gather_f64_mt(const int64_t *gn, const double *origin, const double *spacing, int ncomp,
                       const double *field, const double *pos, int64_t m, const int32_t *trav,
                       const double *coeffs, int n2, int m2, double *out, int nthreads) {
  return gather_body_f64(gn, origin, spacing, ncomp, field, pos, m, trav, coeffs, n2, m2, out,
                         resolve_threads(nthreads));
}
int gbgo_gather_f32_mt(const int64_t *gn, const double *origin, const double *spacing, int ncomp,
                       const float *field, const float *pos, int64_t m, const int32_t *trav,
                       const double *coeffs, int n2, int m2, float *out, int nthreads) {
  return gather_body_f32(gn, origin, spacing, ncomp, field, pos, m, trav, coeffs, n2, m2, out,
                         resolve_threads(nthreads));
}
int gbgo_scatter_f64_mt(const int64_t *gn, const double *origin, const double *spacing, int ncomp,
                        double *field, const double *pos, int64_t m, const double *q,
                        const int32_t *trav, const double *coeffs, int n2, int m2, double alpha,
                        double beta, int nthreads) {
  return scatter_body_f64(gn, origin, spacing, ncomp, field, pos, m, q, trav, coeffs, n2, m2,
                          alpha, beta, resolve_threads(nthreads));
}
int gbgo_scatter_f32_mt(const int64_t *gn, const double *origin, const double *spacing, int ncomp,
                        float *field, const float *pos, int64_t m, const float *q,
                        const int32_t *trav, const double *coeffs, int n2, int m2, double alpha,
                        double beta, int nthreads) {
  return scatter_body_f32(gn, origin, spacing, ncomp, field, pos, m, q, trav, coeffs, n2, m2,
                          alpha, beta, resolve_threads(nthreads));
}

/* ------------------------------------------------------- traversal order */

/* Interpolation.jl:636-642: comparisons in floating point before any conversion. */
int64_t gbgo_tile_index_f64(double coordinate, double origin, double inverse_tile, int64_t tiles) {
  const double u = (coordinate - origin) * inverse_tile;
  if (isnan(u)) return 0;
  if (u <= 0.0) return 0;
  if (u >= (double)tiles) return tiles - 1;
  return (int64_t)u;
}
int64_t gbgo_tile_index_f32(float coordinate, float origin, float inverse_tile, int64_t tiles) {
  const float u = (coordinate - origin) * inverse_tile;
  if (isnan(u)) return 0;
  if (u <= 0.0f) return 0;
  if (u >= (float)tiles) return tiles - 1;
  return (int64_t)u;
}

/* Interpolation.jl:689-692 (tiles), 645-661 (keys), 664-669 (count), 712 (cumsum),
 * 672-684 (place).  Keys are the reference's: 2 + i1 + t1*(i2 + t2*i3). */
#define GBGO_ORDER(T, SUF)                                                                         \
  int gbgo_traversal_order_##SUF(const int64_t *gn, const double *domain, const double *origin,   \
                                 const T *pos, int64_t m, int64_t tile_size, int32_t *order,       \
                                 int64_t *keys_out) {                                              \
    if (tile_size < 1) return GBGO_EARG;                                                           \
    if (m == 0) return GBGO_OK;                                                                    \
    int64_t tiles[3];                                                                              \
    T inv[3], o[3];                                                                                \
    for (int d = 0; d < 3; ++d) {                                                                  \
      int64_t t = (gn[d] + tile_size - 1) / tile_size;                                             \
      tiles[d] = t > 1 ? t : 1;                                                                    \
      inv[d] = (T)tiles[d] / (T)domain[d];                                                         \
      o[d] = (T)origin[d];                                                                         \
    }                                                                                              \
    const int64_t buckets = tiles[0] * tiles[1] * tiles[2] + 2;                                    \
    int64_t *keys = (int64_t *)malloc(sizeof(int64_t) * (size_t)m);                                \
    int64_t *counts = (int64_t *)calloc((size_t)buckets + 1, sizeof(int64_t));                     \
    if (!keys || !counts) { free(keys); free(counts); return GBGO_EARG; }                          \
    for (int64_t p = 0; p < m; ++p) {                                                              \
      const int64_t i1 = gbgo_tile_index_##SUF(pos[p], o[0], inv[0], tiles[0]);                    \
      const int64_t i2 = gbgo_tile_index_##SUF(pos[p + m], o[1], inv[1], tiles[1]);                \
      const int64_t i3 = gbgo_tile_index_##SUF(pos[p + 2 * m], o[2], inv[2], tiles[2]);            \
      keys[p] = 2 + i1 + tiles[0] * (i2 + tiles[1] * i3); /* 1-based bucket + head slot */       \
      counts[keys[p]] += 1;                                                                        \
    }                                                                                              \
    /* inclusive running total (cumsum!), indexed 1-based like the reference */                    \
    for (int64_t b = 2; b <= buckets; ++b) counts[b] += counts[b - 1];                             \
    for (int64_t p = 0; p < m; ++p) {                                                              \
      const int64_t slot = ++counts[keys[p] - 1]; /* 1-based slot */                               \
      order[slot - 1] = (int32_t)(p + 1);                                                          \
    }                                                                                              \
    if (keys_out) memcpy(keys_out, keys, sizeof(int64_t) * (size_t)m);                             \
    free(keys);                                                                                    \
    free(counts);                                                                                  \
    return GBGO_OK;                                                                                \
  }

GBGO_ORDER(double, f64)
GBGO_ORDER(float, f32)

/* ------------------------------------------------------------------ wrap */

/* Julia's float mod (Base: r = rem(x, y); fix the sign toward the divisor). */
static double jl_mod_f64(double x, double y) {
  double r = fmod(x, y);
  if (r == 0.0) return copysign(r, y);
  if ((r > 0) != (y > 0)) return r + y;
  return r;
}
static float jl_mod_f32(float x, float y) {
  float r = fmodf(x, y);
  if (r == 0.0f) return copysignf(r, y);
  if ((r > 0) != (y > 0)) return r + y;
  return r;
}

/* Points.jl:1245-1249. */
double gbgo_wrap_coordinate_f64(double coordinate, double extent, double origin) {
  double offset = jl_mod_f64(coordinate - origin, extent);
  offset = (offset == extent) ? 0.0 : offset;
  return offset + origin;
}
float gbgo_wrap_coordinate_f32(float coordinate, float extent, float origin) {
  float offset = jl_mod_f32(coordinate - origin, extent);
  offset = (offset == extent) ? 0.0f : offset;
  return offset + origin;
}

/* Points.jl:1217-1231, 1382-1440 -- displace!(dst, src, [grid,] (c_1, v_1), ..., (c_K, v_K)):
 * per coordinate dst = (((src + c_1 v_1) + c_2 v_2) + ...), each product and sum rounded
 * in the positions' type (Julia's broadcast fuses no multiply-add; coefficients converted
 * to that type first), then, with wrap, _wrap_coordinate with the axis's extent and origin.
 * All arrays (M, 3) column-major; dst may be src. */
void gbgo_displace_f64(double *dst, const double *src, int64_t m, int32_t nterms, const double *coefficients,
                       const double *const *sections, int32_t wrap, const double *extent, const double *origin) {
  for (int a = 0; a < 3; ++a)
    for (int64_t p = 0; p < m; ++p) {
      double x = src[p + m * a];
      for (int32_t j = 0; j < nterms; ++j) {
        const double prod = coefficients[j] * sections[j][p + m * a];
        x = x + prod;
      }
      dst[p + m * a] = wrap ? gbgo_wrap_coordinate_f64(x, extent[a], origin[a]) : x;
    }
}
void gbgo_displace_f32(float *dst, const float *src, int64_t m, int32_t nterms, const double *coefficients,
                       const float *const *sections, int32_t wrap, const double *extent, const double *origin) {
  for (int a = 0; a < 3; ++a)
    for (int64_t p = 0; p < m; ++p) {
      float x = src[p + m * a];
      for (int32_t j = 0; j < nterms; ++j) {
        const float prod = (float)coefficients[j] * sections[j][p + m * a];
        x = x + prod;
      }
      dst[p + m * a] = wrap ? gbgo_wrap_coordinate_f32(x, (float)extent[a], (float)origin[a]) : x;
    }
}
