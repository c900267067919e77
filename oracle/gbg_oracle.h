/*
 * gbg_oracle.h -- CPU oracle for the particle gather/scatter path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the reference's
 * spline transfer (GBGPeriodicFields.jl, src/Interpolation.jl and src/Points.jl),
 * used by the tests, by smoke() and by the CPU-baseline leg of bench.py as the
 * checker.  No product code path links or calls it.
 *
 * Parity pin: the restatement is checked against every known-answer vector the
 * reference's own tests hold for this path (test/interpolation_transfer.jl:19-87,
 * the TurTLE coefficient pins, the Catmull-Rom closed form, partition of unity,
 * Lagrange cardinal basis, linear m=0 weights) and against the reference's
 * independent hand-written Catmull-Rom gather/scatter
 * (test/exhaustive/references.jl:590-654), restated in tests/.
 *
 * Layouts follow the reference (column-major, 0-based here):
 *   field      : f[x + Nx*y + Nx*Ny*z + N*c]          (Interpolation.jl:1038-1041)
 *   positions  : pos[p + M*d], d = 0,1,2                 (Points.jl:124-133)
 *   point vals : v[p + M*c]                              (Interpolation.jl:1048)
 *   scheme     : coeffs[q + N2*r]  (node q, power r)     (Interpolation.jl:311-312)
 */
#ifndef GBG_ORACLE_H
#define GBG_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
  GBGO_OK = 0,
  GBGO_EARG = 1,        /* ArgumentError in the reference */
  GBGO_ENONFINITE = 2   /* floor(Int, NaN/Inf) throws InexactError in the reference */
};

#define GBGO_MAX_NODES 32
#define GBGO_MAX_POWERS 64

/* Interpolation.jl:326-354 -- Fornberg finite-difference weights.
 * w[i + n*k] = weight of nodes[i] in the order-k derivative at x0. */
int gbgo_fornberg(double x0, const double *nodes, int n, int max_order, double *w);

/* Interpolation.jl:367-392 -- (2n+2) x (2m+2) smooth-spline coefficients. */
int gbgo_hermite_weight_matrix(int n, int m, double *coeffs);

/* Interpolation.jl:403-415 -- (2n+2) x (2n+2) Lagrange cardinal coefficients. */
int gbgo_lagrange_weight_matrix(int n, double *coeffs);

/* Interpolation.jl:244-258 (LalescuSpline) and 293-306 (LagrangeSpline): validate the
 * width/smoothness and fill coeffs; *n2 = nodes per axis, *m2 = number of powers. */
int gbgo_lalescu(int stencil_width, int smoothness, double *coeffs, int *n2, int *m2);
int gbgo_lagrange(int stencil_width, double *coeffs, int *n2, int *m2);

/* Interpolation.jl:440-446 -- Horner evaluation of the N2 per-axis weights at t. */
void gbgo_axis_weights_f64(const double *coeffs, int n2, int m2, double t, double *w);
void gbgo_axis_weights_f32(const float *coeffs, int n2, int m2, float t, float *w);

/* Interpolation.jl:456-460 -- base cell (floor) and fraction in the element type. */
int gbgo_locate_f64(double x, double origin, double spacing, int64_t *base, double *t);
int gbgo_locate_f32(float x, float origin, float spacing, int64_t *base, float *t);

/* Interpolation.jl:1007-1052 (gather) and 1063-1106 (scatter), plus the driver-side
 * beta prescale of anterpolate! (1309-1313).  traversal is NULL or a 1-based
 * permutation (Interpolation.jl:618-627).  Serial: the summation order of the
 * scatter is the point order, which the reference does not fix (atomics).
 * grid_n: Nx,Ny,Nz.  Returns GBGO_ENONFINITE on a non-finite position. */
int gbgo_gather_f64(const int64_t *grid_n, const double *origin, const double *spacing,
                    int ncomp, const double *field, const double *pos, int64_t m,
                    const int32_t *traversal, const double *coeffs, int n2, int m2,
                    double *out);
int gbgo_gather_f32(const int64_t *grid_n, const double *origin, const double *spacing,
                    int ncomp, const float *field, const float *pos, int64_t m,
                    const int32_t *traversal, const double *coeffs, int n2, int m2,
                    float *out);
int gbgo_scatter_f64(const int64_t *grid_n, const double *origin, const double *spacing,
                     int ncomp, double *field, const double *pos, int64_t m,
                     const double *q, const int32_t *traversal, const double *coeffs,
                     int n2, int m2, double alpha, double beta);
int gbgo_scatter_f32(const int64_t *grid_n, const double *origin, const double *spacing,
                     int ncomp, float *field, const float *pos, int64_t m,
                     const float *q, const int32_t *traversal, const double *coeffs,
                     int n2, int m2, double alpha, double beta);

/* Threaded twins (OpenMP over points; scatter through atomic adds, as the reference's
 * KernelAbstractions CPU() launch with Atomix does, docs/ARCHITECTURE.md:793-797).
 * Used only to time the reference's CPU path.  nthreads <= 0 means all cores. */
int gbgo_gather_f64_mt(const int64_t *grid_n, const double *origin, const double *spacing,
                       int ncomp, const double *field, const double *pos, int64_t m,
                       const int32_t *traversal, const double *coeffs, int n2, int m2,
                       double *out, int nthreads);
int gbgo_gather_f32_mt(const int64_t *grid_n, const double *origin, const double *spacing,
                       int ncomp, const float *field, const float *pos, int64_t m,
                       const int32_t *traversal, const double *coeffs, int n2, int m2,
                       float *out, int nthreads);
int gbgo_scatter_f64_mt(const int64_t *grid_n, const double *origin, const double *spacing,
                        int ncomp, double *field, const double *pos, int64_t m,
                        const double *q, const int32_t *traversal, const double *coeffs,
                        int n2, int m2, double alpha, double beta, int nthreads);
int gbgo_scatter_f32_mt(const int64_t *grid_n, const double *origin, const double *spacing,
                        int ncomp, float *field, const float *pos, int64_t m,
                        const float *q, const int32_t *traversal, const double *coeffs,
                        int n2, int m2, double alpha, double beta, int nthreads);

/* Interpolation.jl:636-642 -- saturating tile index. */
int64_t gbgo_tile_index_f64(double coordinate, double origin, double inverse_tile, int64_t tiles);
int64_t gbgo_tile_index_f32(float coordinate, float origin, float inverse_tile, int64_t tiles);

/* Interpolation.jl:645-684, 689-692, 769-785, 816-833 -- the traversal order.  The
 * reference places points within a tile in whatever order its atomics resolve; this
 * serial restatement places them in point order (a stable counting sort), which is
 * one of the orders the reference can produce.  order: 1-based, length m.
 * keys_out (optional, may be NULL): the reference's Int64 bucket key per point. */
int gbgo_traversal_order_f64(const int64_t *grid_n, const double *domain, const double *origin,
                             const double *pos, int64_t m, int64_t tile_size,
                             int32_t *order, int64_t *keys_out);
int gbgo_traversal_order_f32(const int64_t *grid_n, const double *domain, const double *origin,
                             const float *pos, int64_t m, int64_t tile_size,
                             int32_t *order, int64_t *keys_out);

/* Points.jl:1245-1249 -- periodic wrap of one coordinate. */
double gbgo_wrap_coordinate_f64(double coordinate, double extent, double origin);
float gbgo_wrap_coordinate_f32(float coordinate, float extent, float origin);
void gbgo_displace_f64(double *dst, const double *src, int64_t m, int32_t nterms, const double *coefficients,
                       const double *const *sections, int32_t wrap, const double *extent, const double *origin);
void gbgo_displace_f32(float *dst, const float *src, int64_t m, int32_t nterms, const double *coefficients,
                       const float *const *sections, int32_t wrap, const double *extent, const double *origin);

/* Interpolation.jl:1000 + 1025-1027 -- the periodic walk: fills idx[0..width) with
 * mod(base - neighbourhood + t, extent) by the reference's wrapped-start + step rule. */
void gbgo_walk(int64_t base, int64_t neighbourhood, int64_t extent, int width, int64_t *idx);

#ifdef __cplusplus
}
#endif
#endif
