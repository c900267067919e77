// Drop-in transfers on the reference's own array layouts (sm_103a).
//
//   gbg_interpolate             interpolate!            Interpolation.jl:1181-1198, 1007-1052
//   gbg_anterpolate             anterpolate!            Interpolation.jl:1299-1323, 1063-1106
//   gbg_point_traversal_order   point_traversal_order   Interpolation.jl:816-833, 636-684
//   gbg_validate_traversal      PointTraversalOrder     Interpolation.jl:560-589
//
// The gather is one thread per work item, as in the reference, contracting the x
// direction first for every component of the chunk.  The scatter is not the reference's
// atomic push: points are sorted by brick and cell (a stable device counting sort), and each
// brick's nodes are accumulated in shared memory as 128-bit integer sums on a scale local to
// the brick (or, for a stencil wider than the grid, every node pulls its contributions).  No
// float atomics are used, so the scatter is bitwise reproducible and independent of any
// traversal order, and each node keeps the accuracy of an FP64 sum of its own
// contributions.
#include <mutex>
#include <string>

#include <array>
#include <map>
#include <vector>

#include "gbg_common.cuh"

namespace gbg {
namespace {

constexpr int kThreads = 256;

template <typename T>
struct GridT {
  int64_t nx, ny, nz, npf;
  T ox, oy, oz;  // T.(grid.origin)
  T dx, dy, dz;  // T.(grid.grid_spacing)
};

template <typename T>
GridT<T> make_grid(const gbg_grid &g) {
  GridT<T> r;
  r.nx = g.n[0];
  r.ny = g.n[1];
  r.nz = g.n[2];
  r.npf = g.n[0] * g.n[1] * g.n[2];
  r.ox = T(g.origin[0]);
  r.oy = T(g.origin[1]);
  r.oz = T(g.origin[2]);
  r.dx = T(g.spacing[0]);
  r.dy = T(g.spacing[1]);
  r.dz = T(g.spacing[2]);
  return r;
}

template <typename T>
__device__ __forceinline__ T quiet_nan();
template <>
__device__ __forceinline__ double quiet_nan<double>() { return __longlong_as_double(0x7ff8000000000000LL); }
template <>
__device__ __forceinline__ float quiet_nan<float>() { return __int_as_float(0x7fc00000); }

// The wrapped node offsets visited along one axis: the reference's wrapped start
// mod(base - n, N) followed by its step rule (Interpolation.jl:1000, 1025-1027).
template <int N2>
__device__ __forceinline__ void walk_offsets(int64_t base, int64_t extent, int64_t stride,
                                             int64_t (&off)[N2]) {
  int64_t node = imod(base - (N2 - 2) / 2, extent);
#pragma unroll
  for (int i = 0; i < N2; ++i) {
    off[i] = node * stride;
    node = (node + 1 == extent) ? 0 : node + 1;
  }
}

__device__ __forceinline__ int64_t step_up(int64_t node, int64_t extent) {
  return (node + 1 == extent) ? 0 : node + 1;
}
__device__ __forceinline__ int64_t step_down(int64_t node, int64_t extent) {
  return node == 0 ? extent - 1 : node - 1;
}

// Locates a point on the three axes; false if any coordinate is non-finite.
template <typename T>
__device__ __forceinline__ bool locate3(const GridT<T> &g, const T *__restrict__ pos, int64_t p,
                                        int64_t m, int64_t (&b)[3], T (&t)[3]) {
  bool ok = locate(__ldg(pos + p), g.ox, g.dx, b[0], t[0]);
  ok &= locate(__ldg(pos + p + m), g.oy, g.dy, b[1], t[1]);
  ok &= locate(__ldg(pos + p + 2 * m), g.oz, g.dz, b[2], t[2]);
  return ok;
}

// _visit (Interpolation.jl:618-619), bounds-checked instead of trusted.
__device__ __forceinline__ bool visit(const int32_t *__restrict__ trav, int64_t w, int64_t m,
                                      int64_t &p, int32_t *status) {
  p = w;
  if (!trav) return true;
  const int64_t v = (int64_t)__ldg(trav + w) - 1;
  if (v < 0 || v >= m) {
    if (status) atomicOr(status, GBG_DEV_TRAVERSAL);
    return false;
  }
  p = v;
  return true;
}

// ---------------------------------------------------------------- gather

// Horner with fused multiply-adds (one rounding per step instead of the reference's two;
// the weights differ by at most an ulp or so, far inside the transfer's 1e-13 bar).
// M2 > 0: that many powers at compile time; M2 == 0: the scheme's own count.
template <typename T, int N2, int M2>
__device__ __forceinline__ void axis_weights_fma(const SchemeT<T, N2> &s, T t, T (&w)[N2]) {
  if constexpr (M2 > 0) {
#pragma unroll
    for (int q = 0; q < N2; ++q) w[q] = s.c[q + N2 * (M2 - 1)];
#pragma unroll
    for (int p = M2 - 2; p >= 0; --p)
#pragma unroll
      for (int q = 0; q < N2; ++q) w[q] = fma_rn(w[q], t, s.c[q + N2 * p]);
  } else {
#pragma unroll
    for (int q = 0; q < N2; ++q) w[q] = T(0);
#pragma unroll
    for (int p = GBG_MAX_POWERS - 1; p >= 0; --p) {
      if (p < s.m2) {
#pragma unroll
        for (int q = 0; q < N2; ++q) w[q] = fma_rn(w[q], t, s.c[q + N2 * p]);
      }
    }
  }
}

// Compile-time width N2: the (j, i) stencil plane is unrolled, z advances by the
// reference's running walk.  The x direction is contracted first, per (j, k) and
// component, s = sum_i w1[i] f, then acc += (w2[j] w3[k]) s: 22 FP64 operations per
// (j, k) at width 6 and 3 components instead of 25 -- this kernel is FP64-pipe-bound.
template <typename T, int N2, int M2, int CC>
__global__ void __launch_bounds__(kThreads)
    k_gather_plain(GridT<T> g, SchemeT<T, N2> s, int ncomp, const T *__restrict__ field,
                   const T *__restrict__ pos, int64_t m, const int32_t *__restrict__ trav,
                   T *__restrict__ out, int32_t *status) {
  const int64_t nxny = g.nx * g.ny;
  for (int64_t w = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; w < m;
       w += (int64_t)gridDim.x * blockDim.x) {
    int64_t p;
    if (!visit(trav, w, m, p, status)) continue;
    int64_t b[3];
    T t[3];
    const bool ok = locate3(g, pos, p, m, b, t);
    if (!ok && status) atomicOr(status, GBG_DEV_NONFINITE);
    T w1[N2], w2[N2], w3[N2];
    axis_weights_fma<T, N2, M2>(s, t[0], w1);
    axis_weights_fma<T, N2, M2>(s, t[1], w2);
    axis_weights_fma<T, N2, M2>(s, t[2], w3);
    int64_t ix[N2], iy[N2];
    walk_offsets<N2>(b[0], g.nx, 1, ix);
    walk_offsets<N2>(b[1], g.ny, g.nx, iy);
    const int64_t z0 = imod(b[2] - (N2 - 2) / 2, g.nz);
    for (int c0 = 0; c0 < ncomp; c0 += CC) {
      T acc[CC];
#pragma unroll
      for (int c = 0; c < CC; ++c) acc[c] = T(0);
      const T *fc = field + g.npf * c0;
      int64_t node_z = z0;
#pragma unroll 1
      for (int k = 0; k < N2; ++k) {
        T w3k = w3[0];
#pragma unroll
        for (int q = 1; q < N2; ++q)
          if (q == k) w3k = w3[q];
        const T *plane = fc + node_z * nxny;
#pragma unroll
        for (int j = 0; j < N2; ++j) {
          const T wyz = mul_rn(w2[j], w3k);
          const T *row = plane + iy[j];
          T sx[CC];
#pragma unroll
          for (int c = 0; c < CC; ++c) sx[c] = mul_rn(w1[0], __ldg(row + ix[0] + g.npf * c));
#pragma unroll
          for (int i = 1; i < N2; ++i) {
            const T *f = row + ix[i];
#pragma unroll
            for (int c = 0; c < CC; ++c) sx[c] = fma_rn(w1[i], __ldg(f + g.npf * c), sx[c]);
          }
#pragma unroll
          for (int c = 0; c < CC; ++c) acc[c] = fma_rn(wyz, sx[c], acc[c]);
        }
        node_z = step_up(node_z, g.nz);
      }
#pragma unroll
      for (int c = 0; c < CC; ++c) out[p + m * (c0 + c)] = ok ? acc[c] : quiet_nan<T>();
    }
  }
}

// Fixed-point exponent P of the scatter's weights, w * 2^P: |w| <= L (the scheme's
// Bernstein bound with evaluation slack) <= 1.5 * 2^lb, P = 62 - lb.  Then
// |w * 2^P| < 1.5 * 2^62, a product of three weights' high halves stays below
// 3.375 * 2^58, a contribution below 3.375 * 2^56, and a node's sum, shifted by
// bits(K_max) - 5, below 2^63.
int fixed_weight_exp(const gbg_scheme &sch) {
  const double L = weight_bound(sch, std::ldexp(1.0, -40));
  int lb = 0;
  while (1.5 * std::ldexp(1.0, lb) < L && lb < 60) ++lb;
  return 62 - lb;
}

// Run-time width (stencils of 10..16 nodes): nothing unrolled.
template <typename T>
__global__ void __launch_bounds__(kThreads)
    k_gather_plain_dyn(GridT<T> g, SchemeT<T, GBG_MAX_NODES> s, int ncomp,
                       const T *__restrict__ field, const T *__restrict__ pos, int64_t m,
                       const int32_t *__restrict__ trav, T *__restrict__ out, int32_t *status) {
  __shared__ T cs[GBG_MAX_NODES * GBG_MAX_POWERS];
  stage_coeffs(s, cs);
  const int n2 = s.n2, nb = (n2 - 2) / 2;
  for (int64_t w = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; w < m;
       w += (int64_t)gridDim.x * blockDim.x) {
    int64_t p;
    if (!visit(trav, w, m, p, status)) continue;
    int64_t b[3];
    T t[3];
    const bool ok = locate3(g, pos, p, m, b, t);
    if (!ok && status) atomicOr(status, GBG_DEV_NONFINITE);
    T w1[GBG_MAX_NODES], w2[GBG_MAX_NODES], w3[GBG_MAX_NODES];
    axis_weights_dyn(cs, n2, s.m2, t[0], w1);
    axis_weights_dyn(cs, n2, s.m2, t[1], w2);
    axis_weights_dyn(cs, n2, s.m2, t[2], w3);
    const int64_t x0 = imod(b[0] - nb, g.nx), y0 = imod(b[1] - nb, g.ny), z0 = imod(b[2] - nb, g.nz);
#pragma unroll 1
    for (int c = 0; c < ncomp; ++c) {
      T acc = T(0);
      int64_t node_z = z0;
#pragma unroll 1
      for (int k = 0; k < n2; ++k) {
        int64_t node_y = y0;
#pragma unroll 1
        for (int j = 0; j < n2; ++j) {
          const T wyz = mul_rn(w2[j], w3[k]);
          const T *row = field + g.npf * c + g.nx * node_y + g.nx * g.ny * node_z;
          int64_t node_x = x0;
#pragma unroll 1
          for (int i = 0; i < n2; ++i) {
            acc = fma_rn(mul_rn(wyz, w1[i]), __ldg(row + node_x), acc);
            node_x = step_up(node_x, g.nx);
          }
          node_y = step_up(node_y, g.ny);
        }
        node_z = step_up(node_z, g.nz);
      }
      out[p + m * c] = ok ? acc : quiet_nan<T>();
    }
  }
}

// --------------------------------------------------------------- scatter

// The cell (of the base node) each point falls in, and the per-cell point count.
template <typename T>
__global__ void __launch_bounds__(kThreads)
    k_cell_keys(GridT<T> g, const T *__restrict__ pos, int64_t m, uint32_t *__restrict__ keys,
                uint32_t *__restrict__ counts, uint32_t *__restrict__ rank, int32_t *status) {
  for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < m;
       p += (int64_t)gridDim.x * blockDim.x) {
    int64_t b[3];
    T t[3];
    const bool ok = locate3(g, pos, p, m, b, t);
    if (!ok && status) atomicOr(status, GBG_DEV_NONFINITE);
    const uint32_t key =
        (uint32_t)(imod(b[0], g.nx) + g.nx * (imod(b[1], g.ny) + g.ny * imod(b[2], g.nz)));
    keys[p] = key;
    rank[p] = atomicAdd(counts + key, 1u);  // the point's rank within its cell, in no order
  }
}

// Per sorted slot: the point's three weight vectors and its alpha-scaled quantities
// (quantity = T(alpha) * q, Interpolation.jl:1085), laid out slot-major for the pull.
template <typename T>
__global__ void __launch_bounds__(kThreads)
    k_scatter_prep(GridT<T> g, SchemeT<T, GBG_MAX_NODES> s, int ncomp, const T *__restrict__ pos,
                   const T *__restrict__ q, int64_t m, const uint32_t *__restrict__ perm, T alpha,
                   T *__restrict__ rec, T *__restrict__ qs) {
  __shared__ T cs[GBG_MAX_NODES * GBG_MAX_POWERS];
  stage_coeffs(s, cs);
  const int n2 = s.n2;
  for (int64_t sl = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; sl < m;
       sl += (int64_t)gridDim.x * blockDim.x) {
    const int64_t p = perm[sl];
    int64_t b[3];
    T t[3];
    const bool ok = locate3(g, pos, p, m, b, t);
    T *r = rec + sl * 3 * n2;
#pragma unroll 1
    for (int a = 0; a < 3; ++a) {
      T w[GBG_MAX_NODES];
      axis_weights_dyn(cs, n2, s.m2, t[a], w);
#pragma unroll 1
      for (int i = 0; i < n2; ++i) r[a * n2 + i] = ok ? w[i] : quiet_nan<T>();
    }
#pragma unroll 1
    for (int c = 0; c < ncomp; ++c) qs[sl * ncomp + c] = mul_rn(alpha, q[p + m * c]);
  }
}

// One thread per grid node: sum, in a fixed order, the contributions of the points in
// every cell whose stencil reaches this node, then write alpha*W^T q + beta*field.  Weight
// index i reaches node x from the cell (x + n - i) mod N; for a stencil wider than the
// grid a cell is reached through several weight indices and each contributes, exactly as
// the reference's wrapped walk deposits it several times.
template <typename T, int CC>
__global__ void __launch_bounds__(kThreads)
    k_scatter_pull(GridT<T> g, int n2, int ncomp, const uint32_t *__restrict__ cell_start,
                   const T *__restrict__ rec, const T *__restrict__ qs, T *__restrict__ field,
                   T beta, int beta_zero) {
  const int nb = (n2 - 2) / 2;
  const int64_t nxny = g.nx * g.ny;
  for (int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; n < g.npf;
       n += (int64_t)gridDim.x * blockDim.x) {
    const int64_t x = n % g.nx;
    const int64_t yz = n / g.nx;
    const int64_t y = yz % g.ny;
    const int64_t z = yz / g.ny;
    const int64_t cx0 = imod(x + nb, g.nx), cy0 = imod(y + nb, g.ny), cz0 = imod(z + nb, g.nz);
    for (int c0 = 0; c0 < ncomp; c0 += CC) {
      T acc[CC];
#pragma unroll
      for (int c = 0; c < CC; ++c) acc[c] = T(0);
      int64_t cz = cz0;
#pragma unroll 1
      for (int k = 0; k < n2; ++k) {
        int64_t cy = cy0;
#pragma unroll 1
        for (int j = 0; j < n2; ++j) {
          const int64_t rowoff = g.nx * cy + nxny * cz;
          int64_t cx = cx0;
#pragma unroll 1
          for (int i = 0; i < n2; ++i) {
            const int64_t cell = cx + rowoff;
            const uint32_t s0 = __ldg(cell_start + cell), s1 = __ldg(cell_start + cell + 1);
#pragma unroll 1
            for (uint32_t sl = s0; sl < s1; ++sl) {
              const T *r = rec + (int64_t)sl * 3 * n2;
              const T wv = mul_rn(mul_rn(__ldg(r + n2 + j), __ldg(r + 2 * n2 + k)), __ldg(r + i));
              const T *qv = qs + (int64_t)sl * ncomp + c0;
#pragma unroll
              for (int c = 0; c < CC; ++c) acc[c] = fma_rn(wv, __ldg(qv + c), acc[c]);
            }
            cx = step_down(cx, g.nx);
          }
          cy = step_down(cy, g.ny);
        }
        cz = step_down(cz, g.nz);
      }
#pragma unroll
      for (int c = 0; c < CC; ++c) {
        T *f = field + n + g.npf * (c0 + c);
        *f = beta_zero ? acc[c] : add_rn(mul_rn(beta, *f), acc[c]);
      }
    }
  }
}

// The same pull for a compile-time width: the cells of a node's x walk are computed once,
// the x loop is unrolled; the order of every sum is the one above (z, y, x cells, then each
// cell's points in slot order), so the results are the same bits.
template <typename T, int N2, int CC>
__global__ void __launch_bounds__(kThreads)
    k_scatter_pull_n(GridT<T> g, int ncomp, const uint32_t *__restrict__ cell_start, const T *__restrict__ rec,
                     const T *__restrict__ qs, T *__restrict__ field, T beta, int beta_zero) {
  constexpr int nb = (N2 - 2) / 2;
  const int64_t nxny = g.nx * g.ny;
  for (int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; n < g.npf;
       n += (int64_t)gridDim.x * blockDim.x) {
    const int64_t x = n % g.nx;
    const int64_t yz = n / g.nx;
    const int64_t y = yz % g.ny;
    const int64_t z = yz / g.ny;
    int64_t cxs[N2];
    {
      int64_t cx = imod(x + nb, g.nx);
#pragma unroll
      for (int i = 0; i < N2; ++i) {
        cxs[i] = cx;
        cx = step_down(cx, g.nx);
      }
    }
    const int64_t cy0 = imod(y + nb, g.ny), cz0 = imod(z + nb, g.nz);
    for (int c0 = 0; c0 < ncomp; c0 += CC) {
      T acc[CC];
#pragma unroll
      for (int c = 0; c < CC; ++c) acc[c] = T(0);
      int64_t cz = cz0;
#pragma unroll 1
      for (int k = 0; k < N2; ++k) {
        int64_t cy = cy0;
#pragma unroll 1
        for (int j = 0; j < N2; ++j) {
          const int64_t rowoff = g.nx * cy + nxny * cz;
#pragma unroll
          for (int i = 0; i < N2; ++i) {
            const int64_t cell = cxs[i] + rowoff;
            const uint32_t s0 = __ldg(cell_start + cell), s1 = __ldg(cell_start + cell + 1);
#pragma unroll 1
            for (uint32_t sl = s0; sl < s1; ++sl) {
              const T *r = rec + (int64_t)sl * (3 * N2);
              const T wv = mul_rn(mul_rn(__ldg(r + N2 + j), __ldg(r + 2 * N2 + k)), __ldg(r + i));
              const T *qv = qs + (int64_t)sl * ncomp + c0;
#pragma unroll
              for (int c = 0; c < CC; ++c) acc[c] = fma_rn(wv, __ldg(qv + c), acc[c]);
            }
          }
          cy = step_down(cy, g.ny);
        }
        cz = step_down(cz, g.nz);
      }
#pragma unroll
      for (int c = 0; c < CC; ++c) {
        T *f = field + n + g.npf * (c0 + c);
        *f = beta_zero ? acc[c] : add_rn(mul_rn(beta, *f), acc[c]);
      }
    }
  }
}

// ------------------------------------------------------ brick scatter
//
// The default scatter.  Points are sorted by brick and by cell within the brick (a stable
// counting sort, so the order is fixed).  A CTA owns one brick of nodes and accumulates, in
// shared memory, every contribution of the points in the cells whose stencils reach the
// brick (the extended region) as a 128-bit integer, so the sum does not depend on the
// order in which threads add.  Each node is written to HBM once.

struct BrickGeo {
  int32_t b[3];
  int64_t nb[3];
  int64_t bvol;
  // the scatter's shared accumulators: node (x, y, z) of component c at
  // c*slice + z*pp + y*p0 + x, pitches chosen so that a warp's atomics on one point's
  // stencil spread over the banks (choose_acc_pitches)
  int32_t p0 = 0, pp = 0;
  int64_t slice = 0;
  // most runs of consecutive keys along x in one row of any brick's region (brick_segments)
  int32_t nseg = 1;
};

// Binary exponents of the quantities, biased so that 0 means "no non-zero quantity" and
// kENonFinite (above every finite one) a NaN or an infinity: a non-zero finite v has
// 2^(e-1) <= |v| < 2^e and is stored as e + kEBias.
constexpr int kEBias = 2048;
constexpr int kENonFinite = 4095;

__device__ __forceinline__ int biased_exponent(double v) {
  if (v == 0.0) return 0;
  if (!isfinite(v)) return kENonFinite;
  int e = 0;
  frexp(v, &e);
  return e + kEBias;
}

// One pass over the points in their own order: the locate, the brick-major key, the cell
// count (the atomic's value is the point's rank in its cell, for the counting sort), and
// per brick and component the largest exponent of the finite non-zero alpha*q.
template <typename T>
__global__ void __launch_bounds__(kThreads)
    k_brick_keys(GridT<T> g, BrickGeo bg, const T *__restrict__ pos, int64_t m, uint32_t *__restrict__ keys,
                 uint32_t *__restrict__ counts, uint32_t *__restrict__ rank, const T *__restrict__ q, int ncomp,
                 T alpha, uint32_t *__restrict__ ebrick, int32_t *status) {
  const int64_t n[3] = {g.nx, g.ny, g.nz};
  for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < m;
       p += (int64_t)gridDim.x * blockDim.x) {
    int64_t b[3];
    T t[3];
    const bool ok = locate3(g, pos, p, m, b, t);
    if (!ok && status) atomicOr(status, GBG_DEV_NONFINITE);
    int64_t brick = 0, local = 0;
#pragma unroll
    for (int d = 2; d >= 0; --d) {
      const int64_t c = imod(b[d], n[d]);
      brick = brick * bg.nb[d] + c / bg.b[d];
      local = local * bg.b[d] + c % bg.b[d];
    }
    const uint32_t key = (uint32_t)(brick * bg.bvol + local);
    keys[p] = key;
    rank[p] = atomicAdd(counts + key, 1u);
    for (int c = 0; c < ncomp; ++c) {
      const T v = mul_rn(alpha, q[p + m * c]);  // quantity = T(alpha)*q
      const int e = biased_exponent((double)v);
      if (e == kENonFinite) {
        if (status) atomicOr(status, GBG_DEV_NONFINITE);
      } else if (e) {
        atomicMax(ebrick + brick * ncomp + c, (uint32_t)e);
      }
    }
  }
}

// In sorted order, slot by slot: the point's three axes' stencil weights (the reference's
// Horner with fused multiply-adds, once per point) as 64-bit fixed point w * 2^wexp, and
// each alpha*q in floating form of its own: a 64-bit mantissa q * 2^(62 - e) (exact for
// every double) beside its biased exponent e.  The weights are evaluated here, from the
// position read through the permutation, rather than in the key pass, so they are written
// once, already sorted.
template <typename T, int N2, int M2>
__global__ void __launch_bounds__(kThreads)
    k_brick_order(GridT<T> g, SchemeT<T, N2> sch, const T *__restrict__ pos, const uint32_t *__restrict__ perm,
                  int64_t m, int wexp, long long *__restrict__ wts, const T *__restrict__ q, int ncomp, T alpha,
                  long long *__restrict__ qi, int32_t *__restrict__ qe) {
  for (int64_t sl = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; sl < m;
       sl += (int64_t)gridDim.x * blockDim.x) {
    const int64_t p = perm[sl];
    int64_t b[3];
    T t[3];
    const bool ok = locate3(g, pos, p, m, b, t);
    long long *dst = wts + sl * (3 * N2);
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      T w[N2];
      axis_weights_fma<T, N2, M2>(sch, ok ? t[d] : quiet_nan<T>(), w);
#pragma unroll
      for (int k = 0; k < N2; ++k) dst[d * N2 + k] = ok ? fixed_rn((double)w[k], wexp) : 0ll;
    }
    for (int c = 0; c < ncomp; ++c) {
      const T v = mul_rn(alpha, q[p + m * c]);
      const int e = biased_exponent((double)v);
      qi[sl * ncomp + c] = (e && e != kENonFinite) ? fixed_rn((double)v, 62 - (e - kEBias)) : 0ll;
      qe[sl * ncomp + c] = e;
    }
  }
}

// Adds the 128-bit integer (hi:lo) to the sum kept in shared memory as four 32-bit words
// w0 (lowest) .. w3, with native 32-bit atomics: each word's add returns the old value,
// whose wrap is the carry into the next word.  Each add wraps a word at most once, so
// after all adds the words hold the exact 128-bit sum (mod 2^128) in any order, as the
// two-word form atomic_add_split64 does for 64 bits.
__device__ __forceinline__ void atomic_add_split128(uint32_t *w0, uint32_t *w1, uint32_t *w2, uint32_t *w3, int i,
                                                    unsigned long long lo, unsigned long long hi) {
  const uint32_t v0 = (uint32_t)lo, v1 = (uint32_t)(lo >> 32), v2 = (uint32_t)hi, v3 = (uint32_t)(hi >> 32);
  const uint32_t o0 = atomicAdd(w0 + i, v0);
  const uint32_t c1 = (uint32_t)(o0 + v0 < v0);
  const uint32_t s1 = v1 + c1;  // wraps only when v1 == 2^32 - 1 and c1 == 1 (then s1 == 0)
  const uint32_t o1 = atomicAdd(w1 + i, s1);
  const uint32_t c2 = (uint32_t)(s1 < c1) + (uint32_t)(o1 + s1 < s1);
  const uint32_t s2 = v2 + c2;
  const uint32_t o2 = atomicAdd(w2 + i, s2);
  const uint32_t c3 = (uint32_t)(s2 < c2) + (uint32_t)(o2 + s2 < s2);
  atomicAdd(w3 + i, v3 + c3);
}

// One contribution: the node weight wn (64-bit fixed point) times the quantity's mantissa
// mq (exact signed 64 x 64 -> 128-bit product), shifted right by d with rounding (half up),
// added to the node's 128-bit sum.  d >= 127 leaves nothing to add.
__device__ __forceinline__ void add_contribution(uint32_t *a0, uint32_t *a1, uint32_t *a2, uint32_t *a3, int i,
                                                 long long wn, long long mq, int d) {
  if (mq == 0 || wn == 0 || d >= 127) return;
  unsigned long long lo = (unsigned long long)wn * (unsigned long long)mq;
  long long hi = __mul64hi(wn, mq);
  if (d > 0) {
    // + 2^(d-1), then an arithmetic shift right by d
    if (d <= 64) {
      const unsigned long long h = 1ull << (d - 1);
      const unsigned long long s = lo + h;
      hi += (long long)(s < lo);
      lo = s;
    } else {
      hi += (long long)(1ull << (d - 65));
    }
    if (d < 64) {
      lo = (lo >> d) | ((unsigned long long)hi << (64 - d));
      hi >>= d;
    } else if (d == 64) {
      lo = (unsigned long long)hi;
      hi = hi < 0 ? -1ll : 0ll;
    } else {
      lo = (unsigned long long)(hi >> (d - 64));
      hi = hi < 0 ? -1ll : 0ll;
    }
  }
  atomic_add_split128(a0, a1, a2, a3, i, lo, (unsigned long long)hi);
}

template <int N, typename T>
__device__ __forceinline__ T pick_t(const T (&w)[N], int q) {
  T v = w[0];
#pragma unroll
  for (int i = 1; i < N; ++i)
    if (i == q) v = w[i];
  return v;
}

// The default scatter (deterministic, FP64-grade per node).  A CTA owns one brick of
// nodes.  It lists the points of every cell whose stencil reaches the brick (the extended
// region), gives each warp a point (its lanes cover the point's nodes inside the brick),
// and adds every contribution w1*w2*w3*alpha*q to a 128-bit integer accumulator in shared
// memory.
//
// The arithmetic is integer: GB300's FP64 rate is 1/58 of its FP32 rate, while 64-bit
// integer products run on the integer pipes.  The weights are 64-bit fixed point w * 2^P
// (P = 62 - lb, |w| <= 1.5 * 2^lb from the scheme's Bernstein bound), converted once per
// point; a node's weight is hi(wx, hi(wy, wz)), the high halves of two signed 64 x 64-bit
// products (w1 w2 w3 * 2^(3P - 128), to 2^-58 of itself).  Each quantity keeps its own
// binary exponent e_p beside an exact 64-bit mantissa q * 2^(62 - e_p), and every
// component of the brick's region has a scale: the largest exponent e_r among its points.
// A contribution is the exact 128-bit product of the node weight and the mantissa, shifted
// right (rounded) by (e_r - e_p) + sh onto that common scale; sh = max(0, bits(K_max) - 5),
// K_max the brick's largest node coverage, keeps the sum of a node's contributions below
// 2^127 (each is below 3.375 * 2^(120 - sh)).  The largest contribution keeps about
// 120 - sh significant bits and one 2^-k of it keeps 120 - sh - k, so a node's sum has the
// accuracy of an FP64 sum of its own contributions unless the region spans more than about
// 2^60 in magnitude: the scale is local to the brick, not global.  Integer addition is
// associative, so the result does not depend on which thread adds first; the 128-bit sums
// are added as four 32-bit words with carries (atomic_add_split128).  A non-finite quantity
// marks every node its stencil reaches, which is written as NaN (the reference's 0 * NaN
// included).
constexpr int kFlatChunk = 1024;
// the scatter's static shared memory: one count per warp for the block scan
constexpr int kScanSlots = 32;
// quantities of a point the warp-per-point scatter holds in registers (the rest are read per use)
constexpr int kQReg = 4;

template <typename T, int N2>
__global__ void __launch_bounds__(kThreads)
    k_scatter_fixed128(GridT<T> g, BrickGeo bg, int ncomp,
                       const uint32_t *__restrict__ cell_start, const long long *__restrict__ wts,
                       const long long *__restrict__ qi, const int32_t *__restrict__ qe,
                       const uint32_t *__restrict__ ebrick, int wexp, T *__restrict__ field, T beta, int beta_zero) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  constexpr int half = N2 / 2;
  const int E0 = bg.b[0] + N2 - 1, E1 = bg.b[1] + N2 - 1, E2 = bg.b[2] + N2 - 1;
  const int ecount = E0 * E1 * E2;
  const int bvol = (int)bg.bvol;
  // ncomp * slice 128-bit accumulators, comp-major and pitched, as four planes of 32-bit
  // words, lowest first (atomic_add_split128)
  const size_t plane = (size_t)bg.slice * ncomp;
  uint32_t *acc0 = reinterpret_cast<uint32_t *>(smem_raw);
  uint32_t *acc1 = acc0 + plane, *acc2 = acc1 + plane, *acc3 = acc2 + plane;
  uint32_t *off = acc3 + plane;                                              // ecount: exclusive prefix
  // along a row of the region, cells whose keys are consecutive hold consecutive slots, so
  // one base (first slot - prefix) serves each such run of cells (segment)
  uint32_t *segbase = off + ecount;                                          // E1*E2*nseg: slot bases
  uint32_t *pslot = segbase + E1 * E2 * bg.nseg;                             // kFlatChunk: point slot
  uint32_t *pxyz = pslot + kFlatChunk;                                       // kFlatChunk: packed cell
  uint32_t *kx = pxyz + kFlatChunk, *ky = kx + E0, *kz = ky + E1;             // per-axis key tables
  uint32_t *kcnt = kz + E2;                                                   // bvol coverage counts + max
  uint32_t *segx = kcnt + bvol + 1;                                          // E0: segment of each x
  uint32_t *segfirst = segx + E0;                                            // nseg: first x of each
  int32_t *ereg = reinterpret_cast<int32_t *>(segfirst + bg.nseg);           // ncomp: region scales
  uint32_t *poison = reinterpret_cast<uint32_t *>(ereg + ncomp);             // slice: NaN marks
  __shared__ uint32_t warp_tot[kScanSlots];
  const int lane = (int)threadIdx.x & 31, warp = (int)threadIdx.x >> 5, nwarps = (int)blockDim.x >> 5;
  const int64_t nbricks = bg.nb[0] * bg.nb[1] * bg.nb[2];
  const int n[3] = {(int)g.nx, (int)g.ny, (int)g.nz};
  const int nb0 = (int)bg.nb[0], nb1 = (int)bg.nb[1];
  // each thread's first region cell and node, and its stride, as coordinates
  const int ex0 = (int)threadIdx.x % E0, ey0 = ((int)threadIdx.x / E0) % E1, ez0 = (int)threadIdx.x / (E0 * E1);
  const int esx = (int)blockDim.x % E0, esy = ((int)blockDim.x / E0) % E1, esz = (int)blockDim.x / (E0 * E1);
  const int B0 = bg.b[0], B1 = bg.b[1];
  const int lx0 = (int)threadIdx.x % B0, ly0 = ((int)threadIdx.x / B0) % B1, lz0 = (int)threadIdx.x / (B0 * B1);
  const int lsx = (int)blockDim.x % B0, lsy = ((int)blockDim.x / B0) % B1, lsz = (int)blockDim.x / (B0 * B1);
  for (int64_t brick = blockIdx.x; brick < nbricks; brick += gridDim.x) {
    const int bc[3] = {(int)(brick % nb0), (int)((brick / nb0) % nb1), (int)(brick / ((int64_t)nb0 * nb1))};
    const int vx = min(B0, n[0] - bc[0] * B0), vy = min(B1, n[1] - bc[1] * B1), vz = min(bg.b[2], n[2] - bc[2] * bg.b[2]);
    __syncthreads();
    for (int t = threadIdx.x; t < E0 + E1 + E2; t += blockDim.x) {
      const int d = t < E0 ? 0 : (t < E0 + E1 ? 1 : 2);
      const int e = t - (d == 0 ? 0 : (d == 1 ? E0 : E0 + E1));
      int c = (bc[d] * bg.b[d] - half + e) % n[d];
      if (c < 0) c += n[d];
      const uint32_t cb = (uint32_t)c / (uint32_t)bg.b[d], cl = (uint32_t)c - cb * (uint32_t)bg.b[d];
      if (d == 0) kx[e] = cb * (uint32_t)bvol + cl;
      else if (d == 1) ky[e] = cb * (uint32_t)nb0 * (uint32_t)bvol + cl * (uint32_t)B0;
      else kz[e] = cb * (uint32_t)nb1 * (uint32_t)nb0 * (uint32_t)bvol + cl * (uint32_t)(B0 * B1);
    }
    __syncthreads();
    if (warp == 0) {
      // segments along x (E0 <= 32): a new one wherever the key does not step by one
      const bool in = lane < E0;
      const bool brk = in && (lane == 0 || kx[lane] != kx[lane - 1] + 1u);
      const uint32_t starts = __ballot_sync(0xffffffffu, brk);
      if (in) segx[lane] = (uint32_t)__popc(starts & (0xffffffffu >> (31 - lane))) - 1u;
      const int sg = __popc(starts & ((1u << lane) - 1u));
      if (brk && sg < bg.nseg) segfirst[sg] = (uint32_t)lane;
    }
    __syncthreads();
    {
      int ex = ex0, ey = ey0, ez = ez0;
      for (int e = threadIdx.x; e < ecount; e += blockDim.x) {
        const uint32_t key = kx[ex] + ky[ey] + kz[ez];
        const uint32_t r0 = __ldg(cell_start + key);
        const uint32_t sg = segx[ex];
        // first slot, for now (the host's bound on the segments keeps sg below nseg)
        if (segfirst[sg] == (uint32_t)ex && sg < (uint32_t)bg.nseg) segbase[(ez * E1 + ey) * bg.nseg + sg] = r0;
        off[e] = __ldg(cell_start + key + 1) - r0;
        ex += esx;
        ey += esy;
        ez += esz;
        if (ex >= E0) { ex -= E0; ++ey; }
        if (ey >= E1) { ey -= E1; ++ez; }
      }
    }
    __syncthreads();
    // coverage of every node (points whose stencil reaches it): window sums of the cell
    // counts, over x and y into the accumulators as scratch, then over z
    if (threadIdx.x == 0) kcnt[bvol] = 0u;
    uint32_t *scratch = acc0;
    if (E2 <= 4 * bg.b[2] * ncomp) {
      for (int o = threadIdx.x; o < B0 * B1 * E2; o += blockDim.x) {
        const int lx = o % B0, r = o / B0, ly = r % B1, ez = r / B1;
        uint32_t sum = 0;
#pragma unroll
        for (int j = 0; j < N2; ++j) {
          const uint32_t *row = off + (ez * E1 + ly + j) * E0 + lx;
#pragma unroll
          for (int i = 0; i < N2; ++i) sum += row[i];
        }
        scratch[o] = sum;
      }
      __syncthreads();
      for (int nl = threadIdx.x; nl < bvol; nl += blockDim.x) {
        uint32_t sum = 0;
#pragma unroll
        for (int k = 0; k < N2; ++k) sum += scratch[nl + k * B0 * B1];
        kcnt[nl] = sum;
      }
    } else {
      for (int nl = threadIdx.x; nl < bvol; nl += blockDim.x) {
        const int lx = nl % B0, ly = (nl / B0) % B1, lz = nl / (B0 * B1);
        uint32_t sum = 0;
        for (int k = 0; k < N2; ++k)
          for (int j = 0; j < N2; ++j)
            for (int i = 0; i < N2; ++i) sum += off[((lz + k) * E1 + ly + j) * E0 + lx + i];
        kcnt[nl] = sum;
      }
    }
    __syncthreads();
    {
      uint32_t mx = 0;
      for (int nl = threadIdx.x; nl < bvol; nl += blockDim.x) mx = max(mx, kcnt[nl]);
      mx = __reduce_max_sync(0xffffffffu, mx);
      if ((threadIdx.x & 31) == 0) atomicMax(kcnt + bvol, mx);
    }
    for (int i = threadIdx.x; i < 4 * (int)plane; i += blockDim.x) acc0[i] = 0u;
    for (int i = threadIdx.x; i < (int)bg.slice; i += blockDim.x) poison[i] = 0u;
    // each component's scale: the largest exponent in the 27 bricks around this one (the
    // region lies within them; periodic wrap)
    for (int c = threadIdx.x; c < ncomp; c += blockDim.x) {
      uint32_t e = 0;
      for (int d = 0; d < 27; ++d) {
        const int64_t x = (bc[0] + d % 3 - 1 + nb0) % nb0, y = (bc[1] + (d / 3) % 3 - 1 + nb1) % nb1,
                      z = (bc[2] + d / 9 - 1 + bg.nb[2]) % bg.nb[2];
        e = max(e, __ldg(ebrick + ((z * nb1 + y) * nb0 + x) * ncomp + c));
      }
      ereg[c] = (int32_t)e;
    }
    __syncthreads();
    const uint32_t kmax = kcnt[bvol];
    const uint32_t count = block_scan_counts(off, ecount, warp_tot);
    {
      // each segment's base: its first slot less its first cell's prefix
      const int nsg = min((int)segx[E0 - 1] + 1, bg.nseg);
      for (int r = threadIdx.x; r < E1 * E2 * nsg; r += blockDim.x) {
        const int row = r / nsg, sg = r - row * nsg;
        segbase[row * bg.nseg + sg] -= off[row * E0 + (int)segfirst[sg]];
      }
    }
    __syncthreads();
    const int sh = max(0, (32 - __clz((int)kmax)) - 5);
    // a contribution of exponent e_p lands on the component's scale: d = (e_r - e_p) + sh;
    // value = sum * 2^(66 + e_r + sh - 3P) (e_r unbiased), P = wexp
    const bool accumulated = count > 0;
    if (accumulated) {
      for (uint32_t c0 = 0; c0 < count; c0 += kFlatChunk) {
        const uint32_t c1 = min(count, c0 + kFlatChunk);
        {
          int ex = ex0, ey = ey0, ez = ez0;
          for (int e = threadIdx.x; e < ecount; e += blockDim.x) {
            const uint32_t lo = max(off[e], c0), hi = min(e + 1 < ecount ? off[e + 1] : count, c1);
            const uint32_t base = segbase[(ez * E1 + ey) * bg.nseg + min(segx[ex], (uint32_t)bg.nseg - 1u)];
            const uint32_t packed = (uint32_t)ex | ((uint32_t)ey << 8) | ((uint32_t)ez << 16);
            for (uint32_t t = lo; t < hi; ++t) {
              pslot[t - c0] = base + t;
              pxyz[t - c0] = packed;
            }
            ex += esx;
            ey += esy;
            ez += esz;
            if (ex >= E0) { ex -= E0; ++ey; }
            if (ey >= E1) { ey -= E1; ++ez; }
          }
        }
        __syncthreads();
        if constexpr (N2 <= 2) {
          // two-node stencils: a thread per point
          for (uint32_t t = c0 + threadIdx.x; t < c1; t += blockDim.x) {
            const uint32_t sl = pslot[t - c0], packed = pxyz[t - c0];
            const int ex = (int)(packed & 0xffu), ey = (int)((packed >> 8) & 0xffu), ez = (int)(packed >> 16);
            const long long *wp = wts + (int64_t)sl * (3 * N2);
            long long w1[N2], w2[N2], w3[N2];
#pragma unroll
            for (int k = 0; k < N2; ++k) {
              w1[k] = wp[k];
              w2[k] = wp[N2 + k];
              w3[k] = wp[2 * N2 + k];
            }
            const long long *qv = qi + (int64_t)sl * ncomp;
            const int kz0 = max(0, N2 - 1 - ez), kz1 = min(N2, vz + N2 - 1 - ez);
            const int ky0 = max(0, N2 - 1 - ey), ky1 = min(N2, vy + N2 - 1 - ey);
            const int lxb = ex - (N2 - 1);
  #pragma unroll 1
            for (int k = kz0; k < kz1; ++k) {
              const int lz = ez + k - (N2 - 1);
              const long long wz = pick_t(w3, k);
  #pragma unroll 1
              for (int j = ky0; j < ky1; ++j) {
                const int ly = ey + j - (N2 - 1);
                const long long wyz = __mul64hi(pick_t(w2, j), wz);
                const int row = lz * bg.pp + ly * bg.p0;
  #pragma unroll
                for (int i = 0; i < N2; ++i) {
                  const int lx = lxb + i;
                  if (lx < 0 || lx >= vx) continue;
                  const long long w = __mul64hi(w1[i], wyz);
                  for (int c = 0; c < ncomp; ++c) {
                    const int ep = __ldg(qe + (int64_t)sl * ncomp + c);
                    if (ep == kENonFinite) atomicOr(poison + row + lx, 1u << (c & 31));
                    else if (ep) add_contribution(acc0, acc1, acc2, acc3, c * (int)bg.slice + row + lx, w,
                                                  __ldg(qv + c), ereg[c] - ep + sh);
                  }
                }
              }
            }
          }
        } else {
          // a warp per point: its lanes cover the nodes of the point's stencil that lie in
          // the brick (the sub-box i0..i1 x j0..j1 x k0..k1), so every lane of every atomic
          // does work; lanes 0..3*N2-1 load one axis weight each, and each node's three
          // weights arrive by shuffle.  The weight products are formed in the same order as
          // in the gather (wz * S first, then wy, then wx).  The next point's weights and
          // first kQReg quantities are loaded while this one is added.
          uint32_t t = c0 + warp;
          uint32_t sl_n = 0, packed_n = 0;
          long long wl_n = 0ll, q_n[kQReg];
          int e_n[kQReg];
          auto fetch = [&](uint32_t tt) {
            sl_n = pslot[tt - c0];
            packed_n = pxyz[tt - c0];
            wl_n = lane < 3 * N2 ? __ldg(wts + (int64_t)sl_n * (3 * N2) + lane) : 0ll;
#pragma unroll
            for (int r = 0; r < kQReg; ++r) {
              q_n[r] = r < ncomp ? __ldg(qi + (int64_t)sl_n * ncomp + r) : 0ll;
              e_n[r] = r < ncomp ? __ldg(qe + (int64_t)sl_n * ncomp + r) : 0;
            }
          };
          if (t < c1) fetch(t);
          for (; t < c1; t += nwarps) {
            const uint32_t sl = sl_n, packed = packed_n;
            const long long wl = wl_n;
            long long qr[kQReg];
            int er[kQReg];
#pragma unroll
            for (int r = 0; r < kQReg; ++r) {
              qr[r] = q_n[r];
              er[r] = e_n[r];
            }
            if (t + nwarps < c1) fetch(t + nwarps);
            const int ex = (int)(packed & 0xffu), ey = (int)((packed >> 8) & 0xffu), ez = (int)(packed >> 16);
            const int i0 = max(0, N2 - 1 - ex), i1 = min(N2, vx + N2 - 1 - ex);
            const int j0 = max(0, N2 - 1 - ey), j1 = min(N2, vy + N2 - 1 - ey);
            const int k0 = max(0, N2 - 1 - ez), k1 = min(N2, vz + N2 - 1 - ez);
            const int nx = i1 - i0, ny = j1 - j0, nz = k1 - k0;
            if (nx <= 0 || ny <= 0 || nz <= 0) continue;  // warp-uniform
            const long long *qv = qi + (int64_t)sl * ncomp;
            const int32_t *ev = qe + (int64_t)sl * ncomp;
            const int count = nx * ny * nz;
            // idx -> (ii, jj, kk) by multiply-shift division: exact for idx < 4096, divisors <= 8
            const uint32_t rnx = (65536u + nx - 1) / nx, rny = (65536u + ny - 1) / ny;
            const int node0 = (ez - (N2 - 1)) * bg.pp + (ey - (N2 - 1)) * bg.p0 + ex - (N2 - 1);
            for (int base = 0; base < count; base += 32) {
              const int idx = base + lane;
              const int r1 = (int)(((uint32_t)idx * rnx) >> 16), ii = idx - r1 * nx;
              const int kk = (int)(((uint32_t)r1 * rny) >> 16), jj = r1 - kk * ny;
              const int i = min(i0 + ii, N2 - 1), j = min(j0 + jj, N2 - 1), k = min(k0 + kk, N2 - 1);
              const long long wxi = __shfl_sync(0xffffffffu, wl, i);
              const long long wyj = __shfl_sync(0xffffffffu, wl, N2 + j);
              const long long wzk = __shfl_sync(0xffffffffu, wl, 2 * N2 + k);
              if (idx < count) {
                const long long w = __mul64hi(wxi, __mul64hi(wyj, wzk));
                const int node = node0 + k * bg.pp + j * bg.p0 + i;
#pragma unroll
                for (int r = 0; r < kQReg; ++r)
                  if (r < ncomp) {
                    if (er[r] == kENonFinite) atomicOr(poison + node, 1u << (r & 31));
                    else if (er[r]) add_contribution(acc0, acc1, acc2, acc3, r * (int)bg.slice + node, w, qr[r],
                                                     ereg[r] - er[r] + sh);
                  }
                for (int c = kQReg; c < ncomp; ++c) {
                  const int ep = __ldg(ev + c);
                  if (ep == kENonFinite) atomicOr(poison + node, 1u << (c & 31));
                  else if (ep) add_contribution(acc0, acc1, acc2, acc3, c * (int)bg.slice + node, w, __ldg(qv + c),
                                                ereg[c] - ep + sh);
                }
              }
            }
          }
        }
        __syncthreads();
      }
    }
    __syncthreads();
    // write-back in the reference layout: node fastest, so a warp writes a contiguous row
    for (int c = 0; c < ncomp; ++c) {
      int lx = lx0, ly = ly0, lz = lz0;
      for (int nl = threadIdx.x; nl < bvol; nl += blockDim.x) {
        if (lx < vx && ly < vy && lz < vz) {
          const int64_t x = (int64_t)bc[0] * B0 + lx, y = (int64_t)bc[1] * B1 + ly, z = (int64_t)bc[2] * bg.b[2] + lz;
          T *f = field + x + g.nx * (y + g.ny * z) + g.npf * c;
          const int64_t ni = lz * bg.pp + ly * bg.p0 + lx, ai = c * bg.slice + ni;
          // the 128-bit sum as a double (one rounding of the high part, one of the sum)
          const long long hi = (long long)(((unsigned long long)acc3[ai] << 32) | acc2[ai]);
          const unsigned long long lo = ((unsigned long long)acc1[ai] << 32) | acc0[ai];
          const double sum = fma((double)hi, 18446744073709551616.0, (double)lo);
          T v = (accumulated && ereg[c] > 0) ? (T)ldexp(sum, 66 + (ereg[c] - kEBias) + sh - 3 * wexp) : T(0);
          if ((poison[ni] >> (c & 31)) & 1u) v = quiet_nan<T>();
          *f = beta_zero ? v : add_rn(mul_rn(beta, *f), v);
        }
        lx += lsx;
        ly += lsy;
        lz += lsz;
        if (lx >= B0) { lx -= B0; ++ly; }
        if (ly >= B1) { ly -= B1; ++lz; }
      }
    }
  }
}

// ------------------------------------------------------- traversal order

// Interpolation.jl:636-642: the comparisons happen in floating point, before any
// conversion, so non-finite and far-away coordinates saturate into a real tile.
template <typename T>
__device__ __forceinline__ int64_t tile_index(T c, T o, T inv, int64_t tiles) {
  const T u = (c - o) * inv;
  if (isnan(u)) return 0;
  if (u <= T(0)) return 0;
  if (u >= T(tiles)) return tiles - 1;
  return (int64_t)u;
}

template <typename T>
__global__ void __launch_bounds__(kThreads)
    k_tile_keys(const T *__restrict__ pos, int64_t m, T o0, T o1, T o2, T i0, T i1, T i2,
                int64_t t0, int64_t t1, int64_t t2, uint32_t *__restrict__ keys) {
  for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < m;
       p += (int64_t)gridDim.x * blockDim.x) {
    const int64_t a = tile_index(pos[p], o0, i0, t0);
    const int64_t b = tile_index(pos[p + m], o1, i1, t1);
    const int64_t c = tile_index(pos[p + 2 * m], o2, i2, t2);
    keys[p] = (uint32_t)(a + t0 * (b + t1 * c));  // the reference's key less its 2 offset
  }
}

__global__ void k_to_one_based(const uint32_t *__restrict__ perm, int32_t *__restrict__ order,
                               int64_t m) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m;
       i += (int64_t)gridDim.x * blockDim.x)
    order[i] = (int32_t)perm[i] + 1;
}

__global__ void k_validate(const int32_t *__restrict__ order, int64_t m, uint32_t *seen,
                           unsigned long long *stats) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m;
       i += (int64_t)gridDim.x * blockDim.x) {
    const long long v = order[i];
    atomicMin(reinterpret_cast<long long *>(stats), v);
    atomicMax(reinterpret_cast<long long *>(stats + 1), v);
    if (v >= 1 && v <= m && atomicExch(seen + (v - 1), 1u) == 0u) atomicAdd(stats + 2, 1ull);
  }
}

__global__ void k_validate_init(unsigned long long *stats) {
  reinterpret_cast<long long *>(stats)[0] = 0x7fffffffffffffffLL;
  reinterpret_cast<long long *>(stats)[1] = (-0x7fffffffffffffffLL - 1);
  stats[2] = 0ull;
}

__global__ void k_fill_or_scale(void *data, int64_t count, int is_f64, double beta) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count;
       i += (int64_t)gridDim.x * blockDim.x) {
    if (is_f64) {
      double *d = static_cast<double *>(data);
      d[i] = beta == 0.0 ? 0.0 : __dmul_rn(d[i], beta);
    } else {
      float *f = static_cast<float *>(data);
      f[i] = beta == 0.0 ? 0.0f : __fmul_rn(f[i], (float)beta);
    }
  }
}

// ------------------------------------------------------------- dispatch

int chunk_for(int ncomp) { return ncomp % 9 == 0 ? 9 : (ncomp % 3 == 0 ? 3 : 1); }

template <typename T, int N2>
gbg_status launch_gather(const gbg_grid &grid, const gbg_scheme &sch, int ncomp, const void *field,
                         const void *pos, int64_t m, const int32_t *trav, void *out,
                         int32_t *status, cudaStream_t st) {
  const GridT<T> g = make_grid<T>(grid);
  const SchemeT<T, N2> s = make_scheme<T, N2>(sch);
  const int blocks = launch_blocks(m, kThreads);
  const T *f = static_cast<const T *>(field);
  const T *x = static_cast<const T *>(pos);
  T *o = static_cast<T *>(out);
  mark_main_start(st);
  const bool full = sch.num_powers == N2;  // num_powers == width: compile-time Horner
  switch (chunk_for(ncomp) * 2 + (full ? 1 : 0)) {
    case 19: k_gather_plain<T, N2, N2, 9><<<blocks, kThreads, 0, st>>>(g, s, ncomp, f, x, m, trav, o, status); break;
    case 18: k_gather_plain<T, N2, 0, 9><<<blocks, kThreads, 0, st>>>(g, s, ncomp, f, x, m, trav, o, status); break;
    case 7: k_gather_plain<T, N2, N2, 3><<<blocks, kThreads, 0, st>>>(g, s, ncomp, f, x, m, trav, o, status); break;
    case 6: k_gather_plain<T, N2, 0, 3><<<blocks, kThreads, 0, st>>>(g, s, ncomp, f, x, m, trav, o, status); break;
    case 3: k_gather_plain<T, N2, N2, 1><<<blocks, kThreads, 0, st>>>(g, s, ncomp, f, x, m, trav, o, status); break;
    default: k_gather_plain<T, N2, 0, 1><<<blocks, kThreads, 0, st>>>(g, s, ncomp, f, x, m, trav, o, status); break;
  }
  note_launch();
  mark_main_stop(st);
  GBG_CUDA_TRY(cudaGetLastError());
  return GBG_OK;
}

template <typename T>
gbg_status dispatch_gather(const gbg_grid &grid, const gbg_scheme &sch, int ncomp, const void *field,
                           const void *pos, int64_t m, const int32_t *trav, void *out,
                           int32_t *status, cudaStream_t st) {
  switch (sch.stencil_width) {
    case 2: return launch_gather<T, 2>(grid, sch, ncomp, field, pos, m, trav, out, status, st);
    case 4: return launch_gather<T, 4>(grid, sch, ncomp, field, pos, m, trav, out, status, st);
    case 6: return launch_gather<T, 6>(grid, sch, ncomp, field, pos, m, trav, out, status, st);
    case 8: return launch_gather<T, 8>(grid, sch, ncomp, field, pos, m, trav, out, status, st);
    default: {
      const GridT<T> g = make_grid<T>(grid);
      const SchemeT<T, GBG_MAX_NODES> s = make_scheme<T, GBG_MAX_NODES>(sch);
      k_gather_plain_dyn<T><<<launch_blocks(m, kThreads), kThreads, 0, st>>>(
          g, s, ncomp, static_cast<const T *>(field), static_cast<const T *>(pos), m, trav,
          static_cast<T *>(out), status);
      note_launch();
      GBG_CUDA_TRY(cudaGetLastError());
      return GBG_OK;
    }
  }
}

// Which scatter runs, and its bricks: the brick push whenever every axis is at least a
// stencil wide and a brick's accumulators fit in shared memory, else the node pull
// (which also handles a stencil wider than the grid, reached several times per node).
struct ScatterPlan {
  bool bricked = false;
  BrickGeo bg{};
  int64_t nkeys = 0;
  size_t smem = 0;
};

// Pitches of the scatter's shared accumulators.  A warp adds one point's contributions to
// the nodes of its stencil inside the brick, x fastest, 32 nodes at a time, with 32-bit
// atomics on a plane of low words and then a plane of high words (node i's word on bank
// i mod 32); with the brick's own row and plane pitches the stencil's rows fall on the same
// banks.  Over row pitches b0..b0+31 and plane pitches b1*p0..b1*p0+31 whose slice stays
// within max_slice nodes (so that the padding costs no CTA per SM), this takes the pair
// with the fewest shared-memory wavefronts summed over every position of a full n^3
// stencil in the brick.
void choose_acc_pitches(BrickGeo &bg, int n2, int64_t max_slice) {
  const int b0 = bg.b[0], b1 = bg.b[1], b2 = bg.b[2];
  const int nx = std::min(n2, b0), ny = std::min(n2, b1), nz = std::min(n2, b2);
  int64_t best = -1;
  int best_p0 = b0, best_pp = b0 * b1;
  std::vector<int> words;
  for (int p0 = b0; p0 < b0 + 32; ++p0) {
    for (int pp = b1 * p0; pp < b1 * p0 + 32; ++pp) {
      if ((int64_t)b2 * pp > max_slice && !(p0 == b0 && pp == b0 * b1)) continue;
      int64_t total = 0;
      for (int z0 = 0; z0 + nz <= b2; ++z0)
        for (int y0 = 0; y0 + ny <= b1; ++y0)
          for (int x0 = 0; x0 + nx <= b0; ++x0) {
            words.clear();
            for (int k = 0; k < nz; ++k)
              for (int j = 0; j < ny; ++j)
                for (int i = 0; i < nx; ++i) words.push_back((z0 + k) * pp + (y0 + j) * p0 + x0 + i);
            for (size_t c = 0; c < words.size(); c += 32) {
              // wavefronts of one warp instruction: the words are distinct and word w sits on
              // bank w mod 32, so the most words sharing a bank
              int per_bank[32] = {0};
              for (size_t l = c; l < std::min(words.size(), c + 32); ++l) ++per_bank[words[l] & 31];
              int mx = 0;
              for (int q = 0; q < 32; ++q) mx = std::max(mx, per_bank[q]);
              total += mx;
            }
          }
      if (best < 0 || total < best) {
        best = total;
        best_p0 = p0;
        best_pp = pp;
      }
    }
  }
  bg.p0 = best_p0;
  bg.pp = best_pp;
  bg.slice = (int64_t)b2 * best_pp;
}

// The most segments (runs of consecutive keys) along x in one row of any brick's region:
// the region's x cells of brick column bc0 are (bc0*b0 - n2/2 + e) mod n0, e < b0 + n2 - 1,
// keyed by brick * bvol + cell-in-brick, exactly as the scatter kernel keys them.
int brick_segments(const BrickGeo &bg, int64_t n0, int n2) {
  const int e0 = bg.b[0] + n2 - 1;
  int most = 1;
  for (int64_t bc0 = 0; bc0 < bg.nb[0]; ++bc0) {
    int segs = 0;
    int64_t prev = 0;
    for (int e = 0; e < e0; ++e) {
      const int64_t c = imod(bc0 * bg.b[0] - n2 / 2 + e, n0);
      const int64_t key = (c / bg.b[0]) * bg.bvol + c % bg.b[0];
      if (e == 0 || key != prev + 1) ++segs;
      prev = key;
    }
    most = std::max(most, segs);
  }
  return most;
}

ScatterPlan plan_scatter(const gbg_grid &g, int ncomp, size_t esize, int n2) {
  ScatterPlan p;
  const int base[3] = {(size_t)ncomp * esize > 24 ? 8 : 16, 8, 8};
  bool wide_enough = n2 <= 8;
  int64_t nbricks = 1;
  for (int d = 0; d < 3; ++d) {
    p.bg.b[d] = (int32_t)std::min<int64_t>(base[d], g.n[d]);
    p.bg.nb[d] = (g.n[d] + p.bg.b[d] - 1) / p.bg.b[d];
    nbricks *= p.bg.nb[d];
    if (g.n[d] < n2 || g.n[d] >= (int64_t(1) << 31)) wide_enough = false;
  }
  p.bg.bvol = (int64_t)p.bg.b[0] * p.bg.b[1] * p.bg.b[2];
  const int e0 = p.bg.b[0] + n2 - 1, e1 = p.bg.b[1] + n2 - 1, e2 = p.bg.b[2] + n2 - 1;
  const size_t ecount = (size_t)e0 * e1 * e2;
  if (e0 > 32) wide_enough = false;  // the kernel finds the x segments with one warp
  p.bg.nseg = brick_segments(p.bg, g.n[0], n2);
  // shared memory besides the accumulators: region offsets and segment bases, the point
  // chunk, the key tables, the coverage counts, the segment of each x and first x of each,
  // the components' scales and the NaN marks (one word per node of the padded slice, at
  // most the accumulators' slice: bvol words plus the padding counted with the slice)
  const size_t rest = sizeof(uint32_t) * ecount + sizeof(uint32_t) * (size_t)e1 * e2 * p.bg.nseg +
                      2 * sizeof(uint32_t) * kFlatChunk + sizeof(uint32_t) * (size_t)(e0 + e1 + e2) +
                      sizeof(uint32_t) * (size_t)(p.bg.bvol + 1) + sizeof(uint32_t) * (size_t)(e0 + p.bg.nseg) +
                      sizeof(int32_t) * (size_t)ncomp;
  {
    // accumulator pitches that keep the unpadded layout's CTAs per SM (228 KB per SM, 1 KB
    // reserved per CTA by the runtime, the kernel's static scan slots) and its 200 KB cap;
    // they depend on the brick, the width and the components alone, so each is searched once
    const size_t per_node = (size_t)ncomp * 16 + sizeof(uint32_t), sm = 228 * 1024,
                 reserve = 1024 + kScanSlots * sizeof(uint32_t);
    const size_t unpadded = (size_t)p.bg.bvol * per_node + rest;
    const size_t ctas = std::max<size_t>(1, sm / (unpadded + reserve));
    const size_t room = std::min<size_t>(sm / ctas - reserve, 200 * 1024);
    const int64_t max_slice = room > rest ? (int64_t)((room - rest) / per_node) : p.bg.bvol;
    static std::mutex mu;
    static std::map<std::array<int, 5>, std::pair<int, int>> cache;
    const std::array<int, 5> key = {p.bg.b[0], p.bg.b[1], p.bg.b[2], n2, ncomp};
    std::lock_guard<std::mutex> lock(mu);
    auto it = cache.find(key);
    if (it == cache.end()) {
      choose_acc_pitches(p.bg, n2, std::max<int64_t>(max_slice, p.bg.bvol));
      cache[key] = {p.bg.p0, p.bg.pp};
    } else {
      p.bg.p0 = it->second.first;
      p.bg.pp = it->second.second;
      p.bg.slice = (int64_t)p.bg.b[2] * p.bg.pp;
    }
  }
  p.smem = (size_t)p.bg.slice * (ncomp * 16 + sizeof(uint32_t)) + rest;
  (void)esize;
  if (ecount > 65535) wide_enough = false;
  p.bricked = wide_enough && p.smem <= 200 * 1024 && nbricks * p.bg.bvol < (int64_t(1) << 32) - 1;
  p.nkeys = p.bricked ? nbricks * p.bg.bvol : g.n[0] * g.n[1] * g.n[2];
  return p;
}

// The scatter's workspace: keys, per-cell counts (then slot starts), ranks within a cell
// (then the fallback sort's keys), the permutation, the counting sort's long-run flag and
// scratch, the scan's scratch, per sorted slot the three axes' weights (64-bit fixed point
// for the brick scatter) and the quantities (for the brick scatter as mantissas and
// exponents, with per brick the largest exponent of every component).
struct ScatterLayout {
  uint32_t *keys, *counts, *rank, *perm, *flag;
  void *sort_tmp;
  uint32_t *scan_tmp;
  void *rec, *qs;
  long long *qi;
  int32_t *qe;
  uint32_t *ebrick;
};

ScatterLayout scatter_layout(Arena &a, int64_t m, const ScatterPlan &P, int ncomp, int n2, size_t esize) {
  ScatterLayout L;
  L.keys = a.take<uint32_t>((size_t)m);
  L.counts = a.take<uint32_t>((size_t)P.nkeys + 1);
  L.rank = a.take<uint32_t>((size_t)m);
  L.perm = a.take<uint32_t>((size_t)m);
  L.flag = a.take<uint32_t>(4);
  L.sort_tmp = a.take<char>(radix_sort_temp_bytes(m));
  L.scan_tmp = a.take<uint32_t>(scan_temp_elems(P.nkeys + 1));
  const size_t rec_bytes = 3 * (size_t)n2 * (P.bricked ? sizeof(long long) : esize);
  L.rec = a.take<char>((size_t)m * rec_bytes);
  L.qs = P.bricked ? nullptr : a.take<char>((size_t)m * ncomp * esize);
  L.qi = P.bricked ? a.take<long long>((size_t)m * ncomp) : nullptr;
  L.qe = P.bricked ? a.take<int32_t>((size_t)m * ncomp) : nullptr;
  const int64_t nbricks = P.bricked ? P.bg.nb[0] * P.bg.nb[1] * P.bg.nb[2] : 0;
  L.ebrick = P.bricked ? a.take<uint32_t>((size_t)nbricks * ncomp) : nullptr;
  return L;
}

int bits_for(uint64_t max_value) {
  int b = 0;
  while (b < 32 && (max_value >> b) != 0) ++b;
  return b;
}

template <typename T, int N2, bool FIXED>
gbg_status launch_bricked(const GridT<T> &g, const ScatterPlan &P, const gbg_scheme &sch, int ncomp,
                          const T *x, const T *q, int64_t m, double alpha, const ScatterLayout &L, T *field,
                          double beta, int32_t *status, cudaStream_t st) {
  const SchemeT<T, N2> s = make_scheme<T, N2>(sch);
  const int wexp = fixed_weight_exp(sch);
  const int blocks_m = launch_blocks(m, kThreads);
  const int64_t nbricks = P.bg.nb[0] * P.bg.nb[1] * P.bg.nb[2];
  GBG_CUDA_TRY(cudaMemsetAsync(L.ebrick, 0, sizeof(uint32_t) * (size_t)nbricks * ncomp, st));
  GBG_CUDA_TRY(cudaMemsetAsync(L.flag, 0, sizeof(uint32_t), st));
  k_brick_keys<T><<<blocks_m, kThreads, 0, st>>>(g, P.bg, x, m, L.keys, L.counts, L.rank, q, ncomp, T(alpha),
                                                 L.ebrick, status);
  note_launch();
  GBG_CUDA_TRY(cudaGetLastError());
  GBG_TRY(exclusive_scan_u32(L.counts, L.counts, P.nkeys + 1, L.scan_tmp, st));
  GBG_TRY(stable_counting_sort(L.keys, L.rank, L.counts, m, bits_for((uint64_t)(P.nkeys - 1)), L.perm, L.rank,
                               L.flag, L.sort_tmp, st));
  k_brick_order<T, N2, FIXED ? N2 : 0><<<blocks_m, kThreads, 0, st>>>(
      g, s, x, L.perm, m, wexp, static_cast<long long *>(L.rec), q, ncomp, T(alpha), L.qi, L.qe);
  note_launch();
  GBG_CUDA_TRY(cudaGetLastError());
  auto kernel = k_scatter_fixed128<T, N2>;
  GBG_CUDA_TRY(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)P.smem));
  int dev = 0, sms = 1, per_sm = 1;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kThreads, P.smem);
  // the padded pitches only where the occupancy query agrees that they cost no CTA per SM
  BrickGeo bg = P.bg;
  size_t smem = P.smem;
  if (bg.slice != bg.bvol) {
    const size_t flat = smem - (size_t)(bg.slice - bg.bvol) * (ncomp * 16 + sizeof(uint32_t));
    int flat_per_sm = 1;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&flat_per_sm, kernel, kThreads, flat);
    if (flat_per_sm > per_sm) {
      bg.p0 = bg.b[0];
      bg.pp = bg.b[0] * bg.b[1];
      bg.slice = bg.bvol;
      smem = flat;
      per_sm = flat_per_sm;
    }
  }
  const int blocks = (int)std::min<int64_t>(nbricks, (int64_t)sms * std::max(per_sm, 1));
  mark_main_start(st);
  kernel<<<blocks, kThreads, smem, st>>>(g, bg, ncomp, L.counts, static_cast<const long long *>(L.rec), L.qi,
                                         L.qe, L.ebrick, wexp, field, T(beta), beta == 0.0);
  mark_main_stop(st);
  note_launch();
  GBG_CUDA_TRY(cudaGetLastError());
  return GBG_OK;
}


// The deterministic scatter.  The brick push (128-bit integer sums, FP64-grade per node)
// whenever every axis is at least a stencil wide and a brick's accumulators fit in shared
// memory; otherwise the node pull (points sorted by cell, one thread per node summing its
// contributions in T in a fixed order), which also takes a stencil wider than the grid.
template <typename T>
gbg_status dispatch_scatter(const gbg_grid &grid, const gbg_scheme &sch, int ncomp, void *field,
                            const void *pos, int64_t m, const void *q, double alpha, double beta,
                            const ScatterPlan &P, const ScatterLayout &L, int32_t *status, cudaStream_t st) {
  const GridT<T> g = make_grid<T>(grid);
  const T *x = static_cast<const T *>(pos);
  T *f = static_cast<T *>(field);
  GBG_CUDA_TRY(cudaMemsetAsync(L.counts, 0, sizeof(uint32_t) * (size_t)(P.nkeys + 1), st));
  if (P.bricked) {
    const T *qq = static_cast<const T *>(q);
    const int w = sch.stencil_width;
    const bool fixed = sch.num_powers == w;
#define GBG_BRICKED(W)                                                                               \
  return fixed ? launch_bricked<T, W, true>(g, P, sch, ncomp, x, qq, m, alpha, L, f, beta, status, st) \
               : launch_bricked<T, W, false>(g, P, sch, ncomp, x, qq, m, alpha, L, f, beta, status, st)
    if (w == 2) GBG_BRICKED(2);
    if (w == 4) GBG_BRICKED(4);
    if (w == 6) GBG_BRICKED(6);
    GBG_BRICKED(8);
#undef GBG_BRICKED
  }
  const int64_t ncells = g.npf;
  GBG_CUDA_TRY(cudaMemsetAsync(L.flag, 0, sizeof(uint32_t), st));
  const SchemeT<T, GBG_MAX_NODES> s = make_scheme<T, GBG_MAX_NODES>(sch);
  k_cell_keys<T><<<launch_blocks(m, kThreads), kThreads, 0, st>>>(g, x, m, L.keys, L.counts, L.rank, status);
  note_launch();
  GBG_CUDA_TRY(cudaGetLastError());
  GBG_TRY(exclusive_scan_u32(L.counts, L.counts, ncells + 1, L.scan_tmp, st));
  GBG_TRY(stable_counting_sort(L.keys, L.rank, L.counts, m, bits_for((uint64_t)(ncells - 1)), L.perm, L.rank,
                               L.flag, L.sort_tmp, st));
  T *rec = static_cast<T *>(L.rec);
  T *qs = static_cast<T *>(L.qs);
  k_scatter_prep<T><<<launch_blocks(m, kThreads), kThreads, 0, st>>>(
      g, s, ncomp, x, static_cast<const T *>(q), m, L.perm, T(alpha), rec, qs);
  note_launch();
  GBG_CUDA_TRY(cudaGetLastError());
  const int blocks = launch_blocks(ncells, kThreads);
  const int bz = beta == 0.0;
  const int n2 = sch.stencil_width;
  const int cc = chunk_for(ncomp);
  mark_main_start(st);
#define GBG_PULL_N(W)                                                                                                  \
  if (n2 == W) {                                                                                                       \
    if (cc == 9) k_scatter_pull_n<T, W, 9><<<blocks, kThreads, 0, st>>>(g, ncomp, L.counts, rec, qs, f, T(beta), bz);  \
    else if (cc == 3) k_scatter_pull_n<T, W, 3><<<blocks, kThreads, 0, st>>>(g, ncomp, L.counts, rec, qs, f, T(beta), bz); \
    else k_scatter_pull_n<T, W, 1><<<blocks, kThreads, 0, st>>>(g, ncomp, L.counts, rec, qs, f, T(beta), bz);          \
  } else
  GBG_PULL_N(2) GBG_PULL_N(4) GBG_PULL_N(6) GBG_PULL_N(8) {
    switch (cc) {
      case 9: k_scatter_pull<T, 9><<<blocks, kThreads, 0, st>>>(g, n2, ncomp, L.counts, rec, qs, f, T(beta), bz); break;
      case 3: k_scatter_pull<T, 3><<<blocks, kThreads, 0, st>>>(g, n2, ncomp, L.counts, rec, qs, f, T(beta), bz); break;
      default: k_scatter_pull<T, 1><<<blocks, kThreads, 0, st>>>(g, n2, ncomp, L.counts, rec, qs, f, T(beta), bz); break;
    }
  }
#undef GBG_PULL_N
  mark_main_stop(st);
  note_launch();
  GBG_CUDA_TRY(cudaGetLastError());
  return GBG_OK;
}

// ------------------------------------------------------- argument checks

gbg_status check_grid(const gbg_grid *g) {
  if (!g) return set_error(GBG_EARG, "null grid");
  for (int d = 0; d < 3; ++d) {
    if (g->n[d] <= 0) return set_error(GBG_EARG, "grid_size must be positive along every axis");
    if (!(std::isfinite(g->domain[d]) && g->domain[d] > 0))
      return set_error(GBG_EARG, "domain_size must be finite and positive along every axis");
    if (!(std::isfinite(g->spacing[d]) && g->spacing[d] > 0))
      return set_error(GBG_EARG, "grid_spacing must be finite and positive along every axis");
    if (!std::isfinite(g->origin[d])) return set_error(GBG_EARG, "origin must be finite along every axis");
  }
  if (g->n[0] > (int64_t(1) << 31) || g->n[1] > (int64_t(1) << 31) || g->n[2] > (int64_t(1) << 31))
    return set_error(GBG_EUNSUPPORTED, "grid axis longer than 2^31");
  return GBG_OK;
}

gbg_status check_scheme(const gbg_scheme *s) {
  if (!s) return set_error(GBG_EARG, "null scheme");
  if (s->stencil_width < 2 || s->stencil_width % 2 || s->stencil_width > GBG_MAX_NODES)
    return set_error(GBG_EARG, "scheme stencil_width must be even, 2..GBG_MAX_NODES");
  if (s->num_powers < 1 || s->num_powers > GBG_MAX_POWERS)
    return set_error(GBG_EARG, "scheme num_powers must be 1..GBG_MAX_POWERS");
  return GBG_OK;
}

gbg_status check_common(const gbg_grid *grid, gbg_dtype dtype, int32_t ncomp, int64_t m,
                        const gbg_scheme *scheme) {
  GBG_TRY(check_grid(grid));
  GBG_TRY(check_scheme(scheme));
  if (dtype != GBG_F32 && dtype != GBG_F64) return set_error(GBG_EARG, "dtype must be GBG_F32 or GBG_F64");
  if (ncomp < 1) return set_error(GBG_EARG, "ncomp must be at least 1");
  if (m < 0) return set_error(GBG_EDIM, "negative point count");
  if (m > 0x7fffffffLL) return set_error(GBG_EUNSUPPORTED, "more than 2^31-1 points");
  return GBG_OK;
}

}  // namespace
}  // namespace gbg

using namespace gbg;

extern "C" {

gbg_status gbg_interpolate(const gbg_grid *grid, gbg_dtype dtype, int32_t ncomp, const void *field,
                           const void *positions, int64_t npoints, const int32_t *traversal,
                           const gbg_scheme *scheme, void *out, int32_t *device_status,
                           void *stream) {
  clear_error();
  try {
    GBG_TRY(check_common(grid, dtype, ncomp, npoints, scheme));
    if (npoints == 0) return GBG_OK;
    if (!field || !positions || !out) return set_error(GBG_EARG, "interpolate: null array");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (dtype == GBG_F64)
      return dispatch_gather<double>(*grid, *scheme, ncomp, field, positions, npoints, traversal,
                                     out, device_status, st);
    return dispatch_gather<float>(*grid, *scheme, ncomp, field, positions, npoints, traversal, out,
                                  device_status, st);
  } catch (...) {
    return set_error(GBG_ENOMEM, "interpolate: host exception");
  }
}

gbg_status gbg_anterpolate_workspace_size(const gbg_grid *grid, gbg_dtype dtype, int32_t ncomp,
                                          int64_t npoints, const gbg_scheme *scheme, size_t *bytes) {
  clear_error();
  GBG_TRY(check_common(grid, dtype, ncomp, npoints, scheme));
  if (!bytes) return set_error(GBG_EARG, "null bytes");
  const int64_t ncells = grid->n[0] * grid->n[1] * grid->n[2];
  if (ncells >= (int64_t(1) << 32) - 1)
    return set_error(GBG_EUNSUPPORTED, "anterpolate: grids of 2^32 or more cells");
  const size_t es = dtype == GBG_F64 ? 8 : 4;
  const ScatterPlan P = plan_scatter(*grid, ncomp, es, scheme->stencil_width);
  Arena a;
  scatter_layout(a, npoints, P, ncomp, scheme->stencil_width, es);
  *bytes = npoints == 0 ? 0 : a.used + 256;
  return GBG_OK;
}

gbg_status gbg_anterpolate(const gbg_grid *grid, gbg_dtype dtype, int32_t ncomp, void *field,
                           const void *positions, int64_t npoints, const void *quantities,
                           const int32_t *traversal, const gbg_scheme *scheme, double alpha,
                           double beta, void *workspace, size_t workspace_bytes,
                           int32_t *device_status, void *stream) {
  clear_error();
  (void)traversal;  // the deterministic pull is independent of the visiting order
  try {
    size_t need = 0;
    GBG_TRY(gbg_anterpolate_workspace_size(grid, dtype, ncomp, npoints, scheme, &need));
    if (!field) return set_error(GBG_EARG, "anterpolate: null field");
    if (!std::isfinite(alpha) || !std::isfinite(beta)) {
      // allowed by the reference (T(alpha) of an Inf is Inf); passed through as given
    }
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const int64_t total = grid->n[0] * grid->n[1] * grid->n[2] * (int64_t)ncomp;
    if (npoints == 0) {
      // Interpolation.jl:1309-1313: the prescale happens even with no points.
      k_fill_or_scale<<<launch_blocks(total, kThreads), kThreads, 0, st>>>(field, total,
                                                                           dtype == GBG_F64, beta);
      note_launch();
      GBG_CUDA_TRY(cudaGetLastError());
      return GBG_OK;
    }
    if (!positions || !quantities) return set_error(GBG_EARG, "anterpolate: null array");
    Scratch scratch;
    GBG_TRY(scratch.acquire(workspace, workspace_bytes, need, st));
    Arena a;
    a.base = static_cast<char *>(scratch.ptr);
    const size_t es = dtype == GBG_F64 ? 8 : 4;
    const ScatterPlan P = plan_scatter(*grid, ncomp, es, scheme->stencil_width);
    const ScatterLayout L = scatter_layout(a, npoints, P, ncomp, scheme->stencil_width, es);
    if (dtype == GBG_F64)
      return dispatch_scatter<double>(*grid, *scheme, ncomp, field, positions, npoints, quantities,
                                      alpha, beta, P, L, device_status, st);
    return dispatch_scatter<float>(*grid, *scheme, ncomp, field, positions, npoints, quantities,
                                   alpha, beta, P, L, device_status, st);
  } catch (...) {
    return set_error(GBG_ENOMEM, "anterpolate: host exception");
  }
}

// ------------------------------------------------ allocation-free scatter
//
// The scratch of gbg_anterpolate_noalloc: one fixed array per device, part of this
// library's device image, so the entry point never allocates.  Host code must not pass
// the array's name to a kernel (on the host it names a host-side stand-in).  Its device
// address is looked up on every call, in the context current at the call: an address
// kept from an earlier call would be stale after a device reset or in another context.
static __device__ __align__(256) unsigned char g_noalloc_scratch[GBG_NOALLOC_SCRATCH_BYTES];

static gbg_status noalloc_scratch(void **out) {
  void *p = nullptr;
  const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
  if (e != cudaSuccess || !p)
    return set_error(GBG_ECUDA, std::string("cudaGetSymbolAddress of the static scratch failed: ") +
                                    cudaGetErrorString(e));
  *out = p;
  return GBG_OK;
}

gbg_status gbg_anterpolate_noalloc(const gbg_grid *grid, gbg_dtype dtype, int32_t ncomp, void *field,
                                   const void *positions, int64_t npoints, const void *quantities,
                                   const gbg_scheme *scheme, double alpha, double beta,
                                   int32_t *device_status, void *stream) {
  clear_error();
  try {
    size_t need = 0;
    GBG_TRY(gbg_anterpolate_workspace_size(grid, dtype, ncomp, npoints, scheme, &need));
    if (need > GBG_NOALLOC_SCRATCH_BYTES)
      return set_error(GBG_EUNSUPPORTED, "anterpolate (no-alloc): this problem needs " + std::to_string(need) +
                                             " bytes of scratch; the static scratch holds " +
                                             std::to_string((size_t)GBG_NOALLOC_SCRATCH_BYTES));
    void *scratch = nullptr;
    if (need > 0) GBG_TRY(noalloc_scratch(&scratch));
    // The shared path: with a caller workspace it allocates nothing, and it clears the
    // per-cell counts and the sort's flag (the only words that must start at zero) before
    // every use.
    const gbg_status st = gbg_anterpolate(grid, dtype, ncomp, field, positions, npoints, quantities, nullptr,
                                          scheme, alpha, beta, scratch, GBG_NOALLOC_SCRATCH_BYTES,
                                          device_status, stream);
    return st;
  } catch (...) {
    return set_error(GBG_ENOMEM, "anterpolate (no-alloc): host exception");
  }
}

static gbg_status traversal_tiles(const gbg_grid *grid, int64_t tile_size, int64_t tiles[3]) {
  if (tile_size < 1) return set_error(GBG_EARG, "tile_size must be at least 1, got " + std::to_string(tile_size));
  for (int d = 0; d < 3; ++d) {
    const int64_t t = (grid->n[d] + tile_size - 1) / tile_size;
    tiles[d] = t > 1 ? t : 1;
  }
  const double total = (double)tiles[0] * (double)tiles[1] * (double)tiles[2];
  if (total >= 4294967296.0) return set_error(GBG_EUNSUPPORTED, "traversal order: 2^32 or more tiles");
  return GBG_OK;
}

gbg_status gbg_point_traversal_order_workspace_size(const gbg_grid *grid, int64_t npoints,
                                                    int64_t tile_size, size_t *bytes) {
  clear_error();
  GBG_TRY(check_grid(grid));
  int64_t tiles[3];
  GBG_TRY(traversal_tiles(grid, tile_size, tiles));
  if (!bytes) return set_error(GBG_EARG, "null bytes");
  if (npoints < 0 || npoints > 0x7fffffffLL) return set_error(GBG_EUNSUPPORTED, "point count outside 0..2^31-1");
  Arena a;
  a.take<uint32_t>((size_t)npoints);
  a.take<uint32_t>((size_t)npoints);
  a.take<uint32_t>((size_t)npoints);
  a.take<char>(radix_sort_temp_bytes(npoints));
  *bytes = npoints == 0 ? 0 : a.used + 256;
  return GBG_OK;
}

gbg_status gbg_point_traversal_order(const gbg_grid *grid, gbg_dtype dtype, const void *positions,
                                     int64_t npoints, int64_t tile_size, int32_t *order,
                                     void *workspace, size_t workspace_bytes, void *stream) {
  clear_error();
  try {
    size_t need = 0;
    GBG_TRY(gbg_point_traversal_order_workspace_size(grid, npoints, tile_size, &need));
    if (dtype != GBG_F32 && dtype != GBG_F64) return set_error(GBG_EARG, "dtype must be GBG_F32 or GBG_F64");
    if (npoints == 0) return GBG_OK;
    if (!positions || !order) return set_error(GBG_EARG, "traversal order: null array");
    int64_t tiles[3];
    GBG_TRY(traversal_tiles(grid, tile_size, tiles));
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    Scratch scratch;
    GBG_TRY(scratch.acquire(workspace, workspace_bytes, need, st));
    Arena a;
    a.base = static_cast<char *>(scratch.ptr);
    uint32_t *keys = a.take<uint32_t>((size_t)npoints);
    uint32_t *skeys = a.take<uint32_t>((size_t)npoints);
    uint32_t *perm = a.take<uint32_t>((size_t)npoints);
    void *tmp = a.take<char>(radix_sort_temp_bytes(npoints));
    const int blocks = launch_blocks(npoints, kThreads);
    if (dtype == GBG_F64) {
      // inverse_tile = T(tiles) / T(domain), origin = T(origin)  (Interpolation.jl:773-774)
      k_tile_keys<double><<<blocks, kThreads, 0, st>>>(
          static_cast<const double *>(positions), npoints, grid->origin[0], grid->origin[1],
          grid->origin[2], (double)tiles[0] / grid->domain[0], (double)tiles[1] / grid->domain[1],
          (double)tiles[2] / grid->domain[2], tiles[0], tiles[1], tiles[2], keys);
      note_launch();
    } else {
      k_tile_keys<float><<<blocks, kThreads, 0, st>>>(
          static_cast<const float *>(positions), npoints, (float)grid->origin[0],
          (float)grid->origin[1], (float)grid->origin[2], (float)tiles[0] / (float)grid->domain[0],
          (float)tiles[1] / (float)grid->domain[1], (float)tiles[2] / (float)grid->domain[2],
          tiles[0], tiles[1], tiles[2], keys);
      note_launch();
    }
    GBG_CUDA_TRY(cudaGetLastError());
    const uint64_t max_key = (uint64_t)tiles[0] * (uint64_t)tiles[1] * (uint64_t)tiles[2] - 1;
    GBG_TRY(radix_sort_pairs(keys, nullptr, skeys, perm, npoints, bits_for(max_key), tmp, st));
    k_to_one_based<<<blocks, kThreads, 0, st>>>(perm, order, npoints);
    note_launch();
    GBG_CUDA_TRY(cudaGetLastError());
    return GBG_OK;
  } catch (...) {
    return set_error(GBG_ENOMEM, "traversal order: host exception");
  }
}

gbg_status gbg_validate_traversal(const int32_t *order, int64_t npoints, int64_t *host_low,
                                  int64_t *host_high, int64_t *host_visited, void *stream) {
  clear_error();
  if (npoints < 0 || npoints > 0x7fffffffLL) return set_error(GBG_EUNSUPPORTED, "point count outside 0..2^31-1");
  if (npoints == 0) {
    if (host_visited) *host_visited = 0;
    return GBG_OK;
  }
  if (!order) return set_error(GBG_EARG, "validate traversal: null order");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  Scratch scratch;
  const size_t need = 256 + sizeof(uint32_t) * (size_t)npoints;
  GBG_TRY(scratch.acquire(nullptr, 0, need, st));
  unsigned long long *stats = static_cast<unsigned long long *>(scratch.ptr);
  uint32_t *seen = reinterpret_cast<uint32_t *>(static_cast<char *>(scratch.ptr) + 256);
  GBG_CUDA_TRY(cudaMemsetAsync(seen, 0, sizeof(uint32_t) * (size_t)npoints, st));
  k_validate_init<<<1, 1, 0, st>>>(stats);
  note_launch();
  k_validate<<<launch_blocks(npoints, kThreads), kThreads, 0, st>>>(order, npoints, seen, stats);
  note_launch();
  GBG_CUDA_TRY(cudaGetLastError());
  long long h[3];
  GBG_CUDA_TRY(cudaMemcpyAsync(h, stats, sizeof(h), cudaMemcpyDeviceToHost, st));
  GBG_CUDA_TRY(cudaStreamSynchronize(st));
  if (host_low) *host_low = h[0];
  if (host_high) *host_high = h[1];
  if (host_visited) *host_visited = h[2];
  if (h[0] < 1 || h[1] > npoints)
    return set_error(GBG_ETRAVERSAL, "a point traversal order must name points in 1:" + std::to_string(npoints) +
                                         ", but it spans " + std::to_string(h[0]) + ":" + std::to_string(h[1]));
  if (h[2] != npoints)
    return set_error(GBG_ETRAVERSAL, "a point traversal order must name every point exactly once, but it names " +
                                         std::to_string(h[2]) + " of " + std::to_string(npoints));
  return GBG_OK;
}

}  // extern "C"
