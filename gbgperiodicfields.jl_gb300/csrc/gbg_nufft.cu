// NUFFT window transfers on the oversampled grid (sm_103a), and the host-side window
// transform used for the deconvolution.
//
// The reference's fast spectral transfer (src/Interpolation.jl:1611-2070, NUFFT) spreads
// point quantities onto an oversampled (sigma*N) physical grid with the exponential-of-
// semicircle (ES) window, or gathers from it, and does the rest -- the FFT of the
// oversampled grid, the exchange of modes with the reference grid, the division by the
// window's transform -- on whole arrays.  This file holds the two per-point kernels
// (_nufft_gather_kernel!, 1864-1914; _nufft_spread_kernel!, 1919-1950) and the window
// transform (_es_window_transform, 1652-1662); the array steps use cuFFT through the host
// facade.
//
// The FP32 gather bins the points by tile of the oversampled grid; a CTA per tile stages the
// tile's region in shared memory and a warp per point contracts its W^3 stencil there (the
// lanes over the W^2 rows, the x direction first), reduced across the warp.  The FP64 gather
// is a thread per point reading the oversampled field directly (FP64-pipe-bound either way).
//
// The spread is deterministic, unlike the reference's atomic float adds: the window
// weights (evaluated in T as the reference does) and the quantities are converted once per
// point to 64-bit fixed point, every contribution is formed from them with integer high
// products and added as an integer.  Integer addition is associative, so the sums -- and
// the field -- do not depend on the order in which threads add.  The scales leave no
// node's sum able to overflow and keep about M*max|q|*2^-62 of absolute resolution per
// contribution.  The points are binned by tile of the oversampled grid and each tile's sums
// are formed in shared memory before one global add per node: no FP64 arithmetic and no
// global atomic runs per node and point (GB300 runs FP64 at 1/58 of its FP32 rate, while
// 64-bit integer products run on the integer pipes).

#include <algorithm>
#include <cmath>
#include <type_traits>

#include "gbg_common.cuh"

namespace gbg {
namespace {

constexpr int kNThreads = 256;
constexpr int kMaxWidth = 16;
constexpr int kTile = 8;  // points are binned by tiles of kTile^3 oversampled-grid nodes

template <typename T>
struct NGrid {
  int64_t n[3];
  T o[3], d[3];  // T.(origin), T.(grid_spacing) of the oversampled grid
};

template <typename T>
NGrid<T> make_ngrid(const gbg_grid &g) {
  NGrid<T> r;
  for (int a = 0; a < 3; ++a) {
    r.n[a] = g.n[a];
    r.o[a] = T(g.origin[a]);
    r.d[a] = T(g.spacing[a]);
  }
  return r;
}

template <typename T>
__device__ __forceinline__ T nan_t();
template <>
__device__ __forceinline__ double nan_t<double>() { return __longlong_as_double(0x7ff8000000000000LL); }
template <>
__device__ __forceinline__ float nan_t<float>() { return __int_as_float(0x7fc00000); }

__device__ __forceinline__ double div_rn(double a, double b) { return __ddiv_rn(a, b); }
__device__ __forceinline__ float div_rn(float a, float b) { return __fdiv_rn(a, b); }

// Interpolation.jl:1634-1635 -- _stencil_half: the stencil follows the nearer node for an
// odd width.
template <int W, typename T>
__device__ __forceinline__ int stencil_half(T t) {
  return (W % 2 == 1 && t < T(0.5)) ? (W + 1) / 2 : W / 2;
}

// Interpolation.jl:1638-1645 -- _es_weights: node i (1-based) at offset i - half, weight
// exp(beta*(sqrt(max(1 - z^2, 0)) - 1)) with z = 2*(t - (i - half))/W, in T, with the
// reference's separate roundings.
template <int W, typename T>
__device__ __forceinline__ void es_weights(T t, T beta, int half, T (&w)[W]) {
#pragma unroll
  for (int i = 0; i < W; ++i) {
    const T off = T(i + 1 - half);
    const T z = div_rn(mul_rn(T(2), add_rn(t, -off)), T(W));
    const T r = add_rn(T(1), -mul_rn(z, z));
    w[i] = exp(mul_rn(beta, add_rn(sqrt(r > T(0) ? r : T(0)), T(-1))));
  }
}

// _visit (Interpolation.jl:618-619), bounds-checked.
__device__ __forceinline__ bool nvisit(const int32_t *__restrict__ trav, int64_t w, int64_t m, int64_t &p,
                                       int32_t *status) {
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

// A point's weights and wrapped node indices on the three axes.
template <typename T, int W>
struct Stencil {
  T w[3][W];
  int32_t ix[W], iy[W], iz[W];
};

template <typename T, int W>
__device__ __forceinline__ bool point_stencil(const NGrid<T> &g, const T *__restrict__ pos, int64_t p, int64_t m,
                                              T beta, Stencil<T, W> &s) {
  bool ok = true;
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    int64_t base;
    T t;
    ok &= locate(__ldg(pos + p + m * a), g.o[a], g.d[a], base, t);
    const int half = stencil_half<W>(t);
    es_weights<W>(t, beta, half, s.w[a]);
    int32_t *ind = a == 0 ? s.ix : (a == 1 ? s.iy : s.iz);
#pragma unroll
    for (int i = 0; i < W; ++i) ind[i] = (int32_t)imod(base + (i + 1 - half), g.n[a]);
  }
  return ok;
}

// The FP64 gather, a thread per point straight from the oversampled field: the three axes'
// weights, the W^3 stencil with the periodic wrap, the x direction contracted first.  It
// keeps the FP64 pipe busier than the tiled form, whose cross-lane FP64 reductions and
// per-lane window evaluations cost more than the loads it saves.
template <typename T, int W>
__global__ void __launch_bounds__(kNThreads)
    k_nufft_gather(NGrid<T> g, const T *__restrict__ f, const T *__restrict__ pos, int64_t m, int ncomp, T beta,
                   const int32_t *__restrict__ trav, T *__restrict__ out, int32_t *status) {
  const int64_t nxy = g.n[0] * g.n[1], npf = nxy * g.n[2];
  for (int64_t wi = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; wi < m; wi += (int64_t)gridDim.x * blockDim.x) {
    int64_t p;
    if (!nvisit(trav, wi, m, p, status)) continue;
    Stencil<T, W> s;
    if (!point_stencil<T, W>(g, pos, p, m, beta, s)) {
      if (status) atomicOr(status, GBG_DEV_NONFINITE);
      for (int c = 0; c < ncomp; ++c) out[p + m * c] = nan_t<T>();
      continue;
    }
    for (int c = 0; c < ncomp; ++c) {
      const T *fc = f + npf * c;
      T acc = T(0);
#pragma unroll 1
      for (int k = 0; k < W; ++k) {
        const T *plane = fc + nxy * s.iz[k];
#pragma unroll 1
        for (int j = 0; j < W; ++j) {
          const T *row = plane + g.n[0] * s.iy[j];
          T sx = T(0);
#pragma unroll
          for (int i = 0; i < W; ++i) sx = fma_rn(s.w[0][i], __ldg(row + s.ix[i]), sx);
          acc = fma_rn(mul_rn(s.w[1][j], s.w[2][k]), sx, acc);
        }
      }
      out[p + m * c] = acc;
    }
  }
}

// Tiled window gather: a CTA per tile stages the tile's region ((kTile + W - 1)^3 nodes of
// the oversampled field, for a group of components) in shared memory; a warp per point
// evaluates the point's 3W window weights across its lanes, its lanes take the W^2 rows of the
// stencil, contract x first, and the row sums are reduced across the warp.
template <typename T, int W>
__global__ void __launch_bounds__(kNThreads)
    k_nufft_gather_tiles(NGrid<T> g, const T *__restrict__ f, const T *__restrict__ pos, int64_t m, int ncomp,
                         int group, T beta, const int32_t *__restrict__ trav, int64_t nt0, int64_t nt1,
                         int64_t ntiles, const uint32_t *__restrict__ tstart, const uint32_t *__restrict__ order,
                         const int32_t *__restrict__ first, T *__restrict__ out) {
  constexpr int R = kTile + W - 1;
  constexpr int R3 = R * R * R;
  extern __shared__ __align__(16) unsigned char gsm[];
  T *reg = reinterpret_cast<T *>(gsm);  // group x R3 values
  __shared__ T swt[kNThreads / 32][3 * W];
  const int64_t nxy = g.n[0] * g.n[1], npf = nxy * g.n[2];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const uint32_t t0 = tstart[tile], t1 = tstart[tile + 1];
    if (t1 == t0) continue;  // uniform over the CTA
    const int64_t tx = (tile % nt0) * kTile, ty = ((tile / nt0) % nt1) * kTile, tz = (tile / (nt0 * nt1)) * kTile;
    for (int c0 = 0; c0 < ncomp; c0 += group) {
      const int cg = min(group, ncomp - c0);
      __syncthreads();  // the previous group's region is no longer read
      for (int e = threadIdx.x; e < cg * R3; e += blockDim.x) {
        const int cc = e / R3, r = e - cc * R3;
        const int rx = r % R, ry = (r / R) % R, rz = r / (R * R);
        const int64_t x = (tx + rx) % g.n[0], y = (ty + ry) % g.n[1], z = (tz + rz) % g.n[2];
        reg[e] = __ldg(f + npf * (c0 + cc) + z * nxy + y * g.n[0] + x);
      }
      __syncthreads();
      for (uint32_t pt = t0 + warp; pt < t1; pt += nwarps) {
        const uint32_t wi = order[pt];
        int64_t p = wi;
        if (trav) p = (int64_t)__ldg(trav + wi) - 1;
        for (int e = lane; e < 3 * W; e += 32) {  // 3W can exceed the 32 lanes (W > 10)
          const int a = e / W, i = e - a * W;
          int64_t base;
          T t;
          locate(__ldg(pos + p + m * a), g.o[a], g.d[a], base, t);
          const int half = stencil_half<W>(t);
          const T off = T(i + 1 - half);
          const T z = div_rn(mul_rn(T(2), add_rn(t, -off)), T(W));
          const T r = add_rn(T(1), -mul_rn(z, z));
          swt[warp][e] = exp(mul_rn(beta, add_rn(sqrt(r > T(0) ? r : T(0)), T(-1))));
        }
        const int ox = (int)(first[3 * (int64_t)wi] - tx), oy = (int)(first[3 * (int64_t)wi + 1] - ty),
                  oz = (int)(first[3 * (int64_t)wi + 2] - tz);
        __syncwarp();
        T acc[4] = {T(0), T(0), T(0), T(0)};  // up to four components per pass of the rows
        for (int cb = 0; cb < cg; cb += 4) {
          const int nc = min(4, cg - cb);
#pragma unroll
          for (int q = 0; q < 4; ++q) acc[q] = T(0);
          for (int rw = lane; rw < W * W; rw += 32) {
            const int j = rw % W, k = rw / W;
            const T wyz = mul_rn(swt[warp][W + j], swt[warp][2 * W + k]);
            const T *row = reg + ((oz + k) * R + oy + j) * R + ox;
#pragma unroll
            for (int q = 0; q < 4; ++q) {
              if (q < nc) {
                const T *rq = row + (cb + q) * R3;
                T sx = T(0);
#pragma unroll
                for (int i = 0; i < W; ++i) sx = fma_rn(swt[warp][i], rq[i], sx);
                acc[q] = fma_rn(wyz, sx, acc[q]);
              }
            }
          }
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            T v = acc[q];
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
            if (lane == 0 && q < nc) out[p + m * (c0 + cb + q)] = v;
          }
        }
        __syncwarp();
      }
    }
  }
}

// Largest |q| over all points and components, as ordered double bits (NaN above all).
template <typename T>
__global__ void __launch_bounds__(kNThreads)
    k_nufft_qmax(const T *__restrict__ q, int64_t n, unsigned long long *qmax_bits) {
  unsigned long long mx = 0ull;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(fabs((double)q[i]));
    mx = b > mx ? b : mx;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long other = __shfl_xor_sync(0xffffffffu, mx, o);
    mx = other > mx ? other : mx;
  }
  if ((threadIdx.x & 31) == 0) atomicMax(qmax_bits, mx);
}

// The fixed-point scales of a spread.  Weights are w * 2^62 (ES weights lie in [0, 1]);
// quantities q * 2^(62 - eq) with max|q| < 2^eq; a contribution is
// hi(hi(hi(Wy, Wz), Wx), |Q|) = w |q| 2^(56 - eq) < 2^56, shifted right (rounded) by
// s = max(0, em - 6) with M <= 2^em, so that no node's sum of at most M contributions can
// reach 2^62.  A node's value is its sum times 2^(eq + s - 56).
struct SpreadScale {
  int eq, s;
};
__device__ __forceinline__ SpreadScale spread_scale(unsigned long long qmax_bits, int64_t m) {
  int eq = 0, em = 0;
  frexp(__longlong_as_double((long long)qmax_bits), &eq);
  frexp((double)m, &em);
  return {eq, em > 6 ? em - 6 : 0};
}

// Spread, pass 1: each point's window weights (in T, as the reference evaluates them, then
// as 64-bit fixed point) and first stencil node per axis, and its
// tile (kTile^3 nodes holding the first node) with its rank there from an atomic count --
// the order within a tile does not matter, the sums being integer.  A point with a
// non-finite position goes to the extra bucket ntiles, which no tile visits.

// With wbuf == nullptr (the gather) only the tiles and first nodes are kept, and a point
// with a non-finite position gets NaN in out (ncomp components) here.
template <typename T, int W>
__global__ void __launch_bounds__(kNThreads)
    k_nufft_bin(NGrid<T> g, const T *__restrict__ pos, int64_t m, T beta, int64_t nt0, int64_t nt1,
                int64_t ntiles, const int32_t *__restrict__ trav, uint32_t *__restrict__ tcount,
                uint32_t *__restrict__ tkey, uint32_t *__restrict__ rank, int32_t *__restrict__ first,
                unsigned long long *__restrict__ wbuf, int32_t *status, T *__restrict__ out = nullptr,
                int ncomp = 0) {
  for (int64_t wi = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; wi < m; wi += (int64_t)gridDim.x * blockDim.x) {
    int64_t p;
    if (!nvisit(trav, wi, m, p, status)) {
      // a bad traversal entry: the visit slot wi carries no point
      tkey[wi] = (uint32_t)ntiles;
      rank[wi] = atomicAdd(tcount + ntiles, 1u);
      continue;
    }
    bool ok = true;
    int64_t s[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      int64_t base;
      T t;
      ok &= locate(__ldg(pos + p + m * a), g.o[a], g.d[a], base, t);
      const int half = stencil_half<W>(t);
      if (wbuf) {
        T w[W];
        es_weights<W>(t, beta, half, w);
#pragma unroll
        for (int i = 0; i < W; ++i)  // w * 2^62, exact to the rounding of one conversion
          wbuf[(3 * wi + a) * W + i] = ok ? (unsigned long long)fixed_rn((double)w[i], 62) : 0ull;
      }
      s[a] = imod(base + (1 - half), g.n[a]);
      first[3 * wi + a] = (int32_t)s[a];
    }
    if (!ok && status) atomicOr(status, GBG_DEV_NONFINITE);
    if (!ok && out)
      for (int c = 0; c < ncomp; ++c) out[p + m * c] = nan_t<T>();
    const int64_t key = ok ? ((s[2] / kTile) * nt1 + s[1] / kTile) * nt0 + s[0] / kTile : ntiles;
    tkey[wi] = (uint32_t)key;
    rank[wi] = atomicAdd(tcount + key, 1u);
  }
}

// Spread, pass 2: the visit slots in tile order.
__global__ void __launch_bounds__(kNThreads)
    k_nufft_place(int64_t m, const uint32_t *__restrict__ tkey, const uint32_t *__restrict__ rank,
                  const uint32_t *__restrict__ tstart, uint32_t *__restrict__ order) {
  for (int64_t wi = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; wi < m; wi += (int64_t)gridDim.x * blockDim.x)
    order[tstart[tkey[wi]] + rank[wi]] = (uint32_t)wi;
}

// Spread, pass 3: a CTA per tile.  For a group of CG components at a time the tile's
// region ((kTile + W - 1)^3 nodes) is summed in shared memory -- a warp per point, its lanes
// over the point's W^3 nodes, each contribution hi(hi(Wyz, Wx), |Q|) formed with integer
// high products (no FP64 arithmetic per node) and rounded to s bits, then added to the
// node's 64-bit sum as 32-bit low and high words with a carry
// (native 32-bit shared atomics) -- then every nonzero node sum is added to the grid's by
// one global integer atomic.  Integer sums do not depend on the order of the adds.
constexpr int kMaxGroup = 32;

template <int W>
__global__ void __launch_bounds__(kNThreads)
    k_nufft_spread_tiles(NGrid<double> g, int64_t m, const void *__restrict__ qv_, int q_f64,
                         const int32_t *__restrict__ trav, int ncomp, int group, int64_t nt0, int64_t nt1,
                         int64_t ntiles, const uint32_t *__restrict__ tstart, const uint32_t *__restrict__ order,
                         const int32_t *__restrict__ first, const unsigned long long *__restrict__ wbuf,
                         const unsigned long long *__restrict__ qmax_bits, unsigned long long *__restrict__ acc) {
  constexpr int R = kTile + W - 1;
  constexpr int R3 = R * R * R;
  // group x R3 64-bit sums: a plane of low words, then a plane of high words
  extern __shared__ uint32_t sacc_lo[];
  uint32_t *sacc_hi = sacc_lo + group * R3;
  __shared__ unsigned long long swyz[kNThreads / 32][W * W], swx[kNThreads / 32][W];
  __shared__ long long sq[kNThreads / 32][kMaxGroup];
  const double qmax = __longlong_as_double((long long)*qmax_bits);
  if (!isfinite(qmax)) return;  // the field is set to NaN by k_nufft_finish
  const SpreadScale sc = spread_scale(*qmax_bits, m);
  const unsigned long long round = sc.s ? (1ull << (sc.s - 1)) : 0ull;
  const int64_t nxy = g.n[0] * g.n[1], npf = nxy * g.n[2];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const uint32_t t0 = tstart[tile], t1 = tstart[tile + 1];
    if (t1 == t0) continue;  // uniform over the CTA
    const int64_t tx = (tile % nt0) * kTile, ty = ((tile / nt0) % nt1) * kTile, tz = (tile / (nt0 * nt1)) * kTile;
    for (int c0 = 0; c0 < ncomp; c0 += group) {
      const int cg = min(group, ncomp - c0);
      for (int r = threadIdx.x; r < cg * R3; r += blockDim.x) {
        sacc_lo[r] = 0u;
        sacc_hi[r] = 0u;
      }
      __syncthreads();
      for (uint32_t pt = t0 + warp; pt < t1; pt += nwarps) {
        const uint32_t wi = order[pt];
        int64_t p = wi;
        if (trav) p = (int64_t)__ldg(trav + wi) - 1;
        const unsigned long long *wp = wbuf + 3 * (int64_t)wi * W;
        for (int i = lane; i < W; i += 32) swx[warp][i] = wp[i];
        for (int e = lane; e < W * W; e += 32) swyz[warp][e] = __umul64hi(wp[W + e % W], wp[2 * W + e / W]);
        if (lane < cg) {
          const int64_t qi = p + m * (c0 + lane);
          const double q = q_f64 ? static_cast<const double *>(qv_)[qi] : (double)static_cast<const float *>(qv_)[qi];
          sq[warp][lane] = fixed_rn(q, 62 - sc.eq);
        }
        const int ox = (int)(first[3 * (int64_t)wi] - tx), oy = (int)(first[3 * (int64_t)wi + 1] - ty),
                  oz = (int)(first[3 * (int64_t)wi + 2] - tz);
        __syncwarp();
        for (int idx = lane; idx < W * W * W; idx += 32) {
          const int i = idx % W, jk = idx / W, j = jk % W, kk = jk / W;
          const unsigned long long wxyz = __umul64hi(swyz[warp][jk], swx[warp][i]);
          const int r = ((oz + kk) * R + oy + j) * R + ox + i;
          for (int cc = 0; cc < cg; ++cc) {
            const long long qq = sq[warp][cc];
            const unsigned long long mag = (__umul64hi(wxyz, (unsigned long long)(qq < 0 ? -qq : qq)) + round) >> sc.s;
            atomic_add_split64(sacc_lo, sacc_hi, cc * R3 + r, qq < 0 ? (unsigned long long)(-(long long)mag) : mag);
          }
        }
        __syncwarp();
      }
      __syncthreads();
      for (int e = threadIdx.x; e < cg * R3; e += blockDim.x) {
        const unsigned long long v = ((unsigned long long)sacc_hi[e] << 32) | sacc_lo[e];
        if (v == 0ull) continue;
        const int cc = e / R3, r = e - cc * R3;
        const int rx = r % R, ry = (r / R) % R, rz = r / (R * R);
        // the region may pass the end of an axis (and, for a window wider than a small
        // axis, wrap more than once): several region nodes can land on one grid node
        const int64_t x = (tx + rx) % g.n[0], y = (ty + ry) % g.n[1], z = (tz + rz) % g.n[2];
        atomicAdd(acc + npf * (c0 + cc) + z * nxy + y * g.n[0] + x, v);
      }
      __syncthreads();
    }
  }
}

// The oversampled field from the fixed-point sums (NaN everywhere for a non-finite q,
// which the FFT would spread over every mode anyway).
template <typename T>
__global__ void __launch_bounds__(kNThreads)
    k_nufft_finish(const unsigned long long *__restrict__ acc, int64_t n, int64_t m,
                   const unsigned long long *__restrict__ qmax_bits, T *__restrict__ field, int32_t *status) {
  const double qmax = __longlong_as_double((long long)*qmax_bits);
  const bool finite = isfinite(qmax);  // a non-finite quantity is not an error: it yields NaN
  const SpreadScale sc = spread_scale(*qmax_bits, m);
  const int e = sc.eq + sc.s - 56;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    field[i] = finite ? (T)ldexp((double)(long long)acc[i], e) : nan_t<T>();
}

gbg_status check_ngrid(const gbg_grid *g) {
  if (!g) return set_error(GBG_EARG, "null grid");
  for (int a = 0; a < 3; ++a) {
    if (g->n[a] <= 0) return set_error(GBG_EARG, "grid_size must be positive along every axis");
    if (!(std::isfinite(g->spacing[a]) && g->spacing[a] > 0))
      return set_error(GBG_EARG, "grid_spacing must be finite and positive along every axis");
    if (!std::isfinite(g->origin[a])) return set_error(GBG_EARG, "origin must be finite along every axis");
    if (g->n[a] > (int64_t(1) << 30)) return set_error(GBG_EUNSUPPORTED, "grid axis longer than 2^30");
  }
  return GBG_OK;
}

gbg_status check_nufft(const gbg_grid *g, gbg_dtype dtype, int32_t ncomp, int64_t m, int32_t width, double beta) {
  GBG_TRY(check_ngrid(g));
  if (dtype != GBG_F32 && dtype != GBG_F64) return set_error(GBG_EARG, "dtype must be GBG_F32 or GBG_F64");
  if (ncomp < 1) return set_error(GBG_EARG, "ncomp must be at least 1");
  if (m < 0) return set_error(GBG_EDIM, "negative point count");
  if (width < 1) return set_error(GBG_EARG, "NUFFT window_width must be a positive number of nodes");
  if (width > kMaxWidth) return set_error(GBG_EUNSUPPORTED, "NUFFT window_width above 16 nodes");
  if (!(std::isfinite(beta) && beta > 0)) return set_error(GBG_EARG, "NUFFT window_shape must be finite and positive");
  return GBG_OK;
}

// Calls f(std::integral_constant<int, W>) for the run-time width 1..16.
template <typename F>
gbg_status with_width(int32_t width, F &&f) {
  switch (width) {
#define GBG_W(N) \
  case N: return f(std::integral_constant<int, N>{});
    GBG_W(1) GBG_W(2) GBG_W(3) GBG_W(4) GBG_W(5) GBG_W(6) GBG_W(7) GBG_W(8)
    GBG_W(9) GBG_W(10) GBG_W(11) GBG_W(12) GBG_W(13) GBG_W(14) GBG_W(15) GBG_W(16)
#undef GBG_W
    default: return set_error(GBG_EUNSUPPORTED, "NUFFT window_width outside 1..16");
  }
}

// Interpolation.jl:1652-1662 -- _es_window_transform: psi_hat(omega) by the trapezoidal
// rule in theta (z = sin(theta)), in T.
template <typename T>
T es_window_transform(T omega, T beta, int width, int quadrature_points) {
  const T half_width = T(width) / T(2);
  const T pi = T(3.141592653589793238462643383279502884);
  T accumulated = T(0);
  for (int q = 0; q <= quadrature_points; ++q) {
    const T theta = -pi / T(2) + pi * T(q) / T(quadrature_points);
    const T trapezoidal = (q == 0 || q == quadrature_points) ? T(1) / T(2) : T(1);
    accumulated += trapezoidal * std::exp(beta * (std::cos(theta) - T(1))) * std::cos(omega * half_width * std::sin(theta)) *
                   std::cos(theta);
  }
  return half_width * (pi / T(quadrature_points)) * accumulated;
}

template <typename T>
void deconvolution_axis(int64_t n, int64_t stored, bool is_half, int sigma, int width, T beta, double *out) {
  const T pi = T(3.141592653589793238462643383279502884);
  for (int64_t i = 0; i < stored; ++i) {
    const int64_t f = (is_half || i < (n + 1) / 2) ? i : i - n;
    const T omega = T(2) * pi * T(f) / (T(sigma) * T(n));
    out[i] = (double)(T(1) / es_window_transform<T>(omega, beta, width, 256));
  }
  if (n % 2 == 0) out[is_half ? stored - 1 : n / 2] = 0.0;
}

}  // namespace
}  // namespace gbg

using namespace gbg;

extern "C" {

gbg_status gbg_nufft_deconvolution_axis(int64_t n, int32_t is_half, int32_t oversampling, int32_t width,
                                        double beta, gbg_dtype dtype, double *host_out) {
  clear_error();
  if (n < 1) return set_error(GBG_EARG, "grid_size must be positive");
  if (oversampling < 2) return set_error(GBG_EARG, "NUFFT oversampling must be at least 2");
  if (width < 1) return set_error(GBG_EARG, "NUFFT window_width must be a positive number of nodes");
  if (!(std::isfinite(beta) && beta > 0)) return set_error(GBG_EARG, "NUFFT window_shape must be finite and positive");
  if (dtype != GBG_F32 && dtype != GBG_F64) return set_error(GBG_EARG, "dtype must be GBG_F32 or GBG_F64");
  if (!host_out) return set_error(GBG_EARG, "null output");
  const int64_t stored = is_half ? n / 2 + 1 : n;
  if (dtype == GBG_F64)
    deconvolution_axis<double>(n, stored, is_half != 0, oversampling, width, beta, host_out);
  else
    deconvolution_axis<float>(n, stored, is_half != 0, oversampling, width, (float)beta, host_out);
  return GBG_OK;
}

}  // extern "C"

namespace gbg {
namespace {

struct SpreadLayout {
  unsigned long long *acc = nullptr, *qmax = nullptr;
  uint32_t *tcount = nullptr, *scan_tmp = nullptr, *tkey = nullptr, *rank = nullptr, *order = nullptr;
  int32_t *first = nullptr;
  unsigned long long *wbuf = nullptr;
  int64_t nt0 = 0, nt1 = 0, nt2 = 0, ntiles = 0;
};

// The spread's workspace, in order: node sums (ncomp per node), max|q|, tile counts (+ the
// extra bucket and the end), scan scratch, per visit slot its tile, rank and place, first
// stencil nodes (3) and fixed-point window weights (3 W).  With base == nullptr it only sizes.
size_t spread_layout(char *base, const gbg_grid &fine, gbg_dtype dtype, int32_t ncomp, int64_t m, int32_t width,
                     SpreadLayout &L, bool spread = true) {
  Arena a;
  a.base = base;
  L.nt0 = (fine.n[0] + kTile - 1) / kTile;
  L.nt1 = (fine.n[1] + kTile - 1) / kTile;
  L.nt2 = (fine.n[2] + kTile - 1) / kTile;
  L.ntiles = L.nt0 * L.nt1 * L.nt2;
  const int64_t npf = fine.n[0] * fine.n[1] * fine.n[2];
  if (spread) {
    L.acc = a.take<unsigned long long>((size_t)(npf * ncomp));
    L.qmax = a.take<unsigned long long>(1);
  }
  L.tcount = a.take<uint32_t>((size_t)L.ntiles + 2);
  L.scan_tmp = a.take<uint32_t>(scan_temp_elems(L.ntiles + 2));
  const size_t mm = (size_t)(m > 0 ? m : 1);
  L.tkey = a.take<uint32_t>(mm);
  L.rank = a.take<uint32_t>(mm);
  L.order = a.take<uint32_t>(mm);
  L.first = a.take<int32_t>(3 * mm);
  if (spread) L.wbuf = a.take<unsigned long long>(3 * (size_t)width * mm);
  return a.used + 256;
}

// The tiled gather: bin, place, then a CTA per tile over the staged region.
template <typename T, int W>
gbg_status gather_run(const gbg_grid &fine, int32_t ncomp, const T *field, const T *pos, int64_t m,
                      const int32_t *trav, double beta, T *out, const SpreadLayout &L, int32_t *status,
                      cudaStream_t st) {
  const NGrid<T> g = make_ngrid<T>(fine);
  k_nufft_bin<T, W><<<launch_blocks(m, kNThreads), kNThreads, 0, st>>>(
      g, pos, m, (T)beta, L.nt0, L.nt1, L.ntiles, trav, L.tcount, L.tkey, L.rank, L.first, nullptr, status, out,
      ncomp);
  note_launch();
  GBG_CUDA_TRY(cudaGetLastError());
  GBG_TRY(exclusive_scan_u32(L.tcount, L.tcount, L.ntiles + 2, L.scan_tmp, st));
  k_nufft_place<<<launch_blocks(m, kNThreads), kNThreads, 0, st>>>(m, L.tkey, L.rank, L.tcount, L.order);
  note_launch();
  GBG_CUDA_TRY(cudaGetLastError());
  constexpr int R = kTile + W - 1;
  const size_t slice = sizeof(T) * (size_t)R * R * R;
  // components per pass: as many region slices as fit in 96 KB (two CTAs per SM), at least one
  const int group = (int)std::max<size_t>(1, std::min<size_t>((size_t)ncomp, 98304 / slice));
  const size_t smem = slice * group;
  auto kernel = k_nufft_gather_tiles<T, W>;
  GBG_CUDA_TRY(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int per_sm = 1, sms = 0, dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kNThreads, smem);
  const int blocks = (int)std::min<int64_t>(L.ntiles, (int64_t)sms * std::max(per_sm, 1));
  mark_main_start(st);
  kernel<<<blocks, kNThreads, smem, st>>>(g, field, pos, m, ncomp, group, (T)beta, trav, L.nt0, L.nt1, L.ntiles,
                                         L.tcount, L.order, L.first, out);
  mark_main_stop(st);
  note_launch();
  GBG_CUDA_TRY(cudaGetLastError());
  return GBG_OK;
}

template <typename T, int W>
gbg_status spread_run(const gbg_grid &fine, int32_t ncomp, T *field, const T *pos, int64_t m, const T *q,
                      const int32_t *trav, double beta, const SpreadLayout &L, int32_t *status, cudaStream_t st) {
  const NGrid<T> g = make_ngrid<T>(fine);
  const int64_t n = fine.n[0] * fine.n[1] * fine.n[2] * (int64_t)ncomp;
  if (m > 0) {
    const int64_t nq = m * (int64_t)ncomp;
    k_nufft_qmax<T><<<launch_blocks(nq, kNThreads), kNThreads, 0, st>>>(q, nq, L.qmax);
    note_launch();
    k_nufft_bin<T, W><<<launch_blocks(m, kNThreads), kNThreads, 0, st>>>(
        g, pos, m, (T)beta, L.nt0, L.nt1, L.ntiles, trav, L.tcount, L.tkey, L.rank, L.first, L.wbuf, status);
    note_launch();
    GBG_CUDA_TRY(cudaGetLastError());
    GBG_TRY(exclusive_scan_u32(L.tcount, L.tcount, L.ntiles + 2, L.scan_tmp, st));
    k_nufft_place<<<launch_blocks(m, kNThreads), kNThreads, 0, st>>>(m, L.tkey, L.rank, L.tcount, L.order);
    note_launch();
    GBG_CUDA_TRY(cudaGetLastError());
    constexpr int R = kTile + W - 1;
    const size_t slice = sizeof(unsigned long long) * (size_t)R * R * R;
    // components per pass: as many region slices as fit in 96 KB (two CTAs per SM), at least one
    const int group = (int)std::max<size_t>(1, std::min<size_t>({(size_t)ncomp, (size_t)kMaxGroup, 98304 / slice}));
    const size_t smem = slice * group;
    auto kernel = k_nufft_spread_tiles<W>;
    GBG_CUDA_TRY(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int per_sm = 1, sms = 0, dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kNThreads, smem);
    const int blocks = (int)std::min<int64_t>(L.ntiles, (int64_t)sms * std::max(per_sm, 1));
    mark_main_start(st);
    kernel<<<blocks, kNThreads, smem, st>>>(make_ngrid<double>(fine), m, q, sizeof(T) == 8, trav, ncomp, group, L.nt0,
                                           L.nt1, L.ntiles, L.tcount, L.order, L.first, L.wbuf, L.qmax, L.acc);
    mark_main_stop(st);
    note_launch();
    GBG_CUDA_TRY(cudaGetLastError());
  }
  k_nufft_finish<T><<<launch_blocks(n, kNThreads), kNThreads, 0, st>>>(L.acc, n, m > 0 ? m : 1, L.qmax, field, status);
  note_launch();
  GBG_CUDA_TRY(cudaGetLastError());
  return GBG_OK;
}

}  // namespace
}  // namespace gbg

extern "C" {

gbg_status gbg_nufft_interp_workspace_size(const gbg_grid *fine, gbg_dtype dtype, int32_t ncomp, int64_t npoints,
                                           int32_t width, size_t *bytes) {
  clear_error();
  GBG_TRY(check_nufft(fine, dtype, ncomp, npoints, width, 1.0));
  if (!bytes) return set_error(GBG_EARG, "null bytes");
  SpreadLayout L;
  *bytes = spread_layout(nullptr, *fine, dtype, ncomp, npoints, width, L, false);
  return GBG_OK;
}

gbg_status gbg_nufft_interp(const gbg_grid *fine, gbg_dtype dtype, int32_t ncomp, const void *field,
                            const void *positions, int64_t npoints, const int32_t *traversal, int32_t width,
                            double beta, void *out, void *workspace, size_t workspace_bytes, int32_t *device_status,
                            void *stream) {
  clear_error();
  try {
    GBG_TRY(check_nufft(fine, dtype, ncomp, npoints, width, beta));
    if (npoints == 0) return GBG_OK;
    if (!field || !positions || !out) return set_error(GBG_EARG, "nufft_interp: null array");
    if (npoints > 0x7fffffffLL) return set_error(GBG_EUNSUPPORTED, "nufft_interp: more than 2^31-1 points");
    size_t need = 0;
    GBG_TRY(gbg_nufft_interp_workspace_size(fine, dtype, ncomp, npoints, width, &need));
    if (!workspace || workspace_bytes < need) return set_error(GBG_ENOMEM, "nufft_interp: workspace too small");
    if ((reinterpret_cast<uintptr_t>(workspace) & 255u) != 0)
      return set_error(GBG_EARG, "nufft_interp: workspace not 256-byte aligned");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    SpreadLayout L;
    spread_layout(static_cast<char *>(workspace), *fine, dtype, ncomp, npoints, width, L, false);
    GBG_CUDA_TRY(cudaMemsetAsync(L.tcount, 0, sizeof(uint32_t) * ((size_t)L.ntiles + 2), st));
    return with_width(width, [&](auto wc) -> gbg_status {
      constexpr int W = decltype(wc)::value;
      if (dtype == GBG_F64) {
        mark_main_start(st);
        k_nufft_gather<double, W><<<launch_blocks(npoints, kNThreads), kNThreads, 0, st>>>(
            make_ngrid<double>(*fine), static_cast<const double *>(field), static_cast<const double *>(positions),
            npoints, ncomp, beta, traversal, static_cast<double *>(out), device_status);
        mark_main_stop(st);
        note_launch();
        GBG_CUDA_TRY(cudaGetLastError());
        return GBG_OK;
      }
      return gather_run<float, W>(*fine, ncomp, static_cast<const float *>(field), static_cast<const float *>(positions),
                                  npoints, traversal, beta, static_cast<float *>(out), L, device_status, st);
    });
  } catch (...) {
    return set_error(GBG_ENOMEM, "nufft_interp: host exception");
  }
}

gbg_status gbg_nufft_spread_workspace_size(const gbg_grid *fine, gbg_dtype dtype, int32_t ncomp, int64_t npoints,
                                           int32_t width, size_t *bytes) {
  clear_error();
  GBG_TRY(check_nufft(fine, dtype, ncomp, npoints, width, 1.0));
  if (!bytes) return set_error(GBG_EARG, "null bytes");
  SpreadLayout L;
  *bytes = spread_layout(nullptr, *fine, dtype, ncomp, npoints, width, L);
  return GBG_OK;
}

gbg_status gbg_nufft_spread(const gbg_grid *fine, gbg_dtype dtype, int32_t ncomp, void *field,
                            const void *positions, int64_t npoints, const void *quantities,
                            const int32_t *traversal, int32_t width, double beta, void *workspace,
                            size_t workspace_bytes, int32_t *device_status, void *stream) {
  clear_error();
  try {
    GBG_TRY(check_nufft(fine, dtype, ncomp, npoints, width, beta));
    size_t need = 0;
    GBG_TRY(gbg_nufft_spread_workspace_size(fine, dtype, ncomp, npoints, width, &need));
    if (!field) return set_error(GBG_EARG, "nufft_spread: null field");
    if (npoints > 0 && (!positions || !quantities)) return set_error(GBG_EARG, "nufft_spread: null array");
    if (npoints > 0x7fffffffLL) return set_error(GBG_EUNSUPPORTED, "nufft_spread: more than 2^31-1 points");
    if (!workspace || workspace_bytes < need) return set_error(GBG_ENOMEM, "nufft_spread: workspace too small");
    // the layout aligns its pieces to 256 bytes from the workspace's start
    if ((reinterpret_cast<uintptr_t>(workspace) & 255u) != 0)
      return set_error(GBG_EARG, "nufft_spread: workspace not 256-byte aligned");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    SpreadLayout L;
    spread_layout(static_cast<char *>(workspace), *fine, dtype, ncomp, npoints, width, L);
    const int64_t n = fine->n[0] * fine->n[1] * fine->n[2] * (int64_t)ncomp;
    GBG_CUDA_TRY(cudaMemsetAsync(L.acc, 0, (size_t)n * 8, st));
    GBG_CUDA_TRY(cudaMemsetAsync(L.qmax, 0, 8, st));
    GBG_CUDA_TRY(cudaMemsetAsync(L.tcount, 0, sizeof(uint32_t) * ((size_t)L.ntiles + 2), st));
    return with_width(width, [&](auto wc) -> gbg_status {
      constexpr int W = decltype(wc)::value;
      if (dtype == GBG_F64)
        return spread_run<double, W>(*fine, ncomp, static_cast<double *>(field), static_cast<const double *>(positions),
                                     npoints, static_cast<const double *>(quantities), traversal, beta, L,
                                     device_status, st);
      return spread_run<float, W>(*fine, ncomp, static_cast<float *>(field), static_cast<const float *>(positions),
                                  npoints, static_cast<const float *>(quantities), traversal, beta, L, device_status,
                                  st);
    });
  } catch (...) {
    return set_error(GBG_ENOMEM, "nufft_spread: host exception");
  }
}

}  // extern "C"
