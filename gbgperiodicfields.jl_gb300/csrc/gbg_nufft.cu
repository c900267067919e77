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
// The gather is a thread per point: the three axes' W window weights, then the W^3
// stencil with the periodic wrap, the x direction contracted first with FMAs.
//
// The spread is deterministic, unlike the reference's atomic float adds: every
// contribution ((wy*wz)*wx)*q is rounded to a 64-bit fixed-point integer at one scale for
// the whole call, 2^k with k = 61 - e and M*max|q| < 2^e, and added with an integer
// atomic.  Integer addition is associative, so the sums -- and the field -- do not depend
// on the order in which threads add.  No node's sum can reach 2^61 (each window weight is
// at most 1), and a contribution keeps M*max|q|*2^-62 of absolute resolution.

#include <cmath>
#include <type_traits>

#include "gbg_common.cuh"

namespace gbg {
namespace {

constexpr int kNThreads = 256;
constexpr int kMaxWidth = 16;

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

// The fixed-point exponent k of a call: max|q| < 2^eq and M <= 2^em, so M*max|q| < 2^(61-k)
// with k = 61 - eq - em (the exponents are taken apart, so no product can overflow).
__device__ __forceinline__ int spread_exponent(unsigned long long qmax_bits, int64_t m) {
  int eq = 0, em = 0;
  frexp(__longlong_as_double((long long)qmax_bits), &eq);
  frexp((double)m, &em);
  return 61 - eq - em;
}

template <typename T, int W>
__global__ void __launch_bounds__(kNThreads)
    k_nufft_spread(NGrid<T> g, const T *__restrict__ pos, int64_t m, const T *__restrict__ q, int ncomp, T beta,
                   const int32_t *__restrict__ trav, const unsigned long long *__restrict__ qmax_bits,
                   unsigned long long *__restrict__ acc, int32_t *status) {
  const double qmax = __longlong_as_double((long long)*qmax_bits);
  if (!isfinite(qmax)) return;  // the field is set to NaN by k_nufft_finish
  const int k = spread_exponent(*qmax_bits, m);
  const bool plain = k > -1000 && k < 1000;  // 2^k is a finite double: scale by one product
  const double scale = plain ? ldexp(1.0, k) : 0.0;
  const int64_t nxy = g.n[0] * g.n[1], npf = nxy * g.n[2];
  for (int64_t wi = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; wi < m; wi += (int64_t)gridDim.x * blockDim.x) {
    int64_t p;
    if (!nvisit(trav, wi, m, p, status)) continue;
    Stencil<T, W> s;
    if (!point_stencil<T, W>(g, pos, p, m, beta, s)) {
      if (status) atomicOr(status, GBG_DEV_NONFINITE);
      continue;
    }
    for (int c = 0; c < ncomp; ++c) {
      const T qv = q[p + m * c];
      unsigned long long *ac = acc + npf * c;
#pragma unroll 1
      for (int k = 0; k < W; ++k) {
        unsigned long long *plane = ac + nxy * s.iz[k];
#pragma unroll 1
        for (int j = 0; j < W; ++j) {
          unsigned long long *row = plane + g.n[0] * s.iy[j];
          const T wyz = mul_rn(s.w[1][j], s.w[2][k]);
#pragma unroll
          for (int i = 0; i < W; ++i) {
            const T v = mul_rn(mul_rn(wyz, s.w[0][i]), qv);
            const double x = plain ? (double)v * scale : ldexp((double)v, k);
            atomicAdd(row + s.ix[i], (unsigned long long)__double2ll_rn(x));
          }
        }
      }
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
  const bool finite = isfinite(qmax);
  if (!finite && status && blockIdx.x == 0 && threadIdx.x == 0) atomicOr(status, GBG_DEV_NONFINITE);
  const int k = spread_exponent(*qmax_bits, m);
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    field[i] = finite ? (T)ldexp((double)(long long)acc[i], -k) : nan_t<T>();
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

gbg_status gbg_nufft_interp(const gbg_grid *fine, gbg_dtype dtype, int32_t ncomp, const void *field,
                            const void *positions, int64_t npoints, const int32_t *traversal, int32_t width,
                            double beta, void *out, int32_t *device_status, void *stream) {
  clear_error();
  try {
    GBG_TRY(check_nufft(fine, dtype, ncomp, npoints, width, beta));
    if (npoints == 0) return GBG_OK;
    if (!field || !positions || !out) return set_error(GBG_EARG, "nufft_interp: null array");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    return with_width(width, [&](auto wc) -> gbg_status {
      constexpr int W = decltype(wc)::value;
      const int blocks = launch_blocks(npoints, kNThreads);
      mark_main_start(st);
      if (dtype == GBG_F64)
        k_nufft_gather<double, W><<<blocks, kNThreads, 0, st>>>(
            make_ngrid<double>(*fine), static_cast<const double *>(field), static_cast<const double *>(positions),
            npoints, ncomp, beta, traversal, static_cast<double *>(out), device_status);
      else
        k_nufft_gather<float, W><<<blocks, kNThreads, 0, st>>>(
            make_ngrid<float>(*fine), static_cast<const float *>(field), static_cast<const float *>(positions),
            npoints, ncomp, (float)beta, traversal, static_cast<float *>(out), device_status);
      mark_main_stop(st);
      note_launch();
      GBG_CUDA_TRY(cudaGetLastError());
      return GBG_OK;
    });
  } catch (...) {
    return set_error(GBG_ENOMEM, "nufft_interp: host exception");
  }
}

gbg_status gbg_nufft_spread_workspace_size(const gbg_grid *fine, int32_t ncomp, size_t *bytes) {
  clear_error();
  GBG_TRY(check_ngrid(fine));
  if (ncomp < 1) return set_error(GBG_EARG, "ncomp must be at least 1");
  if (!bytes) return set_error(GBG_EARG, "null bytes");
  const int64_t n = fine->n[0] * fine->n[1] * fine->n[2] * (int64_t)ncomp;
  *bytes = (size_t)n * 8 + 256;
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
    GBG_TRY(gbg_nufft_spread_workspace_size(fine, ncomp, &need));
    if (!field) return set_error(GBG_EARG, "nufft_spread: null field");
    if (npoints > 0 && (!positions || !quantities)) return set_error(GBG_EARG, "nufft_spread: null array");
    if (!workspace || workspace_bytes < need) return set_error(GBG_ENOMEM, "nufft_spread: workspace too small");
    if ((reinterpret_cast<uintptr_t>(workspace) & 7u) != 0) return set_error(GBG_EARG, "nufft_spread: workspace not 8-byte aligned");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const int64_t n = fine->n[0] * fine->n[1] * fine->n[2] * (int64_t)ncomp;
    unsigned long long *acc = static_cast<unsigned long long *>(workspace);
    unsigned long long *qmax = acc + n;
    GBG_CUDA_TRY(cudaMemsetAsync(workspace, 0, (size_t)n * 8 + 8, st));
    if (npoints > 0) {
      const int64_t nq = npoints * (int64_t)ncomp;
      if (dtype == GBG_F64)
        k_nufft_qmax<double><<<launch_blocks(nq, kNThreads), kNThreads, 0, st>>>(static_cast<const double *>(quantities), nq, qmax);
      else
        k_nufft_qmax<float><<<launch_blocks(nq, kNThreads), kNThreads, 0, st>>>(static_cast<const float *>(quantities), nq, qmax);
      note_launch();
      GBG_CUDA_TRY(cudaGetLastError());
      GBG_TRY(with_width(width, [&](auto wc) -> gbg_status {
        constexpr int W = decltype(wc)::value;
        const int blocks = launch_blocks(npoints, kNThreads);
        mark_main_start(st);
        if (dtype == GBG_F64)
          k_nufft_spread<double, W><<<blocks, kNThreads, 0, st>>>(
              make_ngrid<double>(*fine), static_cast<const double *>(positions), npoints,
              static_cast<const double *>(quantities), ncomp, beta, traversal, qmax, acc, device_status);
        else
          k_nufft_spread<float, W><<<blocks, kNThreads, 0, st>>>(
              make_ngrid<float>(*fine), static_cast<const float *>(positions), npoints,
              static_cast<const float *>(quantities), ncomp, (float)beta, traversal, qmax, acc, device_status);
        mark_main_stop(st);
        note_launch();
        GBG_CUDA_TRY(cudaGetLastError());
        return GBG_OK;
      }));
    }
    if (dtype == GBG_F64)
      k_nufft_finish<double><<<launch_blocks(n, kNThreads), kNThreads, 0, st>>>(acc, n, npoints > 0 ? npoints : 1, qmax,
                                                                               static_cast<double *>(field), device_status);
    else
      k_nufft_finish<float><<<launch_blocks(n, kNThreads), kNThreads, 0, st>>>(acc, n, npoints > 0 ? npoints : 1, qmax,
                                                                              static_cast<float *>(field), device_status);
    note_launch();
    GBG_CUDA_TRY(cudaGetLastError());
    return GBG_OK;
  } catch (...) {
    return set_error(GBG_ENOMEM, "nufft_spread: host exception");
  }
}

}  // extern "C"
