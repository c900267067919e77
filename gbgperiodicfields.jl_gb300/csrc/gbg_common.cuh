// Internal helpers shared by the sm_103a kernels and the C-ABI layer.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <cmath>
#include <cstddef>
#include <string>

#include "gbg_transfer.h"

namespace gbg {

// ------------------------------------------------------------------ errors

// Records a message for gbg_last_error() (thread-local) and returns the status.
gbg_status set_error(gbg_status status, const std::string &message);
void clear_error();

// Counts kernel launches (gbg_kernel_launches); called next to every <<<...>>>.
void note_launch(int n = 1);

// Record the calling thread's timing events (gbg_set_kernel_timing_events), if any, just
// before and just after the main kernel of a transfer, on that kernel's stream.
void mark_main_start(cudaStream_t st);
void mark_main_stop(cudaStream_t st);

#define GBG_CUDA_TRY(expr)                                                                  \
  do {                                                                                      \
    cudaError_t _e = (expr);                                                                \
    if (_e != cudaSuccess)                                                                  \
      return ::gbg::set_error(GBG_ECUDA, std::string(#expr) + ": " + cudaGetErrorString(_e)); \
  } while (0)

#define GBG_TRY(expr)                 \
  do {                                \
    gbg_status _s = (expr);           \
    if (_s != GBG_OK) return _s;      \
  } while (0)

// ------------------------------------------------------------ arithmetic

// Non-contractible multiply/add, so that the weight polynomials are evaluated with the
// same roundings as the reference's Horner loop (Julia never fuses a*b+c).
__device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float mul_rn(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double add_rn(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ float add_rn(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ double fma_rn(double a, double b, double c) { return fma(a, b, c); }
__device__ __forceinline__ float fma_rn(float a, float b, float c) { return fmaf(a, b, c); }

// Julia's integer mod for a positive divisor: the result lies in [0, n).
// x * 2^e rounded to the nearest integer, ties to even, for finite x with |x| 2^e < 2^63:
// the value __double2ll_rn(x * 2^e) has wherever x * 2^e is exact in double (e >= 0, or no
// underflow), formed from the mantissa and exponent bits on the integer pipes instead of a
// product and a conversion on the FP64 pipe.
__device__ __forceinline__ long long fixed_rn(double x, int e) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const int bexp = (int)((b >> 52) & 0x7ffu);
  const unsigned long long mant = (b & 0xfffffffffffffull) | (bexp ? (1ull << 52) : 0ull);
  const int sh = (bexp ? bexp : 1) - 1075 + e;  // x 2^e = mant 2^sh
  unsigned long long r;
  if (sh >= 0) {
    r = mant << sh;
  } else if (sh < -54) {
    r = 0ull;  // below 2^-2
  } else {
    const int rs = -sh;
    const unsigned long long q = mant >> rs, rem = mant & ((1ull << rs) - 1ull), halfway = 1ull << (rs - 1);
    r = q + (unsigned long long)(rem > halfway || (rem == halfway && (q & 1ull)));
  }
  return (b >> 63) ? -(long long)r : (long long)r;
}

// Adds v to a 64-bit integer kept in shared memory as two 32-bit words, lo[i] and hi[i],
// with native 32-bit atomics: the low word's add returns the old value, whose wrap is the
// carry into the high word.  Each add wraps the low word at most once, so after all adds
// the high word holds the sum of the high parts plus floor(sum of low parts / 2^32) in any
// order: the pair is the exact 64-bit sum, as a 64-bit atomic would leave it.
__device__ __forceinline__ void atomic_add_split64(uint32_t *lo, uint32_t *hi, int i, unsigned long long v) {
  const uint32_t vl = (uint32_t)v, vh = (uint32_t)(v >> 32);
  const uint32_t old = atomicAdd(lo + i, vl);
  atomicAdd(hi + i, vh + (uint32_t)(old + vl < vl));
}

__host__ __device__ __forceinline__ int64_t imod(int64_t a, int64_t n) {
  int64_t r = a % n;
  return r < 0 ? r + n : r;
}

// Interpolation.jl:456-460 -- _locate: ci = (x - o) / dx (IEEE division in T),
// base = floor(ci), t = ci - base.  Returns false for a non-finite or huge ci, for which
// floor(Int, ci) throws in the reference.
template <typename T>
__device__ __forceinline__ bool locate(T x, T o, T d, int64_t &base, T &t) {
  const T ci = (x - o) / d;
  const T fl = floor(ci);
  const bool ok = isfinite(ci) && fabs(fl) < T(9.0e18);
  base = ok ? (int64_t)fl : 0;
  t = ci - fl;
  return ok;
}

// A scheme's coefficients converted to T (Interpolation.jl:1360, _coefficients_as),
// sized for NMAX nodes and passed by value as a kernel parameter.
template <typename T, int NMAX>
struct SchemeT {
  T c[NMAX * GBG_MAX_POWERS];  // [q + n2*p]
  int32_t n2;
  int32_t m2;
};

template <typename T, int NMAX>
inline SchemeT<T, NMAX> make_scheme(const gbg_scheme &s) {
  SchemeT<T, NMAX> r;
  r.n2 = s.stencil_width;
  r.m2 = s.num_powers;
  for (int i = 0; i < NMAX * GBG_MAX_POWERS; ++i) r.c[i] = T(0);
  for (int q = 0; q < s.stencil_width; ++q)
    for (int p = 0; p < s.num_powers; ++p)
      r.c[q + s.stencil_width * p] = T(s.coefficients[q + s.stencil_width * p]);
  return r;
}

// Interpolation.jl:440-446 -- Horner from the highest power, w = w*t + c[:, p], with the
// reference's roundings, for a compile-time width N2.  The loop is unrolled over every
// possible power so that the coefficients stay in the parameter bank; powers >= m2 are
// skipped (w starts at 0, and 0*t + c[:, m2-1] = c[:, m2-1] exactly for finite t).
template <typename T, int N2>
__device__ __forceinline__ void axis_weights(const SchemeT<T, N2> &s, T t, T (&w)[N2]) {
#pragma unroll
  for (int q = 0; q < N2; ++q) w[q] = T(0);
#pragma unroll
  for (int p = GBG_MAX_POWERS - 1; p >= 0; --p) {
    if (p < s.m2) {
#pragma unroll
      for (int q = 0; q < N2; ++q) w[q] = add_rn(mul_rn(w[q], t), s.c[q + N2 * p]);
    }
  }
}

// Horner with a compile-time number of powers M2 (M2 == 0: the guarded form above).
template <typename T, int N2, int M2>
__device__ __forceinline__ void axis_weights_m(const SchemeT<T, N2> &s, T t, T (&w)[N2]) {
  if constexpr (M2 > 0) {
#pragma unroll
    for (int q = 0; q < N2; ++q) w[q] = s.c[q + N2 * (M2 - 1)];
#pragma unroll
    for (int p = M2 - 2; p >= 0; --p)
#pragma unroll
      for (int q = 0; q < N2; ++q) w[q] = add_rn(mul_rn(w[q], t), s.c[q + N2 * p]);
  } else {
    axis_weights<T, N2>(s, t, w);
  }
}

// The same for a run-time width, from coefficients staged in shared memory.
template <typename T>
__device__ __forceinline__ void axis_weights_dyn(const T *c, int n2, int m2, T t, T *w) {
#pragma unroll 1
  for (int q = 0; q < n2; ++q) w[q] = c[q + n2 * (m2 - 1)];
#pragma unroll 1
  for (int p = m2 - 2; p >= 0; --p) {
#pragma unroll 1
    for (int q = 0; q < n2; ++q) w[q] = add_rn(mul_rn(w[q], t), c[q + n2 * p]);
  }
}

// Copies a scheme's coefficients into shared memory (run-time-width kernels).
template <typename T, int NMAX>
__device__ __forceinline__ void stage_coeffs(const SchemeT<T, NMAX> &s, T *c) {
  for (int i = threadIdx.x; i < s.n2 * s.m2; i += blockDim.x) c[i] = s.c[i];
  __syncthreads();
}

// Block-wide exclusive scan of n counts in shared memory (n <= 32 * blockDim.x * 8);
// returns the total.  Every thread must call it.
__device__ __forceinline__ uint32_t block_scan_counts(uint32_t *v, int n, uint32_t *warp_tot) {
  const int per = (n + blockDim.x - 1) / blockDim.x;
  const int lo = threadIdx.x * per, hi = min(n, lo + per);
  uint32_t run = 0;
  for (int i = lo; i < hi; ++i) run += v[i];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t x = run;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) warp_tot[warp] = x;
  __syncthreads();
  if (warp == 0) {
    uint32_t t = lane < (int)(blockDim.x >> 5) ? warp_tot[lane] : 0u;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, t, o);
      if (lane >= o) t += y;
    }
    if (lane < (int)(blockDim.x >> 5)) warp_tot[lane] = t;
  }
  __syncthreads();
  uint32_t prefix = (warp ? warp_tot[warp - 1] : 0u) + x - run;
  const uint32_t total = warp_tot[(blockDim.x >> 5) - 1];
  for (int i = lo; i < hi; ++i) {
    const uint32_t c = v[i];
    v[i] = prefix;
    prefix += c;
  }
  __syncthreads();
  return total;
}

// Bound of |w_q(t)| over the nodes q and t in [0, 1] (Bernstein form), plus horner_slack
// times sum_r |c[q, r]| for the rounding of the weight evaluation.  Used to size the
// fixed-point scales of the deterministic scatters.
double weight_bound(const gbg_scheme &sch, double horner_slack);

// ----------------------------------------------------------- workspace

// Carves aligned sub-buffers out of one workspace; with base == nullptr it only sizes.
struct Arena {
  char *base = nullptr;
  size_t used = 0;
  template <typename U>
  U *take(size_t count) {
    used = (used + 255) & ~size_t(255);
    U *p = base ? reinterpret_cast<U *>(base + used) : nullptr;
    used += count * sizeof(U);
    return p;
  }
};

// Stream-ordered scratch: the caller's workspace when given, else cudaMallocAsync.
struct Scratch {
  void *ptr = nullptr;
  bool owned = false;
  cudaStream_t stream = nullptr;
  gbg_status acquire(void *user, size_t user_bytes, size_t need, cudaStream_t s);
  ~Scratch();
};

// ---------------------------------------------------------------- sort

// Exclusive prefix sum of n uint32 values; tmp must hold scan_temp_elems(n) uint32.
size_t scan_temp_elems(int64_t n);
// With gate, every kernel returns at once unless *gate is non-zero (a device-side switch
// that needs no host synchronization).
gbg_status exclusive_scan_u32(const uint32_t *in, uint32_t *out, int64_t n, uint32_t *tmp,
                              cudaStream_t stream, const uint32_t *gate = nullptr);

// Stable LSD radix sort of (key, value) pairs over the low key_bits bits of the keys.
// vals_in == nullptr means the identity 0..n-1.  Results land in keys_out / vals_out;
// keys_in is not modified.  Scratch sizes come from radix_sort_temp_bytes.
size_t radix_sort_temp_bytes(int64_t n);
gbg_status radix_sort_pairs(const uint32_t *keys_in, const uint32_t *vals_in, uint32_t *keys_out,
                            uint32_t *vals_out, int64_t n, int key_bits, void *temp,
                            cudaStream_t stream, const uint32_t *gate = nullptr);

// Stable sort of point indices by key from a counting pass: rank[p] is what an atomic count
// of keys[p] returned and starts[] the exclusive scan of those counts (starts[k+1] -
// starts[k] points per key).  perm[s] = the point in slot s, points of one key in index
// order -- the order the stable radix sort gives.  *big must be zero on entry; a key with
// more than 1024 points sets it and the radix sort (gated on it) redoes the order, writing
// skeys too.  temp holds radix_sort_temp_bytes(n) bytes.  With rec_user and rec given, the
// placement also writes rec[s] = rec_user[perm[s]] (when *big is left zero; the fallback's
// order is then the caller's to gather).
gbg_status stable_counting_sort(const uint32_t *keys, const uint32_t *rank, const uint32_t *starts, int64_t n,
                                int key_bits, uint32_t *perm, uint32_t *skeys, uint32_t *big, void *temp,
                                cudaStream_t stream, const float4 *rec_user = nullptr, float4 *rec = nullptr);

// Grid-stride launch shape: a multiple of the SM count.
int launch_blocks(int64_t work, int threads, int per_sm = 8);

// Bins whose device memory is taken and returned in stream order (cudaMallocAsync /
// cudaFreeAsync on `stream`), for the serving loop: no call here synchronizes the device.
gbg_status bins_create_async(const gbg_grid &grid, int64_t max_points, const int32_t *brick,
                             cudaStream_t stream, gbg_bins *out, size_t *bytes);
gbg_status bins_destroy_async(gbg_bins bins, cudaStream_t stream);
size_t bins_bytes(const gbg_grid &grid, int64_t max_points, const int32_t *brick);

// The grid, component count and widest stencil of a resident field.
gbg_status field_info(gbg_field f, gbg_grid *grid, int32_t *ncomp, int32_t *max_width);

// Batches whose device tables are allocated in stream order and uploaded from the
// caller's pinned staging memory (at least batch_table_bytes(count) bytes, left untouched
// until the copy has run).
size_t batch_table_bytes(int32_t count);
gbg_status batch_create_async(const gbg_batch_item *items, int32_t count, cudaStream_t stream, void *pinned,
                              size_t pinned_bytes, gbg_batch *out);
gbg_status batch_destroy_async(gbg_batch bt, cudaStream_t stream);

}  // namespace gbg
