// Resident field storage, device cell-binned sort, staged gather and deterministic
// scatter (sm_103a, FP32 storage).
//
// Storage: a field of C components is held as float with the components of a node
// adjacent, padded to CP = 4 or 12 (16-byte multiples), and with a periodic ghost layer
// of halo_lo = n and halo_hi = n+1 nodes (n = max_stencil_width/2 - 1) on every axis:
// node (x, y, z) lives at padded (x + n, y + n, z + n).  Every brick of cells plus the
// halo its stencils reach is then one box of the padded array, which one TMA tensor copy
// stages into shared memory.
//
// Bins: each position is split into a cell and a fraction.  For Float64 positions this
// is done in FP64 (the precision form keeps FP64 only here): u = x*(N/L)*2^32 -
// o*(N/L)*2^32 in one FMA, floor to int64, cell = (u >> 32) mod N, fraction = the low 32
// bits.  Points are then stably radix-sorted by (brick, cell within brick).
//
// Gather: one CTA per brick (persistent; the brick's TMA halo tile double-buffered when
// that keeps as many CTAs per SM), a point per quarter-warp: lane (i, jj) owns the
// x-offset i and the y-offsets 2jj, 2jj+1 for all four z-offsets, reads each node's
// components with 128-bit shared loads (the tile's row pitch makes the 8 lanes of a
// quarter-warp hit 8 distinct 16-byte bank groups), and the quarter-warp reduces its
// partial sums with shuffles.
//
// Scatter: output-driven.  A CTA owns a brick's nodes and a thread a 2x2 quad of them; the
// points of the brick's region are staged in shared memory, and each node sums its points
// in a fixed order in registers (no atomics, bitwise reproducible), then is written once.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <type_traits>
#include <vector>

#include "gbg_common.cuh"

struct gbg_field_s {
  int device = 0;
  gbg_grid grid{};
  int32_t ncomp = 0, cp = 0, max_width = 0, halo = 0;  // halo_lo = halo, halo_hi = halo+1
  int64_t px = 0, py = 0, pz = 0;
  float *data = nullptr;
  size_t bytes = 0;
  CUtensorMap tmap[2];  // [0]: box for width-4 stencils, [1]: box for the field's max width
  int tmap_width[2] = {0, 0};
  int32_t tmap_brick[2][3] = {{0, 0, 0}, {0, 0, 0}};
};

struct gbg_bins_s {
  int device = 0;
  gbg_grid grid{};
  int64_t max_points = 0, npoints = 0;
  int32_t b[3] = {11, 8, 8};
  int64_t nb[3] = {0, 0, 0};
  int64_t nbricks = 0, bvol = 0, nkeys = 0;
  uint32_t *keys = nullptr, *skeys = nullptr, *perm = nullptr, *cell_start = nullptr;
  float4 *rec_user = nullptr, *rec = nullptr;
  void *sort_tmp = nullptr;
  uint32_t *scan_tmp = nullptr;
  float *qs = nullptr;  // sorted, alpha-scaled quantities for the scatter (max_points x 12)
  unsigned *qmax_bits = nullptr;  // largest |alpha q| of the last scatter, as float bits
  void *block = nullptr;
  size_t bytes = 0;
  bool async = false;  // block from cudaMallocAsync (serving loop)
  int32_t gather_threads = 0, scatter_threads = 0;  // 0: the defaults (gbg_bins_set_launch)
  int32_t compensated = 1;  // the scatter's compensated summation (gbg_bins_set_compensated)
  int32_t sparse_regions = 1;  // sparse sets: regions from neighbour lists (gbg_bins_set_sparse_regions)
  uint32_t wait_polls = 0;  // the gather's tile-wait limit, 0: the default (gbg_bins_set_wait_limit)
  // work lists rebuilt with the bins: bricks holding a point (gathers), bricks a point's
  // stencil reaches (scatters with beta == 1; valid when reach_ok), and their lengths
  uint32_t *active = nullptr, *reach = nullptr, *lists_n = nullptr;
  uint32_t *overflow = nullptr;  // the sparse scatter's bricks with too many candidates (count in lists_n[3])
  bool reach_ok = false;
  // corrections of the compensated scatter's regions of several chunks: one slot of
  // bvol * 12 floats per scatter CTA; the scatter launches at most cslots CTAs
  float *cscratch = nullptr;
  int32_t cslots = 1;
};

namespace gbg {
// The arrays of a bins' device block, in order; with a.base == nullptr this only sizes.
inline void bins_layout(Arena &a, gbg_bins_s *b) {
  const int64_t m = b->max_points > 0 ? b->max_points : 1;
  b->keys = a.take<uint32_t>(m);
  b->skeys = a.take<uint32_t>(m);
  b->perm = a.take<uint32_t>(m);
  b->cell_start = a.take<uint32_t>((size_t)b->nkeys + 1);
  b->rec_user = a.take<float4>(m);
  b->rec = a.take<float4>(m);
  b->sort_tmp = a.take<char>(radix_sort_temp_bytes(m));
  b->scan_tmp = a.take<uint32_t>(scan_temp_elems(b->nkeys + 1));
  b->qs = a.take<float>((size_t)m * 12);
  b->qmax_bits = a.take<unsigned>(64);
  b->active = a.take<uint32_t>((size_t)b->nbricks);
  b->reach = a.take<uint32_t>((size_t)b->nbricks);
  b->lists_n = a.take<uint32_t>(4);
  b->overflow = a.take<uint32_t>((size_t)b->nbricks);
  b->cscratch = a.take<float>((size_t)b->cslots * b->bvol * 12);
}
}  // namespace gbg

namespace gbg {
namespace {

constexpr int kThreads = 256;

// Side streams of the library, per device: independent instances of a batch and of a
// batched bins build run on them at the same time, forked from the caller's stream by an
// event and joined back by one event per side stream -- inside a stream capture this
// records parallel branches of the graph.  They are made by gbg_bins_create and
// gbg_batch_create (never inside a capture); the mutex keeps one fork/join at a time.
constexpr int kSideStreams = 8;
struct SidePool {
  cudaStream_t s[kSideStreams];
  cudaEvent_t fork, join[kSideStreams];
  bool ready = false;
};
std::mutex g_side_mu;
SidePool g_side[64];

gbg_status side_pool_ready() {
  int dev = 0;
  GBG_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) return set_error(GBG_EUNSUPPORTED, "device ordinal above 63");
  std::lock_guard<std::mutex> lock(g_side_mu);
  SidePool &p = g_side[dev];
  if (p.ready) return GBG_OK;
  GBG_CUDA_TRY(cudaEventCreateWithFlags(&p.fork, cudaEventDisableTiming));
  for (int i = 0; i < kSideStreams; ++i) {
    GBG_CUDA_TRY(cudaStreamCreateWithFlags(&p.s[i], cudaStreamNonBlocking));
    GBG_CUDA_TRY(cudaEventCreateWithFlags(&p.join[i], cudaEventDisableTiming));
  }
  p.ready = true;
  return GBG_OK;
}

// The caller's stream forked over k side streams: side(i, stream) enqueues side stream i's
// work and then main_work() the caller's stream's own, which overlaps it; every side
// stream is then joined back.
template <typename F, typename G>
gbg_status side_run(cudaStream_t main, int k, F &&side, G &&main_work) {
  int dev = 0;
  GBG_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64 || !g_side[dev].ready)
    return set_error(GBG_EARG, "side streams not made on this device (gbg_bins_create or gbg_batch_create makes them)");
  std::lock_guard<std::mutex> lock(g_side_mu);
  SidePool &p = g_side[dev];
  k = std::max(1, std::min(k, kSideStreams));
  GBG_CUDA_TRY(cudaEventRecord(p.fork, main));
  for (int i = 0; i < k; ++i) GBG_CUDA_TRY(cudaStreamWaitEvent(p.s[i], p.fork, 0));
  gbg_status st = GBG_OK;
  for (int i = 0; i < k && st == GBG_OK; ++i) st = side(i, p.s[i]);
  if (st == GBG_OK) st = main_work();
  for (int i = 0; i < k; ++i) {
    GBG_CUDA_TRY(cudaEventRecord(p.join[i], p.s[i]));
    GBG_CUDA_TRY(cudaStreamWaitEvent(main, p.join[i], 0));
  }
  return st;
}
// scatter CTAs per SM that a launch may use at most: each owns a slot of the compensated
// scatter's correction scratch
constexpr int kScatterSlotsPerSM = 4;

int device_sms() {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) cudaGetLastError();
  return sms > 0 ? sms : 1;
}

int padded_components(int ncomp) { return ncomp <= 4 ? 4 : 12; }

// ------------------------------------------------------------ storage

__global__ void k_import(float *__restrict__ dst, int cp, int ncomp, int64_t px, int64_t py,
                         int64_t pz, int halo, int64_t nx, int64_t ny, int64_t nz,
                         const void *__restrict__ src, int src_f64) {
  const int64_t total = px * py * pz;
  const int64_t npf = nx * ny * nz;
  for (int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; n < total;
       n += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = n % px, j = (n / px) % py, k = n / (px * py);
    const int64_t x = imod(i - halo, nx), y = imod(j - halo, ny), z = imod(k - halo, nz);
    const int64_t s = x + nx * (y + ny * z);
    float *d = dst + n * cp;
    for (int c = 0; c < cp; ++c) {
      float v = 0.0f;
      if (c < ncomp)
        v = src_f64 ? (float)static_cast<const double *>(src)[s + npf * c]
                    : static_cast<const float *>(src)[s + npf * c];
      d[c] = v;
    }
  }
}

__global__ void k_export(const float *__restrict__ srcp, int cp, int ncomp, int64_t px,
                         int64_t py, int halo, int64_t nx, int64_t ny, int64_t nz, void *dst,
                         int dst_f64) {
  const int64_t npf = nx * ny * nz;
  for (int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; s < npf;
       s += (int64_t)gridDim.x * blockDim.x) {
    const int64_t x = s % nx, y = (s / nx) % ny, z = s / (nx * ny);
    const float *p = srcp + ((x + halo) + px * ((y + halo) + py * (z + halo))) * cp;
    for (int c = 0; c < ncomp; ++c) {
      if (dst_f64)
        static_cast<double *>(dst)[s + npf * c] = (double)p[c];
      else
        static_cast<float *>(dst)[s + npf * c] = p[c];
    }
  }
}

// Copies interior nodes into the ghost layer (after a scatter wrote the interior).
// Refreshes the periodic ghost layer from the interior.  Only the ghost nodes are
// visited: the ghost z-planes (whole padded planes), then the ghost y-rows of the
// interior planes, then the ghost x-runs of the interior rows -- about 3 * (2n+1) / N of
// the storage instead of all of it.  Every ghost copies an interior node, so the order
// of the copies does not matter.
__global__ void k_fill_ghosts(float *__restrict__ d, int cp, int64_t px, int64_t py, int64_t pz,
                              int halo, int64_t nx, int64_t ny, int64_t nz) {
  const int64_t gz = pz - nz, gy = py - ny, gx = px - nx;
  const int64_t zs = px * py * gz, ys = px * gy * nz, xs = gx * ny * nz;
  const int64_t total = zs + ys + xs;
  for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < total;
       g += (int64_t)gridDim.x * blockDim.x) {
    int64_t i, j, k;
    if (g < zs) {
      i = g % px;
      const int64_t r = g / px;
      j = r % py;
      const int64_t kk = r / py;
      k = kk < halo ? kk : kk + nz;
    } else if (g < zs + ys) {
      const int64_t h = g - zs;
      i = h % px;
      const int64_t r = h / px, jj = r % gy;
      j = jj < halo ? jj : jj + ny;
      k = r / gy + halo;
    } else {
      const int64_t h = g - zs - ys, ii = h % gx, r = h / gx;
      i = ii < halo ? ii : ii + nx;
      j = r % ny + halo;
      k = r / ny + halo;
    }
    const int64_t x = imod(i - halo, nx) + halo, y = imod(j - halo, ny) + halo,
                  z = imod(k - halo, nz) + halo;
    const float4 *src = reinterpret_cast<const float4 *>(d + (x + px * (y + py * z)) * cp);
    float4 *dst = reinterpret_cast<float4 *>(d + (i + px * (j + py * k)) * cp);
    for (int c = 0; c < cp / 4; ++c) dst[c] = src[c];
  }
}

// Threads for k_fill_ghosts: one per ghost node.
inline int64_t ghost_count(int64_t px, int64_t py, int64_t pz, int64_t nx, int64_t ny, int64_t nz) {
  return px * py * (pz - nz) + px * (py - ny) * nz + (px - nx) * ny * nz;
}

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  if (!fn) {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPoint("cuTensorMapEncodeTiled", &p, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  }
  return fn;
}

// A TMA map over the padded storage whose box is one brick's halo tile for a stencil
// of `width` nodes: (CP, bx+width-1, by+width-1, bz+width-1).
gbg_status tensor_map_for(gbg_field_s *f, int width, const int32_t brick[3], CUtensorMap **out) {
  for (int s = 0; s < 2; ++s)
    if (f->tmap_width[s] == width && f->tmap_brick[s][0] == brick[0] && f->tmap_brick[s][1] == brick[1] &&
        f->tmap_brick[s][2] == brick[2]) {
      *out = &f->tmap[s];
      return GBG_OK;
    }
  auto enc = encode_fn();
  if (!enc) return set_error(GBG_ECUDA, "cuTensorMapEncodeTiled is not available from the driver");
  const int slot = width == 4 ? 0 : 1;
  cuuint64_t dims[4] = {(cuuint64_t)f->cp, (cuuint64_t)f->px, (cuuint64_t)f->py, (cuuint64_t)f->pz};
  cuuint64_t strides[3] = {(cuuint64_t)f->cp * 4, (cuuint64_t)f->cp * 4 * f->px,
                           (cuuint64_t)f->cp * 4 * f->px * f->py};
  cuuint32_t box[4] = {(cuuint32_t)f->cp, (cuuint32_t)(brick[0] + width - 1),
                       (cuuint32_t)(brick[1] + width - 1), (cuuint32_t)(brick[2] + width - 1)};
  cuuint32_t estr[4] = {1, 1, 1, 1};
  for (int d = 1; d < 4; ++d)
    if (box[d] > 256) return set_error(GBG_EUNSUPPORTED, "brick halo tile wider than 256 nodes");
  CUresult r = enc(&f->tmap[slot], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, f->data, dims, strides, box, estr,
                   CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                   CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return set_error(GBG_ECUDA, "cuTensorMapEncodeTiled failed: " + std::to_string((int)r));
  f->tmap_width[slot] = width;
  for (int d = 0; d < 3; ++d) f->tmap_brick[slot][d] = brick[d];
  *out = &f->tmap[slot];
  return GBG_OK;
}

// --------------------------------------------------------------- bins

struct BinGeom {
  int64_t n[3];
  int32_t b[3];
  int64_t nb[3];
  int64_t bvol;
  double scale[3], shift[3];  // FP64: u * 2^32 = x * scale + shift
  float o32[3], d32[3];       // Float32 positions: the reference's _locate in T
};

// floor(u) of a double with |u| < 9.2e18, from its bits by integer instructions (GB300
// runs FP64 compares and conversions at the FP64 rate, a few per clock per SM); ok is
// false for NaN, infinities and |u| >= 9.2e18, and the result is then 0.
__device__ __forceinline__ long long floor_bits(double u, bool &ok) {
  const unsigned long long bits = (unsigned long long)__double_as_longlong(u);
  const unsigned long long a = bits & 0x7FFFFFFFFFFFFFFFull;
  ok = a < 0x43DFEB3DD0676600ull;  // the bits of 9.2e18 (positive doubles order as integers)
  const int ex = (int)(a >> 52);
  const unsigned long long man = (a & 0xFFFFFFFFFFFFFull) | (ex ? 0x10000000000000ull : 0ull);
  const int sh = 1075 - ex;  // |u| = man * 2^-sh
  unsigned long long ip, fr;
  if (sh <= 0) {
    ip = man << (-sh < 11 ? -sh : 0);
    fr = 0;
  } else if (sh >= 64) {
    ip = 0;
    fr = man;
  } else {
    ip = man >> sh;
    fr = man & ((1ull << sh) - 1);
  }
  long long v = (long long)ip;
  if (bits >> 63) v = -v - (fr != 0 ? 1 : 0);
  return ok ? v : 0;
}

// Splits one FP64 coordinate into (cell, fraction) in FP64 fixed point.
__device__ __forceinline__ bool split64(double x, double scale, double shift, int64_t n,
                                        int64_t &cell, float &t) {
  const double u = fma(x, scale, shift);
  bool ok;
  const long long v = floor_bits(u, ok);
  // |u| < 2^63, so the cell word fits 32 bits, and so does n: the periodic wrap in 32-bit
  // arithmetic (a 64-bit remainder costs several times more)
  int32_t r = (int32_t)(v >> 32) % (int32_t)n;
  cell = r < 0 ? r + n : r;
  t = ok ? __uint2float_rz((unsigned)(v & 0xffffffffLL)) * 0x1p-32f : __int_as_float(0x7fc00000);
  return ok;
}

__device__ __forceinline__ bool split32(float x, float o, float d, int64_t n, int64_t &cell, float &t) {
  int64_t base;
  float tt;
  const bool ok = locate(x, o, d, base, tt);
  cell = base >= INT32_MIN && base <= INT32_MAX ? (int64_t)((int32_t)base % (int32_t)n) : imod(base, n);
  if (cell < 0) cell += n;
  t = ok ? tt : __int_as_float(0x7fc00000);
  return ok;
}

// ------------------------------------------------------------ displacement
//
// Points.jl:1217-1231, 1382-1490 -- displace!(dst, src, [grid,] (c_1, v_1), ...): per
// coordinate dst = ((src + c_1 v_1) + c_2 v_2) + ..., every product and sum rounded in the
// positions' type (the reference's broadcast fuses no multiply-add), then, on the torus,
// _wrap_coordinate (Points.jl:1245-1249).

template <typename T>
struct DisplaceArgs {
  const T *src;
  T *dst;
  const T *sec[GBG_MAX_TERMS];
  T coef[GBG_MAX_TERMS];
  int32_t nterms, wrap;
  T extent[3], origin[3];
};

// Julia's floating-point mod (rem, then the sign moved toward the divisor).
template <typename T>
__device__ __forceinline__ T jl_mod(T x, T y) {
  const T r = fmod(x, y);
  if (r == T(0)) return copysign(r, y);
  if ((r > T(0)) != (y > T(0))) return r + y;
  return r;
}

// The excluded endpoint is folded by an equality test, so a non-finite coordinate stays
// non-finite (an infinity becomes NaN, mod's own image of it).
template <typename T>
__device__ __forceinline__ T wrap_coordinate(T x, T extent, T origin) {
  T off = jl_mod(x - origin, extent);
  off = off == extent ? T(0) : off;
  return off + origin;
}

template <typename T>
__device__ __forceinline__ T displaced(const DisplaceArgs<T> &a, int64_t i, int d) {
  T x = a.src[i];
  for (int j = 0; j < a.nterms; ++j) x = add_rn(x, mul_rn(a.coef[j], a.sec[j][i]));
  return a.wrap ? wrap_coordinate(x, a.extent[d], a.origin[d]) : x;
}

template <typename T>
__global__ void __launch_bounds__(kThreads) k_displace(DisplaceArgs<T> a, int64_t m) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < 3 * m; i += (int64_t)gridDim.x * blockDim.x)
    a.dst[i] = displaced(a, i, (int)(i / m));
}

// dst[s + m*c] = src[perm[s] + m*c]: an (m, ncols) column-major array in binned order.
template <typename T>
__global__ void __launch_bounds__(kThreads)
    k_permute(const T *__restrict__ src, T *__restrict__ dst, const uint32_t *__restrict__ perm, int64_t m, int ncols) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m * ncols; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t c = i / m, s = i - c * m;
    dst[i] = src[__ldg(perm + s) + m * c];
  }
}

// A point record's fourth word: the point's cell within its brick as packed coordinates
// (brick edges are at most 64 cells), so readers take it apart with shifts.
__device__ __forceinline__ uint32_t pack_local(uint32_t lx, uint32_t ly, uint32_t lz) {
  return lx | (ly << 8) | (lz << 16);
}
__device__ __forceinline__ void unpack_local(float w, int &lx, int &ly, int &lz) {
  const uint32_t loc = __float_as_uint(w);
  lx = (int)(loc & 0xffu);
  ly = (int)((loc >> 8) & 0xffu);
  lz = (int)(loc >> 16);
}

// Keys, counts (each point keeps the count its atomic returned, its rank within the key
// in no particular order) and per-point records of the bins; with DISP the positions are first
// displaced (and wrapped) from `disp`, written to disp.dst, and binned in the same pass.
template <typename T, bool DISP = false>
__global__ void __launch_bounds__(kThreads)
    k_bin_keys(BinGeom g, const T *__restrict__ pos, int64_t m, uint32_t *__restrict__ keys,
               uint32_t *__restrict__ counts, uint32_t *__restrict__ rank, float4 *__restrict__ rec_user,
               int32_t *status, DisplaceArgs<T> disp = {}) {
  for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < m;
       p += (int64_t)gridDim.x * blockDim.x) {
    int64_t c[3];
    float t[3];
    bool ok = true;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      T x;
      if constexpr (DISP) {
        x = displaced(disp, p + m * d, d);
        disp.dst[p + m * d] = x;
      } else {
        x = pos[p + m * d];
      }
      if constexpr (sizeof(T) == 8)
        ok &= split64((double)x, g.scale[d], g.shift[d], g.n[d], c[d], t[d]);
      else
        ok &= split32((float)x, g.o32[d], g.d32[d], g.n[d], c[d], t[d]);
    }
    if (!ok && status) atomicOr(status, GBG_DEV_NONFINITE);
    // cells, bricks and keys all fit 32 bits (bins hold fewer than 2^32 cells)
    const uint32_t bx = (uint32_t)c[0] / (uint32_t)g.b[0], by = (uint32_t)c[1] / (uint32_t)g.b[1],
                   bz = (uint32_t)c[2] / (uint32_t)g.b[2];
    const uint32_t lx = (uint32_t)c[0] - bx * (uint32_t)g.b[0], ly = (uint32_t)c[1] - by * (uint32_t)g.b[1],
                   lz = (uint32_t)c[2] - bz * (uint32_t)g.b[2];
    const uint32_t local = (lz * (uint32_t)g.b[1] + ly) * (uint32_t)g.b[0] + lx;
    const uint32_t key = ((bz * (uint32_t)g.nb[1] + by) * (uint32_t)g.nb[0] + bx) * (uint32_t)g.bvol + local;
    keys[p] = key;
    rank[p] = atomicAdd(counts + key, 1u);
    rec_user[p] = make_float4(t[0], t[1], t[2], __uint_as_float(pack_local(lx, ly, lz)));
  }
}

// The bins' work lists: bricks holding a point, and bricks whose 27 neighbours (periodic)
// hold one -- the bricks a stencil of up to 8 nodes can reach when every brick (and the
// last, partial one) is at least 4 cells wide (reach_ok).  Their order is whatever the
// atomics give: each list only says which bricks to visit.
__global__ void k_brick_lists(const uint32_t *__restrict__ cell_start, int64_t nbx, int64_t nby, int64_t nbz,
                              int64_t bvol, int reach_ok, uint32_t *__restrict__ active,
                              uint32_t *__restrict__ reach, uint32_t *__restrict__ lists_n) {
  const int64_t nbricks = nbx * nby * nbz;
  auto holds = [&](int64_t b) { return __ldg(cell_start + (b + 1) * bvol) > __ldg(cell_start + b * bvol); };
  for (int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; b < nbricks; b += (int64_t)gridDim.x * blockDim.x) {
    if (holds(b)) active[atomicAdd(lists_n, 1u)] = (uint32_t)b;
    if (!reach_ok) continue;
    const int64_t bx = b % nbx, by = (b / nbx) % nby, bz = b / (nbx * nby);
    bool near = false;
    for (int d = 0; d < 27 && !near; ++d) {
      const int64_t x = (bx + d % 3 - 1 + nbx) % nbx, y = (by + (d / 3) % 3 - 1 + nby) % nby,
                    z = (bz + d / 9 - 1 + nbz) % nbz;
      near = holds((z * nby + y) * nbx + x);
    }
    if (near) reach[atomicAdd(lists_n + 1, 1u)] = (uint32_t)b;
  }
}

__global__ void k_gather_records(const float4 *__restrict__ rec_user, const uint32_t *__restrict__ perm,
                                 int64_t m, float4 *__restrict__ rec, const uint32_t *gate = nullptr) {
  if (gate && __ldg(gate) == 0u) return;  // the stable placement wrote the records
  // four slots a trip: their indices, then their records, then the stores
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; s < m; s += 4 * stride) {
    uint32_t p[4];
    float4 r[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) p[u] = s + u * stride < m ? __ldg(perm + s + u * stride) : 0u;
#pragma unroll
    for (int u = 0; u < 4; ++u) r[u] = s + u * stride < m ? __ldg(rec_user + p[u]) : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
    for (int u = 0; u < 4; ++u)
      if (s + u * stride < m) rec[s + u * stride] = r[u];
  }
}

__global__ void k_order_from_perm(const uint32_t *__restrict__ perm, int32_t *__restrict__ order, int64_t m) {
  for (int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; s < m;
       s += (int64_t)gridDim.x * blockDim.x)
    order[s] = (int32_t)perm[s] + 1;
}

// ------------------------------------------------------------- staged gather

struct StagedGeo {
  int32_t b[3];
  int64_t nb[3];
  int32_t w[3];  // tile = brick + width - 1
  int32_t box_off;  // halo - n: padded coordinate of a brick's first tile node, less b*brick
  int64_t nbricks, bvol, m;
  int32_t ncomp;
  uint32_t wait_polls;  // polls of a tile's mbarrier before the wait gives up (kWaitPolls by default)
};

__device__ __forceinline__ uint32_t smem_addr(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
               : "memory");
}

// Bounded wait on a phase of an mbarrier; false if it did not complete within `polls`
// tries.  A try of the default limit (kWaitPolls) is mbarrier.try_wait, which may suspend
// the thread for a while before it answers; below the default every try is the
// non-blocking mbarrier.test_wait, so that a small limit gives up after about that many
// polls.  The waits on a tile use the launch's limit; the drain of copies still in flight
// after a wait gave up always uses the full kWaitPolls, so no copy outlives the CTA.
constexpr uint32_t kWaitPolls = 1u << 22;
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity, uint32_t polls = kWaitPolls) {
  const uint32_t a = smem_addr(bar);
  const bool block = polls >= kWaitPolls;
  for (uint32_t iter = 0; iter < polls; ++iter) {
    uint32_t done;
    if (block)
      asm volatile(
          "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
          : "=r"(done)
          : "r"(a), "r"(parity)
          : "memory");
    else
      asm volatile(
          "{\n .reg .pred p;\n mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
          : "=r"(done)
          : "r"(a), "r"(parity)
          : "memory");
    if (done) return true;
  }
  return false;
}

__device__ __forceinline__ void tma_load_tile(void *dst, const CUtensorMap *map, int c0, int c1, int c2,
                                              int c3, uint64_t *bar) {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  asm volatile(
      "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, "
      "%4, %5}], [%6];" ::"r"(smem_addr(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(smem_addr(bar))
      : "memory");
}

// All N2 weights at t by Horner (Interpolation.jl:440-446) in FP32.  With a compile-time
// number of powers M2 every coefficient index is a constant (the coefficients stay in the
// parameter bank); M2 == 0 is the guarded fallback for unusual schemes.
template <int N2, int M2>
__device__ __forceinline__ void weights_all(const SchemeT<float, N2> &s, float t, float (&w)[N2]) {
  if constexpr (M2 > 0) {
#pragma unroll
    for (int q = 0; q < N2; ++q) w[q] = s.c[q + N2 * (M2 - 1)];
#pragma unroll
    for (int p = M2 - 2; p >= 0; --p)
#pragma unroll
      for (int q = 0; q < N2; ++q) w[q] = fmaf(w[q], t, s.c[q + N2 * p]);
  } else {
#pragma unroll
    for (int q = 0; q < N2; ++q) w[q] = 0.0f;
#pragma unroll
    for (int p = GBG_MAX_POWERS - 1; p >= 0; --p)
      if (p < s.m2)
#pragma unroll
        for (int q = 0; q < N2; ++q) w[q] = fmaf(w[q], t, s.c[q + N2 * p]);
  }
}

template <int N>
__device__ __forceinline__ float pick(const float (&w)[N], int q) {
  float v = w[0];
#pragma unroll
  for (int i = 1; i < N; ++i)
    if (i == q) v = w[i];
  return v;
}

// Horner for one node q of a compile-time-width scheme (Interpolation.jl:440-446), in FP32.
template <int N2>
__device__ __forceinline__ float poly(const SchemeT<float, N2> &s, int q, float t) {
  float w = 0.0f;
#pragma unroll
  for (int p = GBG_MAX_POWERS - 1; p >= 0; --p) {
    if (p < s.m2) {
      float c = s.c[p * N2];
#pragma unroll
      for (int qq = 1; qq < N2; ++qq)
        if (qq == q) c = s.c[qq + N2 * p];
      w = fmaf(w, t, c);
    }
  }
  return w;
}

template <typename TO>
__device__ __forceinline__ void store_out(TO *out, int64_t idx, float v) { out[idx] = (TO)v; }

// The brick a CTA iteration handles, and whether it holds any point.
__device__ __forceinline__ void brick_coords(const StagedGeo &g, int64_t b, int64_t &bx, int64_t &by, int64_t &bz) {
  bx = b % g.nb[0];
  by = (b / g.nb[0]) % g.nb[1];
  bz = b / (g.nb[0] * g.nb[1]);
}

// One point of a width-4 gather by its quarter-warp: this lane's x node qi and y nodes
// 2jj, 2jj+1 over all four z nodes, then a reduce-scatter of the CP sums over the eight
// lanes.  The nodes are base[(origin + x + y*sy + z*sz) * CP] at stencil-relative
// x, y, z: a brick's tile in shared memory (origin 0) or the field itself; both give the
// same bits.
template <int M2, int CP, typename TO, typename I>
__device__ __forceinline__ void gather4_point(const SchemeT<float, 4> &s, const float (&cx)[M2 > 0 ? M2 : 1],
                                              const float (&cya)[M2 > 0 ? M2 : 1], const float (&cyb)[M2 > 0 ? M2 : 1],
                                              int qi, int jj, int sub, unsigned seg_mask, float4 r, int64_t pt,
                                              const float *base, I sy, I sz, I origin, TO *out, int64_t m, int ncomp) {
  int lx, ly, lz;
  unpack_local(r.w, lx, ly, lz);
  float w1, w2a, w2b, w3[4];
  if constexpr (M2 > 0) {
    // only the weights this lane uses: its x node, its two y nodes, all four z nodes
    w1 = cx[M2 - 1];
    w2a = cya[M2 - 1];
    w2b = cyb[M2 - 1];
#pragma unroll
    for (int p = M2 - 2; p >= 0; --p) {
      w1 = fmaf(w1, r.x, cx[p]);
      w2a = fmaf(w2a, r.y, cya[p]);
      w2b = fmaf(w2b, r.y, cyb[p]);
    }
    weights_all<4, M2>(s, r.z, w3);
  } else {
    float wx[4], wy[4];
    weights_all<4, M2>(s, r.x, wx);
    weights_all<4, M2>(s, r.y, wy);
    weights_all<4, M2>(s, r.z, w3);
    w1 = pick(wx, qi);
    w2a = pick(wy, 2 * jj);
    w2b = pick(wy, 2 * jj + 1);
  }
  float acc[CP];
#pragma unroll
  for (int c = 0; c < CP; ++c) acc[c] = 0.0f;
  const I node0 = origin + lz * sz + (ly + 2 * jj) * sy + lx + qi;
#pragma unroll
  for (int k = 0; k < 4; ++k) {
#pragma unroll
    for (int jp = 0; jp < 2; ++jp) {
      const float w = w1 * (jp ? w2b : w2a) * w3[k];
      const float4 *p = reinterpret_cast<const float4 *>(base + (node0 + k * sz + jp * sy) * CP);
#pragma unroll
      for (int q4 = 0; q4 < CP / 4; ++q4) {
        const float4 v = p[q4];
        acc[4 * q4 + 0] = fmaf(w, v.x, acc[4 * q4 + 0]);
        acc[4 * q4 + 1] = fmaf(w, v.y, acc[4 * q4 + 1]);
        acc[4 * q4 + 2] = fmaf(w, v.z, acc[4 * q4 + 2]);
        acc[4 * q4 + 3] = fmaf(w, v.w, acc[4 * q4 + 3]);
      }
    }
  }
  // reduce-scatter over the 8 lanes: halves by lane bit 2, then bit 1, then sum bit 0
  constexpr int H = CP / 2, Q = CP / 4;
  const bool up2 = sub & 4, up1 = sub & 2;
  float h[H];
#pragma unroll
  for (int v = 0; v < H; ++v) {
    const float keep = up2 ? acc[H + v] : acc[v];
    const float give = up2 ? acc[v] : acc[H + v];
    h[v] = keep + __shfl_xor_sync(seg_mask, give, 4, 8);
  }
  float qv[Q];
#pragma unroll
  for (int v = 0; v < Q; ++v) {
    const float keep = up1 ? h[Q + v] : h[v];
    const float give = up1 ? h[v] : h[Q + v];
    qv[v] = keep + __shfl_xor_sync(seg_mask, give, 2, 8);
  }
#pragma unroll
  for (int v = 0; v < Q; ++v) qv[v] += __shfl_xor_sync(seg_mask, qv[v], 1, 8);
  if ((sub & 1) == 0) {
    const int cbase = (up2 ? H : 0) + (up1 ? Q : 0);
#pragma unroll
    for (int v = 0; v < Q; ++v)
      if (cbase + v < ncomp) store_out(out, pt + m * (cbase + v), qv[v]);
  }
}

// Gather: width-4 stencils, a point per quarter-warp, 512 threads (64 quarter-warps) per
// CTA; each quarter-warp loads its next point's record and index while it computes.  With
// two tile buffers the warps run free of CTA barriers (the warp that releases a buffer last
// refills it); with one (a large tile, two CTAs per SM) the CTA waits at each brick.
constexpr int kGatherThreads = 512;
template <int M2, int CP, typename TO>
__global__ void __launch_bounds__(kGatherThreads, 1)
    k_gather_staged4(const __grid_constant__ CUtensorMap tmap, StagedGeo g, SchemeT<float, 4> s,
                     const uint32_t *__restrict__ cell_start, const float4 *__restrict__ rec,
                     const uint32_t *__restrict__ perm, TO *__restrict__ out, int32_t *status, int nbuf,
                     uint32_t tile_bytes, uint32_t box_bytes, const uint32_t *__restrict__ list,
                     const uint32_t *__restrict__ list_n) {
  extern __shared__ __align__(1024) unsigned char smem[];
  uint64_t *bars = reinterpret_cast<uint64_t *>(smem + nbuf * tile_bytes);
  if (threadIdx.x == 0) {
    for (int i = 0; i < nbuf; ++i) mbar_init(bars + i, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const int sub = lane & 7;
  const int qi = sub & 3, jj = sub >> 2;
  const unsigned seg_mask = 0xFFu << (lane & ~7);
  const int qw = threadIdx.x >> 3;  // quarter-warp id within the CTA
  // this lane's coefficient columns (x node qi, y nodes 2jj and 2jj+1), fixed for the launch
  float cx[M2 > 0 ? M2 : 1], cya[M2 > 0 ? M2 : 1], cyb[M2 > 0 ? M2 : 1];
  if constexpr (M2 > 0) {
#pragma unroll
    for (int p = 0; p < M2; ++p) {
      cx[p] = s.c[qi + 4 * p];
      cya[p] = s.c[2 * jj + 4 * p];
      cyb[p] = s.c[2 * jj + 1 + 4 * p];
    }
  }
  const int nqw = (int)blockDim.x / 8;
  uint32_t phase[2] = {0, 0};
  bool failed = false;

  bool pending[2] = {false, false};  // thread 0's copies issued and not yet waited for
  auto issue = [&](int64_t b, int buf) {
    int64_t bx, by, bz;
    brick_coords(g, b, bx, by, bz);
    pending[buf] = true;
    mbar_expect_tx(bars + buf, box_bytes);
    tma_load_tile(smem + buf * tile_bytes, &tmap, 0, (int)(bx * g.b[0]) + g.box_off,
                  (int)(by * g.b[1]) + g.box_off, (int)(bz * g.b[2]) + g.box_off, bars + buf);
  };
  // the bricks to visit: the bins' list of bricks holding points, or every brick
  const int64_t nunits = list ? (int64_t)__ldg(list_n) : g.nbricks;
  auto unit = [&](int64_t i) -> int64_t { return i >= nunits ? -1 : (list ? (int64_t)__ldg(list + i) : i); };
  if (nbuf == 2) {
    // Two tile buffers and no CTA barrier between bricks: every warp waits for each
    // non-empty brick's tile in turn (so it follows every phase of both mbarriers), takes its
    // quarter-warps' points, and releases the buffer through a shared counter; the warp that
    // releases it last issues the copy of the brick after next into it.  Warps drift across
    // brick boundaries instead of waiting for the slowest one at each.
    __shared__ uint32_t s_rel[2], s_nissue[2], s_fail;
    const uint32_t nwarps = blockDim.x >> 5;
    // the CTA's first non-empty unit at or after i (units i, i + gridDim.x, ...), or nunits
    auto next_unit = [&](int64_t i, uint32_t &a, uint32_t &z) -> int64_t {
      for (; i < nunits; i += gridDim.x) {
        const int64_t b = unit(i);
        a = __ldg(cell_start + b * g.bvol);
        z = __ldg(cell_start + (b + 1) * g.bvol);
        if (z > a) return i;
      }
      a = z = 0u;
      return nunits;
    };
    uint32_t a0 = 0, z0 = 0, a1 = 0, z1 = 0;
    int64_t cur = next_unit(blockIdx.x, a0, z0);
    int64_t nx = cur < nunits ? next_unit(cur + gridDim.x, a1, z1) : nunits;
    if (threadIdx.x == 0) {
      s_rel[0] = s_rel[1] = 0u;
      s_nissue[0] = s_nissue[1] = 0u;
      s_fail = 0u;
      if (cur < nunits) {
        issue(unit(cur), 0);
        s_nissue[0] = 1u;
      }
      if (nx < nunits) {
        issue(unit(nx), 1);
        s_nissue[1] = 1u;
      }
    }
    __syncthreads();
    float4 r_next = make_float4(0.f, 0.f, 0.f, 0.f);
    uint32_t p_next = 0u;
    if (a0 + qw < z0) {
      r_next = __ldg(rec + a0 + qw);
      p_next = __ldg(perm + a0 + qw);
    }
    uint32_t ph[2] = {0u, 0u};
    for (int j = 0; cur < nunits; ++j) {
      const int buf = j & 1;
      uint32_t a2 = 0, z2 = 0;
      const int64_t nx2 = nx < nunits ? next_unit(nx + gridDim.x, a2, z2) : nunits;
      // a warp that gave up stops the others at their next brick; the outcome of the bounded
      // wait is voted so the warp takes one exit
      bool stop = *(volatile uint32_t *)&s_fail != 0u;
      if (!stop) stop = !mbar_wait(bars + buf, ph[buf], g.wait_polls);
      if (__any_sync(0xffffffffu, stop)) {
        if (lane == 0) {
          s_fail = 1u;
          if (status) atomicOr(status, GBG_DEV_TIMEOUT);
        }
        break;
      }
      ph[buf] ^= 1u;
      bool ahead = false;  // this quarter-warp's first record of the next brick is loading
      for (uint32_t sl = a0 + qw; sl < z0; sl += nqw) {
        const float4 r = r_next;
        const int64_t p = p_next;
        if (sl + nqw < z0) {
          r_next = __ldg(rec + sl + nqw);
          p_next = __ldg(perm + sl + nqw);
        } else if (a1 + qw < z1) {
          r_next = __ldg(rec + a1 + qw);
          p_next = __ldg(perm + a1 + qw);
          ahead = true;
        }
        gather4_point<M2, CP>(s, cx, cya, cyb, qi, jj, sub, seg_mask, r, p,
                              reinterpret_cast<const float *>(smem + buf * tile_bytes), g.w[0], g.w[0] * g.w[1], 0,
                              out, g.m, g.ncomp);
      }
      if (!ahead && a1 + qw < z1) {
        r_next = __ldg(rec + a1 + qw);
        p_next = __ldg(perm + a1 + qw);
      }
      __syncwarp();
      if (lane == 0) {
        __threadfence_block();
        if (atomicAdd(&s_rel[buf], 1u) == nwarps - 1u) {
          // every warp is done with this buffer: refill it (reads of the generic proxy are
          // ordered before the copy's writes)
          atomicExch(&s_rel[buf], 0u);
          if (nx2 < nunits) {
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            issue(unit(nx2), buf);
            s_nissue[buf] += 1u;
          }
        }
      }
      cur = nx;
      a0 = a1;
      z0 = z1;
      nx = nx2;
      a1 = a2;
      z1 = z2;
    }
    __syncthreads();
    // every copy issued lands before the CTA's shared memory is released (full limit)
    if (threadIdx.x == 0)
      for (int i = 0; i < 2; ++i)
        if (s_nissue[i]) mbar_wait(bars + i, (s_nissue[i] - 1u) & 1u);
    return;
  }
  // One buffer: the CTA waits at each brick, and thread 0 refills the buffer after the barrier.
  int64_t ui = blockIdx.x;
  // a brick's point range and each quarter-warp's first record are loaded one brick ahead
  uint32_t s0 = 0, s1 = 0;
  float4 r_next = make_float4(0.f, 0.f, 0.f, 0.f);
  uint32_t p_next = 0u;
  if (unit(ui) >= 0) {
    s0 = __ldg(cell_start + unit(ui) * g.bvol);
    s1 = __ldg(cell_start + (unit(ui) + 1) * g.bvol);
    if (threadIdx.x == 0 && s1 > s0) issue(unit(ui), 0);
    if (s0 + qw < s1) {
      r_next = __ldg(rec + s0 + qw);
      p_next = __ldg(perm + s0 + qw);
    }
  }
  for (; ui < nunits; ui += gridDim.x) {
    constexpr int buf = 0;
    const int64_t bn = unit(ui + gridDim.x);
    uint32_t n0 = 0, n1 = 0;
    if (bn >= 0) {
      n0 = __ldg(cell_start + bn * g.bvol);
      n1 = __ldg(cell_start + (bn + 1) * g.bvol);
    }
    bool ahead = false;  // this quarter-warp's first record of the next brick is loading
    if (s1 > s0) {
      // every thread must take the same exit, so the outcome of the bounded wait is voted
      if (__syncthreads_or(!mbar_wait(bars + buf, phase[buf], g.wait_polls))) {
        failed = true;
        if (threadIdx.x == 0 && status) atomicOr(status, GBG_DEV_TIMEOUT);
        break;
      }
      phase[buf] ^= 1;
      pending[buf] = false;
      for (uint32_t sl = s0 + qw; sl < s1; sl += nqw) {
        const float4 r = r_next;
        const int64_t p = p_next;
        if (sl + nqw < s1) {
          r_next = __ldg(rec + sl + nqw);
          p_next = __ldg(perm + sl + nqw);
        } else if (n0 + qw < n1) {
          r_next = __ldg(rec + n0 + qw);
          p_next = __ldg(perm + n0 + qw);
          ahead = true;
        }
        gather4_point<M2, CP>(s, cx, cya, cyb, qi, jj, sub, seg_mask, r, p,
                              reinterpret_cast<const float *>(smem + buf * tile_bytes), g.w[0], g.w[0] * g.w[1], 0,
                              out, g.m, g.ncomp);
      }
    }
    if (!ahead && n0 + qw < n1) {
      r_next = __ldg(rec + n0 + qw);
      p_next = __ldg(perm + n0 + qw);
    }
    __syncthreads();  // every lane is done with this buffer before it is refilled
    if (threadIdx.x == 0 && n1 > n0) issue(bn, 0);
    s0 = n0;
    s1 = n1;
  }
  if (failed && threadIdx.x == 0) {
    // a copy that did not complete in time: let every copy still in flight land (with the
    // full limit) before the CTA's shared memory is released
    for (int i = 0; i < nbuf; ++i)
      if (pending[i]) mbar_wait(bars + i, phase[i]);
  }
}

// One point of a gather of another width, by one thread over its N2^3 stencil; the nodes
// are base[(origin + x + y*sy + z*sz) * CP] as for the width-4 gather.
template <int N2, int M2, int CP, typename TO, typename I>
__device__ __forceinline__ void gather_point(const SchemeT<float, N2> &s, float4 r, int64_t pt, const float *base, I sy,
                                             I sz, I origin, TO *out, int64_t m, int ncomp) {
  int lx, ly, lz;
  unpack_local(r.w, lx, ly, lz);
  float w1[N2], w2[N2], w3[N2];
  weights_all<N2, M2>(s, r.x, w1);
  weights_all<N2, M2>(s, r.y, w2);
  weights_all<N2, M2>(s, r.z, w3);
  float acc[CP];
#pragma unroll
  for (int c = 0; c < CP; ++c) acc[c] = 0.0f;
#pragma unroll 1
  for (int k = 0; k < N2; ++k) {
    float w3k = w3[0];
#pragma unroll
    for (int q = 1; q < N2; ++q)
      if (q == k) w3k = w3[q];
#pragma unroll
    for (int j = 0; j < N2; ++j) {
      const float wyz = w2[j] * w3k;
      const float *row = base + (origin + (lz + k) * sz + (ly + j) * sy + lx) * CP;
#pragma unroll
      for (int i = 0; i < N2; ++i) {
        const float w = wyz * w1[i];
        const float4 *p = reinterpret_cast<const float4 *>(row + i * CP);
#pragma unroll
        for (int q4 = 0; q4 < CP / 4; ++q4) {
          const float4 v = p[q4];
          acc[4 * q4 + 0] = fmaf(w, v.x, acc[4 * q4 + 0]);
          acc[4 * q4 + 1] = fmaf(w, v.y, acc[4 * q4 + 1]);
          acc[4 * q4 + 2] = fmaf(w, v.z, acc[4 * q4 + 2]);
          acc[4 * q4 + 3] = fmaf(w, v.w, acc[4 * q4 + 3]);
        }
      }
    }
  }
#pragma unroll
  for (int c = 0; c < CP; ++c)
    if (c < ncomp) store_out(out, pt + m * c, acc[c]);
}

// Gather for other widths: a point per thread over its N2^3 stencil in the tile.
template <int N2, int M2, int CP, typename TO>
__global__ void __launch_bounds__(kThreads, 1)
    k_gather_staged_generic(const __grid_constant__ CUtensorMap tmap, StagedGeo g, SchemeT<float, N2> s,
                            const uint32_t *__restrict__ cell_start, const float4 *__restrict__ rec,
                            const uint32_t *__restrict__ perm, TO *__restrict__ out, int32_t *status,
                            int nbuf, uint32_t tile_bytes, uint32_t box_bytes, const uint32_t *__restrict__ list,
                            const uint32_t *__restrict__ list_n) {
  extern __shared__ __align__(1024) unsigned char smem[];
  uint64_t *bars = reinterpret_cast<uint64_t *>(smem + nbuf * tile_bytes);
  if (threadIdx.x == 0) {
    for (int i = 0; i < nbuf; ++i) mbar_init(bars + i, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  uint32_t phase[2] = {0, 0};
  bool failed = false;
  bool pending[2] = {false, false};  // thread 0's copies issued and not yet waited for
  auto issue = [&](int64_t b, int buf) {
    int64_t bx, by, bz;
    brick_coords(g, b, bx, by, bz);
    pending[buf] = true;
    mbar_expect_tx(bars + buf, box_bytes);
    tma_load_tile(smem + buf * tile_bytes, &tmap, 0, (int)(bx * g.b[0]) + g.box_off,
                  (int)(by * g.b[1]) + g.box_off, (int)(bz * g.b[2]) + g.box_off, bars + buf);
  };
  // the bricks to visit: the bins' list of bricks holding points, or every brick
  const int64_t nunits = list ? (int64_t)__ldg(list_n) : g.nbricks;
  auto unit = [&](int64_t i) -> int64_t { return i >= nunits ? -1 : (list ? (int64_t)__ldg(list + i) : i); };
  int64_t ui = blockIdx.x;
  // a brick's point range and each thread's first record are loaded one brick ahead
  uint32_t s0 = 0, s1 = 0;
  float4 r_next = make_float4(0.f, 0.f, 0.f, 0.f);
  uint32_t p_next = 0u;
  if (unit(ui) >= 0) {
    s0 = __ldg(cell_start + unit(ui) * g.bvol);
    s1 = __ldg(cell_start + (unit(ui) + 1) * g.bvol);
    if (threadIdx.x == 0 && s1 > s0) issue(unit(ui), 0);
    if (s0 + threadIdx.x < s1) {
      r_next = __ldg(rec + s0 + threadIdx.x);
      p_next = __ldg(perm + s0 + threadIdx.x);
    }
  }
  for (int it = 0; ui < nunits; ++it, ui += gridDim.x) {
    const int buf = nbuf == 2 ? (it & 1) : 0;
    const int64_t bn = unit(ui + gridDim.x);
    uint32_t n0 = 0, n1 = 0;
    if (bn >= 0) {
      n0 = __ldg(cell_start + bn * g.bvol);
      n1 = __ldg(cell_start + (bn + 1) * g.bvol);
    }
    if (nbuf == 2 && threadIdx.x == 0 && n1 > n0) issue(bn, buf ^ 1);
    bool ahead = false;  // this thread's first record of the next brick is loading
    if (s1 > s0) {
      // every thread must take the same exit, so the outcome of the bounded wait is voted
      if (__syncthreads_or(!mbar_wait(bars + buf, phase[buf], g.wait_polls))) {
        failed = true;
        if (threadIdx.x == 0 && status) atomicOr(status, GBG_DEV_TIMEOUT);
        break;
      }
      phase[buf] ^= 1;
      pending[buf] = false;
      for (uint32_t sl = s0 + threadIdx.x; sl < s1; sl += blockDim.x) {
        const float4 r = r_next;
        const int64_t p = p_next;
        if (sl + blockDim.x < s1) {
          r_next = __ldg(rec + sl + blockDim.x);
          p_next = __ldg(perm + sl + blockDim.x);
        } else if (n0 + threadIdx.x < n1) {
          r_next = __ldg(rec + n0 + threadIdx.x);
          p_next = __ldg(perm + n0 + threadIdx.x);
          ahead = true;
        }
        gather_point<N2, M2, CP>(s, r, p, reinterpret_cast<const float *>(smem + buf * tile_bytes), g.w[0],
                                 g.w[0] * g.w[1], 0, out, g.m, g.ncomp);
      }
    }
    if (!ahead && n0 + threadIdx.x < n1) {
      r_next = __ldg(rec + n0 + threadIdx.x);
      p_next = __ldg(perm + n0 + threadIdx.x);
    }
    __syncthreads();
    if (nbuf == 1 && threadIdx.x == 0 && n1 > n0) issue(bn, 0);
    s0 = n0;
    s1 = n1;
  }
  if (failed && threadIdx.x == 0)
    for (int i = 0; i < nbuf; ++i)
      if (pending[i]) mbar_wait(bars + i, phase[i]);
}

// ------------------------------------------------------------ direct gather
//
// For point sets sparse on their grid (a few points per brick) a tile per brick costs more
// than the points' own stencils: these kernels take the points in binned order, all in
// flight at once, and read each point's nodes straight from the field, with the per-point
// arithmetic of the staged kernels (so the same bits).  A point's brick comes from its
// cell key.

__device__ __forceinline__ int64_t direct_origin(const StagedGeo &g, int64_t pf, int64_t py, uint32_t key) {
  const int64_t brick = key / (uint64_t)g.bvol;
  int64_t bx, by, bz;
  brick_coords(g, brick, bx, by, bz);
  return (bx * g.b[0] + g.box_off) + pf * ((by * g.b[1] + g.box_off) + py * (bz * g.b[2] + g.box_off));
}

template <int M2, int CP, typename TO>
__global__ void __launch_bounds__(kThreads)
    k_gather_direct4(StagedGeo g, SchemeT<float, 4> s, const float *__restrict__ field, int64_t px, int64_t py,
                     const float4 *__restrict__ rec, const uint32_t *__restrict__ perm,
                     const uint32_t *__restrict__ keys, TO *__restrict__ out) {
  const int lane = threadIdx.x & 31, sub = lane & 7, qi = sub & 3, jj = sub >> 2;
  const unsigned seg_mask = 0xFFu << (lane & ~7);
  float cx[M2 > 0 ? M2 : 1], cya[M2 > 0 ? M2 : 1], cyb[M2 > 0 ? M2 : 1];
  if constexpr (M2 > 0) {
#pragma unroll
    for (int p = 0; p < M2; ++p) {
      cx[p] = s.c[qi + 4 * p];
      cya[p] = s.c[2 * jj + 4 * p];
      cyb[p] = s.c[2 * jj + 1 + 4 * p];
    }
  }
  const int64_t nq = ((int64_t)gridDim.x * blockDim.x) >> 3;
  for (int64_t sl = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 3; sl < g.m; sl += nq) {
    const float4 r = __ldg(rec + sl);
    const int64_t pt = __ldg(perm + sl);
    const int64_t origin = direct_origin(g, px, py, __ldg(keys + pt));
    gather4_point<M2, CP>(s, cx, cya, cyb, qi, jj, sub, seg_mask, r, pt, field, px, px * py, origin, out, g.m, g.ncomp);
  }
}

template <int N2, int M2, int CP, typename TO>
__global__ void __launch_bounds__(kThreads)
    k_gather_direct(StagedGeo g, SchemeT<float, N2> s, const float *__restrict__ field, int64_t px, int64_t py,
                    const float4 *__restrict__ rec, const uint32_t *__restrict__ perm,
                    const uint32_t *__restrict__ keys, TO *__restrict__ out) {
  for (int64_t sl = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; sl < g.m; sl += (int64_t)gridDim.x * blockDim.x) {
    const float4 r = __ldg(rec + sl);
    const int64_t pt = __ldg(perm + sl);
    const int64_t origin = direct_origin(g, px, py, __ldg(keys + pt));
    gather_point<N2, M2, CP>(s, r, pt, field, px, px * py, origin, out, g.m, g.ncomp);
  }
}

// ------------------------------------------------------------ staged scatter

// Sorted, alpha-scaled quantities: qs[s*CP + c] = T(alpha) * q[perm[s] + M*c].
// Also the largest |alpha q| (as ordered float bits; NaN orders above every number, so a
// NaN quantity shows as a non-finite bound).
template <typename TQ, int CP>
__global__ void k_scatter_qprep(const TQ *__restrict__ q, const uint32_t *__restrict__ perm, int64_t m,
                                int ncomp, float alpha, float *__restrict__ qs, unsigned *__restrict__ qmax_bits) {
  unsigned mx = 0u;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  // two points a trip, every load of both issued before the stores (the loads of one point
  // are independent, so a trip waits for memory once, not once per component group)
  for (int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; s < m; s += 2 * stride) {
    const bool two = s + stride < m;
    const int64_t p0 = perm[s], p1 = perm[two ? s + stride : s];
    float v[2][CP];
#pragma unroll
    for (int c = 0; c < CP; ++c) {
      v[0][c] = c < ncomp ? alpha * (float)q[p0 + m * c] : 0.0f;
      v[1][c] = c < ncomp ? alpha * (float)q[p1 + m * c] : 0.0f;
    }
#pragma unroll
    for (int k = 0; k < 2; ++k) {
      if (k == 1 && !two) break;
      // four components at a time into one 16-byte store
#pragma unroll
      for (int c4 = 0; c4 < CP; c4 += 4) {
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          const unsigned bits = __float_as_uint(fabsf(v[k][c4 + u]));
          mx = bits > mx ? bits : mx;
        }
        reinterpret_cast<float4 *>(qs + (s + k * stride) * CP)[c4 / 4] =
            make_float4(v[k][c4], v[k][c4 + 1], v[k][c4 + 2], v[k][c4 + 3]);
      }
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned other = __shfl_xor_sync(0xffffffffu, mx, o);
    mx = other > mx ? other : mx;
  }
  if ((threadIdx.x & 31) == 0) atomicMax(qmax_bits, mx);
}

// Four-byte asynchronous copies global -> shared (cp.async), their commit and wait.
__device__ __forceinline__ void cp_async4(void *dst, const void *src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(smem_addr(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

// One compensated step (Knuth's TwoSum, every operation rounded on its own): s + x into
// the pair (s, c), c collecting the exact rounding error of each addition.
__device__ __forceinline__ void twosum_add(float &s, float &c, float x) {
  const float t = __fadd_rn(s, x);
  const float z = __fsub_rn(t, s);
  c = __fadd_rn(c, __fadd_rn(__fsub_rn(s, __fsub_rn(t, z)), __fsub_rn(x, z)));
  s = t;
}

struct FixGeo {
  int32_t b[3];
  int32_t nb[3];
  int32_t n[3];
  int32_t e[3];  // extended cell region = brick + width - 1
  int64_t nbricks, bvol;
  int64_t px, py;
  int32_t halo, cp, ncomp;
  int32_t neighbour_skip;  // every brick edge >= width/2: the region lies in the 27 neighbouring bricks
  int32_t chunk;           // points staged in shared memory at a time (a multiple of 4)
  int32_t chunk1;          // the same when the region's points fit at once (no running sums kept)
  int32_t comp;            // compensated: chunk partial sums folded into (sum, correction) by TwoSum
  float *cscratch;         // corrections of regions of several chunks: one slot per CTA
  int64_t cstride;         // floats per slot (>= bvol * CP)
  int32_t sparse;          // few points a brick: regions from the neighbouring bricks' lists
};

// All N2 weights from coefficients in memory ([q + N2*p], M2 == N2 powers).
template <int N2>
__device__ __forceinline__ void weights_ptr(const float *c, float t, float (&w)[N2]) {
#pragma unroll
  for (int q = 0; q < N2; ++q) w[q] = c[q + N2 * (N2 - 1)];
#pragma unroll
  for (int p = N2 - 2; p >= 0; --p)
#pragma unroll
    for (int q = 0; q < N2; ++q) w[q] = fmaf(w[q], t, c[q + N2 * p]);
}

// The same for any number of powers m2.
template <int N2>
__device__ __forceinline__ void weights_rt(const float *c, int m2, float t, float (&w)[N2]) {
#pragma unroll
  for (int q = 0; q < N2; ++q) w[q] = c[q + N2 * (m2 - 1)];
#pragma unroll 1
  for (int p = m2 - 2; p >= 0; --p)
#pragma unroll
    for (int q = 0; q < N2; ++q) w[q] = fmaf(w[q], t, c[q + N2 * p]);
}

// Shared memory of one scatter CTA, in this order: the brick's running sums (CP floats per
// node), one chunk of the region's points (CP quantities and 3*N2+4 weights each), the
// region's per-cell point offsets (+ the total) and first slots, the per-axis key tables
// of the region's cells (this brick's, then the next brick's), and the points' region x
// cells.  (With compensation, a region of several chunks keeps its sums' corrections in the
// CTA's own slot of a global scratch; the next brick's cell table, copied ahead, uses the
// free end of the staging area.)
size_t scatter_nodes_fixed(const FixGeo &g, int cp) {
  const size_t ecount = (size_t)g.e[0] * g.e[1] * g.e[2];
  return sizeof(float) * (size_t)g.bvol * cp +
         sizeof(uint32_t) * (2 * ecount + 1 + 2 * (size_t)(g.e[0] + g.e[1] + g.e[2])) + 16;
}

// Floats of weights per staged point: the N2 x weights, then the y and the z weights each
// with a zero on either side (so that a node's index past the stencil reads a zero),
// rounded up to an odd count: lanes reading the same weight of different points then
// fall in different banks (an even stride such as 16 would put 32 lanes in 2 banks).
template <int N2>
constexpr int kScatterWStride = (3 * N2 + 4) | 1;
inline int scatter_wstride(int n2) { return (3 * n2 + 4) | 1; }

size_t scatter_nodes_smem(const FixGeo &g, int cp, int n2) {
  return scatter_nodes_fixed(g, cp) + sizeof(float) * (size_t)g.chunk * (cp + scatter_wstride(n2)) + (size_t)g.chunk1;
}

// Sets the chunk sizes: the largest chunk (a multiple of 4, 64..1024 points) whose CTA
// fits in `budget` bytes, and the larger one that also takes the running sums' space when
// the whole region fits in one chunk.
void scatter_nodes_chunk(FixGeo &g, int cp, int n2, size_t budget) {
  const size_t per = sizeof(float) * (cp + scatter_wstride(n2)) + 1, fixed = scatter_nodes_fixed(g, cp);
  const size_t fit = budget > fixed ? (budget - fixed) / per : 0;
  g.chunk = (int32_t)std::max<size_t>(64, std::min<size_t>(1024, fit & ~size_t(3)));
  g.chunk1 = g.chunk + (int32_t)(((size_t)g.bvol * cp * sizeof(float) / per) & ~size_t(3));
}

// Shared memory per scatter CTA: half an SM's (two CTAs per SM) less the block's reserved
// and static share, or more when a region of 512 points would not fit one chunk (a brick's
// region holds a few hundred at the usual densities, and each extra chunk re-stages and
// re-walks the rows; a single chunk may also use the running sums' space).  It depends on
// the brick's geometry alone, never on the launch shape: the chunks are where the
// compensated summation folds its partial sums, so the same chunks for every launch keep
// the results bitwise independent of the threads per CTA and of batching.
size_t scatter_nodes_budget(const FixGeo &g, int cp, int n2) {
  const size_t per = sizeof(float) * (cp + scatter_wstride(n2)) + 1;
  const size_t sums = sizeof(float) * (size_t)g.bvol * cp;
  const size_t want = scatter_nodes_fixed(g, cp) + (512 * per > sums ? 512 * per - sums : 0) + 4 * per;
  const size_t half = 228 * 1024 / 2 - 4096;
  return want <= half ? half : std::min<size_t>(200 * 1024, 228 * 1024 - 4096);
}

// Few points a brick (as for the direct gather), and a region no wider than the grid on any
// axis (each region cell a distinct cell): the scatter builds regions from the neighbouring
// bricks' point lists.
int32_t scatter_sparse(const gbg_bins_s *b, const gbg_grid &grid, int n2) {
  if (!b->sparse_regions || b->npoints >= 4 * b->nbricks) return 0;
  for (int d = 0; d < 3; ++d)
    if (b->b[d] + n2 - 1 > grid.n[d]) return 0;
  return 1;
}

// Deterministic scatter, output-driven.  A CTA owns a brick's nodes and a thread owns a
// 2 x 2 quad of nodes in y and z (one node for width 8): it sums, in registers, the
// contributions ((wx*wy)*wz)*alpha*q of every point whose stencil reaches each node, in a
// fixed order per node -- the node's N2 x N2 rows of cells (z outer, y inner), within a
// row the points in their binned order.  A point is loaded once for all the quad's nodes;
// a node that it does not reach adds w == 0 exactly (or, in a chunk holding a non-finite
// value, takes no operation from it), which leaves the node's sum unchanged.  SU points
// per thread are staged per round so that their load latencies overlap.  The
// order depends on the points alone, not on the launch shape, the chunking or the other
// instances of a batch, so the result is reproducible bitwise; no atomics are involved.
//
// The brick's region (its cells widened by N2 - 1) is listed in region order (x fastest)
// with per-cell offsets; its points pass through shared memory in chunks of contiguous
// region positions.  A node's points occupy increasing region positions, so a chunked
// pass continues each node's running sum exactly where the previous chunk left it.
// All index arithmetic is 32-bit: the region's cell keys come from three per-axis tables
// (key = kx[ex] + ky[ey] + kz[ez]).
template <int N2, bool FIXED, int CP, int SU>
__device__ bool scatter_brick_nodes(const FixGeo &g, const float *coef, int m2, int64_t b,
                                    const uint32_t *__restrict__ cell_start, const float4 *__restrict__ rec,
                                    const float *__restrict__ qs, float *__restrict__ field, float beta,
                                    int beta_zero, bool listed, unsigned char *smem, uint32_t *warp_tot,
                                    int64_t next = -1, bool have = false) {
  const int E0 = g.e[0], E1 = g.e[1], E2 = g.e[2];
  const int ecount = E0 * E1 * E2;
  const int bvol = (int)g.bvol;
  // [running sums | chunk: quantities, weights] [offsets, first slots, key tables] [x cells]
  float *sacc = reinterpret_cast<float *>(smem);
  // compensation terms of the running sums (regions of several chunks only): this CTA's slot
  // of the global scratch
  float *scmp = g.cscratch + (size_t)blockIdx.x * g.cstride;
  uint32_t *off = reinterpret_cast<uint32_t *>(sacc + bvol * CP + g.chunk * (CP + kScatterWStride<N2>));
  uint32_t *r0s = off + ecount + 1;
  uint32_t *kx = r0s + ecount, *ky = kx + E0, *kz = ky + E1;
  uint32_t *knx = kz + E2;  // the next brick's per-axis key tables (same layout)
  unsigned char *scx = reinterpret_cast<unsigned char *>(knx + E0 + E1 + E2);
  // the next brick's cell table, copied by cp.async while this brick computes: the last
  // 2 * ecount words of the staging area (first slots, then ends)
  uint32_t *pre_a = off - 2 * ecount, *pre_z = off - ecount;
  if (have) {
    cp_async_wait_all();
    __syncthreads();
  }
  constexpr int half = N2 / 2;
  const int bx = (int)(b % g.nb[0]), by = (int)((b / g.nb[0]) % g.nb[1]), bz = (int)(b / ((int64_t)g.nb[0] * g.nb[1]));
  const int B0 = g.b[0], B1 = g.b[1];
  // nodes of this brick inside the grid
  const int vx = min(B0, g.n[0] - bx * B0), vy = min(B1, g.n[1] - by * B1), vz = min(g.b[2], g.n[2] - bz * g.b[2]);
  // is any point near?  (the 27 neighbouring bricks hold the whole region)  Only a
  // scatter with beta == 1 may leave a brick alone, and a brick taken from the bins' list
  // of bricks in reach of a point is known to be near.
  bool any = true;
  if (g.neighbour_skip && !beta_zero && beta == 1.0f && !listed) {
    bool mine = false;
    if (threadIdx.x < 27) {
      const int dx = (int)threadIdx.x % 3 - 1, dy = ((int)threadIdx.x / 3) % 3 - 1, dz = (int)threadIdx.x / 9 - 1;
      const uint32_t nx = (uint32_t)((bx + dx + g.nb[0]) % g.nb[0]), ny = (uint32_t)((by + dy + g.nb[1]) % g.nb[1]),
                     nz = (uint32_t)((bz + dz + g.nb[2]) % g.nb[2]);
      const uint64_t k = ((uint64_t)nz * (uint32_t)g.nb[1] + ny) * (uint32_t)g.nb[0] + nx;
      mine = __ldg(cell_start + (k + 1) * (uint64_t)bvol) != __ldg(cell_start + k * (uint64_t)bvol);
    }
    any = __syncthreads_or(mine);
  }
  if (!any && !beta_zero && beta == 1.0f) return false;  // the brick keeps its values
  uint32_t count = 0;
  // A point set sparse on its grid: the region's points are taken from the ranges of the
  // 27 neighbouring bricks, kept when their cell lies in the region and put in region
  // order (cell, then slot), instead of building the region's per-cell tables -- the same
  // points in the same order as the tables give.  Too many candidates: the tables.
  constexpr uint32_t kCandScan = 256, kCandKeep = 64;
  uint32_t *sorted_e = off + 32 + kCandKeep, *sorted_s = r0s + 32 + kCandKeep;
  bool sparse = false;
  if (g.sparse && g.neighbour_skip && any && ecount >= 32 + 2 * (int)kCandKeep) {
    uint32_t *nstart = r0s, *npre = off, *cand_e = off + 32, *cand_s = r0s + 32;
    if (threadIdx.x < 32) {
      const int t = threadIdx.x;
      uint32_t a = 0, c = 0;
      if (t < 27) {
        const int dx = t % 3 - 1, dy = (t / 3) % 3 - 1, dz = t / 9 - 1;
        // an axis of one brick has one neighbour (the brick itself), of two bricks two
        const bool dup = (g.nb[0] == 1 && dx != 0) || (g.nb[0] == 2 && dx < 0) || (g.nb[1] == 1 && dy != 0) ||
                         (g.nb[1] == 2 && dy < 0) || (g.nb[2] == 1 && dz != 0) || (g.nb[2] == 2 && dz < 0);
        if (!dup) {
          const uint64_t k = ((uint64_t)((bz + dz + g.nb[2]) % g.nb[2]) * (uint32_t)g.nb[1] +
                              (uint32_t)((by + dy + g.nb[1]) % g.nb[1])) * (uint32_t)g.nb[0] +
                             (uint32_t)((bx + dx + g.nb[0]) % g.nb[0]);
          a = __ldg(cell_start + k * (uint64_t)bvol);
          c = __ldg(cell_start + (k + 1) * (uint64_t)bvol) - a;
        }
      }
      uint32_t x = c;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (t >= o) x += y;
      }
      if (t < 27) {
        nstart[t] = a;
        npre[t + 1] = x;
      }
      if (t == 0) {
        npre[0] = 0;
        warp_tot[1] = 0;
      }
      if (t == 31) warp_tot[0] = x;
    }
    __syncthreads();
    const uint32_t total = warp_tot[0];
    if (total <= kCandScan) {
      for (uint32_t t = threadIdx.x; t < total; t += blockDim.x) {
        int k = 0;
        while (k < 26 && npre[k + 1] <= t) ++k;
        const uint32_t slot = nstart[k] + (t - npre[k]);
        int lx, ly, lz;
        unpack_local(__ldg(rec + slot).w, lx, ly, lz);
        const int dx = k % 3 - 1, dy = (k / 3) % 3 - 1, dz = k / 9 - 1;
        // the point's cell, then its offset from the region's first cell (periodic)
        const int cx = (int)((bx + dx + g.nb[0]) % g.nb[0]) * B0 + lx;
        const int cy = (int)((by + dy + g.nb[1]) % g.nb[1]) * B1 + ly;
        const int cz = (int)((bz + dz + g.nb[2]) % g.nb[2]) * g.b[2] + lz;
        int ex = (cx - (bx * B0 - half)) % g.n[0], ey = (cy - (by * B1 - half)) % g.n[1],
            ez = (cz - (bz * g.b[2] - half)) % g.n[2];
        if (ex < 0) ex += g.n[0];
        if (ey < 0) ey += g.n[1];
        if (ez < 0) ez += g.n[2];
        if (ex < E0 && ey < E1 && ez < E2) {
          const uint32_t i = atomicAdd(warp_tot + 1, 1u);
          if (i < kCandKeep) {
            cand_e[i] = (uint32_t)((ez * E1 + ey) * E0 + ex);
            cand_s[i] = slot;
          }
        }
      }
      __syncthreads();
      const uint32_t kept = warp_tot[1];
      if (kept <= kCandKeep) {
        for (uint32_t i = threadIdx.x; i < kept; i += blockDim.x) {
          const uint32_t e = cand_e[i], sl = cand_s[i];
          uint32_t rank = 0;
          for (uint32_t j = 0; j < kept; ++j) rank += (cand_e[j] < e || (cand_e[j] == e && cand_s[j] < sl)) ? 1u : 0u;
          sorted_e[rank] = e;
          sorted_s[rank] = sl;
        }
        sparse = true;
        count = kept;
      }
      __syncthreads();
    }
  }
  if (any && !sparse) {
    // per-axis key tables of the region's cells (periodic wrap, then brick and local index)
    // this brick's tables (unless its cell table was copied ahead) and the next brick's
    const int ET = E0 + E1 + E2;
    for (int t = threadIdx.x; t < 2 * ET; t += blockDim.x) {
      const bool nxt = t >= ET;
      if (nxt ? next < 0 : have) continue;
      const int tt = nxt ? t - ET : t;
      const int64_t bb = nxt ? next : b;
      const int d = tt < E0 ? 0 : (tt < E0 + E1 ? 1 : 2);
      const int e = tt - (d == 0 ? 0 : (d == 1 ? E0 : E0 + E1));
      const int bc = d == 0 ? (int)(bb % g.nb[0]) : (d == 1 ? (int)((bb / g.nb[0]) % g.nb[1]) : (int)(bb / ((int64_t)g.nb[0] * g.nb[1])));
      int c = (bc * g.b[d] - half + e) % g.n[d];
      if (c < 0) c += g.n[d];
      const uint32_t cb = (uint32_t)c / (uint32_t)g.b[d], cl = (uint32_t)c - cb * (uint32_t)g.b[d];
      uint32_t key;
      if (d == 0) key = cb * (uint32_t)bvol + cl;
      else if (d == 1) key = (cb * (uint32_t)g.nb[0]) * (uint32_t)bvol + cl * (uint32_t)g.b[0];
      else key = (cb * (uint32_t)g.nb[1] * (uint32_t)g.nb[0]) * (uint32_t)bvol + cl * (uint32_t)(g.b[0] * g.b[1]);
      (nxt ? knx : kx)[tt] = key;
    }
    __syncthreads();
    if (have) {
      for (int e = threadIdx.x; e < ecount; e += blockDim.x) {
        const uint32_t a = pre_a[e];
        r0s[e] = a;
        off[e] = pre_z[e] - a;
      }
    } else {
      // eight cells per thread in flight (one round for a 15x8x8 brick's 2178 cells at
      // 256 threads): their keys first, then all sixteen loads
      constexpr int U = 8;
      int ex = (int)threadIdx.x % E0, ey = ((int)threadIdx.x / E0) % E1, ez = (int)threadIdx.x / (E0 * E1);
      const int sx = (int)blockDim.x % E0, sy = ((int)blockDim.x / E0) % E1, sz = (int)blockDim.x / (E0 * E1);
      for (int e = threadIdx.x; e < ecount; e += U * (int)blockDim.x) {
        uint32_t key[U], a[U], z[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
          key[u] = e + u * (int)blockDim.x < ecount ? kx[ex] + ky[ey] + kz[ez] : 0u;
          ex += sx;
          ey += sy;
          ez += sz;
          if (ex >= E0) { ex -= E0; ++ey; }
          if (ey >= E1) { ey -= E1; ++ez; }
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
          a[u] = __ldg(cell_start + key[u]);
          z[u] = __ldg(cell_start + key[u] + 1);
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
          const int eu = e + u * (int)blockDim.x;
          if (eu < ecount) {
            r0s[eu] = a[u];
            off[eu] = z[u] - a[u];
          }
        }
      }
    }
    __syncthreads();
    count = block_scan_counts(off, ecount, warp_tot);
    if (threadIdx.x == 0) off[ecount] = count;
  }
  // a region that fits at once stages over the running sums' space too
  const bool one = count <= (uint32_t)g.chunk1;
  const int P = one ? g.chunk1 : g.chunk;
  float *sq = one ? sacc : sacc + bvol * CP;
  float *sw = sq + P * CP;
  // a thread owns BY x BZ nodes (lx, ly+a, lz+b) and walks the RY x RZ rows of region cells
  // that feed any of them; each point it loads serves up to BY*BZ nodes
  constexpr int BY = N2 <= 6 ? 2 : 1, BZ = BY;
  constexpr int RY = N2 + BY - 1, RZ = N2 + BZ - 1;
  const int QY = (B1 + BY - 1) / BY, QZ = (g.b[2] + BZ - 1) / BZ;
  const int nquads = B0 * QY * QZ, slab = E1 * E0;
  bool issued = false;
  for (uint32_t c0 = 0;; c0 += (uint32_t)P) {
    const uint32_t c1 = min(count, c0 + (uint32_t)P);
    const bool first = c0 == 0, last = c1 == count;
    __syncthreads();  // the previous chunk's points (and off[ecount]) are settled
    // stage the chunk: each point's region cell by binary search of the offsets, its
    // weights (x, then y and z each with a zero either side) and its quantities
    int nonfinite = 0;
    // up to SU points per thread per round: every search first, then every global load,
    // then the weights, so the latencies of the points overlap
    for (uint32_t t0 = c0 + threadIdx.x; t0 < c1; t0 += SU * blockDim.x) {
      if (sparse) break;
      uint32_t sl[SU];
      int cell[SU];
#pragma unroll
      for (int u = 0; u < SU; ++u) {
        const uint32_t t = t0 + u * blockDim.x;
        int lo = 0, hi = ecount;  // the last cell e with off[e] <= t
        if (t < c1) {
          while (hi - lo > 1) {
            const int mid = (lo + hi) >> 1;
            if (off[mid] <= t) lo = mid; else hi = mid;
          }
        }
        cell[u] = lo;
        sl[u] = t < c1 ? r0s[lo] + (t - off[lo]) : 0u;
      }
      float4 r[SU], qv[SU][CP / 4];
#pragma unroll
      for (int u = 0; u < SU; ++u) {
        if (t0 + u * blockDim.x < c1) {
          r[u] = __ldg(rec + sl[u]);
          const float4 *q4 = reinterpret_cast<const float4 *>(qs + (int64_t)sl[u] * CP);
#pragma unroll
          for (int v = 0; v < CP / 4; ++v) qv[u][v] = __ldg(q4 + v);
        }
      }
#pragma unroll
      for (int u = 0; u < SU; ++u) {
        const uint32_t t = t0 + u * blockDim.x;
        if (t >= c1) break;
        const int tl = (int)(t - c0);
        scx[tl] = (unsigned char)(cell[u] % E0);
        float *wt = sw + tl * kScatterWStride<N2>;
        float w[N2];
        if constexpr (FIXED) weights_ptr<N2>(coef, r[u].x, w); else weights_rt<N2>(coef, m2, r[u].x, w);
#pragma unroll
        for (int q = 0; q < N2; ++q) wt[q] = w[q];
        if constexpr (FIXED) weights_ptr<N2>(coef, r[u].y, w); else weights_rt<N2>(coef, m2, r[u].y, w);
        wt[N2] = 0.0f;
#pragma unroll
        for (int q = 0; q < N2; ++q) wt[N2 + 1 + q] = w[q];
        wt[2 * N2 + 1] = 0.0f;
        if constexpr (FIXED) weights_ptr<N2>(coef, r[u].z, w); else weights_rt<N2>(coef, m2, r[u].z, w);
        wt[2 * N2 + 2] = 0.0f;
#pragma unroll
        for (int q = 0; q < N2; ++q) wt[2 * N2 + 3 + q] = w[q];
        wt[3 * N2 + 3] = 0.0f;
        float qa = 0.0f;
#pragma unroll
        for (int v = 0; v < CP / 4; ++v) {
          reinterpret_cast<float4 *>(sq + tl * CP)[v] = qv[u][v];
          qa += fabsf(qv[u][v].x) + fabsf(qv[u][v].y) + fabsf(qv[u][v].z) + fabsf(qv[u][v].w);
        }
        // NaN or infinity in the point's offsets or quantities (the sum is finite otherwise)
        if (!isfinite(r[u].x + r[u].y + r[u].z + qa)) nonfinite = 1;
      }
    }
    if (sparse) {
      // the sorted candidates, staged as above (one chunk: count <= kCandKeep)
      for (uint32_t t = threadIdx.x; t < count; t += blockDim.x) {
        const uint32_t sl = sorted_s[t];
        const float4 r = __ldg(rec + sl);
        scx[t] = (unsigned char)(sorted_e[t] % (uint32_t)E0);
        float *wt = sw + t * kScatterWStride<N2>;
        float w[N2];
        if constexpr (FIXED) weights_ptr<N2>(coef, r.x, w); else weights_rt<N2>(coef, m2, r.x, w);
#pragma unroll
        for (int q = 0; q < N2; ++q) wt[q] = w[q];
        if constexpr (FIXED) weights_ptr<N2>(coef, r.y, w); else weights_rt<N2>(coef, m2, r.y, w);
        wt[N2] = 0.0f;
#pragma unroll
        for (int q = 0; q < N2; ++q) wt[N2 + 1 + q] = w[q];
        wt[2 * N2 + 1] = 0.0f;
        if constexpr (FIXED) weights_ptr<N2>(coef, r.z, w); else weights_rt<N2>(coef, m2, r.z, w);
        wt[2 * N2 + 2] = 0.0f;
#pragma unroll
        for (int q = 0; q < N2; ++q) wt[2 * N2 + 3 + q] = w[q];
        wt[3 * N2 + 3] = 0.0f;
        const float4 *q4 = reinterpret_cast<const float4 *>(qs + (int64_t)sl * CP);
        float qa = 0.0f;
#pragma unroll
        for (int v = 0; v < CP / 4; ++v) {
          const float4 x = __ldg(q4 + v);
          reinterpret_cast<float4 *>(sq + t * CP)[v] = x;
          qa += fabsf(x.x) + fabsf(x.y) + fabsf(x.z) + fabsf(x.w);
        }
        if (!isfinite(r.x + r.y + r.z + qa)) nonfinite = 1;
      }
    }
    // a chunk with a non-finite value takes the exact path: each point only touches the
    // nodes it reaches; otherwise a point adds w*q to all of a quad's nodes, with w == 0
    // exactly for the nodes it does not reach, and fmaf(0, q, s) == s for finite q
    const bool exact = __syncthreads_or(nonfinite);
    // a region staged at once leaves the end of the staging area free while the quads run:
    // the next brick's cell table goes there
    if (one && next >= 0 && !sparse &&
        P * CP + (int)count * kScatterWStride<N2> + 2 * ecount <= bvol * CP + g.chunk * (CP + kScatterWStride<N2>)) {
      int ex = (int)threadIdx.x % E0, ey = ((int)threadIdx.x / E0) % E1, ez = (int)threadIdx.x / (E0 * E1);
      const int sx = (int)blockDim.x % E0, sy = ((int)blockDim.x / E0) % E1, sz = (int)blockDim.x / (E0 * E1);
      const uint32_t *kny = knx + E0, *knz = kny + E1;
      for (int e = threadIdx.x; e < ecount; e += blockDim.x) {
        const uint32_t key = knx[ex] + kny[ey] + knz[ez];
        cp_async4(pre_a + e, cell_start + key);
        cp_async4(pre_z + e, cell_start + key + 1);
        ex += sx;
        ey += sy;
        ez += sz;
        if (ex >= E0) { ex -= E0; ++ey; }
        if (ey >= E1) { ey -= E1; ++ez; }
      }
      cp_async_commit();
      issued = true;
    }
    for (int qi = threadIdx.x; qi < nquads; qi += blockDim.x) {
      const int lx = qi % B0, ly = ((qi / B0) % QY) * BY, lz = (qi / (B0 * QY)) * BZ;
      float acc[BY * BZ][CP];
#pragma unroll
      for (int n = 0; n < BY * BZ; ++n) {
        const int a = n % BY, bb = n / BY;
        const bool mine = ly + a < B1 && lz + bb < g.b[2];
#pragma unroll
        for (int v = 0; v < CP / 4; ++v) {
          float4 s4 = make_float4(0.f, 0.f, 0.f, 0.f);
          // plain sums carry the running sum from chunk to chunk; compensated ones start each
          // chunk at zero and fold it in at the chunk's end
          if (!first && mine && !g.comp)
            s4 = reinterpret_cast<const float4 *>(sacc + (((lz + bb) * B1 + ly + a) * B0 + lx) * CP)[v];
          acc[n][4 * v] = s4.x;
          acc[n][4 * v + 1] = s4.y;
          acc[n][4 * v + 2] = s4.z;
          acc[n][4 * v + 3] = s4.w;
        }
      }
      if (count > 0 && sparse) {
        // the staged candidates in region order: a point feeds this quad when its cell is
        // in the quad's x window and one of its rows (the order of the rows path)
        const int xk = lx + N2 - 1;
        for (uint32_t t = 0; t < count; ++t) {
          const uint32_t e = sorted_e[t];
          const int ex = (int)(e % (uint32_t)E0), ey = (int)((e / (uint32_t)E0) % (uint32_t)E1),
                    ez = (int)(e / (uint32_t)(E0 * E1));
          const int jj = ey - ly, kk = ez - lz;
          if (ex < lx || ex > xk || jj < 0 || jj >= RY || kk < 0 || kk >= RZ) continue;
          const float *wp = sw + t * kScatterWStride<N2>;
          const float *wy = wp + (2 * N2 - jj), *wz = wp + (3 * N2 + 2 - kk);
          const float4 *qp = reinterpret_cast<const float4 *>(sq) + t * (CP / 4);
          const float wx = wp[xk - ex];
          float q[CP];
#pragma unroll
          for (int v = 0; v < CP / 4; ++v) {
            const float4 t4 = qp[v];
            q[4 * v] = t4.x;
            q[4 * v + 1] = t4.y;
            q[4 * v + 2] = t4.z;
            q[4 * v + 3] = t4.w;
          }
#pragma unroll
          for (int n = 0; n < BY * BZ; ++n) {
            const int a = n % BY, bb = n / BY;
            if (exact && !(jj - a >= 0 && jj - a <= N2 - 1 && kk - bb >= 0 && kk - bb <= N2 - 1)) continue;
            const float wgt = (wx * wy[a]) * wz[bb];
#pragma unroll
            for (int c = 0; c < CP; ++c) acc[n][c] = fmaf(wgt, q[c], acc[n][c]);
          }
        }
      } else if (count > 0) {
        // row (jj, kk) holds the region cells (lx..lx+N2-1, ly+jj, lz+kk); its bit in the
        // mask is kk*8 + jj, so bits rise with region order.  Node (lx, ly+a, lz+b) takes a
        // point of that row in region cell ex with stencil indices lx+N2-1-ex on x,
        // N2-1-jj+a on y and N2-1-kk+b on z (a zero weight outside 0..N2-1).  The rows
        // holding points of this chunk are marked, and the loop runs once per point: a
        // lane's trip count is its quad's number of points, not a count per row.
        const int ebase = (lz * E1 + ly) * E0 + lx;
        unsigned long long rows = 0;
#pragma unroll
        for (int kk = 0; kk < RZ; ++kk)
#pragma unroll
          for (int jj = 0; jj < RY; ++jj)
            if (ly + jj < E1 && lz + kk < E2) {
              const int e0 = ebase + kk * slab + jj * E0;
              if (max(off[e0], c0) < min(off[e0 + N2], c1)) rows |= 1ull << (kk * 8 + jj);
            }
        if (rows) {
          const int xk = lx + N2 - 1;
          const float *wp = nullptr, *wy = nullptr, *wz = nullptr;
          const float4 *qp = nullptr;
          const unsigned char *xp = nullptr;
          uint32_t left = 0;
          int jj = 0, kk = 0;
          auto next_row = [&]() {
            const int s = __ffsll((long long)rows) - 1;
            rows &= rows - 1;
            kk = s >> 3;
            jj = s & 7;
            const int e0 = ebase + kk * slab + jj * E0;
            const uint32_t p0 = max(off[e0], c0);
            left = min(off[e0 + N2], c1) - p0;
            const int tl = (int)(p0 - c0);
            wp = sw + tl * kScatterWStride<N2>;
            wy = wp + (2 * N2 - jj);      // y weight of node ly (padded; +1 for node ly+1)
            wz = wp + (3 * N2 + 2 - kk);  // z weight of node lz (padded; +1 for node lz+1)
            qp = reinterpret_cast<const float4 *>(sq) + tl * (CP / 4);
            xp = scx + tl;
          };
          next_row();
          if (!exact) {
            while (true) {
              const float wx = wp[xk - (int)*xp];
              float q[CP];
#pragma unroll
              for (int v = 0; v < CP / 4; ++v) {
                const float4 t4 = qp[v];
                q[4 * v] = t4.x;
                q[4 * v + 1] = t4.y;
                q[4 * v + 2] = t4.z;
                q[4 * v + 3] = t4.w;
              }
#pragma unroll
              for (int n = 0; n < BY * BZ; ++n) {
                const float wgt = (wx * wy[n % BY]) * wz[n / BY];
#pragma unroll
                for (int c = 0; c < CP; ++c) acc[n][c] = fmaf(wgt, q[c], acc[n][c]);
              }
              wp += kScatterWStride<N2>;
              wy += kScatterWStride<N2>;
              wz += kScatterWStride<N2>;
              qp += CP / 4;
              ++xp;
              if (--left == 0) {
                if (!rows) break;
                next_row();
              }
            }
          } else {
            while (true) {
              const float wx = wp[xk - (int)*xp];
              float q[CP];
#pragma unroll
              for (int v = 0; v < CP / 4; ++v) {
                const float4 t4 = qp[v];
                q[4 * v] = t4.x;
                q[4 * v + 1] = t4.y;
                q[4 * v + 2] = t4.z;
                q[4 * v + 3] = t4.w;
              }
#pragma unroll
              for (int n = 0; n < BY * BZ; ++n) {
                const int a = n % BY, bb = n / BY;
                const bool reach = jj - a >= 0 && jj - a <= N2 - 1 && kk - bb >= 0 && kk - bb <= N2 - 1;
                if (reach) {
                  const float wgt = (wx * wy[a]) * wz[bb];
#pragma unroll
                  for (int c = 0; c < CP; ++c) acc[n][c] = fmaf(wgt, q[c], acc[n][c]);
                }
              }
              wp += kScatterWStride<N2>;
              wy += kScatterWStride<N2>;
              wz += kScatterWStride<N2>;
              qp += CP / 4;
              ++xp;
              if (--left == 0) {
                if (!rows) break;
                next_row();
              }
            }
          }
        }
      }
#pragma unroll
      for (int n = 0; n < BY * BZ; ++n) {
        const int a = n % BY, bb = n / BY;
        const int ny = ly + a, nz = lz + bb;
        if (ny >= B1 || nz >= g.b[2]) continue;  // past the brick (odd edge)
        if (g.comp && !first) {
          // fold this chunk's partial sums into the node's (sum, correction)
          float *sp = sacc + ((nz * B1 + ny) * B0 + lx) * CP, *cp2 = scmp + ((nz * B1 + ny) * B0 + lx) * CP;
#pragma unroll
          for (int c = 0; c < CP; ++c) {
            float sum = sp[c], cor = cp2[c];
            twosum_add(sum, cor, acc[n][c]);
            if (last) {
              acc[n][c] = __fadd_rn(sum, cor);
            } else {
              sp[c] = sum;
              cp2[c] = cor;
            }
          }
          if (!last) continue;
        }
        if (last) {
          if (lx >= vx || ny >= vy || nz >= vz) continue;  // past the grid (last brick)
          const int64_t x = (int64_t)bx * B0 + lx, y = (int64_t)by * B1 + ny, z = (int64_t)bz * g.b[2] + nz;
          float4 *d = reinterpret_cast<float4 *>(field + ((x + g.halo) + g.px * ((y + g.halo) + g.py * (z + g.halo))) * CP);
#pragma unroll
          for (int v4 = 0; v4 < CP / 4; ++v4) {
            float v[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) v[u] = 4 * v4 + u < g.ncomp ? acc[n][4 * v4 + u] : 0.0f;
            if (beta_zero) {
              d[v4] = make_float4(v[0], v[1], v[2], v[3]);
            } else {
              const float4 o = d[v4];
              d[v4] = make_float4(__fadd_rn(__fmul_rn(beta, o.x), v[0]), __fadd_rn(__fmul_rn(beta, o.y), v[1]),
                                  __fadd_rn(__fmul_rn(beta, o.z), v[2]), __fadd_rn(__fmul_rn(beta, o.w), v[3]));
            }
          }
        } else {
#pragma unroll
          for (int v = 0; v < CP / 4; ++v) {
            reinterpret_cast<float4 *>(sacc + ((nz * B1 + ny) * B0 + lx) * CP)[v] =
                make_float4(acc[n][4 * v], acc[n][4 * v + 1], acc[n][4 * v + 2], acc[n][4 * v + 3]);
            if (g.comp) reinterpret_cast<float4 *>(scmp + ((nz * B1 + ny) * B0 + lx) * CP)[v] = make_float4(0.f, 0.f, 0.f, 0.f);
          }
        }
      }
    }
    if (last) break;
  }
  __syncthreads();
  return issued;
}

template <int N2, bool FIXED, int CP>
__global__ void __launch_bounds__(kThreads, 2)
    k_scatter_nodes(FixGeo g, SchemeT<float, N2> s, const uint32_t *__restrict__ cell_start,
                    const float4 *__restrict__ rec, const float *__restrict__ qs,
                    const unsigned *__restrict__ qmax_bits, float *__restrict__ field, float beta,
                    int beta_zero, int32_t *status, const uint32_t *__restrict__ list,
                    const uint32_t *__restrict__ list_n) {
  extern __shared__ __align__(16) unsigned char smem_scatter[];
  __shared__ uint32_t warp_tot[32];
  __shared__ float coef[N2 * GBG_MAX_POWERS];
  for (int i = threadIdx.x; i < N2 * s.m2; i += blockDim.x) coef[i] = s.c[i];
  __syncthreads();
  // a non-finite quantity propagates into the nodes it reaches; the status says so
  if (blockIdx.x == 0 && threadIdx.x == 0 && status && !isfinite(__uint_as_float(*qmax_bits)))
    atomicOr(status, GBG_DEV_NONFINITE);
  // the bricks to write: those a point reaches (beta == 1 leaves the others unchanged), or all
  const int64_t nunits = list ? (int64_t)__ldg(list_n) : g.nbricks;
  bool have = false;  // this brick's cell table was copied during the previous brick
  for (int64_t ui = blockIdx.x; ui < nunits; ui += gridDim.x) {
    const int64_t un = ui + gridDim.x;
    const int64_t next = (g.sparse || un >= nunits) ? -1 : (list ? (int64_t)__ldg(list + un) : un);
    have = scatter_brick_nodes<N2, FIXED, CP, CP == 4 ? 3 : 1>(g, coef, s.m2, list ? (int64_t)__ldg(list + ui) : ui, cell_start,
                                                        rec, qs, field, beta, beta_zero, list != nullptr, smem_scatter,
                                                        warp_tot, next, have);
  }
}

gbg_status check_field_bins(const gbg_field_s *f, const gbg_bins_s *b, const gbg_scheme *s) {
  if (!f || !b) return set_error(GBG_EARG, "null field or bins");
  GBG_TRY(s ? GBG_OK : set_error(GBG_EARG, "null scheme"));
  for (int d = 0; d < 3; ++d)
    if (f->grid.n[d] != b->grid.n[d] || f->grid.origin[d] != b->grid.origin[d] ||
        f->grid.domain[d] != b->grid.domain[d])
      return set_error(GBG_EARG, "the bins were built for a different grid than the field's");
  if (s->stencil_width > f->max_width)
    return set_error(GBG_EARG, "the scheme is wider than the field's ghost layer (max_stencil_width " +
                                   std::to_string(f->max_width) + ")");
  if (s->stencil_width < 2 || s->stencil_width % 2 || s->stencil_width > 8)
    return set_error(GBG_EUNSUPPORTED, "resident transfers take stencils of 2..8 nodes");
  if (s->num_powers < 1 || s->num_powers > GBG_MAX_POWERS) return set_error(GBG_EARG, "bad scheme powers");
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev != f->device || dev != b->device)
    return set_error(GBG_EARG, "the field, the bins and the current device must agree");
  return GBG_OK;
}

StagedGeo staged_geo(const gbg_field_s *f, const gbg_bins_s *b, int width) {
  StagedGeo g;
  for (int d = 0; d < 3; ++d) {
    g.b[d] = b->b[d];
    g.nb[d] = b->nb[d];
    g.w[d] = b->b[d] + width - 1;
  }
  g.box_off = f->halo - (width - 2) / 2;
  g.nbricks = b->nbricks;
  g.bvol = b->bvol;
  g.m = b->npoints;
  g.ncomp = f->ncomp;
  g.wait_polls = b->wait_polls ? b->wait_polls : kWaitPolls;
  return g;
}

// Average points per brick below which a gather reads the field directly (the direct
// kernels) instead of staging a tile per brick: at four points a brick a width-4 tile
// (brick + 3 cells) of a 15x8x8 brick is about 8x the bytes of the points' own stencils.
constexpr int64_t kDirectPerBrick = 4;

template <int N2, int M2, typename TO>
gbg_status launch_direct_gather(gbg_field_s *f, gbg_bins_s *b, const gbg_scheme &sch, TO *out, cudaStream_t st) {
  const StagedGeo g = staged_geo(f, b, N2);
  const SchemeT<float, N2> s = make_scheme<float, N2>(sch);
  int sms = 0, dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int64_t lanes = N2 == 4 ? 8 * b->npoints : b->npoints;  // a quarter-warp per width-4 point
  const int blocks = (int)std::max<int64_t>(1, std::min<int64_t>((lanes + kThreads - 1) / kThreads, (int64_t)sms * 8));
  mark_main_start(st);
  if constexpr (N2 == 4) {
    if (f->cp == 4)
      k_gather_direct4<M2, 4, TO><<<blocks, kThreads, 0, st>>>(g, s, f->data, f->px, f->py, b->rec, b->perm, b->keys, out);
    else
      k_gather_direct4<M2, 12, TO><<<blocks, kThreads, 0, st>>>(g, s, f->data, f->px, f->py, b->rec, b->perm, b->keys, out);
  } else {
    if (f->cp == 4)
      k_gather_direct<N2, M2, 4, TO><<<blocks, kThreads, 0, st>>>(g, s, f->data, f->px, f->py, b->rec, b->perm, b->keys, out);
    else
      k_gather_direct<N2, M2, 12, TO><<<blocks, kThreads, 0, st>>>(g, s, f->data, f->px, f->py, b->rec, b->perm, b->keys, out);
  }
  mark_main_stop(st);
  note_launch();
  GBG_CUDA_TRY(cudaGetLastError());
  return GBG_OK;
}

template <int N2, int M2, typename TO>
gbg_status launch_staged_gather(gbg_field_s *f, gbg_bins_s *b, const gbg_scheme &sch, TO *out, int32_t *status,
                                cudaStream_t st) {
  if (b->npoints < kDirectPerBrick * b->nbricks) return launch_direct_gather<N2, M2>(f, b, sch, out, st);
  CUtensorMap *map = nullptr;
  GBG_TRY(tensor_map_for(f, N2, b->b, &map));
  const StagedGeo g = staged_geo(f, b, N2);
  const SchemeT<float, N2> s = make_scheme<float, N2>(sch);
  // the copy's exact byte count (what the mbarrier expects) and the buffer stride
  const uint32_t box_bytes = (uint32_t)((size_t)f->cp * 4 * g.w[0] * g.w[1] * g.w[2]);
  const uint32_t tile_bytes = (box_bytes + 1023u) & ~1023u;
  if ((size_t)tile_bytes + 64 > 227 * 1024) return set_error(GBG_EUNSUPPORTED, "brick halo tile does not fit in shared memory");
  int sms = 0, dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int threads = b->gather_threads ? b->gather_threads : (N2 == 4 ? kGatherThreads : kThreads);
  auto go = [&](auto kernel) -> gbg_status {
    // Double-buffer the tile when that leaves as many CTAs per SM as a single buffer
    // would; otherwise (a large tile whose registers allow two CTAs) keep one buffer per
    // CTA and let the second CTA overlap the first one's copy.
    cudaFuncAttributes fa{};
    cudaFuncGetAttributes(&fa, kernel);
    const size_t smem_sm = 228 * 1024;
    const int by_regs = std::max(1, 65536 / std::max(1, fa.numRegs * threads));
    auto ctas = [&](int nb) {
      const size_t sm = (size_t)nb * tile_bytes + 64 + 1024;  // + the block's static/reserved share
      return std::min<int>(by_regs, (int)(smem_sm / sm));
    };
    const int nbuf = (2 * (size_t)tile_bytes + 64 <= 227 * 1024 && ctas(2) >= ctas(1)) ? 2 : 1;
    const size_t smem = (size_t)nbuf * tile_bytes + 64;
    GBG_CUDA_TRY(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int per_sm = 1;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, smem);
    const int blocks = (int)std::min<int64_t>(b->nbricks, (int64_t)sms * std::max(per_sm, 1));
    mark_main_start(st);
    kernel<<<blocks, threads, smem, st>>>(*map, g, s, b->cell_start, b->rec, b->perm, out, status, nbuf, tile_bytes,
                                           box_bytes, b->active, b->lists_n);
    mark_main_stop(st);
    note_launch();
    GBG_CUDA_TRY(cudaGetLastError());
    return GBG_OK;
  };
  if constexpr (N2 == 4) {
    if (f->cp == 4) return go(k_gather_staged4<M2, 4, TO>);
    return go(k_gather_staged4<M2, 12, TO>);
  } else {
    if (f->cp == 4) return go(k_gather_staged_generic<N2, M2, 4, TO>);
    return go(k_gather_staged_generic<N2, M2, 12, TO>);
  }
}

// True when, on every axis, the region a brick's nodes gather from (half a stencil either
// side) lies within the neighbouring bricks: full bricks and the last, partial one are at
// least half a stencil wide, or the axis is a single brick.
int32_t neighbour_skip_ok(const int32_t *b, const int64_t *nb, const int64_t *n, int width) {
  for (int d = 0; d < 3; ++d) {
    if (nb[d] == 1) continue;
    const int64_t last = n[d] - (nb[d] - 1) * b[d];
    if (b[d] < width / 2 || last < width / 2) return 0;
  }
  return 1;
}

// Sparse scatter, a warp per brick: for point sets with few points a brick the CTA-wide
// setup of a brick is mostly latency, so each warp takes a brick of its own.  It reads the
// point ranges of the 27 neighbouring bricks, keeps the points whose cells lie in the
// brick's region, puts them in region order (cell, then slot) and stages their weights and
// quantities; each lane then owns node quads and adds the staged points in that order,
// exactly as the CTA path does -- the same bits.  A brick with more candidates than a
// warp stages goes to the overflow list, which the CTA kernel takes afterwards.
constexpr uint32_t kWarpScan = 128, kWarpKeep = 32, kWarpMeta = 4 * kWarpKeep + 64;

template <int N2, int CP>
constexpr size_t sparse_warp_smem(int warps) {
  return (size_t)warps * (kWarpKeep * (CP + kScatterWStride<N2>) * sizeof(float) + kWarpMeta * sizeof(uint32_t));
}

template <int N2, bool FIXED, int CP>
__global__ void __launch_bounds__(kThreads)
    k_scatter_sparse(FixGeo g, SchemeT<float, N2> s, const uint32_t *__restrict__ cell_start,
                     const float4 *__restrict__ rec, const float *__restrict__ qs,
                     const unsigned *__restrict__ qmax_bits, float *__restrict__ field, float beta, int beta_zero,
                     int32_t *status, const uint32_t *__restrict__ list, const uint32_t *__restrict__ list_n,
                     uint32_t *__restrict__ overflow, uint32_t *__restrict__ overflow_n) {
  constexpr int W = kScatterWStride<N2>;
  constexpr int BY = N2 <= 6 ? 2 : 1, BZ = BY;
  constexpr int RY = N2 + BY - 1, RZ = N2 + BZ - 1;
  constexpr int half = N2 / 2;
  extern __shared__ __align__(16) unsigned char smem_sparse[];
  __shared__ float coef[N2 * GBG_MAX_POWERS];
  for (int i = threadIdx.x; i < N2 * s.m2; i += blockDim.x) coef[i] = s.c[i];
  __syncthreads();
  if (blockIdx.x == 0 && threadIdx.x == 0 && status && !isfinite(__uint_as_float(*qmax_bits)))
    atomicOr(status, GBG_DEV_NONFINITE);
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5, nwb = blockDim.x >> 5;
  float *sq = reinterpret_cast<float *>(smem_sparse) + (size_t)wib * kWarpKeep * (CP + W);
  float *sw = sq + kWarpKeep * CP;
  uint32_t *meta = reinterpret_cast<uint32_t *>(reinterpret_cast<float *>(smem_sparse) +
                                                (size_t)nwb * kWarpKeep * (CP + W)) + wib * kWarpMeta;
  uint32_t *ce = meta, *cs = ce + kWarpKeep, *re = cs + kWarpKeep, *rs = re + kWarpKeep;
  uint32_t *nst = rs + kWarpKeep, *npre = nst + 28;
  const int B0 = g.b[0], B1 = g.b[1], B2 = g.b[2];
  const int E0 = g.e[0], E1 = g.e[1], E2 = g.e[2];
  const int QY = (B1 + BY - 1) / BY, QZ = (B2 + BZ - 1) / BZ, nquads = B0 * QY * QZ;
  const uint32_t bvol = (uint32_t)g.bvol;
  const int64_t nunits = list ? (int64_t)__ldg(list_n) : g.nbricks;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t ui = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; ui < nunits; ui += nw) {
    const int64_t b = list ? (int64_t)__ldg(list + ui) : ui;
    const int bx = (int)(b % g.nb[0]), by = (int)((b / g.nb[0]) % g.nb[1]),
              bz = (int)(b / ((int64_t)g.nb[0] * g.nb[1]));
    // the 27 neighbours' point ranges (an axis of one brick has one neighbour, of two two)
    uint32_t a = 0, c = 0;
    if (lane < 27) {
      const int dx = lane % 3 - 1, dy = (lane / 3) % 3 - 1, dz = lane / 9 - 1;
      const bool dup = (g.nb[0] == 1 && dx != 0) || (g.nb[0] == 2 && dx < 0) || (g.nb[1] == 1 && dy != 0) ||
                       (g.nb[1] == 2 && dy < 0) || (g.nb[2] == 1 && dz != 0) || (g.nb[2] == 2 && dz < 0);
      if (!dup) {
        const uint64_t k = ((uint64_t)((bz + dz + g.nb[2]) % g.nb[2]) * (uint32_t)g.nb[1] +
                            (uint32_t)((by + dy + g.nb[1]) % g.nb[1])) * (uint32_t)g.nb[0] +
                           (uint32_t)((bx + dx + g.nb[0]) % g.nb[0]);
        a = __ldg(cell_start + k * bvol);
        c = __ldg(cell_start + (k + 1) * bvol) - a;
      }
    }
    uint32_t x = c;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    const uint32_t total = __shfl_sync(0xffffffffu, x, 31);
    if (lane < 27) {
      nst[lane] = a;
      npre[lane + 1] = x;
    }
    if (lane == 0) npre[0] = 0;
    __syncwarp();
    bool over = total > kWarpScan;
    uint32_t kept = 0;
    if (!over) {
      for (uint32_t t0 = 0; t0 < total; t0 += 32) {
        const uint32_t t = t0 + lane;
        bool keep = false;
        uint32_t e = 0, slot = 0;
        if (t < total) {
          int k = 0;
          while (k < 26 && npre[k + 1] <= t) ++k;
          slot = nst[k] + (t - npre[k]);
          int lx, ly, lz;
          unpack_local(__ldg(rec + slot).w, lx, ly, lz);
          const int dx = k % 3 - 1, dy = (k / 3) % 3 - 1, dz = k / 9 - 1;
          const int cx = ((bx + dx + g.nb[0]) % g.nb[0]) * B0 + lx;
          const int cy = ((by + dy + g.nb[1]) % g.nb[1]) * B1 + ly;
          const int cz = ((bz + dz + g.nb[2]) % g.nb[2]) * B2 + lz;
          int ex = (cx - (bx * B0 - half)) % g.n[0], ey = (cy - (by * B1 - half)) % g.n[1],
              ez = (cz - (bz * B2 - half)) % g.n[2];
          if (ex < 0) ex += g.n[0];
          if (ey < 0) ey += g.n[1];
          if (ez < 0) ez += g.n[2];
          keep = ex < E0 && ey < E1 && ez < E2;
          e = (uint32_t)((ez * E1 + ey) * E0 + ex);
        }
        const unsigned ballot = __ballot_sync(0xffffffffu, keep);
        const uint32_t pos = kept + __popc(ballot & ((1u << lane) - 1u));
        if (keep && pos < kWarpKeep) {
          re[pos] = e;
          rs[pos] = slot;
        }
        kept += __popc(ballot);
      }
      over = kept > kWarpKeep;
    }
    if (over) {
      if (lane == 0) overflow[atomicAdd(overflow_n, 1u)] = (uint32_t)b;
      continue;
    }
    __syncwarp();
    // region order: by cell, then slot (binned order within a cell)
    if ((uint32_t)lane < kept) {
      const uint32_t e = re[lane], sl = rs[lane];
      uint32_t rank = 0;
      for (uint32_t j = 0; j < kept; ++j) rank += (re[j] < e || (re[j] == e && rs[j] < sl)) ? 1u : 0u;
      ce[rank] = e;
      cs[rank] = sl;
    }
    __syncwarp();
    // stage the candidates: weights (x, then y and z each with a zero either side) and the
    // quantities, as the CTA path stages them
    int nonfinite = 0;
    if ((uint32_t)lane < kept) {
      const uint32_t sl = cs[lane];
      const float4 r = __ldg(rec + sl);
      float *wt = sw + lane * W;
      float w[N2];
      if constexpr (FIXED) weights_ptr<N2>(coef, r.x, w); else weights_rt<N2>(coef, s.m2, r.x, w);
#pragma unroll
      for (int q = 0; q < N2; ++q) wt[q] = w[q];
      if constexpr (FIXED) weights_ptr<N2>(coef, r.y, w); else weights_rt<N2>(coef, s.m2, r.y, w);
      wt[N2] = 0.0f;
#pragma unroll
      for (int q = 0; q < N2; ++q) wt[N2 + 1 + q] = w[q];
      wt[2 * N2 + 1] = 0.0f;
      if constexpr (FIXED) weights_ptr<N2>(coef, r.z, w); else weights_rt<N2>(coef, s.m2, r.z, w);
      wt[2 * N2 + 2] = 0.0f;
#pragma unroll
      for (int q = 0; q < N2; ++q) wt[2 * N2 + 3 + q] = w[q];
      wt[3 * N2 + 3] = 0.0f;
      const float4 *q4 = reinterpret_cast<const float4 *>(qs + (int64_t)sl * CP);
      float qa = 0.0f;
#pragma unroll
      for (int v = 0; v < CP / 4; ++v) {
        const float4 xq = __ldg(q4 + v);
        reinterpret_cast<float4 *>(sq + lane * CP)[v] = xq;
        qa += fabsf(xq.x) + fabsf(xq.y) + fabsf(xq.z) + fabsf(xq.w);
      }
      if (!isfinite(r.x + r.y + r.z + qa)) nonfinite = 1;
    }
    const bool exact = __any_sync(0xffffffffu, nonfinite);
    __syncwarp();
    const int vx = min(B0, g.n[0] - bx * B0), vy = min(B1, g.n[1] - by * B1), vz = min(B2, g.n[2] - bz * B2);
    for (int qi = lane; qi < nquads; qi += 32) {
      const int lx = qi % B0, ly = ((qi / B0) % QY) * BY, lz = (qi / (B0 * QY)) * BZ;
      float acc[BY * BZ][CP];
#pragma unroll
      for (int n = 0; n < BY * BZ; ++n)
#pragma unroll
        for (int cc = 0; cc < CP; ++cc) acc[n][cc] = 0.0f;
      const int xk = lx + N2 - 1;
      for (uint32_t t = 0; t < kept; ++t) {
        const uint32_t e = ce[t];
        const int ex = (int)(e % (uint32_t)E0), ey = (int)((e / (uint32_t)E0) % (uint32_t)E1),
                  ez = (int)(e / (uint32_t)(E0 * E1));
        const int jj = ey - ly, kk = ez - lz;
        if (ex < lx || ex > xk || jj < 0 || jj >= RY || kk < 0 || kk >= RZ) continue;
        const float *wp = sw + t * W;
        const float *wy = wp + (2 * N2 - jj), *wz = wp + (3 * N2 + 2 - kk);
        const float4 *qp = reinterpret_cast<const float4 *>(sq) + t * (CP / 4);
        const float wx = wp[xk - ex];
        float q[CP];
#pragma unroll
        for (int v = 0; v < CP / 4; ++v) {
          const float4 t4 = qp[v];
          q[4 * v] = t4.x;
          q[4 * v + 1] = t4.y;
          q[4 * v + 2] = t4.z;
          q[4 * v + 3] = t4.w;
        }
#pragma unroll
        for (int n = 0; n < BY * BZ; ++n) {
          const int aa = n % BY, bb = n / BY;
          if (exact && !(jj - aa >= 0 && jj - aa <= N2 - 1 && kk - bb >= 0 && kk - bb <= N2 - 1)) continue;
          const float wgt = (wx * wy[aa]) * wz[bb];
#pragma unroll
          for (int cc = 0; cc < CP; ++cc) acc[n][cc] = fmaf(wgt, q[cc], acc[n][cc]);
        }
      }
#pragma unroll
      for (int n = 0; n < BY * BZ; ++n) {
        const int ny = ly + n % BY, nz = lz + n / BY;
        if (ny >= B1 || nz >= B2 || lx >= vx || ny >= vy || nz >= vz) continue;
        const int64_t X = (int64_t)bx * B0 + lx, Y = (int64_t)by * B1 + ny, Z = (int64_t)bz * B2 + nz;
        float4 *d = reinterpret_cast<float4 *>(field + ((X + g.halo) + g.px * ((Y + g.halo) + g.py * (Z + g.halo))) * CP);
#pragma unroll
        for (int v4 = 0; v4 < CP / 4; ++v4) {
          float v[4];
#pragma unroll
          for (int u = 0; u < 4; ++u) v[u] = 4 * v4 + u < g.ncomp ? acc[n][4 * v4 + u] : 0.0f;
          if (beta_zero) {
            d[v4] = make_float4(v[0], v[1], v[2], v[3]);
          } else {
            const float4 o = d[v4];
            d[v4] = make_float4(__fadd_rn(__fmul_rn(beta, o.x), v[0]), __fadd_rn(__fmul_rn(beta, o.y), v[1]),
                                __fadd_rn(__fmul_rn(beta, o.z), v[2]), __fadd_rn(__fmul_rn(beta, o.w), v[3]));
          }
        }
      }
    }
    __syncwarp();  // the warp's staging is free for its next brick
  }
}

template <int N2, bool FIXED>
gbg_status launch_staged_scatter(gbg_field_s *f, gbg_bins_s *b, const gbg_scheme &sch, double beta,
                                 const unsigned *qmax_bits, int32_t *status, cudaStream_t st) {
  FixGeo g;
  for (int d = 0; d < 3; ++d) {
    g.b[d] = b->b[d];
    g.nb[d] = (int32_t)b->nb[d];
    g.n[d] = (int32_t)f->grid.n[d];
    g.e[d] = b->b[d] + N2 - 1;
  }
  g.neighbour_skip = neighbour_skip_ok(b->b, b->nb, f->grid.n, N2);
  g.comp = b->compensated;
  g.cscratch = b->cscratch;
  g.sparse = scatter_sparse(b, f->grid, N2);
  g.cstride = b->bvol * 12;
  g.nbricks = b->nbricks;
  g.bvol = b->bvol;
  g.px = f->px;
  g.py = f->py;
  g.halo = f->halo;
  g.cp = f->cp;
  g.ncomp = f->ncomp;
  const SchemeT<float, N2> s = make_scheme<float, N2>(sch);
  if (g.e[0] > 255) return set_error(GBG_EUNSUPPORTED, "brick too large for the scatter");
  int sms = 0, dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int threads = b->scatter_threads ? b->scatter_threads : kThreads;
  const bool reach = beta == 1.0 && b->reach_ok;
  auto go = [&](auto kernel) -> gbg_status {
    scatter_nodes_chunk(g, f->cp, N2, scatter_nodes_budget(g, f->cp, N2));
    const size_t smem = scatter_nodes_smem(g, f->cp, N2);
    if (smem > 227 * 1024) return set_error(GBG_EUNSUPPORTED, "brick too large for the scatter's shared memory");
    GBG_CUDA_TRY(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    GBG_CUDA_TRY(cudaFuncSetAttribute(kernel, cudaFuncAttributePreferredSharedMemoryCarveout, 100));
    int per_sm = 1;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, smem);
    const int blocks = (int)std::min<int64_t>(b->cslots, (int64_t)sms * std::max(per_sm, 1));
    mark_main_start(st);
    kernel<<<blocks, threads, smem, st>>>(g, s, b->cell_start, b->rec, b->qs, qmax_bits, f->data, (float)beta,
                                           beta == 0.0, status, reach ? b->reach : nullptr, b->lists_n + 1);
    mark_main_stop(st);
    note_launch();
    GBG_CUDA_TRY(cudaGetLastError());
    return GBG_OK;
  };
  if (g.sparse) {
    // the warp kernel over every brick (or the bricks a point reaches), then the CTA kernel
    // over the bricks it passed on
    GBG_CUDA_TRY(cudaMemsetAsync(b->lists_n + 3, 0, sizeof(uint32_t), st));
    auto sp = [&](auto kernel, size_t smem) -> gbg_status {
      GBG_CUDA_TRY(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
      int per_sm = 1;
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kThreads, smem);
      // a warp per brick; the list of bricks in reach, when there is one, may hold fewer
      const int blocks = (int)std::max<int64_t>(1, std::min<int64_t>((b->nbricks + 7) / 8, (int64_t)sms * std::max(per_sm, 1)));
      kernel<<<blocks, kThreads, smem, st>>>(g, s, b->cell_start, b->rec, b->qs, qmax_bits, f->data, (float)beta,
                                              beta == 0.0, status, reach ? b->reach : nullptr, b->lists_n + 1,
                                              b->overflow, b->lists_n + 3);
      note_launch();
      GBG_CUDA_TRY(cudaGetLastError());
      return GBG_OK;
    };
    mark_main_start(st);
    if (f->cp == 4) GBG_TRY(sp(k_scatter_sparse<N2, FIXED, 4>, sparse_warp_smem<N2, 4>(kThreads / 32)));
    else GBG_TRY(sp(k_scatter_sparse<N2, FIXED, 12>, sparse_warp_smem<N2, 12>(kThreads / 32)));
    auto over = [&](auto kernel) -> gbg_status {
      scatter_nodes_chunk(g, f->cp, N2, scatter_nodes_budget(g, f->cp, N2));
      const size_t smem = scatter_nodes_smem(g, f->cp, N2);
      if (smem > 227 * 1024) return set_error(GBG_EUNSUPPORTED, "brick too large for the scatter's shared memory");
      GBG_CUDA_TRY(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
      GBG_CUDA_TRY(cudaFuncSetAttribute(kernel, cudaFuncAttributePreferredSharedMemoryCarveout, 100));
      int per_sm = 1;
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, smem);
      const int blocks = (int)std::min<int64_t>(b->cslots, (int64_t)sms * std::max(per_sm, 1));
      kernel<<<blocks, threads, smem, st>>>(g, s, b->cell_start, b->rec, b->qs, qmax_bits, f->data, (float)beta,
                                             beta == 0.0, status, b->overflow, b->lists_n + 3);
      note_launch();
      GBG_CUDA_TRY(cudaGetLastError());
      return GBG_OK;
    };
    if (f->cp == 4) GBG_TRY(over(k_scatter_nodes<N2, FIXED, 4>));
    else GBG_TRY(over(k_scatter_nodes<N2, FIXED, 12>));
    mark_main_stop(st);
    return GBG_OK;
  }
  if (f->cp == 4) return go(k_scatter_nodes<N2, FIXED, 4>);
  return go(k_scatter_nodes<N2, FIXED, 12>);
}

// ------------------------------------------------------------ batched form
//
// One persistent launch for the gathers of every instance and one for the scatters.  The
// work list holds (instance, brick) units, largest instances first; CTAs take units from
// a device counter.  The gather keeps one TMA tile in flight ahead of the one it computes.

struct BatchDev {
  StagedGeo g;   // gather geometry (tile = brick + width - 1)
  FixGeo fg;     // scatter geometry
  const uint32_t *cell_start;
  const float4 *rec;
  const uint32_t *perm;
  float *out;    // gather output or null
  float *dest;   // scatter destination storage or null
  const float *qs;
  const unsigned *qmax_bits;
  // the bricks each launch visits: a list and its length on the device, or null for all
  const uint32_t *glist, *gcount, *slist, *scount;
  float coef[8 * 8];  // [q + n2*p], n2 == m2 <= 8
  int32_t n2, cp;
  uint32_t box_bytes;
  float beta;
  int32_t beta_zero;
};

constexpr int kBatchGatherThreads = 512;

// Work unit u of a batch launch -> (instance, brick): the k-th instance in cost order,
// idx[k], owns the units [off[k], off[k+1]) (off[0] = 0, u < off[n]); its j-th unit is
// the j-th brick of its list (gather: the bricks holding points; scatter: the bricks in
// reach of a point when beta == 1), or brick j when it has no list.
template <bool SCATTER>
__device__ __forceinline__ uint2 batch_unit(const BatchDev *__restrict__ items, uint32_t u,
                                            const uint32_t *__restrict__ off, const uint32_t *__restrict__ idx,
                                            int n) {
  int lo = 0, hi = n;
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (__ldg(off + mid) <= u) lo = mid; else hi = mid;
  }
  const uint32_t i = __ldg(idx + lo), j = u - __ldg(off + lo);
  const uint32_t *list = SCATTER ? items[i].slist : items[i].glist;
  return make_uint2(i, list ? __ldg(list + j) : j);
}

// The points of one brick, from its staged tile: a point per quarter-warp (width 4) or
// per thread (other widths), as in the single-instance kernels.
template <int N2, int CP>
__device__ void batch_gather_points(const BatchDev *d, const float *tile, uint32_t s0, uint32_t s1) {
  const StagedGeo &g = d->g;
  if constexpr (N2 == 4) {
    const int lane = threadIdx.x & 31, sub = lane & 7, qi = sub & 3, jj = sub >> 2;
    const unsigned seg_mask = 0xFFu << (lane & ~7);
    for (uint32_t sl = s0 + (threadIdx.x >> 3); sl < s1; sl += kBatchGatherThreads / 8) {
      const float4 r = __ldg(d->rec + sl);
      const int64_t p = __ldg(d->perm + sl);
      int lx, ly, lz;
      unpack_local(r.w, lx, ly, lz);
      float wx[4], wy[4], w3[4];
      weights_ptr<4>(d->coef, r.x, wx);
      weights_ptr<4>(d->coef, r.y, wy);
      weights_ptr<4>(d->coef, r.z, w3);
      const float w1 = pick(wx, qi), w2a = pick(wy, 2 * jj), w2b = pick(wy, 2 * jj + 1);
      float acc[CP];
#pragma unroll
      for (int c = 0; c < CP; ++c) acc[c] = 0.0f;
      const int node0 = (lz * g.w[1] + ly + 2 * jj) * g.w[0] + lx + qi;
#pragma unroll
      for (int k = 0; k < 4; ++k)
#pragma unroll
        for (int jp = 0; jp < 2; ++jp) {
          const float w = w1 * (jp ? w2b : w2a) * w3[k];
          const float4 *pv = reinterpret_cast<const float4 *>(tile + (node0 + (k * g.w[1] + jp) * g.w[0]) * CP);
#pragma unroll
          for (int q4 = 0; q4 < CP / 4; ++q4) {
            const float4 v = pv[q4];
            acc[4 * q4 + 0] = fmaf(w, v.x, acc[4 * q4 + 0]);
            acc[4 * q4 + 1] = fmaf(w, v.y, acc[4 * q4 + 1]);
            acc[4 * q4 + 2] = fmaf(w, v.z, acc[4 * q4 + 2]);
            acc[4 * q4 + 3] = fmaf(w, v.w, acc[4 * q4 + 3]);
          }
        }
      constexpr int H = CP / 2, Q = CP / 4;
      const bool up2 = sub & 4, up1 = sub & 2;
      float h[H];
#pragma unroll
      for (int v = 0; v < H; ++v) {
        const float keep = up2 ? acc[H + v] : acc[v], give = up2 ? acc[v] : acc[H + v];
        h[v] = keep + __shfl_xor_sync(seg_mask, give, 4, 8);
      }
      float qv[Q];
#pragma unroll
      for (int v = 0; v < Q; ++v) {
        const float keep = up1 ? h[Q + v] : h[v], give = up1 ? h[v] : h[Q + v];
        qv[v] = keep + __shfl_xor_sync(seg_mask, give, 2, 8);
      }
#pragma unroll
      for (int v = 0; v < Q; ++v) qv[v] += __shfl_xor_sync(seg_mask, qv[v], 1, 8);
      if ((sub & 1) == 0) {
        const int cbase = (up2 ? H : 0) + (up1 ? Q : 0);
#pragma unroll
        for (int v = 0; v < Q; ++v)
          if (cbase + v < g.ncomp) d->out[p + g.m * (cbase + v)] = qv[v];
      }
    }
  } else {
    for (uint32_t sl = s0 + threadIdx.x; sl < s1; sl += kBatchGatherThreads) {
      const float4 r = __ldg(d->rec + sl);
      int lx, ly, lz;
      unpack_local(r.w, lx, ly, lz);
      float w1[N2], w2[N2], w3[N2];
      weights_ptr<N2>(d->coef, r.x, w1);
      weights_ptr<N2>(d->coef, r.y, w2);
      weights_ptr<N2>(d->coef, r.z, w3);
      float acc[CP];
#pragma unroll
      for (int c = 0; c < CP; ++c) acc[c] = 0.0f;
#pragma unroll 1
      for (int k = 0; k < N2; ++k) {
        const float w3k = pick(w3, k);
#pragma unroll
        for (int j = 0; j < N2; ++j) {
          const float wyz = w2[j] * w3k;
          const float *row = tile + (((lz + k) * g.w[1] + ly + j) * g.w[0] + lx) * CP;
#pragma unroll
          for (int i = 0; i < N2; ++i) {
            const float w = wyz * w1[i];
            const float4 *pv = reinterpret_cast<const float4 *>(row + i * CP);
#pragma unroll
            for (int q4 = 0; q4 < CP / 4; ++q4) {
              const float4 v = pv[q4];
              acc[4 * q4 + 0] = fmaf(w, v.x, acc[4 * q4 + 0]);
              acc[4 * q4 + 1] = fmaf(w, v.y, acc[4 * q4 + 1]);
              acc[4 * q4 + 2] = fmaf(w, v.z, acc[4 * q4 + 2]);
              acc[4 * q4 + 3] = fmaf(w, v.w, acc[4 * q4 + 3]);
            }
          }
        }
      }
      const int64_t p = __ldg(d->perm + sl);
#pragma unroll
      for (int c = 0; c < CP; ++c)
        if (c < g.ncomp) d->out[p + g.m * c] = acc[c];
    }
  }
}

__device__ __forceinline__ bool batch_issue(const BatchDev *items, const CUtensorMap *maps, uint2 u, void *dst,
                                            uint64_t *bar) {
  const BatchDev *d = items + u.x;
  const int64_t b = u.y;
  if (!d->out) return false;
  if (__ldg(d->cell_start + (b + 1) * d->g.bvol) <= __ldg(d->cell_start + b * d->g.bvol)) return false;
  int64_t bx, by, bz;
  brick_coords(d->g, b, bx, by, bz);
  mbar_expect_tx(bar, d->box_bytes);
  tma_load_tile(dst, maps + u.x, 0, (int)(bx * d->g.b[0]) + d->g.box_off, (int)(by * d->g.b[1]) + d->g.box_off,
                (int)(bz * d->g.b[2]) + d->g.box_off, bar);
  return true;
}

__global__ void __launch_bounds__(kBatchGatherThreads, 1)
    k_batch_gather(const BatchDev *__restrict__ items, const CUtensorMap *__restrict__ maps,
                   const uint32_t *__restrict__ off, const uint32_t *__restrict__ idx, int n,
                   uint32_t *counter, uint32_t buf_bytes, int nbuf, int32_t *status) {
  extern __shared__ __align__(1024) unsigned char smem[];
  const uint32_t nwork = off[n];
  uint64_t *bars = reinterpret_cast<uint64_t *>(smem + nbuf * buf_bytes);
  __shared__ uint32_t s_unit[2];
  __shared__ int s_issued[2];
  if (threadIdx.x == 0) {
    mbar_init(bars, 1);
    mbar_init(bars + 1, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    const uint32_t u = atomicAdd(counter, 1u);
    s_unit[0] = u;
    s_issued[0] = u < nwork ? batch_issue(items, maps, batch_unit<false>(items, u, off, idx, n), smem, bars) : 0;
  }
  __syncthreads();
  uint32_t phase[2] = {0, 0};
  int buf = 0;
  bool failed = false;
  while (true) {
    const uint32_t u = s_unit[buf];
    if (u >= nwork) break;
    if (nbuf == 2 && threadIdx.x == 0) {
      const uint32_t un = atomicAdd(counter, 1u);
      s_unit[buf ^ 1] = un;
      s_issued[buf ^ 1] =
          un < nwork ? batch_issue(items, maps, batch_unit<false>(items, un, off, idx, n), smem + (buf ^ 1) * buf_bytes, bars + (buf ^ 1))
                     : 0;
    }
    if (s_issued[buf]) {
      if (__syncthreads_or(!mbar_wait(bars + buf, phase[buf]))) {
        failed = true;
        if (threadIdx.x == 0 && status) atomicOr(status, GBG_DEV_TIMEOUT);
        break;
      }
      phase[buf] ^= 1;
      const uint2 wu = batch_unit<false>(items, u, off, idx, n);
      const BatchDev *d = items + wu.x;
      const uint32_t s0 = __ldg(d->cell_start + (int64_t)wu.y * d->g.bvol);
      const uint32_t s1 = __ldg(d->cell_start + ((int64_t)wu.y + 1) * d->g.bvol);
      const float *tile = reinterpret_cast<const float *>(smem + buf * buf_bytes);
      const int kind = d->n2 * 100 + d->cp;
      switch (kind) {
        case 404: batch_gather_points<4, 4>(d, tile, s0, s1); break;
        case 412: batch_gather_points<4, 12>(d, tile, s0, s1); break;
        case 604: batch_gather_points<6, 4>(d, tile, s0, s1); break;
        case 612: batch_gather_points<6, 12>(d, tile, s0, s1); break;
        case 204: batch_gather_points<2, 4>(d, tile, s0, s1); break;
        case 212: batch_gather_points<2, 12>(d, tile, s0, s1); break;
        case 804: batch_gather_points<8, 4>(d, tile, s0, s1); break;
        default: batch_gather_points<8, 12>(d, tile, s0, s1); break;
      }
    }
    __syncthreads();
    if (nbuf == 1) {
      if (threadIdx.x == 0) {
        const uint32_t un = atomicAdd(counter, 1u);
        s_unit[0] = un;
        s_issued[0] = un < nwork ? batch_issue(items, maps, batch_unit<false>(items, un, off, idx, n), smem, bars) : 0;
      }
      __syncthreads();
    } else {
      buf ^= 1;
    }
  }
  if (failed && threadIdx.x == 0)
    for (int i = 0; i < nbuf; ++i)
      if (s_issued[i]) mbar_wait(bars + i, phase[i]);
}

// The scatter of every listed brick of every instance: units taken from the device counter.
__global__ void __launch_bounds__(kThreads, 2)
    k_batch_scatter(const BatchDev *__restrict__ items, const uint32_t *__restrict__ off,
                    const uint32_t *__restrict__ idx, int n, uint32_t *counter, int32_t *status) {
  extern __shared__ __align__(16) unsigned char bsmem[];
  const uint32_t nwork = off[n];
  __shared__ uint32_t s_u;
  __shared__ uint32_t warp_tot[32];
  while (true) {
    if (threadIdx.x == 0) s_u = atomicAdd(counter, 1u);
    __syncthreads();
    const uint32_t u = s_u;
    __syncthreads();
    if (u >= nwork) break;
    const uint2 wu = batch_unit<true>(items, u, off, idx, n);
    const BatchDev *d = items + wu.x;
    if (threadIdx.x == 0 && status && !isfinite(__uint_as_float(*d->qmax_bits))) atomicOr(status, GBG_DEV_NONFINITE);
    const int kind = d->n2 * 100 + d->cp;
#define GBG_BATCH_SCATTER(N2, CP)                                                                          \
  scatter_brick_nodes<N2, true, CP, 1>(d->fg, d->coef, N2, wu.y, d->cell_start, d->rec, d->qs, d->dest, d->beta, \
                                    d->beta_zero, d->slist != nullptr, bsmem, warp_tot)
    switch (kind) {
      case 404: GBG_BATCH_SCATTER(4, 4); break;
      case 412: GBG_BATCH_SCATTER(4, 12); break;
      case 604: GBG_BATCH_SCATTER(6, 4); break;
      case 612: GBG_BATCH_SCATTER(6, 12); break;
      case 204: GBG_BATCH_SCATTER(2, 4); break;
      case 212: GBG_BATCH_SCATTER(2, 12); break;
      case 804: GBG_BATCH_SCATTER(8, 4); break;
      default: GBG_BATCH_SCATTER(8, 12); break;
    }
#undef GBG_BATCH_SCATTER
  }
}

// Flat index over every destination's points (quantity preparation): item i owns
// [offsets[i], offsets[i+1]).  Each thread keeps a running max per item and flushes it
// with one atomic when its item changes.
__global__ void k_batch_qprep(const BatchDev *__restrict__ items, const float *const *__restrict__ qptrs,
                              const int64_t *__restrict__ offsets, int32_t count, float *const *qs_out,
                              const float *__restrict__ alphas, unsigned *const *qmax_out) {
  const int64_t total = offsets[count];
  unsigned mx = 0u;
  int cur = -1;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    int lo = 0, hi = count;
    while (hi - lo > 1) {
      const int mid = (lo + hi) / 2;
      if (offsets[mid] <= t) lo = mid; else hi = mid;
    }
    if (lo != cur) {
      if (cur >= 0) atomicMax(qmax_out[cur], mx);
      cur = lo;
      mx = 0u;
    }
    const BatchDev *d = items + lo;
    const int64_t s = t - offsets[lo];
    const int64_t m = d->g.m;
    const int64_t p = d->perm[s];
    const int cp = d->cp, nc = d->g.ncomp;
    for (int c = 0; c < cp; ++c) {
      const float v = c < nc ? alphas[lo] * qptrs[lo][p + m * c] : 0.0f;
      qs_out[lo][s * cp + c] = v;
      const unsigned bits = __float_as_uint(fabsf(v));
      mx = bits > mx ? bits : mx;
    }
  }
  if (cur >= 0) atomicMax(qmax_out[cur], mx);
}

// Resets the batch's unit counters and the max|alpha q| word of every destination, and
// lays out the work units: off[k] = the units of the instances before the k-th in cost
// order, from the list lengths the bins' builds left on the device.  One block.
__global__ void k_batch_reset(const BatchDev *__restrict__ items, uint32_t *counters, unsigned *const *qmax_out,
                              int32_t count, const uint32_t *__restrict__ gidx, int32_t ng, uint32_t *goff,
                              const uint32_t *__restrict__ sidx, int32_t ns, uint32_t *soff) {
  __shared__ uint32_t warp_tot[32];
  for (int i = threadIdx.x; i < count; i += blockDim.x)
    if (qmax_out[i]) *qmax_out[i] = 0u;
  if (threadIdx.x < 2) counters[threadIdx.x] = 0u;
  for (int k = threadIdx.x; k <= ng; k += blockDim.x) {
    const BatchDev *d = items + gidx[k < ng ? k : 0];
    goff[k] = k == ng ? 0u : d->glist ? *d->gcount : (uint32_t)d->g.nbricks;
  }
  for (int k = threadIdx.x; k <= ns; k += blockDim.x) {
    const BatchDev *d = items + sidx[k < ns ? k : 0];
    soff[k] = k == ns ? 0u : d->slist ? *d->scount : (uint32_t)d->fg.nbricks;
  }
  __syncthreads();
  block_scan_counts(goff, ng + 1, warp_tot);
  block_scan_counts(soff, ns + 1, warp_tot);
}

}  // namespace
}  // namespace gbg

using namespace gbg;

namespace gbg {

// Geometry and byte count of new bins (no device memory is touched).
gbg_status bins_plan(const gbg_grid &grid, int64_t max_points, const int32_t *brick, gbg_bins_s *b) {
  if (max_points < 0 || max_points > 0x7fffffffLL) return set_error(GBG_EUNSUPPORTED, "point count outside 0..2^31-1");
  cudaGetDevice(&b->device);
  b->grid = grid;
  b->max_points = max_points;
  for (int d = 0; d < 3; ++d) {
    if (brick && brick[d] != 0) b->b[d] = brick[d];
    if (b->b[d] < 1 || b->b[d] > 64) return set_error(GBG_EARG, "brick edges must be 1..64 cells");
    b->nb[d] = (grid.n[d] + b->b[d] - 1) / b->b[d];
  }
  b->bvol = (int64_t)b->b[0] * b->b[1] * b->b[2];
  b->nbricks = b->nb[0] * b->nb[1] * b->nb[2];
  b->nkeys = b->nbricks * b->bvol;
  if (b->nkeys >= (int64_t(1) << 32) - 1) return set_error(GBG_EUNSUPPORTED, "bins: 2^32 or more cells");
  b->reach_ok = neighbour_skip_ok(b->b, b->nb, grid.n, 8) != 0;
  b->cslots = (int32_t)std::min<int64_t>(b->nbricks, (int64_t)kScatterSlotsPerSM * device_sms());
  Arena a;
  bins_layout(a, b);
  b->bytes = a.used + 256;
  return GBG_OK;
}

// Carves the device block of planned bins into its arrays.
void bins_carve(gbg_bins_s *b) {
  Arena a;
  a.base = static_cast<char *>(b->block);
  bins_layout(a, b);
}

gbg_status field_info(gbg_field f, gbg_grid *grid, int32_t *ncomp, int32_t *max_width) {
  if (!f) return set_error(GBG_EARG, "null field");
  if (grid) *grid = f->grid;
  if (ncomp) *ncomp = f->ncomp;
  if (max_width) *max_width = f->max_width;
  return GBG_OK;
}

size_t bins_bytes(const gbg_grid &grid, int64_t max_points, const int32_t *brick) {
  gbg_bins_s b;
  return bins_plan(grid, max_points, brick, &b) == GBG_OK ? b.bytes : 0;
}

gbg_status bins_create_async(const gbg_grid &grid, int64_t max_points, const int32_t *brick, cudaStream_t stream,
                             gbg_bins *out, size_t *bytes) {
  auto *b = new (std::nothrow) gbg_bins_s;
  if (!b) return set_error(GBG_ENOMEM, "host allocation failed");
  gbg_status st = bins_plan(grid, max_points, brick, b);
  if (st) {
    delete b;
    return st;
  }
  if (cudaMallocAsync(&b->block, b->bytes, stream) != cudaSuccess) {
    cudaGetLastError();
    delete b;
    return set_error(GBG_ENOMEM, "cudaMallocAsync of the bins failed");
  }
  bins_carve(b);
  b->async = true;
  if (bytes) *bytes = b->bytes;
  *out = b;
  return GBG_OK;
}

gbg_status bins_destroy_async(gbg_bins b, cudaStream_t stream) {
  if (!b) return GBG_OK;
  const cudaError_t e = b->async ? cudaFreeAsync(b->block, stream) : cudaFree(b->block);
  delete b;
  if (e != cudaSuccess) return set_error(GBG_ECUDA, std::string("freeing the bins: ") + cudaGetErrorString(e));
  return GBG_OK;
}

}  // namespace gbg

extern "C" {

gbg_status gbg_field_create(const gbg_grid *grid, int32_t ncomp, gbg_dtype storage_dtype,
                            int32_t max_stencil_width, gbg_field *out) {
  clear_error();
  if (!grid || !out) return set_error(GBG_EARG, "null argument");
  if (storage_dtype != GBG_F32) return set_error(GBG_EUNSUPPORTED, "resident storage is Float32 in this build");
  if (ncomp < 1 || ncomp > 12) return set_error(GBG_EUNSUPPORTED, "resident fields hold 1..12 components");
  if (max_stencil_width < 2 || max_stencil_width % 2 || max_stencil_width > 8)
    return set_error(GBG_EARG, "max_stencil_width must be even, 2..8");
  for (int d = 0; d < 3; ++d)
    if (grid->n[d] < max_stencil_width)
      return set_error(GBG_EUNSUPPORTED, "resident fields need at least max_stencil_width nodes per axis");
  auto *f = new (std::nothrow) gbg_field_s;
  if (!f) return set_error(GBG_ENOMEM, "host allocation failed");
  cudaGetDevice(&f->device);
  f->grid = *grid;
  f->ncomp = ncomp;
  f->cp = padded_components(ncomp);
  f->max_width = max_stencil_width;
  f->halo = max_stencil_width / 2 - 1;
  f->px = grid->n[0] + 2 * f->halo + 1;
  f->py = grid->n[1] + 2 * f->halo + 1;
  f->pz = grid->n[2] + 2 * f->halo + 1;
  f->bytes = sizeof(float) * (size_t)f->cp * f->px * f->py * f->pz;
  if (cudaMalloc(&f->data, f->bytes) != cudaSuccess) {
    cudaGetLastError();
    delete f;
    return set_error(GBG_ENOMEM, "cudaMalloc of the field storage failed");
  }
  cudaMemset(f->data, 0, f->bytes);
  *out = f;
  return GBG_OK;
}

gbg_status gbg_field_destroy(gbg_field f) {
  clear_error();
  if (!f) return GBG_OK;
  cudaFree(f->data);
  delete f;
  return GBG_OK;
}

gbg_status gbg_field_bytes(gbg_field f, size_t *bytes) {
  if (!f || !bytes) return set_error(GBG_EARG, "null argument");
  *bytes = f->bytes;
  return GBG_OK;
}

gbg_status gbg_field_import(gbg_field f, gbg_dtype src_dtype, const void *src, void *stream) {
  clear_error();
  if (!f || !src) return set_error(GBG_EARG, "null argument");
  if (src_dtype != GBG_F32 && src_dtype != GBG_F64) return set_error(GBG_EARG, "bad dtype");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const int64_t total = f->px * f->py * f->pz;
  k_import<<<launch_blocks(total, kThreads), kThreads, 0, st>>>(f->data, f->cp, f->ncomp, f->px, f->py, f->pz, f->halo,
                                                                f->grid.n[0], f->grid.n[1], f->grid.n[2], src,
                                                                src_dtype == GBG_F64);
  note_launch();
  GBG_CUDA_TRY(cudaGetLastError());
  return GBG_OK;
}

gbg_status gbg_field_export(gbg_field f, gbg_dtype dst_dtype, void *dst, void *stream) {
  clear_error();
  if (!f || !dst) return set_error(GBG_EARG, "null argument");
  if (dst_dtype != GBG_F32 && dst_dtype != GBG_F64) return set_error(GBG_EARG, "bad dtype");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const int64_t npf = f->grid.n[0] * f->grid.n[1] * f->grid.n[2];
  k_export<<<launch_blocks(npf, kThreads), kThreads, 0, st>>>(f->data, f->cp, f->ncomp, f->px, f->py, f->halo,
                                                              f->grid.n[0], f->grid.n[1], f->grid.n[2], dst,
                                                              dst_dtype == GBG_F64);
  note_launch();
  GBG_CUDA_TRY(cudaGetLastError());
  return GBG_OK;
}

gbg_status gbg_bins_create(const gbg_grid *grid, int64_t max_points, const int32_t *brick, gbg_bins *out) {
  clear_error();
  if (!grid || !out) return set_error(GBG_EARG, "null argument");
  auto *b = new (std::nothrow) gbg_bins_s;
  if (!b) return set_error(GBG_ENOMEM, "host allocation failed");
  gbg_status st = bins_plan(*grid, max_points, brick, b);
  if (st) {
    delete b;
    return st;
  }
  if (cudaMalloc(&b->block, b->bytes) != cudaSuccess) {
    cudaGetLastError();
    delete b;
    return set_error(GBG_ENOMEM, "cudaMalloc of the bins failed");
  }
  bins_carve(b);
  cudaMemset(b->cell_start, 0, sizeof(uint32_t) * ((size_t)b->nkeys + 1));
  if (gbg_status e = side_pool_ready()) {
    cudaFree(b->block);
    delete b;
    return e;
  }
  *out = b;
  return GBG_OK;
}

gbg_status gbg_bins_set_wait_limit(gbg_bins b, uint32_t polls) {
  clear_error();
  if (!b) return set_error(GBG_EARG, "null bins");
  b->wait_polls = polls;
  return GBG_OK;
}

gbg_status gbg_bins_set_compensated(gbg_bins b, int32_t compensated) {
  clear_error();
  if (!b) return set_error(GBG_EARG, "null bins");
  b->compensated = compensated ? 1 : 0;
  return GBG_OK;
}

gbg_status gbg_bins_set_sparse_regions(gbg_bins b, int32_t allow) {
  clear_error();
  if (!b) return set_error(GBG_EARG, "null bins");
  b->sparse_regions = allow ? 1 : 0;
  return GBG_OK;
}

gbg_status gbg_bins_set_launch(gbg_bins b, int32_t gather_threads, int32_t scatter_threads) {
  clear_error();
  if (!b) return set_error(GBG_EARG, "null bins");
  if (gather_threads != 0 && gather_threads != 128 && gather_threads != 256 && gather_threads != 512)
    return set_error(GBG_EARG, "gather_threads must be 0, 128, 256 or 512");
  if (scatter_threads != 0 && scatter_threads != 64 && scatter_threads != 128 && scatter_threads != 256)
    return set_error(GBG_EARG, "scatter_threads must be 0, 64, 128 or 256");
  b->gather_threads = gather_threads;
  b->scatter_threads = scatter_threads;
  return GBG_OK;
}

gbg_status gbg_bins_destroy(gbg_bins b) {
  clear_error();
  if (!b) return GBG_OK;
  cudaFree(b->block);
  delete b;
  return GBG_OK;
}

}  // extern "C"

namespace gbg {
namespace {

// Fills the displacement arguments (C ABI terms converted to the positions' type).
template <typename T>
gbg_status make_displace(DisplaceArgs<T> &a, const gbg_grid *grid, T *dst, const T *src, int32_t nterms,
                         const double *coefficients, const void *const *sections) {
  if (nterms < 0 || nterms > GBG_MAX_TERMS)
    return set_error(GBG_EUNSUPPORTED, "displacement: 0.." + std::to_string(GBG_MAX_TERMS) + " terms per call");
  if (nterms > 0 && (!coefficients || !sections)) return set_error(GBG_EARG, "null displacement terms");
  a = DisplaceArgs<T>{};
  a.src = src;
  a.dst = dst;
  a.nterms = nterms;
  for (int j = 0; j < nterms; ++j) {
    if (!sections[j]) return set_error(GBG_EARG, "null displacement section");
    a.sec[j] = static_cast<const T *>(sections[j]);
    a.coef[j] = T(coefficients[j]);
  }
  a.wrap = grid != nullptr;
  for (int d = 0; d < 3; ++d) {
    a.extent[d] = grid ? T(grid->domain[d]) : T(1);
    a.origin[d] = grid ? T(grid->origin[d]) : T(0);
    if (grid && !(a.extent[d] > T(0) && isfinite((double)a.extent[d]) && isfinite((double)a.origin[d])))
      return set_error(GBG_EARG, "displacement: the domain must be finite and positive");
  }
  return GBG_OK;
}

template <typename T>
gbg_status bins_build_impl(gbg_bins_s *b, const T *positions, int64_t npoints, int32_t *device_status,
                           cudaStream_t st, const DisplaceArgs<T> *disp) {
  b->npoints = npoints;
  GBG_CUDA_TRY(cudaMemsetAsync(b->cell_start, 0, sizeof(uint32_t) * ((size_t)b->nkeys + 1), st));
  // the two work-list lengths and the counting sort's long-run flag
  GBG_CUDA_TRY(cudaMemsetAsync(b->lists_n, 0, sizeof(uint32_t) * 3, st));
  if (npoints == 0) return GBG_OK;
  BinGeom g;
  for (int d = 0; d < 3; ++d) {
    g.n[d] = b->grid.n[d];
    g.b[d] = b->b[d];
    g.nb[d] = b->nb[d];
    const double inv = (double)b->grid.n[d] / b->grid.domain[d];
    g.scale[d] = inv * 4294967296.0;
    g.shift[d] = -b->grid.origin[d] * inv * 4294967296.0;
    g.o32[d] = (float)b->grid.origin[d];
    g.d32[d] = (float)b->grid.spacing[d];
  }
  g.bvol = b->bvol;
  const int blocks = launch_blocks(npoints, kThreads);
  // the rank of each point within its key goes to skeys (free until the fallback sort)
  if (disp)
    k_bin_keys<T, true><<<blocks, kThreads, 0, st>>>(g, positions, npoints, b->keys, b->cell_start, b->skeys,
                                                     b->rec_user, device_status, *disp);
  else
    k_bin_keys<T, false><<<blocks, kThreads, 0, st>>>(g, positions, npoints, b->keys, b->cell_start, b->skeys,
                                                      b->rec_user, device_status);
  note_launch();
  GBG_CUDA_TRY(cudaGetLastError());
  int bits = 0;
  while (bits < 32 && ((uint64_t)(b->nkeys - 1) >> bits) != 0) ++bits;
  // one counting pass: the scan of the counts gives every cell its slots, the atomic ranks
  // place the points, and a per-cell pass puts each cell's points in index order (the
  // stable order; a cell of more than 1024 points sends the whole sort to the radix sort)
  GBG_TRY(exclusive_scan_u32(b->cell_start, b->cell_start, b->nkeys + 1, b->scan_tmp, st));
  GBG_TRY(stable_counting_sort(b->keys, b->skeys, b->cell_start, npoints, bits, b->perm, b->skeys, b->lists_n + 2,
                               b->sort_tmp, st, b->rec_user, b->rec));
  // the records in sorted order come with the stable placement; only the radix fallback's
  // order (a cell of more than 1024 points) gathers them again
  k_gather_records<<<blocks, kThreads, 0, st>>>(b->rec_user, b->perm, npoints, b->rec, b->lists_n + 2);
  note_launch();
  k_brick_lists<<<launch_blocks(b->nbricks, kThreads), kThreads, 0, st>>>(
      b->cell_start, b->nb[0], b->nb[1], b->nb[2], b->bvol, b->reach_ok ? 1 : 0, b->active, b->reach, b->lists_n);
  note_launch();
  GBG_CUDA_TRY(cudaGetLastError());
  return GBG_OK;
}

}  // namespace
}  // namespace gbg

extern "C" {

gbg_status gbg_points_displace(const gbg_grid *grid, gbg_dtype dtype, void *dst, const void *src, int64_t npoints,
                               int32_t nterms, const double *coefficients, const void *const *sections,
                               void *stream) {
  clear_error();
  if (dtype != GBG_F32 && dtype != GBG_F64) return set_error(GBG_EARG, "bad dtype");
  if (npoints < 0) return set_error(GBG_EDIM, "negative point count");
  if (npoints > 0 && (!dst || !src)) return set_error(GBG_EARG, "null positions");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  auto go = [&](auto *tag) -> gbg_status {
    using T = std::remove_pointer_t<decltype(tag)>;
    DisplaceArgs<T> a;
    GBG_TRY(make_displace<T>(a, grid, static_cast<T *>(dst), static_cast<const T *>(src), nterms, coefficients,
                             sections));
    if (npoints == 0) return GBG_OK;
    k_displace<T><<<launch_blocks(3 * npoints, kThreads), kThreads, 0, st>>>(a, npoints);
    note_launch();
    GBG_CUDA_TRY(cudaGetLastError());
    return GBG_OK;
  };
  return dtype == GBG_F64 ? go((double *)nullptr) : go((float *)nullptr);
}

gbg_status gbg_bins_build_displaced(gbg_bins b, gbg_dtype dtype, void *dst, const void *src, int64_t npoints,
                                    int32_t nterms, const double *coefficients, const void *const *sections,
                                    int32_t wrap, int32_t *device_status, void *stream) {
  clear_error();
  if (!b) return set_error(GBG_EARG, "null bins");
  if (npoints < 0 || npoints > b->max_points) return set_error(GBG_EDIM, "more points than the bins hold");
  if (dtype != GBG_F32 && dtype != GBG_F64) return set_error(GBG_EARG, "bad dtype");
  if (npoints > 0 && (!dst || !src)) return set_error(GBG_EARG, "null positions");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  auto go = [&](auto *tag) -> gbg_status {
    using T = std::remove_pointer_t<decltype(tag)>;
    DisplaceArgs<T> a;
    GBG_TRY(make_displace<T>(a, wrap ? &b->grid : nullptr, static_cast<T *>(dst), static_cast<const T *>(src), nterms,
                             coefficients, sections));
    return bins_build_impl<T>(b, static_cast<const T *>(dst), npoints, device_status, st, &a);
  };
  return dtype == GBG_F64 ? go((double *)nullptr) : go((float *)nullptr);
}

gbg_status gbg_bins_permute(gbg_bins b, gbg_dtype dtype, int32_t ncols, const void *src, void *dst, void *stream) {
  clear_error();
  if (!b) return set_error(GBG_EARG, "null bins");
  if (dtype != GBG_F32 && dtype != GBG_F64) return set_error(GBG_EARG, "bad dtype");
  if (ncols < 1) return set_error(GBG_EARG, "ncols must be positive");
  if (b->npoints == 0) return GBG_OK;
  if (!src || !dst || src == dst) return set_error(GBG_EARG, "permute needs distinct source and destination");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const int64_t m = b->npoints;
  const int blocks = launch_blocks(m * ncols, kThreads);
  if (dtype == GBG_F64)
    k_permute<double><<<blocks, kThreads, 0, st>>>(static_cast<const double *>(src), static_cast<double *>(dst), b->perm,
                                                   m, ncols);
  else
    k_permute<float><<<blocks, kThreads, 0, st>>>(static_cast<const float *>(src), static_cast<float *>(dst), b->perm,
                                                  m, ncols);
  note_launch();
  GBG_CUDA_TRY(cudaGetLastError());
  return GBG_OK;
}

gbg_status gbg_bins_build(gbg_bins b, gbg_dtype pos_dtype, const void *positions, int64_t npoints,
                          int32_t *device_status, void *stream) {
  clear_error();
  if (!b) return set_error(GBG_EARG, "null bins");
  if (npoints < 0 || npoints > b->max_points) return set_error(GBG_EDIM, "more points than the bins hold");
  if (pos_dtype != GBG_F32 && pos_dtype != GBG_F64) return set_error(GBG_EARG, "bad dtype");
  if (npoints > 0 && !positions) return set_error(GBG_EARG, "null positions");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (pos_dtype == GBG_F64)
    return bins_build_impl<double>(b, static_cast<const double *>(positions), npoints, device_status, st, nullptr);
  return bins_build_impl<float>(b, static_cast<const float *>(positions), npoints, device_status, st, nullptr);
}

gbg_status gbg_bins_build_batch(const gbg_bins *bins, const gbg_dtype *dtypes, const void *const *positions,
                                const int64_t *npoints, int32_t count, int32_t *device_status, void *stream) {
  clear_error();
  if (count < 0 || (count > 0 && (!bins || !dtypes || !positions || !npoints))) return set_error(GBG_EARG, "null argument");
  for (int32_t i = 0; i < count; ++i) {
    if (!bins[i]) return set_error(GBG_EARG, "null bins");
    if (npoints[i] < 0 || npoints[i] > bins[i]->max_points) return set_error(GBG_EDIM, "more points than the bins hold");
    if (dtypes[i] != GBG_F32 && dtypes[i] != GBG_F64) return set_error(GBG_EARG, "bad dtype");
    if (npoints[i] > 0 && !positions[i]) return set_error(GBG_EARG, "null positions");
  }
  if (count == 0) return GBG_OK;
  // the same bins twice build in call order on one side stream
  std::map<const gbg_bins_s *, int> lane;
  std::vector<int> at(count);
  for (int32_t i = 0; i < count; ++i) {
    auto it = lane.find(bins[i]);
    at[i] = it != lane.end() ? it->second : (int)(lane.size() % kSideStreams);
    lane.emplace(bins[i], at[i]);
  }
  const int k = (int)std::min<size_t>(lane.size(), kSideStreams);
  return side_run(
      static_cast<cudaStream_t>(stream), k,
      [&](int side, cudaStream_t s) -> gbg_status {
        for (int32_t i = 0; i < count; ++i) {
          if (at[i] != side) continue;
          if (dtypes[i] == GBG_F64)
            GBG_TRY(bins_build_impl<double>(bins[i], static_cast<const double *>(positions[i]), npoints[i],
                                            device_status, s, nullptr));
          else
            GBG_TRY(bins_build_impl<float>(bins[i], static_cast<const float *>(positions[i]), npoints[i],
                                           device_status, s, nullptr));
        }
        return GBG_OK;
      },
      [] { return GBG_OK; });
}

gbg_status gbg_bins_order(gbg_bins b, int32_t *order, void *stream) {
  clear_error();
  if (!b || (!order && b->npoints)) return set_error(GBG_EARG, "null argument");
  if (b->npoints == 0) return GBG_OK;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  k_order_from_perm<<<launch_blocks(b->npoints, kThreads), kThreads, 0, st>>>(b->perm, order, b->npoints);
  note_launch();
  GBG_CUDA_TRY(cudaGetLastError());
  return GBG_OK;
}

gbg_status gbg_interpolate_binned(gbg_field f, gbg_bins b, const gbg_scheme *scheme, gbg_dtype out_dtype,
                                  void *out, int32_t *device_status, void *stream) {
  clear_error();
  GBG_TRY(check_field_bins(f, b, scheme));
  if (out_dtype != GBG_F32 && out_dtype != GBG_F64) return set_error(GBG_EARG, "bad dtype");
  if (b->npoints == 0) return GBG_OK;
  if (!out) return set_error(GBG_EARG, "null output");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  auto run = [&](auto *o) -> gbg_status {
    switch (scheme->stencil_width) {
      // compile-time (width, powers) for the common schemes, guarded Horner otherwise
      case 2: return scheme->num_powers == 2 ? launch_staged_gather<2, 2>(f, b, *scheme, o, device_status, st)
                                             : launch_staged_gather<2, 0>(f, b, *scheme, o, device_status, st);
      case 4: return scheme->num_powers == 4 ? launch_staged_gather<4, 4>(f, b, *scheme, o, device_status, st)
                                             : launch_staged_gather<4, 0>(f, b, *scheme, o, device_status, st);
      case 6: return scheme->num_powers == 6 ? launch_staged_gather<6, 6>(f, b, *scheme, o, device_status, st)
                     : scheme->num_powers == 4 ? launch_staged_gather<6, 4>(f, b, *scheme, o, device_status, st)
                                               : launch_staged_gather<6, 0>(f, b, *scheme, o, device_status, st);
      default: return scheme->num_powers == 8 ? launch_staged_gather<8, 8>(f, b, *scheme, o, device_status, st)
                                              : launch_staged_gather<8, 0>(f, b, *scheme, o, device_status, st);
    }
  };
  if (out_dtype == GBG_F64) return run(static_cast<double *>(out));
  return run(static_cast<float *>(out));
}

gbg_status gbg_anterpolate_binned(gbg_field f, gbg_bins b, const gbg_scheme *scheme, gbg_dtype q_dtype,
                                  const void *q, double alpha, double beta, int32_t *device_status, void *stream) {
  clear_error();
  GBG_TRY(check_field_bins(f, b, scheme));
  if (q_dtype != GBG_F32 && q_dtype != GBG_F64) return set_error(GBG_EARG, "bad dtype");
  if (b->npoints > 0 && !q) return set_error(GBG_EARG, "null quantities");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const int64_t m = b->npoints;
  GBG_CUDA_TRY(cudaMemsetAsync(b->qmax_bits, 0, sizeof(unsigned), st));
  if (m > 0) {
    const int blocks = launch_blocks(m, kThreads);
    if (q_dtype == GBG_F64) {
      const double *qd = static_cast<const double *>(q);
      if (f->cp == 4) k_scatter_qprep<double, 4><<<blocks, kThreads, 0, st>>>(qd, b->perm, m, f->ncomp, (float)alpha, b->qs, b->qmax_bits);
      else k_scatter_qprep<double, 12><<<blocks, kThreads, 0, st>>>(qd, b->perm, m, f->ncomp, (float)alpha, b->qs, b->qmax_bits);
    } else {
      const float *qf = static_cast<const float *>(q);
      if (f->cp == 4) k_scatter_qprep<float, 4><<<blocks, kThreads, 0, st>>>(qf, b->perm, m, f->ncomp, (float)alpha, b->qs, b->qmax_bits);
      else k_scatter_qprep<float, 12><<<blocks, kThreads, 0, st>>>(qf, b->perm, m, f->ncomp, (float)alpha, b->qs, b->qmax_bits);
    }
    note_launch();
    GBG_CUDA_TRY(cudaGetLastError());
  }
  // With no points the push still runs: it writes beta * field (beta == 0 clears).
  const int w = scheme->stencil_width;
  const bool fixed = scheme->num_powers == w;
  gbg_status s;
  if (w == 2)
    s = fixed ? launch_staged_scatter<2, true>(f, b, *scheme, beta, b->qmax_bits, device_status, st)
              : launch_staged_scatter<2, false>(f, b, *scheme, beta, b->qmax_bits, device_status, st);
  else if (w == 4)
    s = fixed ? launch_staged_scatter<4, true>(f, b, *scheme, beta, b->qmax_bits, device_status, st)
              : launch_staged_scatter<4, false>(f, b, *scheme, beta, b->qmax_bits, device_status, st);
  else if (w == 6)
    s = fixed ? launch_staged_scatter<6, true>(f, b, *scheme, beta, b->qmax_bits, device_status, st)
              : launch_staged_scatter<6, false>(f, b, *scheme, beta, b->qmax_bits, device_status, st);
  else
    s = fixed ? launch_staged_scatter<8, true>(f, b, *scheme, beta, b->qmax_bits, device_status, st)
              : launch_staged_scatter<8, false>(f, b, *scheme, beta, b->qmax_bits, device_status, st);
  GBG_TRY(s);
  const int64_t total = ghost_count(f->px, f->py, f->pz, f->grid.n[0], f->grid.n[1], f->grid.n[2]);
  k_fill_ghosts<<<launch_blocks(total, kThreads), kThreads, 0, st>>>(f->data, f->cp, f->px, f->py, f->pz, f->halo,
                                                                     f->grid.n[0], f->grid.n[1], f->grid.n[2]);
  note_launch();
  GBG_CUDA_TRY(cudaGetLastError());
  return GBG_OK;
}

}  // extern "C"

// ------------------------------------------------------------ batched form: host

struct gbg_batch_s {
  int device = 0;
  int32_t count = 0, ng = 0, ns = 0;  // instances; of them, with a gather / a scatter
  gbg::BatchDev *items = nullptr;
  CUtensorMap *maps = nullptr;
  uint32_t *goff = nullptr, *gidx = nullptr, *soff = nullptr, *sidx = nullptr;
  uint32_t ngwork = 0, nswork = 0;  // bounds on the units (every brick); the lists may hold fewer
  uint32_t *counters = nullptr;
  const float **qptrs = nullptr;
  float **qs_out = nullptr;
  unsigned **qmax_out = nullptr;
  float *alphas = nullptr;
  int64_t *qoff = nullptr;
  int64_t total_q = 0;
  uint32_t buf_bytes = 0;
  int nbuf = 2;
  size_t gather_smem = 0, scatter_smem = 0;
  std::vector<gbg_field> dests;
  // instances large enough to fill the GPU alone: run through the single-instance binned
  // kernels (batch_split), not the persistent launches
  std::vector<gbg_batch_item> direct;
  void *block = nullptr;  // the device tables, one allocation
  size_t bytes = 0;
  bool async = false;     // block from cudaMallocAsync (serving loop)
  // corrections of the pooled scatter's compensated regions of several chunks: cslots
  // slots of cstride floats, one per scatter CTA (a separate allocation, never staged)
  float *cscratch = nullptr;
  int64_t cstride = 0;
  int32_t cslots = 0;
};

namespace gbg {

// Host side of a batch before its tables reach the device.
struct BatchHost {
  std::vector<BatchDev> items;
  std::vector<CUtensorMap> maps;
  std::vector<uint32_t> goff, gidx, soff, sidx;
  std::vector<const float *> qptrs;
  std::vector<float *> qs_out;
  std::vector<unsigned *> qmax_out;
  std::vector<float> alphas;
  std::vector<int64_t> qoff;
};

// Byte offsets of a batch's device tables within its block.
struct BatchLayout {
  size_t items, maps, goff, gidx, soff, sidx, counters, qptrs, qs_out, qmax_out, alphas, qoff, bytes;
};

BatchLayout batch_layout(int32_t n) {
  BatchLayout L;
  size_t at = 0;
  auto take = [&](size_t bytes) {
    const size_t off = (at + 255) & ~size_t(255);
    at = off + bytes;
    return off;
  };
  L.items = take(sizeof(BatchDev) * n);
  L.maps = take(sizeof(CUtensorMap) * n);
  L.goff = take(sizeof(uint32_t) * (n + 1));
  L.gidx = take(sizeof(uint32_t) * n);
  L.soff = take(sizeof(uint32_t) * (n + 1));
  L.sidx = take(sizeof(uint32_t) * n);
  L.counters = take(sizeof(uint32_t) * 64);
  L.qptrs = take(sizeof(const float *) * n);
  L.qs_out = take(sizeof(float *) * n);
  L.qmax_out = take(sizeof(unsigned *) * n);
  L.alphas = take(sizeof(float) * n);
  L.qoff = take(sizeof(int64_t) * (n + 1));
  L.bytes = (at + 255) & ~size_t(255);
  return L;
}

// Checks the items and fills the host tables and the launch shapes of bt.
// The argument rules of one batch item (every item, whichever launch runs it).
gbg_status check_batch_item(const gbg_batch_item &it) {
  gbg_field_s *f = it.field;
  GBG_TRY(check_field_bins(f, it.bins, &it.scheme));
  const int w = it.scheme.stencil_width;
  if (it.scheme.num_powers != w)
    return set_error(GBG_EUNSUPPORTED, "batch: schemes must have num_powers == stencil_width");
  if (it.dest && (it.dest->ncomp != f->ncomp || it.dest->grid.n[0] != f->grid.n[0] ||
                  it.dest->grid.n[1] != f->grid.n[1] || it.dest->grid.n[2] != f->grid.n[2] ||
                  it.dest->max_width < w || !it.q))
    return set_error(GBG_EARG, "batch: the scatter destination must match the field and have quantities");
  return GBG_OK;
}

// Points from which an instance runs through the single-instance binned kernels inside the
// batch: those kernels (tuned per width and component count, double-buffered gather) beat
// the persistent launches, whose one register budget and one gather buffer serve every
// instance -- on 64 instances of 1e3..1e6 points (grids 32^3..256^3) a captured step took
// 53.7 ms all pooled, 45.2 ms with instances of 2^14 points or more direct, 44.3 ms with
// 2^10 or more and with all of them direct.  Instances below 1024 points still share the
// persistent launches, where one launch per instance would cost more than its work.
constexpr int64_t kBatchDirectPoints = 1 << 10;

// Splits a batch's items into those of the persistent launches and the direct ones, after
// checking every item.
gbg_status batch_split(const gbg_batch_item *items, int32_t count, std::vector<gbg_batch_item> &pooled,
                       std::vector<gbg_batch_item> &direct) {
  if (!items || count < 1) return set_error(GBG_EARG, "batch: need at least one item");
  for (int32_t i = 0; i < count; ++i) {
    GBG_TRY(check_batch_item(items[i]));
    (items[i].bins->npoints >= kBatchDirectPoints ? direct : pooled).push_back(items[i]);
  }
  return GBG_OK;
}

gbg_status batch_plan(const gbg_batch_item *items, int32_t count, gbg_batch_s *bt, BatchHost &h) {
  if (!items || count < 1) return set_error(GBG_EARG, "batch: need at least one item");
  cudaGetDevice(&bt->device);
  bt->count = count;
  h.items.resize(count);
  h.maps.resize(count);
  h.qptrs.assign(count, nullptr);
  h.qs_out.assign(count, nullptr);
  h.qmax_out.assign(count, nullptr);
  h.alphas.assign(count, 1.0f);
  h.qoff.assign(count + 1, 0);
  std::vector<double> cost(count);
  uint32_t buf_max = 0;
  size_t scat_max = 0;
  for (int32_t i = 0; i < count; ++i) {
    const gbg_batch_item &it = items[i];
    gbg_field_s *f = it.field;
    gbg_bins_s *b = it.bins;
    GBG_TRY(check_batch_item(it));
    const int w = it.scheme.stencil_width;
    BatchDev &d = h.items[i];
    d = BatchDev{};
    d.g = staged_geo(f, b, w);
    d.cell_start = b->cell_start;
    d.rec = b->rec;
    d.perm = b->perm;
    d.out = it.out;
    d.dest = it.dest ? it.dest->data : nullptr;
    d.qs = b->qs;
    d.qmax_bits = b->qmax_bits;
    d.glist = b->active;
    d.gcount = b->lists_n;
    const bool reach = it.beta == 1.0 && b->reach_ok;
    d.slist = reach ? b->reach : nullptr;
    d.scount = reach ? b->lists_n + 1 : nullptr;
    for (int k = 0; k < 64; ++k) d.coef[k] = 0.0f;
    for (int q = 0; q < w; ++q)
      for (int p = 0; p < w; ++p) d.coef[q + w * p] = (float)it.scheme.coefficients[q + w * p];
    d.n2 = w;
    d.cp = f->cp;
    d.box_bytes = (uint32_t)((size_t)f->cp * 4 * d.g.w[0] * d.g.w[1] * d.g.w[2]);
    d.beta = (float)it.beta;
    d.beta_zero = it.beta == 0.0;
    if (it.dest) {
      gbg_field_s *ds = it.dest;
      for (int k = 0; k < 3; ++k) {
        d.fg.b[k] = b->b[k];
        d.fg.nb[k] = (int32_t)b->nb[k];
        d.fg.n[k] = (int32_t)ds->grid.n[k];
        d.fg.e[k] = b->b[k] + w - 1;
      }
      d.fg.neighbour_skip = neighbour_skip_ok(b->b, b->nb, ds->grid.n, w);
      d.fg.comp = b->compensated;
      d.fg.sparse = scatter_sparse(b, ds->grid, w);
      d.fg.nbricks = b->nbricks;
      d.fg.bvol = b->bvol;
      d.fg.px = ds->px;
      d.fg.py = ds->py;
      d.fg.halo = ds->halo;
      d.fg.cp = ds->cp;
      d.fg.ncomp = ds->ncomp;
      scatter_nodes_chunk(d.fg, ds->cp, w, scatter_nodes_budget(d.fg, ds->cp, w));
      scat_max = std::max(scat_max, scatter_nodes_smem(d.fg, ds->cp, w));
      bt->cstride = std::max<int64_t>(bt->cstride, b->bvol * 12);
      if (d.fg.e[0] > 255) return set_error(GBG_EUNSUPPORTED, "batch: brick too large for the scatter");
      h.qptrs[i] = it.q;
      h.qs_out[i] = b->qs;
      h.qmax_out[i] = b->qmax_bits;
      h.alphas[i] = (float)it.alpha;
      bt->dests.push_back(it.dest);
      h.qoff[i + 1] = b->npoints;
    }
    if (it.out) {
      CUtensorMap *m = nullptr;
      GBG_TRY(tensor_map_for(f, w, b->b, &m));
      h.maps[i] = *m;
      buf_max = std::max(buf_max, (d.box_bytes + 1023u) & ~1023u);
    } else {
      std::memset(&h.maps[i], 0, sizeof(CUtensorMap));
    }
    cost[i] = (double)b->npoints * w * w * w * f->cp + (double)b->nbricks;
  }
  for (int32_t i = 0; i < count; ++i) h.qoff[i + 1] += h.qoff[i];
  bt->total_q = h.qoff[count];
  // instances in cost order, largest first; the offsets written here (every brick) are
  // the bounds the launch shapes use, k_batch_reset rewrites them from the lists
  std::vector<int32_t> order(count);
  for (int32_t i = 0; i < count; ++i) order[i] = i;
  std::stable_sort(order.begin(), order.end(), [&](int32_t a, int32_t c) { return cost[a] > cost[c]; });
  uint64_t ng = 0, ns = 0;
  h.goff.assign(1, 0);
  h.soff.assign(1, 0);
  for (int32_t i : order) {
    const uint64_t nb = (uint64_t)items[i].bins->nbricks;
    if (items[i].out) {
      h.gidx.push_back((uint32_t)i);
      ng += nb;
      h.goff.push_back((uint32_t)ng);
    }
    if (items[i].dest) {
      h.sidx.push_back((uint32_t)i);
      ns += nb;
      h.soff.push_back((uint32_t)ns);
    }
  }
  if (ng >= 0xffffffffull || ns >= 0xffffffffull) return set_error(GBG_EUNSUPPORTED, "batch: 2^32 or more bricks");
  bt->ng = (int32_t)h.gidx.size();
  bt->ns = (int32_t)h.sidx.size();
  h.goff.resize(count + 1, (uint32_t)ng);
  h.gidx.resize(count, 0);
  h.soff.resize(count + 1, (uint32_t)ns);
  h.sidx.resize(count, 0);
  bt->ngwork = (uint32_t)ng;
  bt->nswork = (uint32_t)ns;
  bt->buf_bytes = buf_max;
  bt->nbuf = 2 * (size_t)buf_max + 64 <= 227 * 1024 ? 2 : 1;
  bt->gather_smem = (size_t)bt->nbuf * buf_max + 64;
  bt->scatter_smem = scat_max;
  if (bt->gather_smem > 227 * 1024 || bt->scatter_smem > 227 * 1024)
    return set_error(GBG_EUNSUPPORTED, "batch: a brick's tile does not fit in shared memory");
  bt->bytes = batch_layout(count).bytes;
  bt->cslots = ns ? (int32_t)std::min<uint64_t>(ns, (uint64_t)kScatterSlotsPerSM * device_sms()) : 0;
  return GBG_OK;
}

// Points bt at its device block and writes the tables' image (the bytes the block must
// hold) into host memory of bt->bytes bytes.
void batch_fill(gbg_batch_s *bt, const BatchHost &h, char *image) {
  const int32_t n = bt->count;
  char *dev = static_cast<char *>(bt->block);
  const BatchLayout L = batch_layout(n);
  std::memset(image, 0, bt->bytes);
  auto put = [&](auto *&dst, size_t off, const void *src, size_t bytes) {
    if (bytes) std::memcpy(image + off, src, bytes);
    dst = reinterpret_cast<std::remove_reference_t<decltype(dst)>>(dev + off);
  };
  put(bt->items, L.items, h.items.data(), sizeof(BatchDev) * n);
  put(bt->maps, L.maps, h.maps.data(), sizeof(CUtensorMap) * n);
  put(bt->goff, L.goff, h.goff.data(), sizeof(uint32_t) * (n + 1));
  put(bt->gidx, L.gidx, h.gidx.data(), sizeof(uint32_t) * n);
  put(bt->soff, L.soff, h.soff.data(), sizeof(uint32_t) * (n + 1));
  put(bt->sidx, L.sidx, h.sidx.data(), sizeof(uint32_t) * n);
  put(bt->counters, L.counters, nullptr, 0);
  put(bt->qptrs, L.qptrs, h.qptrs.data(), sizeof(const float *) * n);
  put(bt->qs_out, L.qs_out, h.qs_out.data(), sizeof(float *) * n);
  put(bt->qmax_out, L.qmax_out, h.qmax_out.data(), sizeof(unsigned *) * n);
  put(bt->alphas, L.alphas, h.alphas.data(), sizeof(float) * n);
  put(bt->qoff, L.qoff, h.qoff.data(), sizeof(int64_t) * (n + 1));
  BatchDev *items = reinterpret_cast<BatchDev *>(image + L.items);
  for (int32_t i = 0; i < n; ++i) {
    items[i].fg.cscratch = bt->cscratch;
    items[i].fg.cstride = bt->cstride;
  }
}

size_t batch_scratch_bytes(const gbg_batch_s *bt) { return sizeof(float) * (size_t)bt->cslots * bt->cstride; }

gbg_status batch_create_async(const gbg_batch_item *items, int32_t count, cudaStream_t stream, void *pinned,
                              size_t pinned_bytes, gbg_batch *out) {
  std::vector<gbg_batch_item> pooled, direct;
  GBG_TRY(batch_split(items, count, pooled, direct));
  auto *bt = new (std::nothrow) gbg_batch_s;
  if (!bt) return set_error(GBG_ENOMEM, "host allocation failed");
  bt->direct = direct;
  if (pooled.empty()) {
    cudaGetDevice(&bt->device);
    *out = bt;
    return GBG_OK;
  }
  BatchHost h;
  gbg_status st = batch_plan(pooled.data(), (int32_t)pooled.size(), bt, h);
  if (st == GBG_OK && bt->bytes > pinned_bytes) st = set_error(GBG_ENOMEM, "batch: staging buffer too small");
  if (st) {
    delete bt;
    return st;
  }
  if (cudaMallocAsync(&bt->block, bt->bytes, stream) != cudaSuccess) {
    cudaGetLastError();
    delete bt;
    return set_error(GBG_ENOMEM, "batch: cudaMallocAsync failed");
  }
  bt->async = true;
  if (bt->cslots && cudaMallocAsync(&bt->cscratch, batch_scratch_bytes(bt), stream) != cudaSuccess) {
    cudaGetLastError();
    cudaFreeAsync(bt->block, stream);
    delete bt;
    return set_error(GBG_ENOMEM, "batch: cudaMallocAsync of the scatter scratch failed");
  }
  batch_fill(bt, h, static_cast<char *>(pinned));
  const cudaError_t e = cudaMemcpyAsync(bt->block, pinned, bt->bytes, cudaMemcpyHostToDevice, stream);
  if (e != cudaSuccess) {
    cudaFreeAsync(bt->block, stream);
    if (bt->cscratch) cudaFreeAsync(bt->cscratch, stream);
    delete bt;
    return set_error(GBG_ECUDA, std::string("batch: copy failed: ") + cudaGetErrorString(e));
  }
  *out = bt;
  return GBG_OK;
}

size_t batch_table_bytes(int32_t count) { return batch_layout(count).bytes; }

gbg_status batch_destroy_async(gbg_batch bt, cudaStream_t stream) {
  if (!bt) return GBG_OK;
  cudaError_t e = !bt->block ? cudaSuccess : bt->async ? cudaFreeAsync(bt->block, stream) : cudaFree(bt->block);
  if (bt->cscratch) {
    const cudaError_t e2 = bt->async ? cudaFreeAsync(bt->cscratch, stream) : cudaFree(bt->cscratch);
    if (e == cudaSuccess) e = e2;
  }
  delete bt;
  if (e != cudaSuccess) return set_error(GBG_ECUDA, std::string("freeing the batch: ") + cudaGetErrorString(e));
  return GBG_OK;
}

}  // namespace gbg

extern "C" {

gbg_status gbg_batch_create(const gbg_batch_item *items, int32_t count, gbg_batch *out) {
  clear_error();
  if (!out) return set_error(GBG_EARG, "null argument");
  GBG_TRY(side_pool_ready());
  std::vector<gbg_batch_item> pooled, direct;
  GBG_TRY(batch_split(items, count, pooled, direct));
  auto *bt = new (std::nothrow) gbg_batch_s;
  if (!bt) return set_error(GBG_ENOMEM, "host allocation failed");
  bt->direct = direct;
  if (pooled.empty()) {
    cudaGetDevice(&bt->device);
    *out = bt;
    return GBG_OK;
  }
  BatchHost h;
  gbg_status st = batch_plan(pooled.data(), (int32_t)pooled.size(), bt, h);
  if (st) {
    delete bt;
    return st;
  }
  if (cudaMalloc(&bt->block, bt->bytes) != cudaSuccess) {
    cudaGetLastError();
    delete bt;
    return set_error(GBG_ENOMEM, "batch: cudaMalloc failed");
  }
  if (bt->cslots && cudaMalloc(&bt->cscratch, batch_scratch_bytes(bt)) != cudaSuccess) {
    cudaGetLastError();
    cudaFree(bt->block);
    delete bt;
    return set_error(GBG_ENOMEM, "batch: cudaMalloc of the scatter scratch failed");
  }
  std::vector<char> image(bt->bytes);
  batch_fill(bt, h, image.data());
  const cudaError_t e = cudaMemcpy(bt->block, image.data(), bt->bytes, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    cudaFree(bt->block);
    if (bt->cscratch) cudaFree(bt->cscratch);
    delete bt;
    return set_error(GBG_ECUDA, std::string("batch: copy failed: ") + cudaGetErrorString(e));
  }
  *out = bt;
  return GBG_OK;
}

gbg_status gbg_batch_run(gbg_batch bt, int32_t *device_status, void *stream) {
  clear_error();
  if (!bt) return set_error(GBG_EARG, "null batch");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const bool pooled = bt->count > 0;
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, bt->device);
  // the direct instances spread over the side streams: gathers by output, scatters by bins
  // (their sorted quantities) and destination, items sharing either on one side stream
  std::vector<int> glane, slane;
  int gk = 0, sk = 0;
  {
    std::map<const void *, int> seen;
    for (const gbg_batch_item &it : bt->direct) {
      int l = -1;
      if (it.out) {
        auto f = seen.find(it.out);
        l = f != seen.end() ? f->second : gk++ % kSideStreams;
        seen.emplace(it.out, l);
      }
      glane.push_back(l);
    }
    seen.clear();
    for (const gbg_batch_item &it : bt->direct) {
      int l = -1;
      if (it.dest) {
        auto fb = seen.find(it.bins), fd = seen.find(it.dest);
        if (fb != seen.end() && fd != seen.end() && fb->second != fd->second) l = -2;  // tied to two lanes
        else l = fb != seen.end() ? fb->second : fd != seen.end() ? fd->second : sk++ % kSideStreams;
        if (l >= 0) {
          seen.emplace(it.bins, l);
          seen.emplace(it.dest, l);
        }
      }
      slane.push_back(l);
    }
    gk = std::min(gk, kSideStreams);
    sk = std::min(sk, kSideStreams);
  }
  // a destination shared with a pooled instance, or an item tied to two lanes: the direct
  // scatters run one after another after the pooled scatter
  bool serial_scatters = std::count(slane.begin(), slane.end(), -2) > 0;
  for (const gbg_batch_item &it : bt->direct)
    if (it.dest && std::find(bt->dests.begin(), bt->dests.end(), it.dest) != bt->dests.end()) serial_scatters = true;
  auto pooled_gather = [&]() -> gbg_status {
    if (!pooled) return GBG_OK;
    k_batch_reset<<<1, 256, 0, st>>>(bt->items, bt->counters, bt->qmax_out, bt->count, bt->gidx, bt->ng, bt->goff,
                                     bt->sidx, bt->ns, bt->soff);
    note_launch();
    GBG_CUDA_TRY(cudaGetLastError());
    if (bt->nswork > 0 && bt->total_q > 0) {
      k_batch_qprep<<<launch_blocks(bt->total_q, kThreads), kThreads, 0, st>>>(
          bt->items, bt->qptrs, bt->qoff, bt->count, bt->qs_out, bt->alphas, bt->qmax_out);
      note_launch();
      GBG_CUDA_TRY(cudaGetLastError());
    }
    if (bt->ngwork > 0) {
      GBG_CUDA_TRY(cudaFuncSetAttribute(k_batch_gather, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)bt->gather_smem));
      const int blocks = (int)std::min<uint32_t>(bt->ngwork, (uint32_t)sms);
      k_batch_gather<<<blocks, kBatchGatherThreads, bt->gather_smem, st>>>(
          bt->items, bt->maps, bt->goff, bt->gidx, bt->ng, bt->counters, bt->buf_bytes, bt->nbuf, device_status);
      note_launch();
      GBG_CUDA_TRY(cudaGetLastError());
    }
    return GBG_OK;
  };
  auto pooled_scatter = [&]() -> gbg_status {
    if (!pooled || bt->nswork == 0) return GBG_OK;
    GBG_CUDA_TRY(cudaFuncSetAttribute(k_batch_scatter, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)bt->scatter_smem));
    GBG_CUDA_TRY(cudaFuncSetAttribute(k_batch_scatter, cudaFuncAttributePreferredSharedMemoryCarveout, 100));
    int per_sm = 1;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_batch_scatter, kThreads, bt->scatter_smem);
    const int blocks = (int)std::min<uint32_t>((uint32_t)bt->cslots, (uint32_t)(std::max(per_sm, 1) * sms));
    k_batch_scatter<<<blocks, kThreads, bt->scatter_smem, st>>>(bt->items, bt->soff, bt->sidx, bt->ns,
                                                                bt->counters + 1, device_status);
    note_launch();
    GBG_CUDA_TRY(cudaGetLastError());
    for (gbg_field_s *f : bt->dests) {
      const int64_t total = ghost_count(f->px, f->py, f->pz, f->grid.n[0], f->grid.n[1], f->grid.n[2]);
      k_fill_ghosts<<<launch_blocks(total, kThreads), kThreads, 0, st>>>(f->data, f->cp, f->px, f->py, f->pz, f->halo,
                                                                         f->grid.n[0], f->grid.n[1], f->grid.n[2]);
      note_launch();
    }
    GBG_CUDA_TRY(cudaGetLastError());
    return GBG_OK;
  };
  // every gather before any scatter, as one persistent gather launch followed by one
  // persistent scatter launch would order them (a destination may be another item's field)
  if (gk > 0) {
    GBG_TRY(side_run(st, gk, [&](int side, cudaStream_t s) -> gbg_status {
      for (size_t i = 0; i < bt->direct.size(); ++i)
        if (glane[i] == side) {
          const gbg_batch_item &it = bt->direct[i];
          GBG_TRY(gbg_interpolate_binned(it.field, it.bins, &it.scheme, GBG_F32, it.out, device_status, s));
        }
      return GBG_OK;
    }, pooled_gather));
  } else {
    GBG_TRY(pooled_gather());
  }
  if (sk > 0 && !serial_scatters) {
    GBG_TRY(side_run(st, sk, [&](int side, cudaStream_t s) -> gbg_status {
      for (size_t i = 0; i < bt->direct.size(); ++i)
        if (slane[i] == side) {
          const gbg_batch_item &it = bt->direct[i];
          GBG_TRY(gbg_anterpolate_binned(it.dest, it.bins, &it.scheme, GBG_F32, it.q, it.alpha, it.beta, device_status, s));
        }
      return GBG_OK;
    }, pooled_scatter));
  } else {
    GBG_TRY(pooled_scatter());
    for (const gbg_batch_item &it : bt->direct)
      if (it.dest) GBG_TRY(gbg_anterpolate_binned(it.dest, it.bins, &it.scheme, GBG_F32, it.q, it.alpha, it.beta, device_status, stream));
  }
  return GBG_OK;
}

gbg_status gbg_batch_destroy(gbg_batch bt) {
  clear_error();
  return batch_destroy_async(bt, nullptr);
}

}  // extern "C"
