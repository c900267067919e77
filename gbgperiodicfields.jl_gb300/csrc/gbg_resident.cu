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
// Gather: one CTA per brick (persistent, double-buffered TMA halo tiles), a point per
// quarter-warp: lane (i, jj) owns the x-offset i and the y-offsets 2jj, 2jj+1 for all
// four z-offsets, reads each node's components with 128-bit shared loads (the tile's row
// pitch makes the 8 lanes of a quarter-warp hit 8 distinct 16-byte bank groups), and the
// quarter-warp reduces its partial sums with shuffles.
//
// Scatter: a CTA per brick stages the point ranges of the cells around the brick in
// shared memory; each thread owns grid nodes and pulls, in a fixed order, the weighted
// quantities of the points whose stencils reach them, with Neumaier-compensated FP32
// sums.  No float atomics: the result is bitwise reproducible.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <string>

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
  void *block = nullptr;
  size_t bytes = 0;
};

namespace gbg {
namespace {

constexpr int kThreads = 256;

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
__global__ void k_fill_ghosts(float *__restrict__ d, int cp, int64_t px, int64_t py, int64_t pz,
                              int halo, int64_t nx, int64_t ny, int64_t nz) {
  const int64_t total = px * py * pz;
  for (int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; n < total;
       n += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = n % px, j = (n / px) % py, k = n / (px * py);
    const bool interior = i >= halo && i < halo + nx && j >= halo && j < halo + ny && k >= halo &&
                          k < halo + nz;
    if (interior) continue;
    const int64_t x = imod(i - halo, nx) + halo, y = imod(j - halo, ny) + halo,
                  z = imod(k - halo, nz) + halo;
    const float4 *s = reinterpret_cast<const float4 *>(d + (x + px * (y + py * z)) * cp);
    float4 *t = reinterpret_cast<float4 *>(d + n * cp);
    for (int c = 0; c < cp / 4; ++c) t[c] = s[c];
  }
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

// Splits one FP64 coordinate into (cell, fraction) in FP64 fixed point.
__device__ __forceinline__ bool split64(double x, double scale, double shift, int64_t n,
                                        int64_t &cell, float &t) {
  const double u = fma(x, scale, shift);
  const bool ok = isfinite(u) && fabs(u) < 9.2e18;
  const long long v = ok ? __double2ll_rd(u) : 0;
  cell = imod((int64_t)(v >> 32), n);
  t = ok ? __uint2float_rz((unsigned)(v & 0xffffffffLL)) * 0x1p-32f : __int_as_float(0x7fc00000);
  return ok;
}

__device__ __forceinline__ bool split32(float x, float o, float d, int64_t n, int64_t &cell, float &t) {
  int64_t base;
  float tt;
  const bool ok = locate(x, o, d, base, tt);
  cell = imod(base, n);
  t = ok ? tt : __int_as_float(0x7fc00000);
  return ok;
}

template <typename T>
__global__ void __launch_bounds__(kThreads)
    k_bin_keys(BinGeom g, const T *__restrict__ pos, int64_t m, uint32_t *__restrict__ keys,
               uint32_t *__restrict__ counts, float4 *__restrict__ rec_user, int32_t *status) {
  for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < m;
       p += (int64_t)gridDim.x * blockDim.x) {
    int64_t c[3];
    float t[3];
    bool ok = true;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      if constexpr (sizeof(T) == 8)
        ok &= split64((double)pos[p + m * d], g.scale[d], g.shift[d], g.n[d], c[d], t[d]);
      else
        ok &= split32((float)pos[p + m * d], g.o32[d], g.d32[d], g.n[d], c[d], t[d]);
    }
    if (!ok && status) atomicOr(status, GBG_DEV_NONFINITE);
    const int64_t bx = c[0] / g.b[0], by = c[1] / g.b[1], bz = c[2] / g.b[2];
    const uint32_t local = (uint32_t)((c[2] - bz * g.b[2]) * g.b[1] * g.b[0] +
                                      (c[1] - by * g.b[1]) * g.b[0] + (c[0] - bx * g.b[0]));
    const uint32_t key = (uint32_t)(((bz * g.nb[1] + by) * g.nb[0] + bx) * g.bvol + local);
    keys[p] = key;
    atomicAdd(counts + key, 1u);
    rec_user[p] = make_float4(t[0], t[1], t[2], __uint_as_float(local));
  }
}

__global__ void k_gather_records(const float4 *__restrict__ rec_user, const uint32_t *__restrict__ perm,
                                 int64_t m, float4 *__restrict__ rec) {
  for (int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; s < m;
       s += (int64_t)gridDim.x * blockDim.x)
    rec[s] = __ldg(rec_user + perm[s]);
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

// Bounded wait on a phase of an mbarrier; false if it did not complete.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity) {
  const uint32_t a = smem_addr(bar);
  for (int iter = 0; iter < (1 << 22); ++iter) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
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

// Gather: width-4 stencils, a point per quarter-warp.
template <int CP, typename TO>
__global__ void __launch_bounds__(kThreads, 1)
    k_gather_staged4(const __grid_constant__ CUtensorMap tmap, StagedGeo g, SchemeT<float, 4> s,
                     const uint32_t *__restrict__ cell_start, const float4 *__restrict__ rec,
                     const uint32_t *__restrict__ perm, TO *__restrict__ out, int32_t *status, int nbuf,
                     uint32_t tile_bytes, uint32_t box_bytes) {
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
  const int nqw = kThreads / 8;
  uint32_t phase[2] = {0, 0};
  bool failed = false;

  auto issue = [&](int64_t b, int buf) {
    int64_t bx, by, bz;
    brick_coords(g, b, bx, by, bz);
    mbar_expect_tx(bars + buf, box_bytes);
    tma_load_tile(smem + buf * tile_bytes, &tmap, 0, (int)(bx * g.b[0]) + g.box_off,
                  (int)(by * g.b[1]) + g.box_off, (int)(bz * g.b[2]) + g.box_off, bars + buf);
  };
  auto nonempty = [&](int64_t b) { return __ldg(cell_start + (b + 1) * g.bvol) > __ldg(cell_start + b * g.bvol); };

  int64_t b = blockIdx.x;
  if (threadIdx.x == 0 && b < g.nbricks && nonempty(b)) issue(b, 0);
  for (int it = 0; b < g.nbricks; ++it, b += gridDim.x) {
    const int buf = nbuf == 2 ? (it & 1) : 0;
    const int64_t bn = b + gridDim.x;
    const uint32_t s0 = __ldg(cell_start + b * g.bvol), s1 = __ldg(cell_start + (b + 1) * g.bvol);
    if (nbuf == 2 && threadIdx.x == 0 && bn < g.nbricks && nonempty(bn)) issue(bn, buf ^ 1);
    if (s1 > s0) {
      if (!mbar_wait(bars + buf, phase[buf])) {
        failed = true;
        if (threadIdx.x == 0 && status) atomicOr(status, GBG_DEV_TIMEOUT);
        break;
      }
      phase[buf] ^= 1;
      const float *tile = reinterpret_cast<const float *>(smem + buf * tile_bytes);
      for (uint32_t sl = s0 + qw; sl < s1; sl += nqw) {
        const float4 r = __ldg(rec + sl);
        const uint32_t loc = __float_as_uint(r.w);
        const int lx = loc % g.b[0], ly = (loc / g.b[0]) % g.b[1], lz = loc / (g.b[0] * g.b[1]);
        const float w1 = poly<4>(s, qi, r.x);
        const float w2a = poly<4>(s, 2 * jj, r.y), w2b = poly<4>(s, 2 * jj + 1, r.y);
        float w3[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) w3[k] = poly<4>(s, k, r.z);
        float acc[CP];
#pragma unroll
        for (int c = 0; c < CP; ++c) acc[c] = 0.0f;
        const int node0 = (lz * g.w[1] + ly + 2 * jj) * g.w[0] + lx + qi;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
#pragma unroll
          for (int jp = 0; jp < 2; ++jp) {
            const float w = w1 * (jp ? w2b : w2a) * w3[k];
            const float4 *p = reinterpret_cast<const float4 *>(tile + (node0 + (k * g.w[1] + jp) * g.w[0]) * CP);
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
          const int64_t p = perm[sl];
          const int cbase = (up2 ? H : 0) + (up1 ? Q : 0);
#pragma unroll
          for (int v = 0; v < Q; ++v)
            if (cbase + v < g.ncomp) store_out(out, p + g.m * (cbase + v), qv[v]);
        }
      }
    }
    __syncthreads();  // every lane is done with this buffer before it is refilled
    if (nbuf == 1 && threadIdx.x == 0 && bn < g.nbricks && nonempty(bn)) issue(bn, 0);
  }
  if (failed) {
    // a copy that never completed: give any other in-flight copy a bounded chance to land
    for (int i = 0; i < nbuf; ++i) mbar_wait(bars + i, phase[i]);
  }
}

// Gather for other widths: a point per thread over its N2^3 stencil in the tile.
template <int N2, int CP, typename TO>
__global__ void __launch_bounds__(kThreads, 1)
    k_gather_staged_generic(const __grid_constant__ CUtensorMap tmap, StagedGeo g, SchemeT<float, N2> s,
                            const uint32_t *__restrict__ cell_start, const float4 *__restrict__ rec,
                            const uint32_t *__restrict__ perm, TO *__restrict__ out, int32_t *status,
                            int nbuf, uint32_t tile_bytes, uint32_t box_bytes) {
  extern __shared__ __align__(1024) unsigned char smem[];
  uint64_t *bars = reinterpret_cast<uint64_t *>(smem + nbuf * tile_bytes);
  if (threadIdx.x == 0) {
    for (int i = 0; i < nbuf; ++i) mbar_init(bars + i, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  uint32_t phase[2] = {0, 0};
  bool failed = false;
  auto issue = [&](int64_t b, int buf) {
    int64_t bx, by, bz;
    brick_coords(g, b, bx, by, bz);
    mbar_expect_tx(bars + buf, box_bytes);
    tma_load_tile(smem + buf * tile_bytes, &tmap, 0, (int)(bx * g.b[0]) + g.box_off,
                  (int)(by * g.b[1]) + g.box_off, (int)(bz * g.b[2]) + g.box_off, bars + buf);
  };
  auto nonempty = [&](int64_t b) { return __ldg(cell_start + (b + 1) * g.bvol) > __ldg(cell_start + b * g.bvol); };
  int64_t b = blockIdx.x;
  if (threadIdx.x == 0 && b < g.nbricks && nonempty(b)) issue(b, 0);
  for (int it = 0; b < g.nbricks; ++it, b += gridDim.x) {
    const int buf = nbuf == 2 ? (it & 1) : 0;
    const int64_t bn = b + gridDim.x;
    const uint32_t s0 = __ldg(cell_start + b * g.bvol), s1 = __ldg(cell_start + (b + 1) * g.bvol);
    if (nbuf == 2 && threadIdx.x == 0 && bn < g.nbricks && nonempty(bn)) issue(bn, buf ^ 1);
    if (s1 > s0) {
      if (!mbar_wait(bars + buf, phase[buf])) {
        failed = true;
        if (threadIdx.x == 0 && status) atomicOr(status, GBG_DEV_TIMEOUT);
        break;
      }
      phase[buf] ^= 1;
      const float *tile = reinterpret_cast<const float *>(smem + buf * tile_bytes);
      for (uint32_t sl = s0 + threadIdx.x; sl < s1; sl += kThreads) {
        const float4 r = __ldg(rec + sl);
        const uint32_t loc = __float_as_uint(r.w);
        const int lx = loc % g.b[0], ly = (loc / g.b[0]) % g.b[1], lz = loc / (g.b[0] * g.b[1]);
        float w1[N2], w2[N2], w3[N2];
#pragma unroll
        for (int q = 0; q < N2; ++q) {
          w1[q] = poly<N2>(s, q, r.x);
          w2[q] = poly<N2>(s, q, r.y);
          w3[q] = poly<N2>(s, q, r.z);
        }
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
            const float *row = tile + (((lz + k) * g.w[1] + ly + j) * g.w[0] + lx) * CP;
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
        const int64_t p = perm[sl];
#pragma unroll
        for (int c = 0; c < CP; ++c)
          if (c < g.ncomp) store_out(out, p + g.m * c, acc[c]);
      }
    }
    __syncthreads();
    if (nbuf == 1 && threadIdx.x == 0 && bn < g.nbricks && nonempty(bn)) issue(bn, 0);
  }
  if (failed)
    for (int i = 0; i < nbuf; ++i) mbar_wait(bars + i, phase[i]);
}

// ------------------------------------------------------------ staged scatter

// Sorted, alpha-scaled quantities: qs[s*CP + c] = T(alpha) * q[perm[s] + M*c].
template <typename TQ>
__global__ void k_scatter_qprep(const TQ *__restrict__ q, const uint32_t *__restrict__ perm, int64_t m,
                                int ncomp, int cp, float alpha, float *__restrict__ qs) {
  for (int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; s < m;
       s += (int64_t)gridDim.x * blockDim.x) {
    const int64_t p = perm[s];
    for (int c = 0; c < cp; ++c) qs[s * cp + c] = c < ncomp ? alpha * (float)q[p + m * c] : 0.0f;
  }
}

struct PullGeo {
  int32_t b[3];
  int64_t nb[3];
  int64_t n[3];
  int32_t e[3];  // extended cell region = brick + width - 1
  int64_t nbricks, bvol;
  int64_t px, py;
  int32_t halo, cp;
};

__device__ __forceinline__ void neumaier(float &sum, float &comp, float v) {
  const float t = __fadd_rn(sum, v);
  if (fabsf(sum) >= fabsf(v))
    comp = __fadd_rn(comp, __fadd_rn(__fsub_rn(sum, t), v));
  else
    comp = __fadd_rn(comp, __fadd_rn(__fsub_rn(v, t), sum));
  sum = t;
}

// One CTA per brick (persistent): stage the point ranges of the cells whose stencils
// reach the brick, then each thread pulls for its nodes.  Weight index i reaches node x
// from cell x + n - i; in the extended region that cell is at ex = lx + N2 - 1 - i.
template <int N2, int CP>
__global__ void __launch_bounds__(kThreads)
    k_scatter_pull_staged(PullGeo g, SchemeT<float, N2> s, const uint32_t *__restrict__ cell_start,
                          const float4 *__restrict__ rec, const float *__restrict__ qs, float *__restrict__ field,
                          float beta, int beta_zero, int compensated) {
  extern __shared__ uint32_t ranges[];  // 2 per extended cell
  constexpr int nbw = (N2 - 2) / 2;
  const int ecount = g.e[0] * g.e[1] * g.e[2];
  for (int64_t b = blockIdx.x; b < g.nbricks; b += gridDim.x) {
    const int64_t bx = b % g.nb[0], by = (b / g.nb[0]) % g.nb[1], bz = b / (g.nb[0] * g.nb[1]);
    __syncthreads();
    for (int e = threadIdx.x; e < ecount; e += blockDim.x) {
      const int ex = e % g.e[0], ey = (e / g.e[0]) % g.e[1], ez = e / (g.e[0] * g.e[1]);
      const int64_t cx = imod(bx * g.b[0] - nbw - 1 + ex, g.n[0]);
      const int64_t cy = imod(by * g.b[1] - nbw - 1 + ey, g.n[1]);
      const int64_t cz = imod(bz * g.b[2] - nbw - 1 + ez, g.n[2]);
      const int64_t kb = ((cz / g.b[2]) * g.nb[1] + cy / g.b[1]) * g.nb[0] + cx / g.b[0];
      const int64_t key = kb * g.bvol + ((cz % g.b[2]) * g.b[1] + cy % g.b[1]) * g.b[0] + cx % g.b[0];
      ranges[2 * e] = __ldg(cell_start + key);
      ranges[2 * e + 1] = __ldg(cell_start + key + 1);
    }
    __syncthreads();
    const int nodes = g.b[0] * g.b[1] * g.b[2];
    for (int nl = threadIdx.x; nl < nodes; nl += blockDim.x) {
      const int lx = nl % g.b[0], ly = (nl / g.b[0]) % g.b[1], lz = nl / (g.b[0] * g.b[1]);
      const int64_t x = bx * g.b[0] + lx, y = by * g.b[1] + ly, z = bz * g.b[2] + lz;
      if (x >= g.n[0] || y >= g.n[1] || z >= g.n[2]) continue;
      float sum[CP], comp[CP];
#pragma unroll
      for (int c = 0; c < CP; ++c) sum[c] = comp[c] = 0.0f;
#pragma unroll 1
      for (int k = 0; k < N2; ++k) {
#pragma unroll 1
        for (int j = 0; j < N2; ++j) {
#pragma unroll 1
          for (int i = 0; i < N2; ++i) {
            const int e = ((lz + N2 - 1 - k) * g.e[1] + (ly + N2 - 1 - j)) * g.e[0] + (lx + N2 - 1 - i);
            const uint32_t r0 = ranges[2 * e], r1 = ranges[2 * e + 1];
            for (uint32_t sl = r0; sl < r1; ++sl) {
              const float4 r = __ldg(rec + sl);
              const float w = __fmul_rn(__fmul_rn(poly<N2>(s, j, r.y), poly<N2>(s, k, r.z)), poly<N2>(s, i, r.x));
              const float4 *qv = reinterpret_cast<const float4 *>(qs + (int64_t)sl * CP);
#pragma unroll
              for (int q4 = 0; q4 < CP / 4; ++q4) {
                const float4 v = __ldg(qv + q4);
                const float vv[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                  const float add = __fmul_rn(w, vv[u]);
                  if (compensated)
                    neumaier(sum[4 * q4 + u], comp[4 * q4 + u], add);
                  else
                    sum[4 * q4 + u] = __fadd_rn(sum[4 * q4 + u], add);
                }
              }
            }
          }
        }
      }
      float *d = field + ((x + g.halo) + g.px * ((y + g.halo) + g.py * (z + g.halo))) * CP;
#pragma unroll
      for (int c = 0; c < CP; ++c) {
        const float total = __fadd_rn(sum[c], comp[c]);
        d[c] = beta_zero ? total : __fadd_rn(__fmul_rn(beta, d[c]), total);
      }
    }
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
  return g;
}

template <int N2, typename TO>
gbg_status launch_staged_gather(gbg_field_s *f, gbg_bins_s *b, const gbg_scheme &sch, TO *out, cudaStream_t st) {
  CUtensorMap *map = nullptr;
  GBG_TRY(tensor_map_for(f, N2, b->b, &map));
  const StagedGeo g = staged_geo(f, b, N2);
  const SchemeT<float, N2> s = make_scheme<float, N2>(sch);
  // the copy's exact byte count (what the mbarrier expects) and the buffer stride
  const uint32_t box_bytes = (uint32_t)((size_t)f->cp * 4 * g.w[0] * g.w[1] * g.w[2]);
  const uint32_t tile_bytes = (box_bytes + 1023u) & ~1023u;
  const int nbuf = (2 * (size_t)tile_bytes + 64 <= 200 * 1024) ? 2 : 1;
  const size_t smem = (size_t)nbuf * tile_bytes + 64;
  if (smem > 227 * 1024) return set_error(GBG_EUNSUPPORTED, "brick halo tile does not fit in shared memory");
  int sms = 0, dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int blocks = (int)std::min<int64_t>(b->nbricks, (int64_t)sms);
  int32_t *status = nullptr;
  auto go = [&](auto kernel) -> gbg_status {
    GBG_CUDA_TRY(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    kernel<<<blocks, kThreads, smem, st>>>(*map, g, s, b->cell_start, b->rec, b->perm, out, status, nbuf, tile_bytes,
                                            box_bytes);
    note_launch();
    GBG_CUDA_TRY(cudaGetLastError());
    return GBG_OK;
  };
  if constexpr (N2 == 4) {
    if (f->cp == 4) return go(k_gather_staged4<4, TO>);
    return go(k_gather_staged4<12, TO>);
  } else {
    if (f->cp == 4) return go(k_gather_staged_generic<N2, 4, TO>);
    return go(k_gather_staged_generic<N2, 12, TO>);
  }
}

template <int N2>
gbg_status launch_staged_scatter(gbg_field_s *f, gbg_bins_s *b, const gbg_scheme &sch, double beta,
                                 cudaStream_t st) {
  PullGeo g;
  for (int d = 0; d < 3; ++d) {
    g.b[d] = b->b[d];
    g.nb[d] = b->nb[d];
    g.n[d] = f->grid.n[d];
    g.e[d] = b->b[d] + N2 - 1;
  }
  g.nbricks = b->nbricks;
  g.bvol = b->bvol;
  g.px = f->px;
  g.py = f->py;
  g.halo = f->halo;
  g.cp = f->cp;
  const SchemeT<float, N2> s = make_scheme<float, N2>(sch);
  const size_t smem = sizeof(uint32_t) * 2 * g.e[0] * g.e[1] * g.e[2];
  if (smem > 200 * 1024) return set_error(GBG_EUNSUPPORTED, "brick too large for the scatter's cell ranges");
  int sms = 0, dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int blocks = (int)std::min<int64_t>(b->nbricks, (int64_t)sms * 4);
  auto go = [&](auto kernel) -> gbg_status {
    GBG_CUDA_TRY(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    kernel<<<blocks, kThreads, smem, st>>>(g, s, b->cell_start, b->rec, b->qs, f->data, (float)beta, beta == 0.0, 1);
    note_launch();
    GBG_CUDA_TRY(cudaGetLastError());
    return GBG_OK;
  };
  if (f->cp == 4) return go(k_scatter_pull_staged<N2, 4>);
  return go(k_scatter_pull_staged<N2, 12>);
}

}  // namespace
}  // namespace gbg

using namespace gbg;

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
  if (max_points < 0 || max_points > 0x7fffffffLL) return set_error(GBG_EUNSUPPORTED, "point count outside 0..2^31-1");
  auto *b = new (std::nothrow) gbg_bins_s;
  if (!b) return set_error(GBG_ENOMEM, "host allocation failed");
  cudaGetDevice(&b->device);
  b->grid = *grid;
  b->max_points = max_points;
  for (int d = 0; d < 3; ++d) {
    if (brick) b->b[d] = brick[d];
    if (b->b[d] < 1 || b->b[d] > 64) {
      delete b;
      return set_error(GBG_EARG, "brick edges must be 1..64 cells");
    }
    b->nb[d] = (grid->n[d] + b->b[d] - 1) / b->b[d];
  }
  b->bvol = (int64_t)b->b[0] * b->b[1] * b->b[2];
  b->nbricks = b->nb[0] * b->nb[1] * b->nb[2];
  b->nkeys = b->nbricks * b->bvol;
  if (b->nkeys >= (int64_t(1) << 32) - 1) {
    delete b;
    return set_error(GBG_EUNSUPPORTED, "bins: 2^32 or more cells");
  }
  const int64_t m = max_points > 0 ? max_points : 1;
  Arena a;
  a.take<uint32_t>(m);
  a.take<uint32_t>(m);
  a.take<uint32_t>(m);
  a.take<uint32_t>((size_t)b->nkeys + 1);
  a.take<float4>(m);
  a.take<float4>(m);
  a.take<char>(radix_sort_temp_bytes(m));
  a.take<uint32_t>(scan_temp_elems(b->nkeys + 1));
  a.take<float>((size_t)m * 12);
  b->bytes = a.used + 256;
  if (cudaMalloc(&b->block, b->bytes) != cudaSuccess) {
    cudaGetLastError();
    delete b;
    return set_error(GBG_ENOMEM, "cudaMalloc of the bins failed");
  }
  a.base = static_cast<char *>(b->block);
  a.used = 0;
  b->keys = a.take<uint32_t>(m);
  b->skeys = a.take<uint32_t>(m);
  b->perm = a.take<uint32_t>(m);
  b->cell_start = a.take<uint32_t>((size_t)b->nkeys + 1);
  b->rec_user = a.take<float4>(m);
  b->rec = a.take<float4>(m);
  b->sort_tmp = a.take<char>(radix_sort_temp_bytes(m));
  b->scan_tmp = a.take<uint32_t>(scan_temp_elems(b->nkeys + 1));
  b->qs = a.take<float>((size_t)m * 12);
  cudaMemset(b->cell_start, 0, sizeof(uint32_t) * ((size_t)b->nkeys + 1));
  *out = b;
  return GBG_OK;
}

gbg_status gbg_bins_destroy(gbg_bins b) {
  clear_error();
  if (!b) return GBG_OK;
  cudaFree(b->block);
  delete b;
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
  b->npoints = npoints;
  GBG_CUDA_TRY(cudaMemsetAsync(b->cell_start, 0, sizeof(uint32_t) * ((size_t)b->nkeys + 1), st));
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
  if (pos_dtype == GBG_F64)
    k_bin_keys<double><<<blocks, kThreads, 0, st>>>(g, static_cast<const double *>(positions), npoints, b->keys,
                                                    b->cell_start, b->rec_user, device_status);
  else
    k_bin_keys<float><<<blocks, kThreads, 0, st>>>(g, static_cast<const float *>(positions), npoints, b->keys,
                                                   b->cell_start, b->rec_user, device_status);
  note_launch();
  GBG_CUDA_TRY(cudaGetLastError());
  int bits = 0;
  while (bits < 32 && ((uint64_t)(b->nkeys - 1) >> bits) != 0) ++bits;
  GBG_TRY(radix_sort_pairs(b->keys, nullptr, b->skeys, b->perm, npoints, bits, b->sort_tmp, st));
  GBG_TRY(exclusive_scan_u32(b->cell_start, b->cell_start, b->nkeys + 1, b->scan_tmp, st));
  k_gather_records<<<blocks, kThreads, 0, st>>>(b->rec_user, b->perm, npoints, b->rec);
  note_launch();
  GBG_CUDA_TRY(cudaGetLastError());
  return GBG_OK;
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
                                  void *out, void *stream) {
  clear_error();
  GBG_TRY(check_field_bins(f, b, scheme));
  if (out_dtype != GBG_F32 && out_dtype != GBG_F64) return set_error(GBG_EARG, "bad dtype");
  if (b->npoints == 0) return GBG_OK;
  if (!out) return set_error(GBG_EARG, "null output");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  auto run = [&](auto *o) -> gbg_status {
    switch (scheme->stencil_width) {
      case 2: return launch_staged_gather<2>(f, b, *scheme, o, st);
      case 4: return launch_staged_gather<4>(f, b, *scheme, o, st);
      case 6: return launch_staged_gather<6>(f, b, *scheme, o, st);
      default: return launch_staged_gather<8>(f, b, *scheme, o, st);
    }
  };
  if (out_dtype == GBG_F64) return run(static_cast<double *>(out));
  return run(static_cast<float *>(out));
}

gbg_status gbg_anterpolate_binned(gbg_field f, gbg_bins b, const gbg_scheme *scheme, gbg_dtype q_dtype,
                                  const void *q, double alpha, double beta, void *stream) {
  clear_error();
  GBG_TRY(check_field_bins(f, b, scheme));
  if (q_dtype != GBG_F32 && q_dtype != GBG_F64) return set_error(GBG_EARG, "bad dtype");
  if (b->npoints > 0 && !q) return set_error(GBG_EARG, "null quantities");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const int64_t m = b->npoints;
  if (m > 0) {
    const int blocks = launch_blocks(m, kThreads);
    if (q_dtype == GBG_F64)
      k_scatter_qprep<double><<<blocks, kThreads, 0, st>>>(static_cast<const double *>(q), b->perm, m, f->ncomp, f->cp,
                                                           (float)alpha, b->qs);
    else
      k_scatter_qprep<float><<<blocks, kThreads, 0, st>>>(static_cast<const float *>(q), b->perm, m, f->ncomp, f->cp,
                                                          (float)alpha, b->qs);
    note_launch();
    GBG_CUDA_TRY(cudaGetLastError());
  }
  // With no points the pull still runs: it writes beta * field (beta == 0 clears).
  gbg_status s;
  switch (scheme->stencil_width) {
    case 2: s = launch_staged_scatter<2>(f, b, *scheme, beta, st); break;
    case 4: s = launch_staged_scatter<4>(f, b, *scheme, beta, st); break;
    case 6: s = launch_staged_scatter<6>(f, b, *scheme, beta, st); break;
    default: s = launch_staged_scatter<8>(f, b, *scheme, beta, st); break;
  }
  GBG_TRY(s);
  const int64_t total = f->px * f->py * f->pz;
  k_fill_ghosts<<<launch_blocks(total, kThreads), kThreads, 0, st>>>(f->data, f->cp, f->px, f->py, f->pz, f->halo,
                                                                     f->grid.n[0], f->grid.n[1], f->grid.n[2]);
  note_launch();
  GBG_CUDA_TRY(cudaGetLastError());
  return GBG_OK;
}

}  // extern "C"
