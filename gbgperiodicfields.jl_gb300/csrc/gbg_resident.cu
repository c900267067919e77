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
// Scatter: a CTA owns a brick's nodes and adds every contribution of the points whose
// stencils reach the brick into two-level int32 fixed-point accumulators in shared memory
// (exact, order-independent integer sums: no float atomics, bitwise reproducible), then
// writes each node once.
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
  unsigned *qmax_bits = nullptr;  // largest |alpha q| of the last scatter, as float bits
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

// Gather: width-4 stencils, a point per quarter-warp, 512 threads (64 quarter-warps) per
// CTA; each quarter-warp loads its next point's record and index while it computes.
constexpr int kGatherThreads = 512;
template <int M2, int CP, typename TO>
__global__ void __launch_bounds__(kGatherThreads, 1)
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
  const int nqw = kGatherThreads / 8;
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
      uint32_t sl = s0 + qw;
      float4 r_next = sl < s1 ? __ldg(rec + sl) : make_float4(0.f, 0.f, 0.f, 0.f);
      uint32_t p_next = sl < s1 ? __ldg(perm + sl) : 0u;
      for (; sl < s1; sl += nqw) {
        const float4 r = r_next;
        const int64_t p = p_next;
        if (sl + nqw < s1) {
          r_next = __ldg(rec + sl + nqw);
          p_next = __ldg(perm + sl + nqw);
        }
        const uint32_t loc = __float_as_uint(r.w);
        const int lx = loc % g.b[0], ly = (loc / g.b[0]) % g.b[1], lz = loc / (g.b[0] * g.b[1]);
        float wx[4], wy[4], w3[4];
        weights_all<4, M2>(s, r.x, wx);
        weights_all<4, M2>(s, r.y, wy);
        weights_all<4, M2>(s, r.z, w3);
        const float w1 = pick(wx, qi);
        const float w2a = pick(wy, 2 * jj), w2b = pick(wy, 2 * jj + 1);
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
template <int N2, int M2, int CP, typename TO>
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
// Also the largest |alpha q| (as ordered float bits; NaN orders above every number, so a
// NaN quantity shows as a non-finite bound).
template <typename TQ>
__global__ void k_scatter_qprep(const TQ *__restrict__ q, const uint32_t *__restrict__ perm, int64_t m,
                                int ncomp, int cp, float alpha, float *__restrict__ qs,
                                unsigned *__restrict__ qmax_bits) {
  unsigned mx = 0u;
  for (int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; s < m;
       s += (int64_t)gridDim.x * blockDim.x) {
    const int64_t p = perm[s];
    for (int c = 0; c < cp; ++c) {
      const float v = c < ncomp ? alpha * (float)q[p + m * c] : 0.0f;
      qs[s * cp + c] = v;
      const unsigned bits = __float_as_uint(fabsf(v));
      mx = bits > mx ? bits : mx;
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned other = __shfl_xor_sync(0xffffffffu, mx, o);
    mx = other > mx ? other : mx;
  }
  if ((threadIdx.x & 31) == 0) atomicMax(qmax_bits, mx);
}

struct FixGeo {
  int32_t b[3];
  int64_t nb[3];
  int64_t n[3];
  int32_t e[3];  // extended cell region = brick + width - 1
  int64_t nbricks, bvol;
  int64_t px, py;
  int32_t halo, cp, ncomp;
  double l3;  // bound on |w1*w2*w3|: (max_q sum_r |c[q,r]|)^3
};

// Deterministic scatter.  A CTA owns a brick's nodes; it walks the points of every cell
// whose stencil reaches the brick (the extended region) and adds each contribution
// w*alpha*q to fixed-point accumulators in shared memory.  Integer addition is
// associative, so the sums -- and the result -- do not depend on the order in which the
// threads add, and no float atomics are involved.
//
// Each contribution x = w*q*S1 (S1 a power of two) is split into its nearest integer hi
// and the residual r = x - hi, |r| <= 1/2, kept as lo = round(r * 2^k); hi and lo go to
// two int32 accumulators.  Both roundings use the float "magic number" 1.5*2^23 (an FMA
// lands the value where the float's ulp is 1), so no slow int64 conversion or atomic is
// needed.  S1 and k come from bounds on one contribution (max|alpha q| * l3) and on a
// node's sum (points in the region times that), so neither accumulator can overflow; the
// result carries about 2^-41 of max|alpha q| * l3 per contribution.
constexpr float kMagic = 12582912.0f;  // 1.5 * 2^23
constexpr int kMagicBits = 0x4B400000;

__device__ __forceinline__ void add_fixed(int *hi_acc, int *lo_acc, int idx, float w, float q, float lo_scale) {
  const float h = fmaf(w, q, kMagic);
  const float hi_f = h - kMagic;  // exact: an integer below 2^22
  const float r = fmaf(w, q, -hi_f);
  const float l = fmaf(r, lo_scale, kMagic);
  atomicAdd(hi_acc + idx, __float_as_int(h) - kMagicBits);
  atomicAdd(lo_acc + idx, __float_as_int(l) - kMagicBits);
}

template <int N2, int M2, int CP>
__global__ void __launch_bounds__(kThreads, 2)
    k_scatter_fixed(FixGeo g, SchemeT<float, N2> s, const uint32_t *__restrict__ cell_start,
                    const float4 *__restrict__ rec, const float *__restrict__ qs,
                    const unsigned *__restrict__ qmax_bits, float *__restrict__ field, float beta,
                    int beta_zero, int32_t *status) {
  extern __shared__ int acc_hi[];  // bvol * CP hi, bvol * CP lo, then the cell ranges
  int *acc_lo = acc_hi + g.bvol * CP;
  uint32_t *ranges = reinterpret_cast<uint32_t *>(acc_lo + g.bvol * CP);
  __shared__ unsigned int s_count;
  constexpr int nbw = (N2 - 2) / 2;
  const int ecount = g.e[0] * g.e[1] * g.e[2];
  const float qmax = __uint_as_float(*qmax_bits);
  for (int64_t b = blockIdx.x; b < g.nbricks; b += gridDim.x) {
    const int64_t bx = b % g.nb[0], by = (b / g.nb[0]) % g.nb[1], bz = b / (g.nb[0] * g.nb[1]);
    __syncthreads();
    for (int64_t i = threadIdx.x; i < 2 * g.bvol * CP; i += blockDim.x) acc_hi[i] = 0;
    if (threadIdx.x == 0) s_count = 0u;
    __syncthreads();
    unsigned mine = 0;
    for (int e = threadIdx.x; e < ecount; e += blockDim.x) {
      const int ex = e % g.e[0], ey = (e / g.e[0]) % g.e[1], ez = e / (g.e[0] * g.e[1]);
      const int64_t cx = imod(bx * g.b[0] - nbw - 1 + ex, g.n[0]);
      const int64_t cy = imod(by * g.b[1] - nbw - 1 + ey, g.n[1]);
      const int64_t cz = imod(bz * g.b[2] - nbw - 1 + ez, g.n[2]);
      const int64_t kb = ((cz / g.b[2]) * g.nb[1] + cy / g.b[1]) * g.nb[0] + cx / g.b[0];
      const int64_t key = kb * g.bvol + ((cz % g.b[2]) * g.b[1] + cy % g.b[1]) * g.b[0] + cx % g.b[0];
      const uint32_t r0 = __ldg(cell_start + key), r1 = __ldg(cell_start + key + 1);
      ranges[2 * e] = r0;
      ranges[2 * e + 1] = r1;
      mine += r1 - r0;
    }
    atomicAdd(&s_count, mine);
    __syncthreads();
    const unsigned count = s_count;
    const double one = (double)qmax * g.l3;        // bound on one contribution
    const double bound = one * (double)count;      // bound on a node's sum
    const bool finite = isfinite(bound);
    if (!finite && threadIdx.x == 0 && status) atomicOr(status, GBG_DEV_NONFINITE);
    int e1 = 0, es = 0;
    frexp(one, &e1);
    frexp(bound, &es);
    int s1 = min(20 - e1, 29 - es);
    s1 = max(-120, min(120, s1));
    const int kbits = min(21, 30 - (32 - __clz((int)count)));
    const float S1 = exp2f((float)s1), LS = exp2f((float)kbits);
    if (finite && count > 0 && one > 0.0) {
      if constexpr (N2 == 4) {
        const int qw = threadIdx.x >> 3, sub = threadIdx.x & 7, qi = sub & 3, jj = sub >> 2;
        for (int e = qw; e < ecount; e += kThreads / 8) {
          const uint32_t r0 = ranges[2 * e], r1 = ranges[2 * e + 1];
          if (r0 == r1) continue;
          const int ex = e % g.e[0], ey = (e / g.e[0]) % g.e[1], ez = e / (g.e[0] * g.e[1]);
          const int lx = ex + qi - 3;
          const bool inx = lx >= 0 && lx < g.b[0] && bx * g.b[0] + lx < g.n[0];
          for (uint32_t sl = r0; sl < r1; ++sl) {
            const float4 r = __ldg(rec + sl);
            float wx[4], wy[4], wz[4];
            weights_all<4, M2>(s, r.x, wx);
            weights_all<4, M2>(s, r.y, wy);
            weights_all<4, M2>(s, r.z, wz);
            const float w1s = pick(wx, qi) * S1;
            float q[CP];
            const float4 *q4 = reinterpret_cast<const float4 *>(qs + (int64_t)sl * CP);
#pragma unroll
            for (int v = 0; v < CP / 4; ++v) {
              const float4 t = __ldg(q4 + v);
              q[4 * v] = t.x;
              q[4 * v + 1] = t.y;
              q[4 * v + 2] = t.z;
              q[4 * v + 3] = t.w;
            }
            if (!inx) continue;
#pragma unroll
            for (int jp = 0; jp < 2; ++jp) {
              const int ly = ey + 2 * jj + jp - 3;
              if (ly < 0 || ly >= g.b[1] || by * g.b[1] + ly >= g.n[1]) continue;
              const float wxy = w1s * pick(wy, 2 * jj + jp);
#pragma unroll
              for (int k = 0; k < 4; ++k) {
                const int lz = ez + k - 3;
                if (lz < 0 || lz >= g.b[2] || bz * g.b[2] + lz >= g.n[2]) continue;
                const float w = wxy * wz[k];
                const int node = (lz * g.b[1] + ly) * g.b[0] + lx;
#pragma unroll
                for (int c = 0; c < CP; ++c) add_fixed(acc_hi, acc_lo, c * (int)g.bvol + node, w, q[c], LS);
              }
            }
          }
        }
      } else {
        for (int e = threadIdx.x; e < ecount; e += kThreads) {
          const uint32_t r0 = ranges[2 * e], r1 = ranges[2 * e + 1];
          if (r0 == r1) continue;
          const int ex = e % g.e[0], ey = (e / g.e[0]) % g.e[1], ez = e / (g.e[0] * g.e[1]);
          for (uint32_t sl = r0; sl < r1; ++sl) {
            const float4 r = __ldg(rec + sl);
            float wx[N2], wy[N2], wz[N2];
            weights_all<N2, M2>(s, r.x, wx);
            weights_all<N2, M2>(s, r.y, wy);
            weights_all<N2, M2>(s, r.z, wz);
            const float *q = qs + (int64_t)sl * CP;
#pragma unroll 1
            for (int k = 0; k < N2; ++k) {
              const int lz = ez + k - (N2 - 1);
              if (lz < 0 || lz >= g.b[2] || bz * g.b[2] + lz >= g.n[2]) continue;
#pragma unroll 1
              for (int j = 0; j < N2; ++j) {
                const int ly = ey + j - (N2 - 1);
                if (ly < 0 || ly >= g.b[1] || by * g.b[1] + ly >= g.n[1]) continue;
#pragma unroll
                for (int i = 0; i < N2; ++i) {
                  const int lx = ex + i - (N2 - 1);
                  if (lx < 0 || lx >= g.b[0] || bx * g.b[0] + lx >= g.n[0]) continue;
                  const float w = wx[i] * wy[j] * wz[k] * S1;
                  const int node = (lz * g.b[1] + ly) * g.b[0] + lx;
                  for (int c = 0; c < CP; ++c) add_fixed(acc_hi, acc_lo, c * (int)g.bvol + node, w, __ldg(q + c), LS);
                }
              }
            }
          }
        }
      }
    }
    __syncthreads();
    // ordered write-back: every node of the brick is written once (in FP32: the value is
    // hi * 2^-s1 + lo * 2^-(s1+k); both products are exact scalings)
    const float to_value = exp2f((float)-s1), lo_value = exp2f((float)(-s1 - kbits));
    for (int64_t i = threadIdx.x; i < g.bvol * CP; i += blockDim.x) {
      const int64_t nl = i / CP;
      const int c = (int)(i - nl * CP);
      const int lx = (int)(nl % g.b[0]), ly = (int)((nl / g.b[0]) % g.b[1]), lz = (int)(nl / (g.b[0] * g.b[1]));
      const int64_t x = bx * g.b[0] + lx, y = by * g.b[1] + ly, z = bz * g.b[2] + lz;
      if (x >= g.n[0] || y >= g.n[1] || z >= g.n[2]) continue;
      float *d = field + ((x + g.halo) + g.px * ((y + g.halo) + g.py * (z + g.halo))) * CP + c;
      const int64_t a = (int64_t)c * g.bvol + nl;
      float v = finite ? fmaf((float)acc_hi[a], to_value, (float)acc_lo[a] * lo_value) : __int_as_float(0x7fc00000);
      if (c >= g.ncomp) v = 0.0f;
      *d = beta_zero ? v : __fadd_rn(__fmul_rn(beta, *d), v);
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

template <int N2, int M2, typename TO>
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
  const int threads = N2 == 4 ? kGatherThreads : kThreads;
  auto go = [&](auto kernel) -> gbg_status {
    GBG_CUDA_TRY(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    kernel<<<blocks, threads, smem, st>>>(*map, g, s, b->cell_start, b->rec, b->perm, out, status, nbuf, tile_bytes,
                                           box_bytes);
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

// Per-axis weight bound of a scheme: max over nodes of sum_r |c[q, r]| (|t| <= 1).
double axis_bound(const gbg_scheme &sch) {
  double best = 0.0;
  for (int q = 0; q < sch.stencil_width; ++q) {
    double s = 0.0;
    for (int r = 0; r < sch.num_powers; ++r) s += std::fabs(sch.coefficients[q + sch.stencil_width * r]);
    best = s > best ? s : best;
  }
  return best;
}

template <int N2, int M2>
gbg_status launch_staged_scatter(gbg_field_s *f, gbg_bins_s *b, const gbg_scheme &sch, double beta,
                                 const unsigned *qmax_bits, int32_t *status, cudaStream_t st) {
  FixGeo g;
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
  g.ncomp = f->ncomp;
  const double L = axis_bound(sch);
  g.l3 = L * L * L;
  const SchemeT<float, N2> s = make_scheme<float, N2>(sch);
  const size_t smem = 2 * sizeof(int) * (size_t)g.bvol * f->cp +
                      sizeof(uint32_t) * 2 * (size_t)g.e[0] * g.e[1] * g.e[2];
  if (smem > 200 * 1024) return set_error(GBG_EUNSUPPORTED, "brick too large for the scatter's shared accumulators");
  int sms = 0, dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int blocks = (int)std::min<int64_t>(b->nbricks, (int64_t)sms * 2);
  auto go = [&](auto kernel) -> gbg_status {
    GBG_CUDA_TRY(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    kernel<<<blocks, kThreads, smem, st>>>(g, s, b->cell_start, b->rec, b->qs, qmax_bits, f->data, (float)beta,
                                           beta == 0.0, status);
    note_launch();
    GBG_CUDA_TRY(cudaGetLastError());
    return GBG_OK;
  };
  if (f->cp == 4) return go(k_scatter_fixed<N2, M2, 4>);
  return go(k_scatter_fixed<N2, M2, 12>);
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
  a.take<unsigned>(64);
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
  b->qmax_bits = a.take<unsigned>(64);
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
      // compile-time (width, powers) for the common schemes, guarded Horner otherwise
      case 2: return scheme->num_powers == 2 ? launch_staged_gather<2, 2>(f, b, *scheme, o, st)
                                             : launch_staged_gather<2, 0>(f, b, *scheme, o, st);
      case 4: return scheme->num_powers == 4 ? launch_staged_gather<4, 4>(f, b, *scheme, o, st)
                                             : launch_staged_gather<4, 0>(f, b, *scheme, o, st);
      case 6: return scheme->num_powers == 6 ? launch_staged_gather<6, 6>(f, b, *scheme, o, st)
                     : scheme->num_powers == 4 ? launch_staged_gather<6, 4>(f, b, *scheme, o, st)
                                               : launch_staged_gather<6, 0>(f, b, *scheme, o, st);
      default: return scheme->num_powers == 8 ? launch_staged_gather<8, 8>(f, b, *scheme, o, st)
                                              : launch_staged_gather<8, 0>(f, b, *scheme, o, st);
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
  GBG_CUDA_TRY(cudaMemsetAsync(b->qmax_bits, 0, sizeof(unsigned), st));
  if (m > 0) {
    const int blocks = launch_blocks(m, kThreads);
    if (q_dtype == GBG_F64)
      k_scatter_qprep<double><<<blocks, kThreads, 0, st>>>(static_cast<const double *>(q), b->perm, m, f->ncomp, f->cp,
                                                           (float)alpha, b->qs, b->qmax_bits);
    else
      k_scatter_qprep<float><<<blocks, kThreads, 0, st>>>(static_cast<const float *>(q), b->perm, m, f->ncomp, f->cp,
                                                          (float)alpha, b->qs, b->qmax_bits);
    note_launch();
    GBG_CUDA_TRY(cudaGetLastError());
  }
  // With no points the push still runs: it writes beta * field (beta == 0 clears).
  const int w = scheme->stencil_width, p = scheme->num_powers;
  gbg_status s;
  if (w == 2)
    s = p == 2 ? launch_staged_scatter<2, 2>(f, b, *scheme, beta, b->qmax_bits, nullptr, st)
               : launch_staged_scatter<2, 0>(f, b, *scheme, beta, b->qmax_bits, nullptr, st);
  else if (w == 4)
    s = p == 4 ? launch_staged_scatter<4, 4>(f, b, *scheme, beta, b->qmax_bits, nullptr, st)
               : launch_staged_scatter<4, 0>(f, b, *scheme, beta, b->qmax_bits, nullptr, st);
  else if (w == 6)
    s = p == 6 ? launch_staged_scatter<6, 6>(f, b, *scheme, beta, b->qmax_bits, nullptr, st)
               : launch_staged_scatter<6, 0>(f, b, *scheme, beta, b->qmax_bits, nullptr, st);
  else
    s = p == 8 ? launch_staged_scatter<8, 8>(f, b, *scheme, beta, b->qmax_bits, nullptr, st)
               : launch_staged_scatter<8, 0>(f, b, *scheme, beta, b->qmax_bits, nullptr, st);
  GBG_TRY(s);
  const int64_t total = f->px * f->py * f->pz;
  k_fill_ghosts<<<launch_blocks(total, kThreads), kThreads, 0, st>>>(f->data, f->cp, f->px, f->py, f->pz, f->halo,
                                                                     f->grid.n[0], f->grid.n[1], f->grid.n[2]);
  note_launch();
  GBG_CUDA_TRY(cudaGetLastError());
  return GBG_OK;
}

}  // extern "C"
