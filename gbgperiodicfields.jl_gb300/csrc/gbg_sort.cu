// Device prefix sum and stable LSD radix sort (sm_103a).
//
// The reference's traversal order is a counting sort whose placement goes through
// atomics, so points within a tile land in an unspecified order
// (Interpolation.jl:672-684).  Here the placement is a stable LSD radix sort of
// (key, point index) pairs: within a key the points keep their index order, which makes
// the order -- and every float sum that follows it -- identical run to run.
#include "gbg_common.cuh"

namespace gbg {

namespace {

constexpr int kScanThreads = 256;
constexpr int kScanItems = 8;
constexpr int kScanTile = kScanThreads * kScanItems;  // 2048

constexpr int kRsThreads = 256;
constexpr int kRsItems = 16;
constexpr int kRsWarps = kRsThreads / 32;
constexpr int kRsTile = kRsThreads * kRsItems;  // 4096
constexpr int kRsBins = 256;

// Block-wide exclusive scan of one value per thread; returns the block total via *total.
__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t v, uint32_t *warp_sums,
                                                         uint32_t *total) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) warp_sums[warp] = x;
  __syncthreads();
  if (warp == 0) {
    uint32_t s = lane < (int)(blockDim.x >> 5) ? warp_sums[lane] : 0u;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      uint32_t y = __shfl_up_sync(0xffffffffu, s, o);
      if (lane >= o) s += y;
    }
    if (lane < (int)(blockDim.x >> 5)) warp_sums[lane] = s;  // inclusive over warps
  }
  __syncthreads();
  const uint32_t warp_prefix = warp ? warp_sums[warp - 1] : 0u;
  *total = warp_sums[(blockDim.x >> 5) - 1];
  return warp_prefix + x - v;
}

__global__ void __launch_bounds__(kScanThreads) k_block_sums(const uint32_t *in, int64_t n,
                                                             uint32_t *sums, const uint32_t *gate) {
  if (gate && __ldg(gate) == 0u) return;
  __shared__ uint32_t ws[32];
  const int64_t base = (int64_t)blockIdx.x * kScanTile;
  uint32_t s = 0;
#pragma unroll
  for (int r = 0; r < kScanItems; ++r) {
    const int64_t i = base + r * kScanThreads + threadIdx.x;
    if (i < n) s += in[i];
  }
  uint32_t total;
  block_exclusive_scan(s, ws, &total);
  if (threadIdx.x == 0) sums[blockIdx.x] = total;
}

// Scans one tile (coalesced through shared memory) and adds offsets[blockIdx.x] if given.
// in may equal out: a block only reads and writes its own tile.
__global__ void __launch_bounds__(kScanThreads) k_scan_tile(const uint32_t *in, uint32_t *out,
                                                            int64_t n, const uint32_t *offsets,
                                                            const uint32_t *gate) {
  if (gate && __ldg(gate) == 0u) return;
  __shared__ uint32_t tile[kScanTile];
  __shared__ uint32_t ws[32];
  const int64_t base = (int64_t)blockIdx.x * kScanTile;
#pragma unroll
  for (int r = 0; r < kScanItems; ++r) {
    const int64_t i = base + r * kScanThreads + threadIdx.x;
    tile[r * kScanThreads + threadIdx.x] = i < n ? in[i] : 0u;
  }
  __syncthreads();
  uint32_t v[kScanItems];
  uint32_t s = 0;
#pragma unroll
  for (int r = 0; r < kScanItems; ++r) {
    v[r] = tile[threadIdx.x * kScanItems + r];
    s += v[r];
  }
  uint32_t total;
  uint32_t run = block_exclusive_scan(s, ws, &total) + (offsets ? offsets[blockIdx.x] : 0u);
#pragma unroll
  for (int r = 0; r < kScanItems; ++r) {
    tile[threadIdx.x * kScanItems + r] = run;
    run += v[r];
  }
  __syncthreads();
#pragma unroll
  for (int r = 0; r < kScanItems; ++r) {
    const int64_t i = base + r * kScanThreads + threadIdx.x;
    if (i < n) out[i] = tile[r * kScanThreads + threadIdx.x];
  }
}

__global__ void __launch_bounds__(kRsThreads) k_rs_hist(const uint32_t *keys, int64_t n, int shift,
                                                        uint32_t *hist, int64_t nb, const uint32_t *gate) {
  if (gate && __ldg(gate) == 0u) return;
  __shared__ uint32_t h[kRsWarps][kRsBins];
  for (int i = threadIdx.x; i < kRsWarps * kRsBins; i += kRsThreads) (&h[0][0])[i] = 0u;
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t seg = (int64_t)blockIdx.x * kRsTile + warp * (kRsItems * 32);
#pragma unroll 4
  for (int r = 0; r < kRsItems; ++r) {
    const int64_t i = seg + r * 32 + lane;
    if (i < n) atomicAdd(&h[warp][(keys[i] >> shift) & 0xFFu], 1u);
  }
  __syncthreads();
  for (int d = threadIdx.x; d < kRsBins; d += kRsThreads) {
    uint32_t s = 0;
#pragma unroll
    for (int w = 0; w < kRsWarps; ++w) s += h[w][d];
    hist[(int64_t)d * nb + blockIdx.x] = s;
  }
}

// Stable scatter of one digit pass.  Each warp owns a contiguous run of 512 items of the
// tile and ranks them in index order, so equal digits keep their relative order.  The tile
// is first put in digit order in shared memory, then every digit's run is written out
// contiguously (coalesced) at its global offset.
__global__ void __launch_bounds__(kRsThreads) k_rs_scatter(const uint32_t *keys_in,
                                                           const uint32_t *vals_in, int64_t n,
                                                           int shift, const uint32_t *offsets,
                                                           int64_t nb, uint32_t *keys_out,
                                                           uint32_t *vals_out, const uint32_t *gate) {
  static_assert(kRsThreads == kRsBins, "one thread per digit in the tile's digit scan");
  if (gate && __ldg(gate) == 0u) return;
  __shared__ uint32_t wh[kRsWarps][kRsBins];
  __shared__ uint32_t sbase[kRsBins], goff[kRsBins], ws[32];
  __shared__ uint32_t skey[kRsTile], sval[kRsTile];
  for (int i = threadIdx.x; i < kRsWarps * kRsBins; i += kRsThreads) (&wh[0][0])[i] = 0u;
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t tile0 = (int64_t)blockIdx.x * kRsTile;
  const int64_t seg = tile0 + warp * (kRsItems * 32);
  uint32_t key[kRsItems];
#pragma unroll
  for (int r = 0; r < kRsItems; ++r) {
    const int64_t i = seg + r * 32 + lane;
    key[r] = i < n ? keys_in[i] : 0u;
    if (i < n) atomicAdd(&wh[warp][(key[r] >> shift) & 0xFFu], 1u);
  }
  __syncthreads();
  {
    // thread d: the tile's digit-d items start at sbase[d] (an exclusive scan over digits);
    // warp w's start at sbase[d] plus the counts of the warps before it
    const int d = threadIdx.x;
    uint32_t cnt = 0;
#pragma unroll
    for (int w = 0; w < kRsWarps; ++w) cnt += wh[w][d];
    uint32_t total;
    uint32_t run = block_exclusive_scan(cnt, ws, &total);
    sbase[d] = run;
    goff[d] = offsets[(int64_t)d * nb + blockIdx.x];
#pragma unroll
    for (int w = 0; w < kRsWarps; ++w) {
      const uint32_t c = wh[w][d];
      wh[w][d] = run;
      run += c;
    }
  }
  __syncthreads();
  const uint32_t lower = (1u << lane) - 1u;
#pragma unroll
  for (int r = 0; r < kRsItems; ++r) {
    const int64_t i = seg + r * 32 + lane;
    const bool valid = i < n;
    const uint32_t digit = valid ? ((key[r] >> shift) & 0xFFu) : 0x100u;
    const uint32_t peers = __match_any_sync(0xffffffffu, digit);
    uint32_t pos = 0;
    if (valid) pos = wh[warp][digit] + __popc(peers & lower);
    __syncwarp();
    if (valid && lane == 31 - __clz(peers)) wh[warp][digit] += __popc(peers);
    __syncwarp();
    if (valid) {
      skey[pos] = key[r];
      sval[pos] = vals_in ? vals_in[i] : (uint32_t)i;
    }
  }
  __syncthreads();
  const int count = (int)min((int64_t)kRsTile, n - tile0);
  for (int j = threadIdx.x; j < count; j += kRsThreads) {
    const uint32_t k = skey[j];
    const uint32_t d = (k >> shift) & 0xFFu;
    const uint32_t gp = goff[d] + (uint32_t)j - sbase[d];
    keys_out[gp] = k;
    vals_out[gp] = sval[j];
  }
}

int sm_count_cached() {
  static int cached[64] = {0};
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= 64) dev = 0;
  if (!cached[dev]) {
    int v = 0;
    cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
    cached[dev] = v > 0 ? v : 1;
  }
  return cached[dev];
}

// Counting placement.  Every point p already holds rank[p], the value an atomic count of
// its key returned (unique within the key, but in no particular order), and starts[] is the
// exclusive scan of the counts: the slot starts[key] + rank is free for it.
__global__ void k_place_unstable(const uint32_t *__restrict__ keys, const uint32_t *__restrict__ rank,
                                 const uint32_t *__restrict__ starts, int64_t n, uint32_t *__restrict__ perm_u) {
  // four points a trip: keys and ranks, then the keys' starts, then the stores
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < n; p += 4 * stride) {
    uint32_t k[4], r[4], a[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const bool in = p + u * stride < n;
      k[u] = in ? __ldg(keys + p + u * stride) : 0u;
      r[u] = in ? __ldg(rank + p + u * stride) : 0u;
    }
#pragma unroll
    for (int u = 0; u < 4; ++u) a[u] = p + u * stride < n ? __ldg(starts + k[u]) : 0u;
#pragma unroll
    for (int u = 0; u < 4; ++u)
      if (p + u * stride < n) perm_u[a[u] + r[u]] = (uint32_t)(p + u * stride);
  }
}

// Makes the placement stable: the point in slot s moves to the position, within its key's
// run of slots, given by the number of the run's points with a smaller index.  Runs longer
// than kPlaceMaxRun are left alone and raise *big instead (the radix sort then redoes the
// whole order), so no thread does more than kPlaceMaxRun steps.
constexpr uint32_t kPlaceMaxRun = 1024;
__global__ void k_place_stable(const uint32_t *__restrict__ keys, const uint32_t *__restrict__ starts,
                               const uint32_t *__restrict__ perm_u, int64_t n, uint32_t *__restrict__ perm,
                               uint32_t *big, const float4 *__restrict__ rec_user, float4 *__restrict__ rec) {
  // two slots a trip, each level of their loads issued together
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t s0 = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; s0 < n; s0 += 2 * stride) {
    uint32_t pv[2], kv[2], av[2], cv[2];
    float4 rv[2] = {make_float4(0.f, 0.f, 0.f, 0.f), make_float4(0.f, 0.f, 0.f, 0.f)};
#pragma unroll
    for (int u = 0; u < 2; ++u) pv[u] = s0 + u * stride < n ? __ldg(perm_u + s0 + u * stride) : 0u;
#pragma unroll
    for (int u = 0; u < 2; ++u) {
      kv[u] = s0 + u * stride < n ? __ldg(keys + pv[u]) : 0u;
      if (rec && s0 + u * stride < n) rv[u] = __ldg(rec_user + pv[u]);
    }
#pragma unroll
    for (int u = 0; u < 2; ++u) {
      av[u] = s0 + u * stride < n ? __ldg(starts + kv[u]) : 0u;
      cv[u] = s0 + u * stride < n ? __ldg(starts + kv[u] + 1) - av[u] : 0u;
    }
#pragma unroll
    for (int u = 0; u < 2; ++u) {
      const int64_t s = s0 + u * stride;
      if (s >= n) continue;
      const uint32_t p = pv[u], a = av[u], c = cv[u];
      if (c == 1u) {
        perm[s] = p;
        if (rec) rec[s] = rv[u];
        continue;
      }
      if (c > kPlaceMaxRun) {
        atomicOr(big, 1u);
        continue;
      }
      uint32_t r = 0;
      for (uint32_t t = 0; t < c; ++t) r += __ldg(perm_u + a + t) < p ? 1u : 0u;
      perm[a + r] = p;
      if (rec) rec[a + r] = rv[u];
    }
  }
}

}  // namespace

int launch_blocks(int64_t work, int threads, int per_sm) {
  const int64_t want = (work + threads - 1) / threads;
  const int64_t cap = (int64_t)sm_count_cached() * per_sm;
  const int64_t b = want < cap ? want : cap;
  return (int)(b > 0 ? b : 1);
}

size_t scan_temp_elems(int64_t n) {
  size_t total = 0;
  int64_t m = n;
  while (m > kScanTile) {
    m = (m + kScanTile - 1) / kScanTile;
    total += (size_t)m + 64;
  }
  return total + 64;
}

gbg_status exclusive_scan_u32(const uint32_t *in, uint32_t *out, int64_t n, uint32_t *tmp,
                              cudaStream_t stream, const uint32_t *gate) {
  if (n <= 0) return GBG_OK;
  const int64_t nb = (n + kScanTile - 1) / kScanTile;
  if (nb == 1) {
    k_scan_tile<<<1, kScanThreads, 0, stream>>>(in, out, n, nullptr, gate);
    note_launch();
    GBG_CUDA_TRY(cudaGetLastError());
    return GBG_OK;
  }
  uint32_t *sums = tmp;
  uint32_t *rest = tmp + nb + 64;
  k_block_sums<<<(unsigned)nb, kScanThreads, 0, stream>>>(in, n, sums, gate);
  note_launch();
  GBG_CUDA_TRY(cudaGetLastError());
  GBG_TRY(exclusive_scan_u32(sums, sums, nb, rest, stream, gate));
  k_scan_tile<<<(unsigned)nb, kScanThreads, 0, stream>>>(in, out, n, sums, gate);
  note_launch();
  GBG_CUDA_TRY(cudaGetLastError());
  return GBG_OK;
}

size_t radix_sort_temp_bytes(int64_t n) {
  const int64_t nb = (n + kRsTile - 1) / kRsTile;
  Arena a;
  a.take<uint32_t>((size_t)(kRsBins * nb));
  a.take<uint32_t>(scan_temp_elems(kRsBins * nb));
  a.take<uint32_t>((size_t)n);
  a.take<uint32_t>((size_t)n);
  return a.used + 256;
}

gbg_status radix_sort_pairs(const uint32_t *keys_in, const uint32_t *vals_in, uint32_t *keys_out,
                            uint32_t *vals_out, int64_t n, int key_bits, void *temp,
                            cudaStream_t stream, const uint32_t *gate) {
  if (n <= 0) return GBG_OK;
  if (n > 0x7fffffffLL) return set_error(GBG_EUNSUPPORTED, "radix sort: more than 2^31-1 points");
  const int64_t nb = (n + kRsTile - 1) / kRsTile;
  Arena a;
  a.base = static_cast<char *>(temp);
  uint32_t *hist = a.take<uint32_t>((size_t)(kRsBins * nb));
  uint32_t *scan_tmp = a.take<uint32_t>(scan_temp_elems(kRsBins * nb));
  uint32_t *kt = a.take<uint32_t>((size_t)n);
  uint32_t *vt = a.take<uint32_t>((size_t)n);
  int passes = (key_bits + 7) / 8;
  if (passes < 1) passes = 1;
  const uint32_t *kin = keys_in;
  const uint32_t *vin = vals_in;
  for (int p = 0; p < passes; ++p) {
    const bool to_out = ((passes - 1 - p) % 2) == 0;
    uint32_t *kout = to_out ? keys_out : kt;
    uint32_t *vout = to_out ? vals_out : vt;
    k_rs_hist<<<(unsigned)nb, kRsThreads, 0, stream>>>(kin, n, 8 * p, hist, nb, gate);
    note_launch();
    GBG_CUDA_TRY(cudaGetLastError());
    GBG_TRY(exclusive_scan_u32(hist, hist, kRsBins * nb, scan_tmp, stream, gate));
    k_rs_scatter<<<(unsigned)nb, kRsThreads, 0, stream>>>(kin, vin, n, 8 * p, hist, nb, kout, vout, gate);
    note_launch();
    GBG_CUDA_TRY(cudaGetLastError());
    kin = kout;
    vin = vout;
  }
  return GBG_OK;
}


gbg_status stable_counting_sort(const uint32_t *keys, const uint32_t *rank, const uint32_t *starts, int64_t n,
                                int key_bits, uint32_t *perm, uint32_t *skeys, uint32_t *big, void *temp,
                                cudaStream_t stream, const float4 *rec_user, float4 *rec) {
  if (n <= 0) return GBG_OK;
  if (n > 0x7fffffffLL) return set_error(GBG_EUNSUPPORTED, "counting sort: more than 2^31-1 points");
  // the unstable placement lives at the start of the radix sort's scratch, which only the
  // fallback (after the stable pass has read it) writes
  uint32_t *perm_u = static_cast<uint32_t *>(temp);
  const int blocks = launch_blocks(n, 256);
  k_place_unstable<<<blocks, 256, 0, stream>>>(keys, rank, starts, n, perm_u);
  note_launch();
  k_place_stable<<<blocks, 256, 0, stream>>>(keys, starts, perm_u, n, perm, big, rec_user, rec);
  note_launch();
  GBG_CUDA_TRY(cudaGetLastError());
  return radix_sort_pairs(keys, nullptr, skeys, perm, n, key_bits, temp, stream, big);
}

}  // namespace gbg
