// grid.cu — the neighbour grid of one step: predict + cell hash, per-cell
// counts, a stable LSD radix sort of (cell id, particle index), and the
// exclusive prefix of cell counts that gives every cell its sorted range.
//
// Replaces buildGridHash (fluids/Simulator.cu:178-211): thrust::transform with
// getGridId, thrust::sort_by_key over zip(pos, vel, npos, nvel, iid), the two
// cudaMemsets and computeGridRange (fluids/Simulator_kernel.cuh:21-50).
// Instead of moving 52 B of payload through every sort pass, only the 4-byte
// index travels; the payload is gathered once afterwards (solver.cu: reorder).
// Ties keep input order (LSD radix passes are stable), which is the order the
// reference's in-place stable sort leaves.
#include "pbf_internal.cuh"

namespace pbf {

namespace {

constexpr int kRadixBits = 8;
constexpr int kRadix = 1 << kRadixBits;
constexpr int kSortThreads = 256;
constexpr int kSortItems = kSortTile / kSortThreads;  // 8
constexpr int kSortWarps = kSortThreads / 32;
constexpr int kScanThreads = 256;
constexpr int kScanItems = kScanTile / kScanThreads;  // 8
constexpr int kTopThreads = 1024;

static_assert(kSortThreads == kRadix, "one thread per digit in the rank-offset step");

// Exclusive scan of one value per thread across a block of THREADS threads.
// Returns the exclusive prefix; *total receives the block sum.
template <int THREADS>
__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t v, uint32_t* smem,
                                                         uint32_t* total) {
  static_assert(THREADS % 32 == 0 && THREADS / 32 <= 32, "block size");
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) smem[warp] = x;
  __syncthreads();
  if (warp == 0) {
    uint32_t w = lane < THREADS / 32 ? smem[lane] : 0u;
    uint32_t s = w;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      uint32_t y = __shfl_up_sync(0xffffffffu, s, o);
      if (lane >= o) s += y;
    }
    if (lane < THREADS / 32) smem[lane] = s - w;
    if (lane == THREADS / 32 - 1) smem[THREADS / 32] = s;
  }
  __syncthreads();
  *total = smem[THREADS / 32];
  uint32_t r = smem[warp] + x - v;
  __syncthreads();
  return r;
}

// ---- exclusive scan of a uint32 array (reduce, scan partials, downsweep) -------

__global__ void __launch_bounds__(kScanThreads)
k_scan_reduce(const uint32_t* __restrict__ in, int len, uint32_t* __restrict__ partials) {
  __shared__ uint32_t smem[kScanThreads / 32 + 1];
  const int base = blockIdx.x * kScanTile + threadIdx.x * kScanItems;
  uint32_t sum = 0;
#pragma unroll
  for (int k = 0; k < kScanItems; ++k)
    if (base + k < len) sum += in[base + k];
  uint32_t total;
  block_exclusive_scan<kScanThreads>(sum, smem, &total);
  if (threadIdx.x == 0) partials[blockIdx.x] = total;
}

__global__ void __launch_bounds__(kTopThreads)
k_scan_top(uint32_t* __restrict__ partials, int count) {
  __shared__ uint32_t smem[kTopThreads / 32 + 1];
  constexpr int kItems = kMaxScanPartials / kTopThreads;
  const int base = threadIdx.x * kItems;
  uint32_t v[kItems];
  uint32_t sum = 0;
#pragma unroll
  for (int k = 0; k < kItems; ++k) {
    v[k] = base + k < count ? partials[base + k] : 0u;
    sum += v[k];
  }
  uint32_t total;
  uint32_t run = block_exclusive_scan<kTopThreads>(sum, smem, &total);
#pragma unroll
  for (int k = 0; k < kItems; ++k) {
    if (base + k < count) partials[base + k] = run;
    run += v[k];
  }
}

__global__ void __launch_bounds__(kScanThreads)
k_scan_down(const uint32_t* in, int len, const uint32_t* __restrict__ partials, uint32_t* out) {
  // in and out may alias (in-place scan): every thread reads its items before
  // writing them, and no thread touches another thread's items.
  __shared__ uint32_t smem[kScanThreads / 32 + 1];
  const int base = blockIdx.x * kScanTile + threadIdx.x * kScanItems;
  uint32_t v[kScanItems];
  uint32_t sum = 0;
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    v[k] = base + k < len ? in[base + k] : 0u;
    sum += v[k];
  }
  uint32_t total;
  uint32_t run = block_exclusive_scan<kScanThreads>(sum, smem, &total) + partials[blockIdx.x];
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    if (base + k < len) out[base + k] = run;
    run += v[k];
  }
}


}  // namespace

cudaError_t exclusive_scan(const uint32_t* in, uint32_t* out, int len, uint32_t* partials,
                           cudaStream_t stream) {
  const int tiles = (len + kScanTile - 1) / kScanTile;
  if (tiles > kMaxScanPartials) return cudaErrorInvalidValue;
  k_scan_reduce<<<tiles, kScanThreads, 0, stream>>>(in, len, partials);
  k_scan_top<<<1, kTopThreads, 0, stream>>>(partials, tiles);
  k_scan_down<<<tiles, kScanThreads, 0, stream>>>(in, len, partials, out);
  return cudaGetLastError();
}

namespace {

// ---- predict + hash ---------------------------------------------------------------

// advect_kernel (fluids/Simulator_kernel.cuh:7-19) fused with getGridId
// (fluids/Simulator.cu:56-73): v' = fma(dt, g, v), x* = fma(dt, v', x),
// key = cell id of x*.  Also counts particles per cell (integer atomics:
// order-independent, so the counts are deterministic).
template <bool kPredict>
__global__ void __launch_bounds__(256)
k_hash(const float4* __restrict__ pos, const float4* __restrict__ vel, int n, StepConsts c,
       Geometry G, uint32_t* __restrict__ keys, uint32_t* __restrict__ cell_count) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float4 x = pos[i];
  if (kPredict) {
    const float4 v = vel[i];
    const float vx = fmaf(c.dt, c.g[0], v.x), vy = fmaf(c.dt, c.g[1], v.y),
                vz = fmaf(c.dt, c.g[2], v.z);
    x.x = fmaf(c.dt, vx, x.x);
    x.y = fmaf(c.dt, vy, x.y);
    x.z = fmaf(c.dt, vz, x.z);
  }
  const SceneGeom g = geom_of(c, G, i);
  const int3 q = cell_of(c, g, x);
  const uint32_t key = (uint32_t)cell_index(g, q.x, q.y, q.z);
  keys[i] = key;
  // one atomic per cell and warp (the particles are in last step's cell order,
  // so a warp's lanes mostly share a few cells)
  const unsigned same = __match_any_sync(__activemask(), key);
  if ((threadIdx.x & 31) == __ffs(same) - 1) atomicAdd(&cell_count[key], (uint32_t)__popc(same));
}

// ---- stable LSD radix sort of (key, index) ------------------------------------

// Per-tile digit histogram, stored digit-major: counts[d * ntiles + tile].
__global__ void __launch_bounds__(kSortThreads)
k_radix_upsweep(const uint32_t* __restrict__ keys, int n, int shift,
                uint32_t* __restrict__ counts, int ntiles) {
  __shared__ uint32_t hist[kRadix];
  hist[threadIdx.x] = 0;
  __syncthreads();
  const int base = blockIdx.x * kSortTile;
  const unsigned lane = threadIdx.x & 31;
#pragma unroll
  for (int k = 0; k < kSortItems; ++k) {
    const int idx = base + k * kSortThreads + threadIdx.x;
    const uint32_t d = idx < n ? (keys[idx] >> shift) & (kRadix - 1) : (uint32_t)kRadix;
    const unsigned peers = __match_any_sync(0xffffffffu, d);
    if (d < (uint32_t)kRadix && (peers & ((1u << lane) - 1)) == 0)
      atomicAdd(&hist[d], (uint32_t)__popc(peers));
  }
  __syncthreads();
  counts[threadIdx.x * ntiles + blockIdx.x] = hist[threadIdx.x];
}

// Stable scatter of one tile.  Warp w owns tile items [w*256, w*256+256) in
// 8 rounds of 32 (idx order = (warp, round, lane)); ranks within a round come
// from __match_any_sync, across rounds from a per-warp digit counter, across
// warps from an exclusive scan of those counters, across tiles from the
// scanned digit-major counts.
__global__ void __launch_bounds__(kSortThreads)
k_radix_downsweep(const uint32_t* __restrict__ keys_in, const uint32_t* __restrict__ vals_in,
                  uint32_t* __restrict__ keys_out, uint32_t* __restrict__ vals_out, int n,
                  int shift, const uint32_t* __restrict__ counts_scanned, int ntiles) {
  __shared__ uint32_t whist[kSortWarps][kRadix];
  const int warp = threadIdx.x >> 5;
  const unsigned lane = threadIdx.x & 31;
  const unsigned lt = (1u << lane) - 1;
  for (int k = threadIdx.x; k < kSortWarps * kRadix; k += kSortThreads) (&whist[0][0])[k] = 0;
  __syncthreads();
  const int base = blockIdx.x * kSortTile + warp * (kSortItems * 32);
  uint32_t key[kSortItems], val[kSortItems], rank[kSortItems];
#pragma unroll
  for (int k = 0; k < kSortItems; ++k) {
    const int idx = base + k * 32 + lane;
    const bool valid = idx < n;
    key[k] = valid ? keys_in[idx] : 0u;
    val[k] = valid ? (vals_in ? vals_in[idx] : (uint32_t)idx) : 0u;
    const uint32_t d = valid ? (key[k] >> shift) & (kRadix - 1) : (uint32_t)kRadix;
    const unsigned peers = __match_any_sync(0xffffffffu, d);
    const uint32_t r = __popc(peers & lt);
    const uint32_t b = whist[warp][valid ? d : 0u];  // index stays inside the table
    __syncwarp();
    if (valid && r == 0) whist[warp][d] = b + __popc(peers);
    __syncwarp();
    rank[k] = b + r;
  }
  __syncthreads();
  {
    const int d = threadIdx.x;
    uint32_t run = counts_scanned[d * ntiles + blockIdx.x];
#pragma unroll
    for (int w = 0; w < kSortWarps; ++w) {
      const uint32_t t = whist[w][d];
      whist[w][d] = run;
      run += t;
    }
  }
  __syncthreads();
#pragma unroll
  for (int k = 0; k < kSortItems; ++k) {
    const int idx = base + k * 32 + lane;
    if (idx < n) {
      const uint32_t d = (key[k] >> shift) & (kRadix - 1);
      const uint32_t dst = whist[warp][d] + rank[k];
      if (dst < (uint32_t)n) {  // always true for consistent counts; never write out of range
        if (keys_out) keys_out[dst] = key[k];
        vals_out[dst] = val[k];
      }
    }
  }
}

__global__ void k_export_ranges(const uint32_t* __restrict__ cs, int cells,
                                uint32_t* __restrict__ start, uint32_t* __restrict__ end) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= cells) return;
  const uint32_t s = cs[k], e = cs[k + 1];
  start[k] = e > s ? s : 0u;
  end[k] = e > s ? e : 0u;
}

int key_bits(int cells) {
  int b = 0;
  while (b < 32 && ((uint64_t)1 << b) < (uint64_t)cells) ++b;
  return b;
}

}  // namespace

int grid_launches(const StepConsts& c, int n) {
  (void)n;
  const int bits = key_bits(c.cells);
  const int passes = bits > 0 ? (bits + kRadixBits - 1) / kRadixBits : 1;
  return 1 + 3 + passes * (1 + 3 + 1);  // hash, cell scan, passes x (upsweep, scan, downsweep)
}

int sort_tiles(int n) { return (n + kSortTile - 1) / kSortTile; }

size_t radix_counts_len(int max_particles) {
  return (size_t)kRadix * (size_t)(sort_tiles(max_particles) > 0 ? sort_tiles(max_particles) : 1);
}

cudaError_t build_grid(const StepConsts& c, const Geometry& G, const float4* pos, const float4* vel,
                       const float4* xstar, int n, GridScratch& s, const uint32_t** perm_out,
                       uint32_t* keys_copy, cudaStream_t stream) {
  cudaError_t err;
  const int cells1 = c.cells + 1;
  if ((err = cudaMemsetAsync(s.cell_count, 0, sizeof(uint32_t) * cells1, stream)) != cudaSuccess)
    return err;
  const int blocks = (n + 255) / 256;
  if (xstar)
    k_hash<false><<<blocks, 256, 0, stream>>>(xstar, nullptr, n, c, G, s.keys_a, s.cell_count);
  else
    k_hash<true><<<blocks, 256, 0, stream>>>(pos, vel, n, c, G, s.keys_a, s.cell_count);
  if ((err = cudaGetLastError()) != cudaSuccess) return err;
  if (keys_copy &&
      (err = cudaMemcpyAsync(keys_copy, s.keys_a, sizeof(uint32_t) * n, cudaMemcpyDeviceToDevice,
                             stream)) != cudaSuccess)
    return err;
  if ((err = exclusive_scan(s.cell_count, s.cell_start, cells1, s.scan_partials, stream)) !=
      cudaSuccess)
    return err;

  // LSD passes over the key bits; at least one pass so perm is always written.
  const int bits = key_bits(c.cells);
  const int passes = bits > 0 ? (bits + kRadixBits - 1) / kRadixBits : 1;
  const int ntiles = sort_tiles(n);
  const int clen = kRadix * ntiles;
  uint32_t* kin = s.keys_a;
  uint32_t* kout = s.keys_b;
  uint32_t* vin = nullptr;
  uint32_t* vout = s.vals_a;
  for (int p = 0; p < passes; ++p) {
    const int shift = p * kRadixBits;
    const bool last = p == passes - 1;  // its keys stay: the passes flag cells by them
    k_radix_upsweep<<<ntiles, kSortThreads, 0, stream>>>(kin, n, shift, s.radix_counts, ntiles);
    if ((err = exclusive_scan(s.radix_counts, s.radix_counts, clen, s.scan_partials, stream)) !=
        cudaSuccess)
      return err;
    k_radix_downsweep<<<ntiles, kSortThreads, 0, stream>>>(kin, vin, kout, vout, n, shift,
                                                           s.radix_counts, ntiles);
    if (last) s.keys_sorted = kout;
    if ((err = cudaGetLastError()) != cudaSuccess) return err;
    uint32_t* t = kin;
    kin = kout;
    kout = t;
    vin = vout;
    vout = (vout == s.vals_a) ? s.vals_b : s.vals_a;
  }
  *perm_out = vin;
  return cudaSuccess;
}

cudaError_t export_ranges(const StepConsts& c, const uint32_t* cell_start, uint32_t* start,
                          uint32_t* end, cudaStream_t stream) {
  if (c.cells <= 0) return cudaSuccess;
  k_export_ranges<<<(c.cells + 255) / 256, 256, 0, stream>>>(cell_start, c.cells, start, end);
  return cudaGetLastError();
}

}  // namespace pbf
