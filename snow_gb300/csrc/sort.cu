// Particle binning for SNOW_MODE_FAST on sm_103a: cell keys, a stable LSD
// radix sort of (key, particle index) pairs, the permutation of the particle
// streams into key order and the P2G work items (home block, particle range).
//
// The reference has no sort (it scatters every (particle, neighbour) pair with
// global int atomics, p2gTransfer.cpp:22-23); binning is what makes the
// shared-memory tiling of this implementation possible. Cell of a particle: ivec3((x - gGridPos) /
// gridSpacing) as p2gTransfer.glsl:76-81 computes it (truncation toward
// zero), clamped into the grid. Key: block-major cell index
//   key = block(i>>2, j>>2, k>>2) * 64 + (i&3) + 4 (j&3) + 16 (k&3)
// with blocks numbered x fastest. The sort is stable, so the permutation is
// the one std::stable_sort gives on the same keys.
//
// Radix sort: 8-bit digits; per pass an upsweep (per-tile digit histograms,
// digit-major), an exclusive scan of the histograms and a downsweep that ranks
// each tile's keys stably with warp match/ballot and per-warp digit counters,
// then scatters.
#include <mutex>

#include "snow_internal.h"

namespace snow {
namespace {

constexpr int kRsThreads = 256;
constexpr int kRsWarps = kRsThreads / 32;
constexpr int kRsKpt = 16;                         // keys per thread
constexpr int kRsTile = kRsThreads * kRsKpt;       // 4096 keys per tile
constexpr int kRsPerWarp = kRsTile / kRsWarps;     // 512
constexpr int kScanChunk = 4096;                   // entries per scan CTA

__global__ void __launch_bounds__(kRsThreads) k_rs_hist(const uint32_t* __restrict__ keys, size_t n, int shift,
                                                        uint32_t* __restrict__ hist, int ntiles) {
  __shared__ uint32_t h[256];
  for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    h[threadIdx.x] = 0;
    __syncthreads();
    const size_t base = (size_t)tile * kRsTile;
    for (int i = threadIdx.x; i < kRsTile; i += kRsThreads) {
      const size_t idx = base + i;
      if (idx < n) atomicAdd(&h[(keys[idx] >> shift) & 255u], 1u);
    }
    __syncthreads();
    hist[(size_t)threadIdx.x * ntiles + tile] = h[threadIdx.x];
    __syncthreads();
  }
}

// ---- exclusive scan of a uint32 array, three phases ----------------------
__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t v, uint32_t* total) {
  __shared__ uint32_t wsum[32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  uint32_t x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) wsum[w] = x;
  __syncthreads();
  if (w == 0) {
    const int nw = blockDim.x >> 5;
    uint32_t s = lane < nw ? wsum[lane] : 0u;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, s, o);
      if (lane >= o) s += y;
    }
    if (lane < nw) wsum[lane] = s;
  }
  __syncthreads();
  const uint32_t before = (w > 0 ? wsum[w - 1] : 0u) + x - v;
  if (total) *total = wsum[(blockDim.x >> 5) - 1];
  __syncthreads();
  return before;
}

__global__ void __launch_bounds__(256) k_scan_reduce(const uint32_t* __restrict__ a, size_t len,
                                                     uint32_t* __restrict__ partial) {
  const size_t base = (size_t)blockIdx.x * kScanChunk;
  uint32_t s = 0;
  for (int i = threadIdx.x; i < kScanChunk; i += blockDim.x) {
    const size_t idx = base + i;
    if (idx < len) s += a[idx];
  }
  uint32_t total;
  block_exclusive_scan(s, &total);
  if (threadIdx.x == 0) partial[blockIdx.x] = total;
}

__global__ void __launch_bounds__(1024) k_scan_partials(uint32_t* __restrict__ partial, int np) {
  __shared__ uint32_t carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int base = 0; base < np; base += blockDim.x) {
    const int i = base + threadIdx.x;
    const uint32_t v = i < np ? partial[i] : 0u;
    uint32_t total;
    const uint32_t ex = block_exclusive_scan(v, &total);
    if (i < np) partial[i] = carry + ex;
    __syncthreads();
    if (threadIdx.x == 0) carry += total;
    __syncthreads();
  }
}

__global__ void __launch_bounds__(256) k_scan_down(uint32_t* __restrict__ a, size_t len,
                                                   const uint32_t* __restrict__ partial) {
  constexpr int per = kScanChunk / 256;
  const size_t base = (size_t)blockIdx.x * kScanChunk + (size_t)threadIdx.x * per;
  uint32_t v[per];
  uint32_t s = 0;
#pragma unroll
  for (int j = 0; j < per; j++) {
    v[j] = (base + j < len) ? a[base + j] : 0u;
    s += v[j];
  }
  uint32_t run = partial[blockIdx.x] + block_exclusive_scan(s, nullptr);
#pragma unroll
  for (int j = 0; j < per; j++) {
    if (base + j < len) a[base + j] = run;
    run += v[j];
  }
}

void exclusive_scan(uint32_t* a, size_t len, uint32_t* partial, cudaStream_t st) {
  const int chunks = (int)((len + kScanChunk - 1) / kScanChunk);
  k_scan_reduce<<<chunks, 256, 0, st>>>(a, len, partial);
  k_scan_partials<<<1, 1024, 0, st>>>(partial, chunks);
  k_scan_down<<<chunks, 256, 0, st>>>(a, len, partial);
}

__global__ void __launch_bounds__(kRsThreads) k_rs_scatter(const uint32_t* __restrict__ kin,
                                                           const uint32_t* __restrict__ vin,
                                                           uint32_t* __restrict__ kout, uint32_t* __restrict__ vout,
                                                           size_t n, int shift,
                                                           const uint32_t* __restrict__ offsets, int ntiles) {
  __shared__ uint32_t wcount[kRsWarps][256];
  __shared__ uint32_t gbase[256];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const uint32_t lt = (1u << lane) - 1u;
  for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    for (int i = threadIdx.x; i < kRsWarps * 256; i += kRsThreads) (&wcount[0][0])[i] = 0u;
    gbase[threadIdx.x] = offsets[(size_t)threadIdx.x * ntiles + tile];
    __syncthreads();
    const size_t base = (size_t)tile * kRsTile + (size_t)w * kRsPerWarp;
    uint32_t key[kRsKpt], val[kRsKpt], rank[kRsKpt];
#pragma unroll
    for (int j = 0; j < kRsKpt; j++) {
      const size_t idx = base + (size_t)j * 32 + lane;
      const bool valid = idx < n;
      key[j] = valid ? kin[idx] : 0u;
      val[j] = valid ? vin[idx] : 0u;
      const uint32_t d = valid ? ((key[j] >> shift) & 255u) : 256u;
      const uint32_t peers = __match_any_sync(0xffffffffu, d);
      const uint32_t before = d < 256u ? wcount[w][d] : 0u;
      __syncwarp();
      if (d < 256u && (peers & lt) == 0u) wcount[w][d] = before + __popc(peers);
      __syncwarp();
      rank[j] = valid ? before + __popc(peers & lt) : 0xffffffffu;
    }
    __syncthreads();
    {
      const int d = threadIdx.x;  // one thread per digit
      uint32_t run = 0;
#pragma unroll
      for (int ww = 0; ww < kRsWarps; ww++) {
        const uint32_t t = wcount[ww][d];
        wcount[ww][d] = run;
        run += t;
      }
    }
    __syncthreads();
#pragma unroll
    for (int j = 0; j < kRsKpt; j++) {
      if (rank[j] == 0xffffffffu) continue;
      const uint32_t d = (key[j] >> shift) & 255u;
      const uint32_t pos = gbase[d] + wcount[w][d] + rank[j];
      kout[pos] = key[j];
      vout[pos] = val[j];
    }
    __syncthreads();
  }
}

// ---- keys, permutation, work items -----------------------------------------
__global__ void k_keys(const SceneDev* __restrict__ sd, uint32_t* __restrict__ keys, uint32_t* __restrict__ vals) {
  const SceneDev& S = *sd;
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < S.n; p += gridDim.x * blockDim.x) {
    const float4 xm = S.xm[p];
    const float x[3] = {xm.x, xm.y, xm.z};
    int c[3];
#pragma unroll
    for (int k = 0; k < 3; k++) {
      int v = (int)((x[k] - S.gpos[k]) / S.h);
      v = v < 0 ? 0 : (v > S.dim[k] - 1 ? S.dim[k] - 1 : v);
      c[k] = v;
    }
    const uint32_t b = ((uint32_t)(c[2] >> 2) * (uint32_t)S.bdim[1] + (uint32_t)(c[1] >> 2)) * (uint32_t)S.bdim[0] +
                       (uint32_t)(c[0] >> 2);
    keys[p] = b * 64u + (uint32_t)(c[0] & 3) + 4u * (uint32_t)(c[1] & 3) + 16u * (uint32_t)(c[2] & 3);
    vals[p] = (uint32_t)p;
  }
}

// Gathers the particle streams into key order (into the scratch copies;
// k_heads copies them back, or the step's fused kernel reads them there)
// and zeroes the item and home counters.
__global__ void k_permute(const SceneDev* __restrict__ sd, const uint32_t* __restrict__ perm, float4* __restrict__ xm,
                          float4* __restrict__ vv, float4* __restrict__ fa, float4* __restrict__ fb,
                          float2* __restrict__ fc, uint32_t* __restrict__ pid, float4* __restrict__ vq) {
  const SceneDev& S = *sd;
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    S.counters[CNT_ITEMS] = 0;
    S.counters[CNT_HOME] = 0;
  }
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < S.n; i += gridDim.x * blockDim.x) {
    const uint32_t src = perm[i];
    xm[i] = S.xm[src];
    vv[i] = S.vv[src];
    fa[i] = S.fa[src];
    fb[i] = S.fb[src];
    fc[i] = S.fc[src];
    pid[i] = S.pid[src];
    vq[i] = S.vq[src];
  }
}

// Block ranges of the sorted keys and the list of home blocks; also copies
// the permuted particle ids back, and with copy_back the permuted streams
// (else the particles stay in the binned copies, flagged by CNT_BINNED, for
// the step's fused kernel to read and write back).
__global__ void k_heads(const SceneDev* __restrict__ sd, const uint32_t* __restrict__ keys, int* __restrict__ bstart,
                        int* __restrict__ bend, int* __restrict__ home, const float4* __restrict__ xm,
                        const float4* __restrict__ vv, const float4* __restrict__ fa, const float4* __restrict__ fb,
                        const float2* __restrict__ fc, const uint32_t* __restrict__ pid,
                        const float4* __restrict__ vq, int copy_back) {
  const SceneDev& S = *sd;
  const int n = S.n;
  if (!copy_back && blockIdx.x == 0 && threadIdx.x == 0) S.counters[CNT_BINNED] = 1;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    S.pid[i] = pid[i];
    if (copy_back) {
      S.xm[i] = xm[i];
      S.vv[i] = vv[i];
      S.fa[i] = fa[i];
      S.fb[i] = fb[i];
      S.fc[i] = fc[i];
      S.vq[i] = vq[i];
    }
    const uint32_t b = keys[i] >> 6;
    if (i == 0 || (keys[i - 1] >> 6) != b) {
      bstart[b] = i;
      home[atomicAdd(&S.counters[CNT_HOME], 1)] = (int)b;
    }
    if (i == n - 1 || (keys[i + 1] >> 6) != b) bend[b] = i + 1;
  }
}

__global__ void k_items(const SceneDev* __restrict__ sd, const int* __restrict__ bstart, const int* __restrict__ bend,
                        const int* __restrict__ home, int items_max) {
  const SceneDev& S = *sd;
  const int nh = S.counters[CNT_HOME];
  for (int h = blockIdx.x * blockDim.x + threadIdx.x; h < nh; h += gridDim.x * blockDim.x) {
    const int b = home[h];
    const int s = bstart[b], e = bend[b];
    // split the block's particles into nit near-equal items of <= items_max
    const int cnt = e - s;
    const int nit = (cnt + items_max - 1) / items_max;
    const int at = atomicAdd(&S.counters[CNT_ITEMS], nit);
    for (int j = 0; j < nit; j++) {
      if (at + j >= S.item_cap) break;  // cannot happen: item_cap covers the bound
      const int first = s + (int)(((long long)j * cnt) / nit);
      const int last = s + (int)(((long long)(j + 1) * cnt) / nit);
      S.items[at + j] = make_int4(b, first, last - first, 0);
    }
  }
}

int grid_for(size_t n, int threads, int per_sm) {
  size_t g = (n + threads - 1) / threads;
  const size_t cap = (size_t)num_sms() * per_sm;
  if (g > cap) g = cap;
  return (int)(g < 1 ? 1 : g);
}

}  // namespace

size_t radix_tiles(size_t n) { return (n + kRsTile - 1) / kRsTile; }

void radix_sort_pairs(uint32_t* k[2], uint32_t* v[2], size_t n, int key_bits, uint32_t* hist, uint32_t* scan_tmp,
                      cudaStream_t st, int start) {
  if (n == 0) return;
  const int ntiles = (int)radix_tiles(n);
  const int passes = (key_bits + 7) / 8;
  int cur = start;
  const int g = grid_for((size_t)ntiles * kRsThreads, kRsThreads, 8);
  for (int pass = 0; pass < passes; pass++) {
    const int shift = 8 * pass;
    k_rs_hist<<<g, kRsThreads, 0, st>>>(k[cur], n, shift, hist, ntiles);
    exclusive_scan(hist, (size_t)256 * ntiles, scan_tmp, st);
    k_rs_scatter<<<g, kRsThreads, 0, st>>>(k[cur], v[cur], k[cur ^ 1], v[cur ^ 1], n, shift, hist, ntiles);
    cur ^= 1;
  }
  if (cur == 1) {
    cudaMemcpyAsync(k[0], k[1], n * sizeof(uint32_t), cudaMemcpyDeviceToDevice, st);
    cudaMemcpyAsync(v[0], v[1], n * sizeof(uint32_t), cudaMemcpyDeviceToDevice, st);
  }
}

void fast_sort_keys(const SceneDev& sd, const SceneDev* sd_dev, BinScratch& b, int key_bits, cudaStream_t st) {
  if (sd.n <= 0) return;
  // an odd number of passes starts from the second buffer so that the
  // result lands in the first without a copy
  const int start = ((key_bits + 7) / 8) & 1;
  k_keys<<<grid_for(sd.n, 256, 8), 256, 0, st>>>(sd_dev, b.keys[start], b.vals[start]);
  radix_sort_pairs(b.keys, b.vals, (size_t)sd.n, key_bits, b.hist, b.scan_tmp, st, start);
}

void fast_apply_bins(const SceneDev& sd, const SceneDev* sd_dev, BinScratch& b, int items_max, bool copy_back,
                     cudaStream_t st) {
  if (sd.n <= 0) return;
  const size_t n = (size_t)sd.n;
  k_permute<<<grid_for(n, 256, 8), 256, 0, st>>>(sd_dev, b.vals[0], b.tmp4[0], b.tmp4[1], b.tmp4[2], b.tmp4[3],
                                                  b.tmp2, b.tmp_pid, b.tmp4[4]);
  k_heads<<<grid_for(n, 256, 8), 256, 0, st>>>(sd_dev, b.keys[0], b.bstart, b.bend, b.home, b.tmp4[0], b.tmp4[1],
                                                b.tmp4[2], b.tmp4[3], b.tmp2, b.tmp_pid, b.tmp4[4], copy_back ? 1 : 0);
  const size_t maxhome = n < (size_t)sd.nblocks ? n : (size_t)sd.nblocks;
  k_items<<<grid_for(maxhome, 256, 4), 256, 0, st>>>(sd_dev, b.bstart, b.bend, b.home, items_max);
}

}  // namespace snow

// ---------------------------------------------------------------------------
// snow_sort_keys_static: the stable radix sort above for callers that cannot
// allocate device memory. Its scratch (the second key/value buffer of the
// ping-pong passes, the digit histograms and the scan partials) lives in one
// file-scope __device__ array, sized for SNOW_SORT_STATIC_MAX_KEYS keys; every
// GPU that loads the library holds it (about 2.1 MB) until the process exits.
// ---------------------------------------------------------------------------
namespace snow {
namespace {

constexpr size_t kStaticKeys = SNOW_SORT_STATIC_MAX_KEYS;
constexpr size_t kStaticTiles = (kStaticKeys + kRsTile - 1) / kRsTile;
constexpr size_t kStaticHist = 256 * kStaticTiles;
constexpr size_t kStaticPartials = (kStaticHist + kScanChunk - 1) / kScanChunk + 1;
// layout: [keys kStaticKeys][vals kStaticKeys][hist kStaticHist][partials]
constexpr size_t kStaticWords = 2 * kStaticKeys + kStaticHist + kStaticPartials;

__device__ __align__(256) uint32_t g_sort_scratch[kStaticWords];

__global__ void k_iota(uint32_t* __restrict__ v, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    v[i] = (uint32_t)i;
}

// The driver's id of the calling thread's current context (0 if none). Ids
// are never reused in a process, so a context created after a reset (which
// reloads the module and moves g_sort_scratch) gets a new id.
unsigned long long current_context_id() {
  using GetCurrent = int (*)(void**);
  using GetId = int (*)(void*, unsigned long long*);
  static GetCurrent get_current = nullptr;
  static GetId get_id = nullptr;
  static bool looked_up = false;
  if (!looked_up) {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_current = reinterpret_cast<GetCurrent>(f);
    f = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_id = reinterpret_cast<GetId>(f);
    looked_up = true;
  }
  void* c = nullptr;
  unsigned long long id = 0;
  if (!get_current || !get_id || get_current(&c) != 0 || !c || get_id(c, &id) != 0) return 0;
  return id;
}

// Device address of g_sort_scratch in the current context. Host code only
// sees a host-side stand-in for the symbol, so the address is looked up
// (cudaGetSymbolAddress) and cached per context: a reset of the device's
// primary context reloads the module at another address, and the new
// context's different id makes the cache look the address up again.
cudaError_t static_scratch(uint32_t** out) {
  static std::mutex mu;
  static unsigned long long ctx_id[64] = {};
  static uint32_t* addr[64] = {};
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(mu);
  const unsigned long long id = current_context_id();
  if (!addr[dev] || id == 0 || id != ctx_id[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_sort_scratch);  // also makes the primary context current
    if (e != cudaSuccess) return e;
    addr[dev] = static_cast<uint32_t*>(p);
    ctx_id[dev] = current_context_id();
  }
  *out = addr[dev];
  return cudaSuccess;
}

// Whether the byte ranges [a, a + n) and [b, b + n) of 32-bit words overlap.
bool ranges_overlap(const void* a, const void* b, size_t n) {
  const uintptr_t x = reinterpret_cast<uintptr_t>(a), y = reinterpret_cast<uintptr_t>(b);
  const uintptr_t bytes = n * sizeof(uint32_t);
  return x < y + bytes && y < x + bytes;
}

}  // namespace
}  // namespace snow

extern "C" snow_status snow_sort_keys_static(const uint32_t* keys, uint32_t* sorted_keys, uint32_t* perm, size_t n,
                                             int key_bits, void* stream) {
  using namespace snow;
  if (!keys || !sorted_keys || !perm || key_bits < 1 || key_bits > 32) return SNOW_EINVAL;
  if (n > kStaticKeys) return SNOW_EINVAL;
  if (n == 0) return SNOW_OK;
  // perm is written before the keys are read: it may not share memory with
  // either key array; keys and sorted_keys may only coincide exactly
  if (ranges_overlap(perm, keys, n) || ranges_overlap(perm, sorted_keys, n) ||
      (keys != sorted_keys && ranges_overlap(keys, sorted_keys, n)))
    return SNOW_EINVAL;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  uint32_t* scratch = nullptr;
  if (static_scratch(&scratch) != cudaSuccess) {
    cudaGetLastError();
    return SNOW_ECUDA;
  }
  uint32_t* k[2] = {sorted_keys, scratch};
  uint32_t* v[2] = {perm, scratch + kStaticKeys};
  uint32_t* hist = scratch + 2 * kStaticKeys;
  uint32_t* partials = hist + kStaticHist;
  if (sorted_keys != keys &&
      cudaMemcpyAsync(sorted_keys, keys, n * sizeof(uint32_t), cudaMemcpyDeviceToDevice, st) != cudaSuccess) {
    cudaGetLastError();
    return SNOW_ECUDA;
  }
  k_iota<<<grid_for(n, 256, 4), 256, 0, st>>>(perm, n);
  radix_sort_pairs(k, v, n, key_bits, hist, partials, st);
  if (cudaGetLastError() != cudaSuccess) return SNOW_ECUDA;
  return SNOW_OK;
}
