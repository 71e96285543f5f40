// Device-wide primitives of the set-up passes: a stable LSD radix sort of
// (key, value) pairs, an exclusive prefix sum and a run-length encoding of
// sorted keys.  The gridding (cell keys of (visibility, tap) pairs), the
// weighting schemes (cell keys of visibilities) and the problem set-up
// (the locality order of the visibilities) sort with them.
//
// Radix sort: 8-bit digits, one pass per digit from the lowest bit up, each
// pass three launches and no waits between blocks:
//   k_radix_count   the digits of tile b (a contiguous run of chunks) are
//                   counted by kSplit blocks, each with every thread's keys
//                   of a chunk in flight at once, per-warp histograms (one
//                   shared add per key, or one per warp when its 32 digits
//                   agree), and one global add per digit into
//                   counts[b][digit];
//   k_radix_digit   block d scans counts[.][d] over the tiles (where tile
//                   b's first key of digit d goes among the keys of d) and
//                   writes the digit's total;
//   k_radix_scatter block b walks tile b's chunks (4096 keys, 2048 for
//                   64-bit pairs) in order with the next chunk's loads in
//                   flight, ranks each key among the chunk's keys of its
//                   digit in input order (a warp's equal digits from eight
//                   ballots, per-warp counters),
//                   stages the chunk sorted by digit in shared memory and
//                   writes each digit's keys as one contiguous run, at the
//                   digit's base (an exclusive scan of the 256 totals) plus
//                   the tile's offset.
// Equal digits keep their input order within a chunk, across a block's
// chunks and across blocks, so the sort is stable and its output is unique:
// the same as any other stable sort on the same bits.  Bits at and above
// end_bit do not take part in the order; the keys are moved whole.
#include <algorithm>
#include <cstdint>

#include "gv_internal.cuh"

namespace gv {
namespace {

constexpr int kThreads = 256;  // = the number of 8-bit digit values
constexpr int kWarps = kThreads / 32;
constexpr int kBins = 256;
constexpr int kNoDigit = kBins;  // the lanes past the end of the input

template <class K, class V>
struct Tile {
  static constexpr int kItems = (sizeof(K) + sizeof(V) > 8) ? 8 : 16;  // per thread
  static constexpr int kChunk = kThreads * kItems;
  static constexpr int kMinBlocks = 2;  // resident per SM
};
constexpr int kSplit = 4;  // counting blocks per tile

__device__ __forceinline__ uint32_t lanes_below(int lane) { return (1u << lane) - 1u; }

// the valid lanes of the warp whose 8-bit digit equals this lane's: one
// ballot per digit bit (cheaper than a general match of 32-bit values)
__device__ __forceinline__ uint32_t digit_peers(uint32_t d, bool valid) {
  uint32_t m = __ballot_sync(0xffffffffu, valid);
#pragma unroll
  for (int b = 0; b < 8; b++) {
    const uint32_t bit = (d >> b) & 1u;
    const uint32_t bb = __ballot_sync(0xffffffffu, bit);
    m &= bit ? bb : ~bb;
  }
  return m;
}
__device__ __forceinline__ int64_t dmin(int64_t a, int64_t b) { return a < b ? a : b; }

template <class K>
__device__ __forceinline__ uint32_t digit_of(K k, int shift, uint32_t mask) {
  return (uint32_t)(k >> shift) & mask;
}

// exclusive scan over the 256 threads of a block; *total = the sum
__device__ __forceinline__ uint32_t block_exclusive_256(uint32_t v, uint32_t* total) {
  __shared__ uint32_t ws[kWarps];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  uint32_t x = v;
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) ws[w] = x;
  __syncthreads();
  uint32_t wbase = 0u, all = 0u;
#pragma unroll
  for (int v2 = 0; v2 < kWarps; v2++) {
    const uint32_t s = ws[v2];
    if (v2 < w) wbase += s;
    all += s;
  }
  *total = all;
  __syncthreads();
  return wbase + x - v;
}

// the chunk at `start` (its keys below b1), warp-striped: item i of lane l
// of warp w is the chunk's key w * 32 * kItems + i * 32 + l
template <class K, class V, int kItems>
__device__ __forceinline__ void load_chunk(const K* __restrict__ kin, const V* __restrict__ vin,
                                           int64_t start, int64_t b1, int w, int lane, K* key,
                                           V* val) {
#pragma unroll
  for (int i = 0; i < kItems; i++) {
    const int64_t idx = start + w * 32 * kItems + i * 32 + lane;
    if (idx < b1) {
      key[i] = kin[idx];
      val[i] = vin[idx];
    }
  }
}

// counts[b][d] += keys of digit d in this block's part of tile b
template <class K, int kItems>
__global__ void __launch_bounds__(kThreads) k_radix_count(const K* __restrict__ keys, int64_t n,
                                                          int shift, uint32_t mask,
                                                          int64_t per_block, int64_t per_sub,
                                                          uint32_t* __restrict__ counts) {
  constexpr int kChunk = kThreads * kItems;
  __shared__ uint32_t h[kWarps][kBins];
  for (int i = threadIdx.x; i < kWarps * kBins; i += kThreads) (&h[0][0])[i] = 0u;
  __syncthreads();
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t c0 = (int64_t)blockIdx.x * per_block + (int64_t)blockIdx.y * per_sub;
  const int64_t c1 = dmin((int64_t)(blockIdx.x + 1) * per_block, c0 + per_sub);
  const int64_t e1 = dmin(n, c1 * kChunk);
  for (int64_t base = c0 * kChunk; base < e1; base += kChunk) {
    uint32_t dig[kItems];
#pragma unroll
    for (int i = 0; i < kItems; i++) {
      const int64_t idx = base + w * 32 * kItems + i * 32 + lane;
      dig[i] = idx < e1 ? digit_of(__ldg(keys + idx), shift, mask) : (uint32_t)kNoDigit;
    }
#pragma unroll
    for (int i = 0; i < kItems; i++) {
      // one add for a warp of equal digits (the skewed passes), else one
      // per lane (few collisions among 256 bins)
      const uint32_t d0 = __shfl_sync(0xffffffffu, dig[i], 0);
      if (__all_sync(0xffffffffu, dig[i] == d0)) {
        if (lane == 0 && d0 != (uint32_t)kNoDigit) atomicAdd(&h[w][d0], 32u);
      } else if (dig[i] != (uint32_t)kNoDigit) {
        atomicAdd(&h[w][dig[i]], 1u);
      }
    }
  }
  __syncthreads();
  uint32_t c = 0u;
#pragma unroll
  for (int v = 0; v < kWarps; v++) c += h[v][threadIdx.x];
  if (c) atomicAdd(counts + (int64_t)blockIdx.x * kBins + threadIdx.x, c);
}

// block d: counts[b][d] -> keys of digit d in the tiles before b;
// totals[d] = keys of digit d
__global__ void __launch_bounds__(kThreads) k_radix_digit(uint32_t* __restrict__ counts, int nb,
                                                          uint32_t* __restrict__ totals) {
  const int d = blockIdx.x;
  const int q = (nb + kThreads - 1) / kThreads;
  const int b0 = min(nb, (int)threadIdx.x * q), b1 = min(nb, b0 + q);
  uint32_t s = 0u;
  for (int b = b0; b < b1; b++) s += counts[(int64_t)b * kBins + d];
  uint32_t total = 0u;
  uint32_t run = block_exclusive_256(s, &total);
  for (int b = b0; b < b1; b++) {
    const uint32_t c = counts[(int64_t)b * kBins + d];
    counts[(int64_t)b * kBins + d] = run;
    run += c;
  }
  if (threadIdx.x == 0) totals[d] = total;
}

template <class K, class V>
__global__ void __launch_bounds__(kThreads, (Tile<K, V>::kMinBlocks)) k_radix_scatter(
    const K* __restrict__ kin, const V* __restrict__ vin, K* __restrict__ kout,
    V* __restrict__ vout, int64_t n, int shift, uint32_t mask, int64_t per_block,
    const uint32_t* __restrict__ offsets, const uint32_t* __restrict__ totals) {
  constexpr int kItems = Tile<K, V>::kItems;
  constexpr int kChunk = Tile<K, V>::kChunk;
  __shared__ K sk[kChunk];
  __shared__ V sv[kChunk];
  __shared__ uint32_t cnt[kWarps][kBins];  // per-warp digit counts, then prefixes
  __shared__ uint32_t start[kBins];        // first sorted position of the digit in the chunk
  __shared__ uint32_t goff[kBins];         // where the digit's next key goes in kout
  const int t = threadIdx.x, w = t >> 5, lane = t & 31;
  {
    uint32_t all = 0u;
    const uint32_t base_d = block_exclusive_256(totals[t], &all);
    goff[t] = base_d + offsets[(int64_t)blockIdx.x * kBins + t];
  }
  const int64_t b0 = (int64_t)blockIdx.x * per_block * kChunk;
  const int64_t b1 = dmin(n, b0 + per_block * kChunk);
  // warp-striped: item i of lane l of warp w is the chunk's key
  // w * 32 * kItems + i * 32 + l, so (w, i, l) is the input order
  K key[kItems];
  V val[kItems];
  load_chunk<K, V, kItems>(kin, vin, b0, b1, w, lane, key, val);
  for (int64_t base = b0; base < b1; base += kChunk) {
    const int m = (int)dmin(kChunk, b1 - base);
    for (int i = t; i < kWarps * kBins; i += kThreads) (&cnt[0][0])[i] = 0u;
    __syncthreads();
    uint32_t rank[kItems];
#pragma unroll
    for (int i = 0; i < kItems; i++) {
      const bool valid = w * 32 * kItems + i * 32 + lane < m;
      const uint32_t d = valid ? digit_of(key[i], shift, mask) : (uint32_t)kNoDigit;
      const uint32_t peers = digit_peers(d, valid);
      const uint32_t below = peers & lanes_below(lane);
      const uint32_t prev = valid ? cnt[w][d] : 0u;
      rank[i] = prev + (uint32_t)__popc(below);
      __syncwarp();
      if (valid && below == 0u) cnt[w][d] = prev + (uint32_t)__popc(peers);
      __syncwarp();
    }
    __syncthreads();
    // thread t = digit t: the warps' exclusive prefixes, the chunk's total,
    // and the digit's first position in the chunk
    uint32_t tot = 0u;
#pragma unroll
    for (int v = 0; v < kWarps; v++) {
      const uint32_t c = cnt[v][t];
      cnt[v][t] = tot;
      tot += c;
    }
    uint32_t all = 0u;
    start[t] = block_exclusive_256(tot, &all);
    __syncthreads();
#pragma unroll
    for (int i = 0; i < kItems; i++) {
      if (w * 32 * kItems + i * 32 + lane < m) {
        const uint32_t d = digit_of(key[i], shift, mask);
        const uint32_t pos = start[d] + cnt[w][d] + rank[i];
        if (pos < (uint32_t)kChunk) {  // always: the ranks of the chunk's m keys are 0..m-1
          sk[pos] = key[i];
          sv[pos] = val[i];
        }
      }
    }
    // the next chunk's loads go out before this one is written
    load_chunk<K, V, kItems>(kin, vin, base + kChunk, b1, w, lane, key, val);
    __syncthreads();
    // sorted position p holds a key of digit d: its place in kout is the
    // digit's running offset plus its rank among the chunk's keys of d
#pragma unroll
    for (int j = 0; j < kItems; j++) {
      const int p = j * kThreads + t;
      if (p < m) {
        const K k = sk[p];
        const uint32_t d = digit_of(k, shift, mask);
        const int64_t dst = (int64_t)goff[d] + (p - (int)start[d]);
        if (dst >= 0 && dst < n) {  // always, when the counts agree with the keys
          kout[dst] = k;
          vout[dst] = sv[p];
        }
      }
    }
    __syncthreads();
    goff[t] += tot;
    // the next chunk's first barrier orders this update before its reads
  }
}

// ---- exclusive scan -------------------------------------------------------

constexpr int kScanItems = 16;  // per thread of a 256-thread tile
constexpr int kScanTile = kThreads * kScanItems;

// Exclusive prefix sum of a[0..m) in place, one block of 1024 threads, each
// owning a contiguous segment (the tile sums of a scan: at most a few tens
// of thousands of words, resident in L2)
constexpr int kScanThreads = 1024;
__global__ void __launch_bounds__(kScanThreads) k_scan_sums(uint32_t* __restrict__ a, int64_t m) {
  __shared__ uint32_t ws[32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int64_t seg = (m + kScanThreads - 1) / kScanThreads;
  const int64_t s0 = dmin(m, seg * threadIdx.x);
  const int64_t s1 = dmin(m, s0 + seg);
  uint32_t sum = 0u;
  for (int64_t i = s0; i < s1; i++) sum += a[i];
  uint32_t x = sum;
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) ws[w] = x;
  __syncthreads();
  if (w == 0) {
    uint32_t v = ws[lane];
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, v, o);
      if (lane >= o) v += y;
    }
    ws[lane] = v;
  }
  __syncthreads();
  uint32_t run = (w > 0 ? ws[w - 1] : 0u) + x - sum;
  for (int64_t i = s0; i < s1; i++) {
    const uint32_t c = a[i];
    a[i] = run;
    run += c;
  }
}

// tile sums of in[0..n)
template <class T>
__global__ void __launch_bounds__(kThreads) k_scan_tiles(const T* __restrict__ in, int64_t n,
                                                         uint32_t* __restrict__ sums) {
  const int64_t base = (int64_t)blockIdx.x * kScanTile;
  uint32_t s = 0u;
#pragma unroll
  for (int j = 0; j < kScanItems; j++) {
    const int64_t i = base + j * kThreads + threadIdx.x;
    if (i < n) s += (uint32_t)in[i];
  }
  uint32_t total = 0u;
  block_exclusive_256(s, &total);
  if (threadIdx.x == 0) sums[blockIdx.x] = total;
}

// out = exclusive prefix sum of in, given the tiles' exclusive offsets;
// thread t owns kScanItems consecutive entries of its tile
template <class T>
__global__ void __launch_bounds__(kThreads) k_scan_apply(const T* __restrict__ in, int64_t n,
                                                         const uint32_t* __restrict__ tile_off,
                                                         T* __restrict__ out) {
  const int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanItems;
  uint32_t v[kScanItems];
  uint32_t s = 0u;
#pragma unroll
  for (int j = 0; j < kScanItems; j++) {
    const int64_t i = base + j;
    v[j] = i < n ? (uint32_t)in[i] : 0u;
    s += v[j];
  }
  uint32_t total = 0u;
  uint32_t run = tile_off[blockIdx.x] + block_exclusive_256(s, &total);
#pragma unroll
  for (int j = 0; j < kScanItems; j++) {
    const int64_t i = base + j;
    if (i < n) out[i] = (T)run;
    run += v[j];
  }
}

// ---- run-length encoding of sorted keys -----------------------------------

// heads (first keys of runs) per scan tile
__global__ void __launch_bounds__(kThreads) k_rle_tiles(const uint32_t* __restrict__ keys,
                                                        int64_t n, uint32_t* __restrict__ sums) {
  const int64_t base = (int64_t)blockIdx.x * kScanTile;
  uint32_t s = 0u;
#pragma unroll
  for (int j = 0; j < kScanItems; j++) {
    const int64_t i = base + j * kThreads + threadIdx.x;
    if (i < n) s += (i == 0 || __ldg(keys + i) != __ldg(keys + i - 1)) ? 1u : 0u;
  }
  uint32_t total = 0u;
  block_exclusive_256(s, &total);
  if (threadIdx.x == 0) sums[blockIdx.x] = total;
}

// thread t of a tile owns kScanItems consecutive keys: each head's run
// index is the number of heads before it; the run's key and first position
// are written (runs at or past cap are counted, not written)
__global__ void __launch_bounds__(kThreads) k_rle_apply(const uint32_t* __restrict__ keys,
                                                        int64_t n,
                                                        const uint32_t* __restrict__ tile_off,
                                                        int64_t cap, uint32_t* __restrict__ rkey,
                                                        uint32_t* __restrict__ rstart,
                                                        int* __restrict__ nruns) {
  const int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanItems;
  uint32_t k[kScanItems];
  uint32_t heads = 0u;
  uint32_t prev = (base > 0 && base < n) ? __ldg(keys + base - 1) : 0u;
#pragma unroll
  for (int j = 0; j < kScanItems; j++) {
    const int64_t i = base + j;
    k[j] = i < n ? __ldg(keys + i) : 0u;
    if (i < n && (i == 0 || k[j] != prev)) heads |= 1u << j;
    prev = k[j];
  }
  uint32_t total = 0u;
  uint32_t run = tile_off[blockIdx.x] + block_exclusive_256((uint32_t)__popc(heads), &total);
#pragma unroll
  for (int j = 0; j < kScanItems; j++) {
    if ((heads >> j) & 1u) {
      if ((int64_t)run < cap) {
        rkey[run] = k[j];
        rstart[run] = (uint32_t)(base + j);
      }
      run++;
    }
  }
  if (base <= n - 1 && n - 1 < base + kScanItems) *nruns = (int)run;
}

// run r ends where run r + 1 starts; the last run written (r = cap - 1 of
// more runs) ends where its key does
__global__ void k_rle_counts(int64_t n, const uint32_t* __restrict__ keys,
                             const uint32_t* __restrict__ rstart, const int* __restrict__ nruns,
                             int64_t cap, uint32_t* __restrict__ rcount) {
  const int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t nr = *nruns;
  if (r >= nr || r >= cap) return;
  int64_t e;
  if (r + 1 >= nr) {
    e = n;
  } else if (r + 1 < cap) {
    e = rstart[r + 1];
  } else {
    const uint32_t k0 = keys[rstart[r]];
    e = (int64_t)rstart[r] + 1;
    while (e < n && keys[e] == k0) e++;
  }
  rcount[r] = (uint32_t)(e - rstart[r]);
}

size_t align_up(size_t b) { return (b + 255) & ~(size_t)255; }

// tiles of a sort pass: as many as scatter blocks are resident at once
// (each walks its tile of chunks), fewer for short inputs
template <class K, class V>
int radix_tiles(int64_t chunks) {
  static int cap = 0;
  if (cap == 0) {
    int dev = 0, sms = 0, occ = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
        sms <= 0)
      sms = 132;
    cudaFuncSetAttribute(k_radix_scatter<K, V>, cudaFuncAttributePreferredSharedMemoryCarveout,
                         (int)cudaSharedmemCarveoutMaxShared);
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_radix_scatter<K, V>, kThreads, 0) !=
            cudaSuccess ||
        occ <= 0)
      occ = 2;
    (void)cudaGetLastError();
    cap = sms * occ;
  }
  return (int)std::max<int64_t>(1, std::min<int64_t>(chunks, cap));
}

}  // namespace

template <class K, class V>
size_t radix_sort_scratch(int64_t n) {
  constexpr int kChunk = Tile<K, V>::kChunk;
  const int64_t chunks = (n + kChunk - 1) / kChunk;
  const int nb = radix_tiles<K, V>(chunks);
  return align_up(sizeof(K) * n) + align_up(sizeof(V) * n) +
         align_up(sizeof(uint32_t) * kBins * (nb + 1));
}

template <class K, class V>
gv_status radix_sort_pairs(void* scratch, size_t bytes, const K* kin, K* kout, const V* vin,
                           V* vout, int64_t n, int begin_bit, int end_bit, cudaStream_t st) {
  constexpr int kItems = Tile<K, V>::kItems;
  constexpr int kChunk = Tile<K, V>::kChunk;
  if (n <= 0) return GV_OK;
  if (n > (int64_t)UINT32_MAX || begin_bit < 0 || end_bit > (int)(8 * sizeof(K)) ||
      bytes < radix_sort_scratch<K, V>(n)) {
    set_error("radix_sort_pairs: size, bit range or scratch out of range");
    return GV_ERR_INVALID;
  }
  const int passes = end_bit > begin_bit ? (end_bit - begin_bit + 7) / 8 : 0;
  if (passes == 0) {
    GV_CUDA(cudaMemcpyAsync(kout, kin, sizeof(K) * n, cudaMemcpyDeviceToDevice, st));
    GV_CUDA(cudaMemcpyAsync(vout, vin, sizeof(V) * n, cudaMemcpyDeviceToDevice, st));
    return GV_OK;
  }
  char* p = static_cast<char*>(scratch);
  K* kalt = reinterpret_cast<K*>(p);
  p += align_up(sizeof(K) * n);
  V* valt = reinterpret_cast<V*>(p);
  p += align_up(sizeof(V) * n);
  const int64_t chunks = (n + kChunk - 1) / kChunk;
  int nb = radix_tiles<K, V>(chunks);
  const int64_t per_block = (chunks + nb - 1) / nb;
  nb = (int)((chunks + per_block - 1) / per_block);
  const int64_t per_sub = (per_block + kSplit - 1) / kSplit;
  uint32_t* counts = reinterpret_cast<uint32_t*>(p);  // [nb][256]
  uint32_t* totals = counts + (int64_t)kBins * nb;    // [256]
  const K* ks = kin;
  const V* vs = vin;
  for (int q = 0; q < passes; q++) {
    const int shift = begin_bit + 8 * q;
    const int bits = std::min(8, end_bit - shift);
    const uint32_t mask = (1u << bits) - 1u;
    // the last pass writes kout: passes alternate kout and the scratch copy
    const bool to_out = ((passes - 1 - q) % 2) == 0;
    K* kd = to_out ? kout : kalt;
    V* vd = to_out ? vout : valt;
    GV_CUDA(cudaMemsetAsync(counts, 0, sizeof(uint32_t) * kBins * nb, st));
    k_radix_count<K, kItems><<<dim3(nb, kSplit), kThreads, 0, st>>>(ks, n, shift, mask,
                                                                     per_block, per_sub, counts);
    GV_LAUNCH("k_radix_count");
    k_radix_digit<<<kBins, kThreads, 0, st>>>(counts, nb, totals);
    GV_LAUNCH("k_radix_digit");
    k_radix_scatter<K, V><<<nb, kThreads, 0, st>>>(ks, vs, kd, vd, n, shift, mask, per_block,
                                                   counts, totals);
    GV_LAUNCH("k_radix_scatter");
    ks = kd;
    vs = vd;
  }
  return GV_OK;
}

template size_t radix_sort_scratch<uint32_t, uint32_t>(int64_t);
template size_t radix_sort_scratch<unsigned long long, int64_t>(int64_t);
template gv_status radix_sort_pairs<uint32_t, uint32_t>(void*, size_t, const uint32_t*,
                                                        uint32_t*, const uint32_t*, uint32_t*,
                                                        int64_t, int, int, cudaStream_t);
template gv_status radix_sort_pairs<unsigned long long, int64_t>(
    void*, size_t, const unsigned long long*, unsigned long long*, const int64_t*, int64_t*,
    int64_t, int, int, cudaStream_t);

size_t scan_scratch(int64_t n) {
  const int64_t tiles = std::max<int64_t>(1, (n + kScanTile - 1) / kScanTile);
  return align_up(sizeof(uint32_t) * tiles);
}

template <class T>
gv_status exclusive_scan(void* scratch, size_t bytes, const T* in, T* out, int64_t n,
                         cudaStream_t st) {
  if (n <= 0) return GV_OK;
  const int64_t tiles = (n + kScanTile - 1) / kScanTile;
  if (n > (int64_t)INT32_MAX || bytes < scan_scratch(n)) {
    set_error("exclusive_scan: size or scratch out of range");
    return GV_ERR_INVALID;
  }
  uint32_t* sums = static_cast<uint32_t*>(scratch);
  k_scan_tiles<T><<<(unsigned)tiles, kThreads, 0, st>>>(in, n, sums);
  GV_LAUNCH("k_scan_tiles");
  k_scan_sums<<<1, kScanThreads, 0, st>>>(sums, tiles);
  GV_LAUNCH("k_scan_sums");
  k_scan_apply<T><<<(unsigned)tiles, kThreads, 0, st>>>(in, n, sums, out);
  GV_LAUNCH("k_scan_apply");
  return GV_OK;
}

template gv_status exclusive_scan<int>(void*, size_t, const int*, int*, int64_t, cudaStream_t);
template gv_status exclusive_scan<uint32_t>(void*, size_t, const uint32_t*, uint32_t*, int64_t,
                                            cudaStream_t);

size_t rle_scratch(int64_t n) { return scan_scratch(n); }

gv_status run_length_encode(void* scratch, size_t bytes, const uint32_t* keys, int64_t n,
                            uint32_t* rkey, uint32_t* rstart, uint32_t* rcount, int64_t cap,
                            int* nruns, cudaStream_t st) {
  if (n <= 0) {
    GV_CUDA(cudaMemsetAsync(nruns, 0, sizeof(int), st));
    return GV_OK;
  }
  if (n > (int64_t)UINT32_MAX || bytes < rle_scratch(n)) {
    set_error("run_length_encode: size or scratch out of range");
    return GV_ERR_INVALID;
  }
  uint32_t* sums = static_cast<uint32_t*>(scratch);
  const int64_t tiles = (n + kScanTile - 1) / kScanTile;
  k_rle_tiles<<<(unsigned)tiles, kThreads, 0, st>>>(keys, n, sums);
  GV_LAUNCH("k_rle_tiles");
  k_scan_sums<<<1, kScanThreads, 0, st>>>(sums, tiles);
  GV_LAUNCH("k_scan_sums");
  k_rle_apply<<<(unsigned)tiles, kThreads, 0, st>>>(keys, n, sums, cap, rkey, rstart, nruns);
  GV_LAUNCH("k_rle_apply");
  const int64_t rc = std::min<int64_t>(n, cap);
  if (rc > 0) {
    k_rle_counts<<<(unsigned)((rc + 255) / 256), 256, 0, st>>>(n, keys, rstart, nruns, cap,
                                                                rcount);
    GV_LAUNCH("k_rle_counts");
  }
  return GV_OK;
}

}  // namespace gv

// ---- C ABI (tests and tools) ------------------------------------------------

namespace {
struct Scratch {
  void* p = nullptr;
  ~Scratch() {
    if (p) cudaFree(p);
  }
};

template <class K, class V>
gv_status sort_entry(const K* kin, K* kout, const V* vin, V* vout, int64_t n, int32_t b0,
                     int32_t b1, void* stream) {
  if (n < 0 || (n > 0 && (!kin || !kout || !vin || !vout))) {
    gv::set_error("radix sort: null buffer or negative size");
    return GV_ERR_INVALID;
  }
  if (n == 0) return GV_OK;
  cudaStream_t st = (cudaStream_t)stream;
  const size_t bytes = gv::radix_sort_scratch<K, V>(n);
  Scratch s;
  GV_CUDA(cudaMalloc(&s.p, bytes));
  GV_TRY((gv::radix_sort_pairs<K, V>(s.p, bytes, kin, kout, vin, vout, n, b0, b1, st)));
  GV_CUDA(cudaStreamSynchronize(st));
  return GV_OK;
}
}  // namespace

extern "C" {

gv_status gv_radix_sort_pairs_u32(const uint32_t* d_keys_in, uint32_t* d_keys_out,
                                  const uint32_t* d_vals_in, uint32_t* d_vals_out, int64_t n,
                                  int32_t begin_bit, int32_t end_bit, void* stream) {
  return sort_entry<uint32_t, uint32_t>(d_keys_in, d_keys_out, d_vals_in, d_vals_out, n,
                                        begin_bit, end_bit, stream);
}

gv_status gv_radix_sort_pairs_u64(const uint64_t* d_keys_in, uint64_t* d_keys_out,
                                  const int64_t* d_vals_in, int64_t* d_vals_out, int64_t n,
                                  int32_t begin_bit, int32_t end_bit, void* stream) {
  return sort_entry<unsigned long long, int64_t>(
      reinterpret_cast<const unsigned long long*>(d_keys_in),
      reinterpret_cast<unsigned long long*>(d_keys_out), d_vals_in, d_vals_out, n, begin_bit,
      end_bit, stream);
}

gv_status gv_exclusive_scan_i32(const int32_t* d_in, int32_t* d_out, int64_t n, void* stream) {
  if (n < 0 || (n > 0 && (!d_in || !d_out))) {
    gv::set_error("exclusive scan: null buffer or negative size");
    return GV_ERR_INVALID;
  }
  if (n == 0) return GV_OK;
  cudaStream_t st = (cudaStream_t)stream;
  const size_t bytes = gv::scan_scratch(n);
  Scratch s;
  GV_CUDA(cudaMalloc(&s.p, bytes));
  GV_TRY(gv::exclusive_scan<int>(s.p, bytes, d_in, d_out, n, st));
  GV_CUDA(cudaStreamSynchronize(st));
  return GV_OK;
}

gv_status gv_run_length_encode_u32(const uint32_t* d_keys, int64_t n, uint32_t* d_run_keys,
                                   uint32_t* d_run_starts, uint32_t* d_run_lengths, int64_t cap,
                                   int32_t* d_nruns, void* stream) {
  if (n < 0 || cap < 0 || !d_nruns ||
      (n > 0 && (!d_keys || !d_run_keys || !d_run_starts || !d_run_lengths))) {
    gv::set_error("run-length encode: null buffer or negative size");
    return GV_ERR_INVALID;
  }
  cudaStream_t st = (cudaStream_t)stream;
  const size_t bytes = gv::rle_scratch(n);
  Scratch s;
  GV_CUDA(cudaMalloc(&s.p, bytes));
  GV_TRY(gv::run_length_encode(s.p, bytes, d_keys, n, d_run_keys, d_run_starts, d_run_lengths,
                               cap, d_nruns, st));
  GV_CUDA(cudaStreamSynchronize(st));
  return GV_OK;
}

}  // extern "C"
