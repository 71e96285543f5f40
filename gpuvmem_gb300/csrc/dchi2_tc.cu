// DChi2 on the 5th-generation tensor cores (tcgen05, sm_103a).
//
// The reference's direct sum (src/functions.cu:3698-3791)
//   S(i,j) = sum_k w_k Re(conj(Vr_k) e^{2 pi i theta_k(i,j)}),
//   theta_k(i,j) = x_j u_k + y_i v_k + (z_ij - 1) w_k,
// is a complex GEMM once the phase is split into per-row and per-column
// factors: with (z-1) = -(x^2+y^2)/2 + rho and |w rho| below 1e-7 cycles
// (checked at set-up),
//   e^{2 pi i theta} = b_k(i) a_k(j),  b_k(i) = e^{2 pi i (y_i v_k - w_k y_i^2/2)},
//                                     a_k(j) = e^{2 pi i (x_j u_k - w_k x_j^2/2)},
//   S(i,j) = Re sum_k b_k(i) x_k(j),  x_k(j) = conj(w_k Vr_k) a_k(j),
// i.e. a real GEMM D = A B with K = 2V:  A[i][2k] = Re b, A[i][2k+1] = Im b,
// B[2k][j] = Re x, B[2k+1][j] = -Im x.
//
// Operands are never materialised in HBM.  Per chunk of 32 visibilities the
// generator warps build the 128 x 64 A tile and the TN x 64 B tile in shared
// memory: each thread produces 8 consecutive rows for one visibility from an
// exact fixed-point anchor (the linear phase is reduced mod 1 with 32-bit
// integer products) and a chirp recurrence in FP32.  Each operand is split
// into FP16 hi + lo parts and the tile is accumulated with three MMAs
// (hi*hi + hi*lo + lo*hi) into an FP32 accumulator in TMEM.  Operand tiles are
// MN-major with the 128-byte swizzle.
//
// Thread-block clusters of CS CTAs (CS = 1, 2 or 4) work on CS consecutive
// row tiles of the same column tile and visibility range, so they need the
// same B tile: each CTA generates 1/CS of B and writes it into the shared
// memory of every CTA of its cluster (distributed shared memory); A stays
// local.  Each CTA runs its own cta_group::1 MMAs on its own TMEM.  An MMA
// commit is multicast to every CTA's "stage empty" barrier, since every
// CTA writes into every stage.
//
// Warp roles (no block-wide barrier per chunk):
//   generator warps  wait for the chunk's visibility constants and a stage
//                    free in all CTAs of the cluster, generate, arrive on the
//                    "stage full" barrier of every CTA; warps 0..7 also drain
//                    the accumulator every `slab` chunks into a running sum
//                    in the other half of TMEM, and at the end of a channel
//                    apply the epilogue factor (beam, fg_scale, chain rule)
//                    and add it to this split's partial image;
//   control warp     its lanes load the visibility constants of chunks up to
//                    three ahead into a 4-slot ring; its lane 0 issues the
//                    MMAs of each full stage and commits them.
// Split-K partials are summed in FP64 in a fixed order, so results are
// deterministic.
//
// Every wait is bounded: on timeout the kernel records an error word, every
// warp stops, the MMAs in flight are waited for (bounded), the cluster
// meets at a final barrier so no CTA exits while a peer may still write into
// its shared memory, TMEM is freed and the kernel returns; the host turns
// the word into GV_ERR_DEVICE.
#include <cuda_fp16.h>

#include <algorithm>
#include <cstdint>
#include <cstdlib>

#include "gv_internal.cuh"

namespace gv {

namespace tc {

constexpr int kTM = 128;            // image rows per tile (MMA M)
constexpr int kChunkVis = 32;       // visibilities per chunk
constexpr int kKC = 2 * kChunkVis;  // K elements per chunk
constexpr int kDrainWarps = 8;      // warps that drain TMEM (4 lane quarters x 2 halves)
constexpr int kVisSlots = 4;
constexpr int kLookahead = kVisSlots - 1;
constexpr int kSlab = 4;            // default chunks accumulated before a drain
constexpr uint32_t kTmemCols = 512;
constexpr long long kWaitCycles = 4000000000LL;  // ~2 s at 2 GHz

// generator warps per CTA: every warp gets the same number of warp-tasks per
// chunk.  A warp-task is 64 rows x 4*vpl visibilities (vpl = visibilities
// per lane, generated as independent instruction streams for ILP); for
// TN = 256 a chunk has 16/vpl A tasks and 32/(cs*vpl) B tasks.
__host__ __device__ constexpr int gen_warps(int cs, int vpl) {
  return vpl == 2 ? 12 : (cs == 4 ? 12 : 16);
}
__host__ __device__ constexpr int threads_for(int cs, int vpl) {
  return gen_warps(cs, vpl) * 32 + 32;
}

struct VisEntry {
  uint32_t FU, FV;
  float GU, GV;
  float2 Eu, Ev;
  float2 c;      // conj(w Vr) * global scale / chunk scale
  float ascale;  // chunk scale 2^e (e <= 0) applied to the A operand
  float pad;
};

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

// ---- cluster / tcgen05 / mbarrier wrappers (inline PTX) ---------------------
__device__ __forceinline__ uint32_t cluster_rank() {
  uint32_t r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}
__device__ __forceinline__ uint32_t cluster_id() {
  uint32_t r;
  asm volatile("mov.u32 %0, %%clusterid.x;" : "=r"(r));
  return r;
}
__device__ __forceinline__ uint32_t num_clusters() {
  uint32_t r;
  asm volatile("mov.u32 %0, %%nclusterid.x;" : "=r"(r));
  return r;
}
__device__ __forceinline__ void cluster_sync() {
  asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::
                   : "memory");
}
// shared::cluster address of `local` in CTA `rank` of this cluster
__device__ __forceinline__ uint32_t map_rank(uint32_t local, uint32_t rank) {
  uint32_t r;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(local), "r"(rank));
  return r;
}
__device__ __forceinline__ void st_cluster_v4(uint32_t addr, uint4 v) {
  asm volatile("st.shared::cluster.v4.b32 [%0], {%1, %2, %3, %4};" ::"r"(addr), "r"(v.x),
               "r"(v.y), "r"(v.z), "r"(v.w)
               : "memory");
}
__device__ __forceinline__ void mbar_init(uint64_t* m, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(m)), "r"(count));
}
__device__ __forceinline__ void mbar_arrive(uint64_t* m) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(m)) : "memory");
}
// arrive, with release at cluster scope, on a barrier of any CTA of the cluster
__device__ __forceinline__ void mbar_arrive_cluster(uint32_t cluster_addr) {
  asm volatile("mbarrier.arrive.release.cluster.shared::cluster.b64 _, [%0];" ::"r"(cluster_addr)
               : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* m, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.acquire.cluster.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}\n"
      : "=r"(ok)
      : "r"(smem_u32(m)), "r"(parity)
      : "memory");
  return ok != 0;
}
// bounded wait; returns false on timeout or when another warp gave up
__device__ __forceinline__ bool mbar_wait(uint64_t* m, uint32_t parity, volatile int* abort,
                                          uint32_t* err, uint32_t code) {
  if (mbar_try_wait(m, parity)) return true;
  const long long t0 = clock64();
  for (uint32_t it = 1;; it++) {
    if (mbar_try_wait(m, parity)) return true;
    if ((it & 15) == 0) {
      if (*abort) return false;
      if (clock64() - t0 > kWaitCycles) {
        atomicExch(err, code);
        *abort = 1;
        return false;
      }
    }
  }
}
// warp-level wait: lane 0 waits, the warp reconverges (memory ordering of
// __syncwarp carries lane 0's acquire to the other lanes)
__device__ __forceinline__ bool warp_wait(uint64_t* m, uint32_t parity, volatile int* abort,
                                          uint32_t* err, uint32_t code) {
  int ok = 1;
  if ((threadIdx.x & 31) == 0) ok = mbar_wait(m, parity, abort, err, code) ? 1 : 0;
  return __shfl_sync(0xffffffffu, ok, 0) != 0;
}
// warp-level arrive (barriers counted in warps)
__device__ __forceinline__ void warp_arrive(uint64_t* m) {
  __syncwarp();
  if ((threadIdx.x & 31) == 0) mbar_arrive(m);
}
__device__ __forceinline__ void tmem_alloc(uint32_t* slot, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                   smem_u32(slot)),
               "r"(ncols)
               : "memory");
}
__device__ __forceinline__ void tmem_relinquish() {
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols)
               : "memory");
}
__device__ __forceinline__ void fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
// generic-proxy writes (local and remote shared memory) -> async proxy
__device__ __forceinline__ void fence_proxy_async() {
  asm volatile("fence.proxy.async;" ::: "memory");
}
__device__ __forceinline__ void mma_f16(uint32_t dtmem, uint64_t adesc, uint64_t bdesc,
                                        uint32_t idesc, uint32_t accum) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(dtmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accum)
      : "memory");
}
__device__ __forceinline__ void mma_commit(uint64_t* mbar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
          smem_u32(mbar))
      : "memory");
}
// commit arriving on the barrier at the same offset in every CTA of `mask`
__device__ __forceinline__ void mma_commit_multicast(uint64_t* mbar, uint16_t mask) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.multicast::cluster.b64 "
      "[%0], %1;" ::"r"(smem_u32(mbar)),
      "h"(mask)
      : "memory");
}
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float* v) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
      "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
      "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),
        "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]),
        "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
        "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]),
        "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int k = 0; k < 32; k++) v[k] = __uint_as_float(r[k]);
}
__device__ __forceinline__ void tmem_st32(uint32_t taddr, const float* v) {
  asm volatile(
      "tcgen05.st.sync.aligned.32x32b.x32.b32 [%0], "
      "{%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,"
      "%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31,%32};" ::"r"(taddr),
      "r"(__float_as_uint(v[0])), "r"(__float_as_uint(v[1])), "r"(__float_as_uint(v[2])),
      "r"(__float_as_uint(v[3])), "r"(__float_as_uint(v[4])), "r"(__float_as_uint(v[5])),
      "r"(__float_as_uint(v[6])), "r"(__float_as_uint(v[7])), "r"(__float_as_uint(v[8])),
      "r"(__float_as_uint(v[9])), "r"(__float_as_uint(v[10])), "r"(__float_as_uint(v[11])),
      "r"(__float_as_uint(v[12])), "r"(__float_as_uint(v[13])), "r"(__float_as_uint(v[14])),
      "r"(__float_as_uint(v[15])), "r"(__float_as_uint(v[16])), "r"(__float_as_uint(v[17])),
      "r"(__float_as_uint(v[18])), "r"(__float_as_uint(v[19])), "r"(__float_as_uint(v[20])),
      "r"(__float_as_uint(v[21])), "r"(__float_as_uint(v[22])), "r"(__float_as_uint(v[23])),
      "r"(__float_as_uint(v[24])), "r"(__float_as_uint(v[25])), "r"(__float_as_uint(v[26])),
      "r"(__float_as_uint(v[27])), "r"(__float_as_uint(v[28])), "r"(__float_as_uint(v[29])),
      "r"(__float_as_uint(v[30])), "r"(__float_as_uint(v[31]))
      : "memory");
  asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
}

// Shared-memory matrix descriptor (tcgen05): start address, leading byte
// offset (stride between 64-element MN atoms for MN-major swizzled layouts),
// stride byte offset (stride between 8-row K atoms), version 1, 128-byte
// swizzle.
__device__ __forceinline__ uint64_t make_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);
  d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
  d |= (uint64_t)1 << 46;
  d |= (uint64_t)2 << 61;
  return d;
}

// Instruction descriptor of kind::f16: D = F32, A = B = F16, both MN-major.
__host__ __device__ constexpr uint32_t make_idesc(int M, int N) {
  return (1u << 4) | (0u << 7) | (0u << 10) | (1u << 15) | (1u << 16) |
         ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

// byte offset of the 16-byte chunk holding rows 8*oct..8*oct+7 of MN atom
// `matom` at K index kk, in an MN-major 128B-swizzled tile whose MN atoms
// (64 rows) are 1024 B apart and K atoms (8 rows) are sbo apart
__device__ __forceinline__ uint32_t tile_off(int matom, int oct, int kk, uint32_t sbo) {
  const int katom = kk >> 3, krow = kk & 7;
  return (uint32_t)(katom * sbo + matom * 1024 + krow * 128 + ((oct ^ krow) << 4));
}

struct TcParams {
  int N;  // image is N x N
  int64_t MN;
  int x0, y0;  // int-truncated centre (DChi2 coordinates)
  float xobs, yobs, nu_0, D, pbf, pbcut, fg_scale, threshold;
  int pb;
  double DELTAX, DELTAY;
  int normalize, flag_opt, mode;
  int fast_anchor;  // 1: anchor phasor from the SFU (__sincosf), 0: sincospif
  int slab;         // chunks accumulated in TMEM by the tensor core before a drain
  int ntile_i, ntile_j, nsplit;
  int C;
  int64_t Ktot;               // kept visibilities over all channels
  const int64_t* kc_off;      // [C+1] compact offsets of kept visibilities
  const ChanRange* ranges;    // [C]
  const float* chfreq;
  const int64_t* chnvis;
  const uint4* ph;
  const float4* E;
  const float2* cvr;
  const float4* deg;
  const float2* vo;
  const uint8_t* mask;
  const float* img;
  const uint32_t* cmax_bits;  // max |c| (float bits)
  float* partial;             // [nsplit][MN]
  uint32_t* err;
};

template <int TN>
struct Layout {
  static constexpr uint32_t kSboA = (kTM / 64) * 1024;  // bytes between K atoms of A
  static constexpr uint32_t kSboB = (TN / 64) * 1024;
  static constexpr uint32_t kTileA = kSboA * (kKC / 8);  // one A part (hi or lo)
  static constexpr uint32_t kTileB = kSboB * (kKC / 8);
  static constexpr uint32_t kStage = 2 * kTileA + 2 * kTileB;
  static constexpr uint32_t kVis = kVisSlots * kChunkVis * sizeof(VisEntry);
  static constexpr uint32_t kBars = 16 * 8;
  static constexpr uint32_t kSmem = 1024 + 2 * kStage + kVis + kBars + 16;
};

// Epilogue factor of one pixel for channel c (mode 0: gradient with chain
// rule; 1: raw channel DChi2; 2: dirty image), divided by the operand scale.
__device__ __forceinline__ float epi_factor(const TcParams& p, int c, int i, int j, float inv_s) {
  if (p.mode == 2) return inv_s;
  const int64_t q = (int64_t)p.N * i + j;
  if (!(p.mask[q] & kMaskIn)) return 0.0f;
  const float freq = p.chfreq[c];
  const float atten = attenuation(i, j, p.xobs, p.yobs, p.DELTAX, p.DELTAY, freq, p.D, p.pbf,
                                  p.pbcut, p.pb);
  float f = -(p.fg_scale * atten) * inv_s;
  if (p.normalize) f /= (float)p.chnvis[c];
  if (p.mode == 1) return f;
  const float nudiv = freq / p.nu_0;
  const float i0 = p.img[q], al = p.img[p.MN + q];
  const float pw = powf(nudiv, al);
  if (p.flag_opt % 2 == 0) return f * pw;
  if (i0 > p.threshold) return f * (i0 * pw * p.fg_scale * logf(nudiv));
  return 0.0f;
}

struct Octet {
  uint4 hre, him, lre, lim;
};

// 8 consecutive rows of one operand for one visibility: FP16 hi/lo parts of
// Re and (sign-adjusted) Im, packed for 16-byte stores.
template <bool kIsB>
__device__ __forceinline__ Octet gen_octet(const VisEntry& ve, int r0, bool fast) {
  const uint32_t F = kIsB ? ve.FU : ve.FV;
  const float G = kIsB ? ve.GU : ve.GV;
  const float2 E = kIsB ? ve.Eu : ve.Ev;
  const float rf = (float)r0;
  const uint32_t lin = (uint32_t)r0 * F;
  float th = (float)(int32_t)lin * 2.3283064365386963e-10f;
  th = fmaf(-rf * rf, G, th);
  // th is in [-0.5, 0.5] cycles: the SFU's sin/cos of 2 pi th are within
  // ~4e-7 absolute, below the FP16 hi/lo split's own error budget
  float sn, cs;
  if (fast)
    __sincosf(6.283185307179586f * th, &sn, &cs);
  else
    sincospif(2.0f * th, &sn, &cs);
  float2 v = make_float2(cs, sn);
  if (kIsB)
    v = cmul(v, ve.c);
  else
    v = make_float2(v.x * ve.ascale, v.y * ve.ascale);
  // d = e^{2 pi i (f - G (2 r0 + 1))}, q = e^{-4 pi i G}; the chirp angles
  // are below 1e-3 rad, so second-order expansions are exact in FP32
  const float eps = -6.283185307179586f * G * (2.0f * rf + 1.0f);
  float2 d = cmul(E, make_float2(fmaf(-0.5f * eps, eps, 1.0f), eps));
  const float eq = -12.566370614359172f * G;
  float re[8], im[8];
#pragma unroll
  for (int t = 0; t < 8; t++) {
    re[t] = v.x;
    im[t] = kIsB ? -v.y : v.y;
    if (t < 7) {
      v = cmul(v, d);
      d = make_float2(fmaf(-eq, d.y, d.x), fmaf(eq, d.x, d.y));
    }
  }
  uint32_t hre[4], him[4], lre[4], lim[4];
#pragma unroll
  for (int t = 0; t < 4; t++) {
    const __half2 h_re = __floats2half2_rn(re[2 * t], re[2 * t + 1]);
    const __half2 h_im = __floats2half2_rn(im[2 * t], im[2 * t + 1]);
    const float2 b_re = __half22float2(h_re);
    const float2 b_im = __half22float2(h_im);
    const __half2 l_re = __floats2half2_rn(re[2 * t] - b_re.x, re[2 * t + 1] - b_re.y);
    const __half2 l_im = __floats2half2_rn(im[2 * t] - b_im.x, im[2 * t + 1] - b_im.y);
    hre[t] = *reinterpret_cast<const uint32_t*>(&h_re);
    him[t] = *reinterpret_cast<const uint32_t*>(&h_im);
    lre[t] = *reinterpret_cast<const uint32_t*>(&l_re);
    lim[t] = *reinterpret_cast<const uint32_t*>(&l_im);
  }
  Octet o;
  o.hre = make_uint4(hre[0], hre[1], hre[2], hre[3]);
  o.him = make_uint4(him[0], him[1], him[2], him[3]);
  o.lre = make_uint4(lre[0], lre[1], lre[2], lre[3]);
  o.lim = make_uint4(lim[0], lim[1], lim[2], lim[3]);
  return o;
}

// The chunk sequence every warp of every CTA of a cluster walks in the same
// order: the cluster's work items (row-tile group, column tile, split), the
// channels each split overlaps, and 32-visibility chunks within a channel.
struct ChunkIter {
  int item, c, n, nchunks;
  int64_t goff, nvis;
  bool valid;
};

__device__ __forceinline__ void item_range(const TcParams& p, int item, int64_t* ks,
                                           int64_t* ke) {
  const int split = item % p.nsplit;
  *ks = p.Ktot * split / p.nsplit;
  *ke = p.Ktot * (split + 1) / p.nsplit;
}

// position `it` on the first chunk at or after (item, channel c); returns
// false when the cluster has no more chunks
__device__ bool iter_seek(const TcParams& p, int nitems, int stride, ChunkIter& it) {
  while (it.item < nitems) {
    int64_t ks, ke;
    item_range(p, it.item, &ks, &ke);
    for (; it.c < p.C; it.c++) {
      const int64_t cs = p.kc_off[it.c], ce = p.kc_off[it.c + 1];
      const int64_t a = ks > cs ? ks : cs, b = ke < ce ? ke : ce;
      if (a < b) {
        it.goff = p.ranges[it.c].off + (a - cs);
        it.nvis = b - a;
        it.nchunks = (int)((it.nvis + kChunkVis - 1) / kChunkVis);
        it.n = 0;
        it.valid = true;
        return true;
      }
    }
    it.item += stride;
    it.c = 0;
  }
  it.valid = false;
  return false;
}

__device__ __forceinline__ void iter_next(const TcParams& p, int nitems, int stride,
                                          ChunkIter& it) {
  if (++it.n < it.nchunks) return;
  it.c++;
  iter_seek(p, nitems, stride, it);
}

template <int TN, int CS, int VPL>
__global__ void __launch_bounds__(threads_for(CS, VPL), 1) k_dchi2_tc(TcParams p) {
  using L = Layout<TN>;
  constexpr int GW = gen_warps(CS, VPL);
  constexpr int kMB = TN / 64;        // MN atoms of B
  constexpr int kMBown = kMB / CS;    // B atoms this CTA generates
  extern __shared__ uint8_t smem_raw[];
  const uint32_t raw = smem_u32(smem_raw);
  uint8_t* base = smem_raw + (((raw + 1023u) & ~1023u) - raw);
  VisEntry* s_vis = reinterpret_cast<VisEntry*>(base + 2 * L::kStage);
  uint64_t* bars = reinterpret_cast<uint64_t*>(base + 2 * L::kStage + L::kVis);
  uint64_t* op_full = bars;       // [2]  one arrive per generator warp per CTA of the cluster
  uint64_t* op_empty = bars + 2;  // [2]  one MMA commit per CTA of the cluster
  uint64_t* vis_full = bars + 4;  // [4]  32 arrives (control lanes)
  uint64_t* vis_empty = bars + 8; // [4]  one arrive per generator warp
  uint64_t* drained = bars + 12;  // [1]  one arrive per draining warp
  uint32_t* tslot = reinterpret_cast<uint32_t*>(bars + 16);
  __shared__ int s_abort;
  volatile int* abort = &s_abort;

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const uint32_t rank = CS > 1 ? cluster_rank() : 0u;
  const int cid = CS > 1 ? (int)cluster_id() : (int)blockIdx.x;
  const int ncl = CS > 1 ? (int)num_clusters() : (int)gridDim.x;
  if (warp == 0) {
    tmem_alloc(tslot, kTmemCols);
    tmem_relinquish();
  }
  if (tid == 0) {
    mbar_init(&op_full[0], GW * CS);
    mbar_init(&op_full[1], GW * CS);
    mbar_init(&op_empty[0], CS);
    mbar_init(&op_empty[1], CS);
    for (int s = 0; s < kVisSlots; s++) {
      mbar_init(&vis_full[s], 32);
      mbar_init(&vis_empty[s], GW);
    }
    mbar_init(drained, kDrainWarps);
    s_abort = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  fence_before();
  __syncthreads();
  if (CS > 1) cluster_sync();  // peers' barriers are initialised before any remote access
  fence_after();
  const uint32_t tbase = *tslot;
  const uint32_t t_acc = tbase;
  const uint32_t t_run = tbase + 256;

  // operand scale: c * 2^-e with max |c| * 2^-e <= 1
  const float cmax = __uint_as_float(*p.cmax_bits);
  int e = 0;
  if (cmax > 0.0f) frexpf(cmax, &e);
  const float scale = ldexpf(1.0f, -e);
  const float inv_s = ldexpf(1.0f, e);
  const int nitems = (p.ntile_i / CS) * p.ntile_j * p.nsplit;
  uint32_t nch = 0;  // position in the cluster's chunk sequence

  if (warp == GW) {
    // ------------------------------- control warp --------------------------
    ChunkIter ld{cid, 0, 0, 0, 0, 0, false};
    ChunkIter mm = ld;
    iter_seek(p, nitems, ncl, ld);
    iter_seek(p, nitems, ncl, mm);
    uint32_t nld = 0, ndrain = 0;
    const uint32_t idesc = make_idesc(kTM, TN);
    bool ok = true;
    auto load_one = [&](const ChunkIter& it, uint32_t q) -> bool {
      const int slot = q % kVisSlots;
      if (q >= kVisSlots) {
        if (!mbar_wait(&vis_empty[slot], ((q / kVisSlots) - 1) & 1, abort, p.err, 4u)) return false;
      }
      VisEntry ve;
      const int64_t kidx = (int64_t)it.n * kChunkVis + lane;
      if (kidx < it.nvis) {
        const int64_t g = it.goff + kidx;
        const uint4 ph = p.ph[g];
        const float4 E = p.E[g];
        float2 cc;
        if (p.mode == 2) {
          const float4 d = p.deg[g];
          const float2 o = p.vo[g];
          cc = make_float2(d.w * o.x, -(d.w * o.y));
        } else {
          const float2 r = p.cvr[g];
          cc = make_float2(r.x, -r.y);
        }
        ve.FU = ph.x;
        ve.FV = ph.y;
        ve.GU = __uint_as_float(ph.z);
        ve.GV = __uint_as_float(ph.w);
        ve.Eu = make_float2(E.x, E.y);
        ve.Ev = make_float2(E.z, E.w);
        ve.c = make_float2(cc.x * scale, cc.y * scale);
      } else {
        ve.FU = ve.FV = 0u;
        ve.GU = ve.GV = 0.0f;
        ve.Eu = ve.Ev = make_float2(1.0f, 0.0f);
        ve.c = make_float2(0.0f, 0.0f);
      }
      // chunk scale: B carries c / 2^e, A carries b * 2^e (powers of two,
      // exact), so small residuals keep FP16's relative precision
      float m = fmaxf(fabsf(ve.c.x), fabsf(ve.c.y));
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
      int ce = 0;
      if (m > 0.0f) frexpf(m, &ce);
      ce = ce < -24 ? -24 : (ce > 0 ? 0 : ce);
      ve.ascale = ldexpf(1.0f, ce);
      ve.c = make_float2(ldexpf(ve.c.x, -ce), ldexpf(ve.c.y, -ce));
      ve.pad = 0.0f;
      s_vis[slot * kChunkVis + lane] = ve;
      mbar_arrive(&vis_full[slot]);
      return true;
    };
    // prime the ring
    while (ok && ld.valid && nld < (uint32_t)kLookahead) {
      ok = load_one(ld, nld);
      nld++;
      iter_next(p, nitems, ncl, ld);
    }
    while (ok && mm.valid) {
      if (ld.valid) {
        ok = load_one(ld, nld);
        nld++;
        iter_next(p, nitems, ncl, ld);
        if (!ok) break;
      }
      const int st = nch & 1;
      const bool fresh = (mm.n % p.slab) == 0;
      const bool drain = (mm.n == mm.nchunks - 1) || ((mm.n % p.slab) == p.slab - 1);
      if (lane == 0) {
        ok = mbar_wait(&op_full[st], (nch >> 1) & 1, abort, p.err, 5u);
        if (ok && fresh && nch > 0) ok = mbar_wait(drained, (ndrain - 1) & 1, abort, p.err, 6u);
        if (ok) {
          fence_after();
          uint8_t* sp = base + st * L::kStage;
          const uint32_t sa_hi = smem_u32(sp), sa_lo = sa_hi + L::kTileA;
          const uint32_t sb_hi = sa_hi + 2 * L::kTileA, sb_lo = sb_hi + L::kTileB;
#pragma unroll
          for (int t = 0; t < kKC / 16; t++) {
            const uint64_t ah = make_desc(sa_hi + t * 2 * L::kSboA, 1024, L::kSboA);
            const uint64_t al = make_desc(sa_lo + t * 2 * L::kSboA, 1024, L::kSboA);
            const uint64_t bh = make_desc(sb_hi + t * 2 * L::kSboB, 1024, L::kSboB);
            const uint64_t bl = make_desc(sb_lo + t * 2 * L::kSboB, 1024, L::kSboB);
            mma_f16(t_acc, ah, bh, idesc, (fresh && t == 0) ? 0u : 1u);
            mma_f16(t_acc, ah, bl, idesc, 1u);
            mma_f16(t_acc, al, bh, idesc, 1u);
          }
          if (CS > 1)
            mma_commit_multicast(&op_empty[st], (uint16_t)((1u << CS) - 1u));
          else
            mma_commit(&op_empty[st]);
        }
      }
      ok = __shfl_sync(0xffffffffu, ok ? 1 : 0, 0) != 0;
      if (drain) ndrain++;
      nch++;
      iter_next(p, nitems, ncl, mm);
    }
    // retire: no MMA of this CTA may be in flight when TMEM is freed (the
    // barrier also counts the peers' commits, which only makes this later)
    if (lane == 0 && nch > 0) {
      const uint32_t q = nch - 1;
      const long long t0 = clock64();
      while (!mbar_try_wait(&op_empty[q & 1], (q >> 1) & 1)) {
        if (clock64() - t0 > kWaitCycles) {
          atomicExch(p.err, 7u);
          break;
        }
      }
    }
  } else {
    // ----------------------------- generator warps -------------------------
    const int oct = lane & 7, kq = lane >> 3;
    const bool fast = p.fast_anchor != 0;
    constexpr int kVq = kChunkVis / (4 * VPL);  // visibility groups per chunk
    constexpr int kTasksA = (kTM / 64) * kVq;
    constexpr int kTasksB = kMBown * kVq;
    constexpr int kCols = TN / 2;             // epilogue columns per draining thread
    const bool drainer = warp < kDrainWarps;
    const int lq = warp & 3, half = (warp >> 2) & 1;
    const uint32_t lane_off = (uint32_t)(32 * lq) << 16;
    // shared::cluster addresses of both stages' B tiles and op_full barriers
    // in every CTA of the cluster
    uint32_t bhi_r[2][CS], blo_r[2][CS], full_r[2][CS];
#pragma unroll
    for (int s = 0; s < 2; s++) {
      const uint32_t lb = smem_u32(base + s * L::kStage + 2 * L::kTileA);
#pragma unroll
      for (int r = 0; r < CS; r++) {
        bhi_r[s][r] = CS > 1 ? map_rank(lb, r) : lb;
        blo_r[s][r] = CS > 1 ? map_rank(lb + L::kTileB, r) : lb + L::kTileB;
        full_r[s][r] = CS > 1 ? map_rank(smem_u32(&op_full[s]), r) : smem_u32(&op_full[s]);
      }
    }
    bool ok = true;
    for (int item = cid; item < nitems && ok; item += ncl) {
      const int split = item % p.nsplit;
      const int tile = item / p.nsplit;
      const int tig = tile / p.ntile_j, tj = tile % p.ntile_j;
      const int i0 = (tig * CS + (int)rank) * kTM, j0 = tj * TN;
      int64_t ks, ke;
      item_range(p, item, &ks, &ke);
      bool first_channel = true;
      const int ei = i0 + 32 * lq + lane;
      const int ej0 = j0 + half * kCols;
      float* prow = p.partial + (int64_t)split * p.MN + (int64_t)p.N * ei + ej0;
      for (int c = 0; c < p.C && ok; c++) {
        const int64_t cs = p.kc_off[c], ce = p.kc_off[c + 1];
        const int64_t a = ks > cs ? ks : cs, b = ke < ce ? ke : ce;
        if (a >= b) continue;
        const int nchunks = (int)((b - a + kChunkVis - 1) / kChunkVis);
        bool run_empty = true;
        for (int n = 0; n < nchunks && ok; n++) {
          const int st = nch & 1;
          const int slot = nch % kVisSlots;
          if (nch >= 2) ok = warp_wait(&op_empty[st], ((nch >> 1) - 1) & 1, abort, p.err, 1u);
          if (ok) ok = warp_wait(&vis_full[slot], (nch / kVisSlots) & 1, abort, p.err, 2u);
          if (!ok) break;
          uint8_t* sp = base + st * L::kStage;
          uint8_t* a_hi = sp;
          uint8_t* a_lo = sp + L::kTileA;
          const VisEntry* sv = s_vis + slot * kChunkVis;
          for (int wt = warp; wt < kTasksA + kTasksB; wt += GW) {
            if (wt < kTasksA) {
              const int matom = wt / kVq;
              const int kv0 = (wt % kVq) * 4 * VPL + kq;
              const int r0 = i0 + matom * 64 + oct * 8 - p.y0;
              Octet o[VPL];
#pragma unroll
              for (int v = 0; v < VPL; v++) o[v] = gen_octet<false>(sv[kv0 + 4 * v], r0, fast);
#pragma unroll
              for (int v = 0; v < VPL; v++) {
                const int kv = kv0 + 4 * v;
                const uint32_t ore = tile_off(matom, oct, 2 * kv, L::kSboA);
                const uint32_t oim = tile_off(matom, oct, 2 * kv + 1, L::kSboA);
                *reinterpret_cast<uint4*>(a_hi + ore) = o[v].hre;
                *reinterpret_cast<uint4*>(a_hi + oim) = o[v].him;
                *reinterpret_cast<uint4*>(a_lo + ore) = o[v].lre;
                *reinterpret_cast<uint4*>(a_lo + oim) = o[v].lim;
              }
            } else {
              const int w2 = wt - kTasksA;
              const int matom = (int)rank * kMBown + w2 / kVq;
              const int kv0 = (w2 % kVq) * 4 * VPL + kq;
              const int r0 = j0 + matom * 64 + oct * 8 - p.x0;
              Octet o[VPL];
#pragma unroll
              for (int v = 0; v < VPL; v++) o[v] = gen_octet<true>(sv[kv0 + 4 * v], r0, fast);
#pragma unroll
              for (int v = 0; v < VPL; v++) {
                const int kv = kv0 + 4 * v;
                const uint32_t ore = tile_off(matom, oct, 2 * kv, L::kSboB);
                const uint32_t oim = tile_off(matom, oct, 2 * kv + 1, L::kSboB);
                if (CS == 1) {
                  uint8_t* b_hi = sp + 2 * L::kTileA;
                  uint8_t* b_lo = b_hi + L::kTileB;
                  *reinterpret_cast<uint4*>(b_hi + ore) = o[v].hre;
                  *reinterpret_cast<uint4*>(b_hi + oim) = o[v].him;
                  *reinterpret_cast<uint4*>(b_lo + ore) = o[v].lre;
                  *reinterpret_cast<uint4*>(b_lo + oim) = o[v].lim;
                } else {
#pragma unroll
                  for (int r = 0; r < CS; r++) {
                    st_cluster_v4(bhi_r[st][r] + ore, o[v].hre);
                    st_cluster_v4(bhi_r[st][r] + oim, o[v].him);
                    st_cluster_v4(blo_r[st][r] + ore, o[v].lre);
                    st_cluster_v4(blo_r[st][r] + oim, o[v].lim);
                  }
                }
              }
            }
          }
          fence_proxy_async();
          __syncwarp();
          if (lane == 0) {
#pragma unroll
            for (int r = 0; r < CS; r++) mbar_arrive_cluster(full_r[st][r]);
          }
          warp_arrive(&vis_empty[slot]);
          const bool last = (n == nchunks - 1);
          const bool drain = last || ((n % p.slab) == p.slab - 1);
          const uint32_t my = nch;
          nch++;
          if (!drain || !drainer) continue;
          ok = warp_wait(&op_empty[my & 1], (my >> 1) & 1, abort, p.err, 3u);
          if (!ok) break;
          fence_after();
          // running sum += accumulator (short FP32 chains)
#pragma unroll 1
          for (int cb = 0; cb < kCols; cb += 32) {
            const uint32_t col = (uint32_t)(half * kCols + cb);
            float acc[32], run[32];
            tmem_ld32(t_acc + lane_off + col, acc);
            if (!run_empty) {
              tmem_ld32(t_run + lane_off + col, run);
#pragma unroll
              for (int k = 0; k < 32; k++) acc[k] += run[k];
            }
            tmem_st32(t_run + lane_off + col, acc);
          }
          run_empty = false;
          fence_before();
          warp_arrive(drained);
          if (last) {
            // channel epilogue: partial (+)= factor * running sum
#pragma unroll 1
            for (int cb = 0; cb < kCols; cb += 32) {
              const uint32_t col = (uint32_t)(half * kCols + cb);
              float run[32];
              tmem_ld32(t_run + lane_off + col, run);
#pragma unroll 4
              for (int k = 0; k < 32; k++) {
                const float f = epi_factor(p, c, ei, ej0 + cb + k, inv_s);
                const float v = f * run[k];
                if (first_channel)
                  prow[cb + k] = v;
                else
                  prow[cb + k] += v;
              }
            }
            first_channel = false;
          }
        }
      }
      if (ok && first_channel && drainer) {
        // no visibilities in this split for this tile: its partial is zero
        for (int k = 0; k < kCols; k++) prow[k] = 0.0f;
      }
    }
  }
  fence_before();
  __syncthreads();
  if (CS > 1) cluster_sync();  // no CTA leaves while a peer may still write into it
  fence_after();
  if (warp == 0) tmem_dealloc(tbase, kTmemCols);
}

// result[plane][q] += sum_s partial[s][q] (FP64, fixed order)
__global__ void k_reduce_partials(int64_t MN, int nsplit, const float* __restrict__ partial,
                                  float* __restrict__ out) {
  const int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (q >= MN) return;
  double s = 0.0;
  for (int k = 0; k < nsplit; k++) s += (double)partial[(int64_t)k * MN + q];
  out[q] += (float)s;
}

template <int TN, int CS, int VPL>
gv_status launch_tc(const Problem& P, const TcParams& p, int nitems) {
  auto kern = k_dchi2_tc<TN, CS, VPL>;
  const size_t smem = Layout<TN>::kSmem;
  GV_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  cudaLaunchConfig_t cfg = {};
  cudaLaunchAttribute attr[1];
  cfg.blockDim = dim3(threads_for(CS, VPL), 1, 1);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = P.stream;
  int nclusters = P.num_sms / CS;
  if (CS > 1) {
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = CS;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    cfg.gridDim = dim3(CS * nclusters, 1, 1);
    int active = 0;
    GV_CUDA(cudaOccupancyMaxActiveClusters(&active, kern, &cfg));
    if (active <= 0) {
      set_error("no cluster of the tensor-core DChi2 kernel fits on this device");
      return GV_ERR_UNSUPPORTED;
    }
    nclusters = std::min(nclusters, active);
  }
  nclusters = std::max(1, std::min(nclusters, nitems));
  cfg.gridDim = dim3(CS * nclusters, 1, 1);
  GV_CUDA(cudaLaunchKernelEx(&cfg, kern, p));
  GV_LAUNCH("k_dchi2_tc");
  return GV_OK;
}

}  // namespace tc

bool dchi2_tc_supported(const Problem& P) {
  return P.N >= 128 && P.N == P.M && P.max_wrho < 1e-7 && P.tc_partial != nullptr;
}

int tc_tile_n(const Problem& P) { return P.N >= 256 ? 256 : 128; }

// cluster size: the largest of 4, 2, 1 dividing the row tiles and the B atoms
int tc_cluster(const Problem& P) {
  const int TN = tc_tile_n(P);
  const int ntile_i = P.N / tc::kTM;
  // measured on GB300 (2048^2, 35.28M visibilities): 1 CTA 2.30 s, clusters
  // of 2 3.44 s, of 4 5.48 s -- the remote 16-byte stores of the shared B
  // tile cost more than the generation they save -- so clusters are opt-in
  int cs = 1;
  const char* env = std::getenv("GV_TC_CLUSTER");
  if (env) cs = std::atoi(env);
  while (cs > 1 && (ntile_i % cs != 0 || (TN / 64) % cs != 0 || (cs != 2 && cs != 4))) cs /= 2;
  return cs < 1 ? 1 : cs;
}

gv_status dchi2_tc(Problem& P, const float* d_img, int flag_opt, float* d_result,
                   int only_channel, int mode) {
  if (!dchi2_tc_supported(P)) {
    set_error("tensor-core DChi2 engine not supported for this problem");
    return GV_ERR_UNSUPPORTED;
  }
  tc::TcParams p;
  p.N = P.N;
  p.MN = (int64_t)P.M * P.N;
  p.x0 = (int)P.xobs;
  p.y0 = (int)P.yobs;
  p.xobs = P.xobs;
  p.yobs = P.yobs;
  p.nu_0 = P.nu_0;
  p.D = P.D;
  p.pbf = P.pbf;
  p.pbcut = P.pbcut;
  p.fg_scale = P.fg_scale;
  p.threshold = P.threshold;
  p.pb = P.pb;
  p.DELTAX = P.DELTAX;
  p.DELTAY = P.DELTAY;
  p.normalize = P.normalize;
  p.flag_opt = flag_opt;
  p.mode = mode;
  p.fast_anchor = P.tc_fast_anchor;
  {
    const char* sl = std::getenv("GV_TC_SLAB");
    p.slab = sl ? std::max(1, std::atoi(sl)) : tc::kSlab;
  }
  const int TN = tc_tile_n(P);
  const int CS = tc_cluster(P);
  p.ntile_i = P.N / tc::kTM;
  p.ntile_j = P.N / TN;
  p.nsplit = P.tc_nsplit;
  p.ranges = P.d_ranges;
  p.chfreq = P.d_chfreq;
  p.chnvis = P.d_chnvis;
  p.ph = P.d_ph;
  p.E = P.d_E;
  p.cvr = P.d_cvr;
  p.deg = P.d_deg;
  p.vo = P.d_vo;
  p.mask = P.d_mask;
  p.img = d_img;
  p.partial = P.tc_partial;
  p.err = P.d_flags + kFlagErr;
  p.cmax_bits = P.d_flags + (mode == 2 ? kFlagDirtyMax : kFlagCvrMax);
  if (only_channel >= 0) {
    p.C = 1;
    p.kc_off = P.d_kc_one + 2 * only_channel;
    p.ranges = P.d_ranges + only_channel;
    p.chfreq = P.d_chfreq + only_channel;
    p.chnvis = P.d_chnvis + only_channel;
    p.Ktot = P.chans[only_channel].ngrid;
  } else {
    p.C = (int)P.chans.size();
    p.kc_off = P.d_kc_off;
    p.Ktot = P.Vgrid;
  }
  const int nitems = (p.ntile_i / CS) * p.ntile_j * p.nsplit;
  // visibilities per generator lane (independent chains for ILP)
  int vpl = 2;
  if (const char* v = std::getenv("GV_TC_VPL")) vpl = std::atoi(v) == 1 ? 1 : 2;
  gv_status s;
  if (TN == 256) {
    if (CS == 4) s = tc::launch_tc<256, 4, 1>(P, p, nitems);
    else if (CS == 2) s = tc::launch_tc<256, 2, 1>(P, p, nitems);
    else if (vpl == 2) s = tc::launch_tc<256, 1, 2>(P, p, nitems);
    else s = tc::launch_tc<256, 1, 1>(P, p, nitems);
  } else {
    if (CS == 2) s = tc::launch_tc<128, 2, 1>(P, p, nitems);
    else if (vpl == 2) s = tc::launch_tc<128, 1, 2>(P, p, nitems);
    else s = tc::launch_tc<128, 1, 1>(P, p, nitems);
  }
  if (s != GV_OK) return s;
  float* out = d_result + (mode == 0 ? (int64_t)(flag_opt % 2) * p.MN : 0);
  tc::k_reduce_partials<<<(unsigned)((p.MN + 255) / 256), 256, 0, P.stream>>>(
      p.MN, p.nsplit, P.tc_partial, out);
  GV_LAUNCH("k_reduce_partials");
  return GV_OK;
}

}  // namespace gv
