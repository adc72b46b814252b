// SPDX-License-Identifier: MPL-2.0
// BF16 tensor-core mean-shift bulk iterations on sm_103a (tcgen05 + TMEM).
//
// Flash-style: per (tile of 128 seeds, chunk of 128 votes)
//   MMA1  D[128x128] = S'[128x16] . X'[128x16]^T      (seed-vote dot products)
//   epilogue: tcgen05.ld D, w = max(0, 1 - (|s'|^2 + |x'|^2 - 2 s'.x') / h^2)
//             (Epanechnikov, packed FP32 FMAs), written as BF16 into shared
//             memory
//   MMA2  ACC[128x32] += W[128x128] . [x_hi, 1, x_lo][128x32]
// S' and X' are centred on the chunk's centre c (X' once per vote set, S' per
// chunk), which keeps |s'|, |x'| small so the expanded distance does not lose
// its digits in BF16; MMA2 uses the uncentred x split into a BF16 value and
// its BF16 residue, plus a ones column, so sum w x and sum w come out of TMEM.
// Votes are pre-arranged per chunk in the canonical no-swizzle K-major
// core-matrix layout (8 rows x 16 bytes per core matrix), so one TMA bulk copy
// (cp.async.bulk + mbarrier complete_tx) stages a chunk.  Accumulators live
// in TMEM (256 columns per CTA: D at 0..127, ACC at 128..143).  Every
// mbarrier wait is bounded; on timeout the CTA records a status, drains and
// frees its TMEM.
#include "meanshift_fast.cuh"
#include "primitives.cuh"

#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <vector>

namespace sym {
namespace {

// --------------------------------------------------------------- PTX glue
__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

constexpr uint32_t kSpinLimit = 1u << 24;

// Bounded wait: false when the barrier phase never completed.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity) {
  for (uint32_t i = 0; i < kSpinLimit; ++i)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}

__device__ __forceinline__ void tma_bulk_load(void *dst, const void *src, uint32_t bytes,
                                              uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ void fence_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

// Whole warp: allocate `cols` TMEM columns, address written to shared memory.
__device__ __forceinline__ void tmem_alloc(uint32_t *dst, uint32_t cols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                   smem_u32(dst)),
               "r"(cols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t cols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(cols)
               : "memory");
}

// Shared-memory matrix descriptor (sm_100 family): start address, leading
// (K-direction core-matrix) byte offset, stride (M/N-direction 8-row group)
// byte offset, descriptor version 1, no swizzle.
__device__ __forceinline__ uint64_t smem_desc(const void *p, uint32_t lbo, uint32_t sbo) {
  uint64_t d = (uint64_t(smem_u32(p)) >> 4) & 0x3FFFull;
  d |= uint64_t((lbo >> 4) & 0x3FFFu) << 16;
  d |= uint64_t((sbo >> 4) & 0x3FFFu) << 32;
  d |= uint64_t(1) << 46;
  return d;
}

// Instruction descriptor of kind::f16: F32 accumulator, BF16 A and B, both
// K-major, N >> 3 at bit 17, M >> 4 at bit 24.
__host__ __device__ constexpr uint32_t idesc_bf16(uint32_t m, uint32_t n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((n >> 3) << 17) | ((m >> 4) << 24);
}

__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc,
                                         uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
      "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
      : "memory");
}

__device__ __forceinline__ void mma_commit(uint64_t *bar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
          smem_u32(bar))
      : "memory");
}

// 32 consecutive FP32 columns of this thread's TMEM lane.
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32]) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
      "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
      "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]),
        "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]),
        "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
  for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

// ------------------------------------------------------------- layouts
// Canonical no-swizzle K-major tile of 16-bit elements: core matrices of 8
// rows x 8 elements (16 bytes per row), `lbo` bytes between K-adjacent core
// matrices, `sbo` bytes between row groups.
__host__ __device__ constexpr uint32_t kmajor_offset(uint32_t row, uint32_t k, uint32_t lbo,
                                                     uint32_t sbo) {
  return (row / 8) * sbo + (k / 8) * lbo + (row % 8) * 16 + (k % 8) * 2;
}

// Chunk image (one TMA bulk copy):
//   B1   X' = x - c as 128 votes x 16 features, K-major (LBO 128, SBO 256)
//   B2   32 "features" x 128 votes, K-major (LBO 128, SBO 2048): rows 0..5
//        BF16(x), row 6 ones, rows 16..21 the BF16 rounding residue of x;
//        MMA2 then yields sum w x (hi + lo) and sum w directly in TMEM
//   XX   |x'|^2 of the rounded X' (128 floats; far away for padding votes)
//   CEN  the chunk centre c (8 floats)
constexpr uint32_t kB1Bytes = 4096, kB2Bytes = 8192, kXXBytes = 512, kCenBytes = 32;
constexpr uint32_t kImage = kB1Bytes + kB2Bytes + kXXBytes + kCenBytes;  // 12832
static_assert(kImage % 16 == 0, "TMA bulk copies move multiples of 16 bytes");

__global__ void build_images(const float *desc, uint64_t q, uint64_t nchunks, const float *cbox,
                             uint8_t *images) {
  uint64_t c = blockIdx.x;
  int t = threadIdx.x;  // vote in chunk
  if (c >= nchunks) return;
  const float *b = cbox + c * 12;
  float cen[6];
  for (int d = 0; d < 6; ++d) cen[d] = 0.5f * (b[d] + b[6 + d]);
  uint64_t v = c * kChunk + t;
  bool live = v < q;
  uint8_t *img = images + c * kImage;
  __nv_bfloat16 *b1 = reinterpret_cast<__nv_bfloat16 *>(img);
  __nv_bfloat16 *b2 = reinterpret_cast<__nv_bfloat16 *>(img + kB1Bytes);
  float *xx = reinterpret_cast<float *>(img + kB1Bytes + kB2Bytes);
  float *ce = reinterpret_cast<float *>(img + kB1Bytes + kB2Bytes + kXXBytes);
  if (t < 8) ce[t] = t < 6 ? cen[t] : 0.f;
  float n2 = 0;
  for (int k = 0; k < 16; ++k) {
    float x = live && k < 6 ? desc[v * 8 + k] - cen[k] : 0.f;
    __nv_bfloat16 h = __float2bfloat16_rn(x);
    float r = __bfloat162float(h);
    n2 += r * r;
    b1[kmajor_offset(t, k, 128, 256) / 2] = h;
  }
  for (int k = 0; k < 32; ++k) {
    float val = 0.f;
    if (live && k < 6) {
      val = desc[v * 8 + k];
    } else if (live && k == 6) {
      val = 1.f;
    } else if (live && k >= 16 && k < 22) {
      float x = desc[v * 8 + (k - 16)];
      val = x - __bfloat162float(__float2bfloat16_rn(x));
    }
    b2[kmajor_offset(k, t, 128, 2048) / 2] = __float2bfloat16_rn(val);
  }
  xx[t] = live ? n2 : 1e30f;  // padding votes sit infinitely far away
}

// Shared-memory plan of the self-test (one tile, one stage, N = 16 MMA2).
constexpr uint32_t kSelfB2 = 4096;
constexpr uint32_t kOffA1 = 0, kOffA2 = 4096, kOffStage = 4096 + 32768;
constexpr uint32_t kOffBars = kOffStage + 2 * 8704;
constexpr uint32_t kOffMisc = kOffBars + 64;
constexpr uint32_t kSmemRequest = 100 * 1024;
constexpr uint32_t kTmemCols = 256, kColD = 0, kColAcc = 128;

__device__ __forceinline__ float box_gap2_tc(const float *lo, const float *hi, const float *b) {
  float g = 0;
  for (int k = 0; k < 6; ++k) {
    float d = fmaxf(fmaxf(b[k] - hi[k], lo[k] - b[6 + k]), 0.f);
    g += d * d;
  }
  return g;
}

// ------------------------------------------------- work lists per tile
// Box of each tile's active seeds (one block of kChunk threads per tile).
__global__ void tile_boxes(const float *means, const int32_t *ids, uint64_t nactive, float *boxes) {
  __shared__ float part[4][12];
  uint64_t slot = uint64_t(blockIdx.x) * kChunk + threadIdx.x;
  bool live = slot < nactive;
  float lo[6], hi[6];
  for (int d = 0; d < 6; ++d) {
    float m = live ? means[uint64_t(ids[slot]) * 8 + d] : 0.f;
    lo[d] = live ? m : INFINITY, hi[d] = live ? m : -INFINITY;
  }
  for (int o = 16; o; o >>= 1)
    for (int d = 0; d < 6; ++d) {
      lo[d] = fminf(lo[d], __shfl_xor_sync(0xffffffffu, lo[d], o));
      hi[d] = fmaxf(hi[d], __shfl_xor_sync(0xffffffffu, hi[d], o));
    }
  int warp = threadIdx.x >> 5;
  if ((threadIdx.x & 31) == 0)
    for (int d = 0; d < 6; ++d) part[warp][d] = lo[d], part[warp][6 + d] = hi[d];
  __syncthreads();
  if (threadIdx.x < 12) {
    float v = part[0][threadIdx.x];
    for (int w = 1; w < 4; ++w)
      v = threadIdx.x < 6 ? fminf(v, part[w][threadIdx.x]) : fmaxf(v, part[w][threadIdx.x]);
    boxes[blockIdx.x * 12 + threadIdx.x] = v;
  }
}

// need[t * nchunks + c]: chunk c lies within the bandwidth of tile t's box.
__global__ void tile_needs(const float *boxes, const float *cbox, uint64_t nchunks, float skip_gap2,
                           uint8_t *need) {
  uint64_t c = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  uint64_t t = blockIdx.y;
  if (c >= nchunks) return;
  const float *tb = boxes + t * 12;
  need[t * nchunks + c] = box_gap2_tc(tb, tb + 6, cbox + c * 12) <= skip_gap2;
}

// offsets[t] = first list entry of tile t (entries are t * nchunks + c,
// ascending); offsets[tiles] = list length.
__global__ void tile_offsets(const int32_t *list, const uint64_t *count, uint64_t tiles,
                             uint64_t nchunks, uint64_t *offsets) {
  uint64_t t = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (t > tiles) return;
  uint64_t n = *count;
  if (t == tiles) {
    offsets[t] = n;
    return;
  }
  uint64_t key = t * nchunks, lo = 0, hi = n;
  while (lo < hi) {
    uint64_t mid = (lo + hi) / 2;
    if (uint64_t(list[mid]) < key) lo = mid + 1;
    else hi = mid;
  }
  offsets[t] = lo;
}

// --------------------------------------------- pipelined tensor kernel
// Warp roles: warps 0..15 form four epilogue warpgroups (warpgroup g owns
// D columns 32g..32g+31 of every row; warp w reads TMEM lanes 32(w%4)..),
// warp 16 is the producer (TMA, A1 staging, MMA issue).
//   stages   3 TMA buffers of one chunk image each
//   D[2]     two TMEM accumulators for MMA1 (columns 0..127, 128..255)
//   ACC      TMEM columns 256..271
//   A1[2]    seeds centred on the chunk, A2[2] BF16 weights
// Handshakes (mbarriers): load_full[s] (TMA bytes), d_full[b] (MMA1 done),
// d_free[b] (epilogue read D[b]), a2_full[b] (epilogue wrote A2[b]),
// a2_free[b] and stage_free[s] (MMA2 done), acc_done.
constexpr int kStages = 3;
constexpr int kEpiWarps = 16, kThreads2 = (kEpiWarps + 1) * 32;
constexpr uint32_t kT2A1 = 0;                                 // 2 x 4096
constexpr uint32_t kT2A2 = 8192;                              // 2 x 32768
constexpr uint32_t kT2Stage = kT2A2 + 2 * 32768;              // 3 x kImage
constexpr uint32_t kT2Bars = kT2Stage + kStages * kImage;     // 15 barriers
constexpr uint32_t kT2Misc = kT2Bars + 16 * 8;
constexpr uint32_t kT2Seeds = kT2Misc + 64;                   // 128 x 8 floats
constexpr uint32_t kT2Smem = kT2Seeds + 128 * 8 * 4;
static_assert(kT2Stage % 128 == 0 && (kT2Stage + kImage) % 16 == 0, "TMA alignment");
constexpr uint32_t kT2Cols = 512, kT2ColAcc = 256;

struct Tc2Args {
  const uint8_t *images;
  uint64_t nchunks;
  const int32_t *list;      // needed (tile, chunk) entries, t * nchunks + c
  const uint64_t *offsets;  // tiles + 1
  uint64_t splits;
  const float *means;
  const int32_t *ids;
  uint64_t nactive;
  float inv_h2;
  float *partial;
  unsigned long long *evals;
  int *status;
};

__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

// d = a * b + c on two FP32 lanes at once.
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) {
  unsigned long long ra, rb, rc, rd;
  memcpy(&ra, &a, 8), memcpy(&rb, &b, 8), memcpy(&rc, &c, 8);
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(rd) : "l"(ra), "l"(rb), "l"(rc));
  float2 d;
  memcpy(&d, &rd, 8);
  return d;
}

__global__ void __launch_bounds__(kThreads2, 1) ms_tile_tc2(Tc2Args a) {
  extern __shared__ __align__(1024) uint8_t smem[];
  uint8_t *A1 = smem + kT2A1, *A2 = smem + kT2A2, *stage = smem + kT2Stage;
  uint64_t *bars = reinterpret_cast<uint64_t *>(smem + kT2Bars);
  uint64_t *load_full = bars, *stage_free = bars + 3, *d_full = bars + 6, *d_free = bars + 8;
  uint64_t *a2_full = bars + 10, *a2_free = bars + 12, *acc_done = bars + 14;
  uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(smem + kT2Misc);
  float *seeds = reinterpret_cast<float *>(smem + kT2Seeds);

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const uint64_t tile = blockIdx.x, split = blockIdx.y;
  const uint64_t slots = uint64_t(gridDim.x) * kChunk;
  const uint64_t lt0 = a.offsets[tile], lt1 = a.offsets[tile + 1], len = lt1 - lt0;
  const uint64_t e0 = lt0 + len * split / a.splits, e1 = lt0 + len * (split + 1) / a.splits;
  const uint32_t n = uint32_t(e1 - e0);
  const uint64_t tbase = tile * a.nchunks;

  if (tid < kChunk) {  // seed means of the tile -> shared memory
    uint64_t slot = tile * kChunk + tid;
    bool live = slot < a.nactive;
    int32_t sd = live ? a.ids[slot] : 0;
    for (int d = 0; d < 8; ++d) seeds[tid * 8 + d] = live && d < 6 ? a.means[uint64_t(sd) * 8 + d] : 0.f;
  }
  if (tid == 0) {
    for (int s = 0; s < kStages; ++s) mbar_init(&load_full[s], 1), mbar_init(&stage_free[s], 1);
    for (int b = 0; b < 2; ++b) {
      mbar_init(&d_full[b], 1);
      mbar_init(&d_free[b], kEpiWarps);
      mbar_init(&a2_full[b], kEpiWarps);
      mbar_init(&a2_free[b], 1);
    }
    mbar_init(acc_done, 1);
    fence_mbar_init();
  }
  if (warp == 0 && n) tmem_alloc(tmem_slot, kT2Cols);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = n ? *tmem_slot : 0;
  bool ok = true;

  if (warp == kEpiWarps) {
    // ------------------------------------------------------- producer
    auto chunk_of = [&](uint32_t i) { return uint64_t(a.list[e0 + i]) - tbase; };
    for (uint32_t i = 0; i < n && i < uint32_t(kStages); ++i)
      if (lane == 0) {
        mbar_expect_tx(&load_full[i], kImage);
        tma_bulk_load(stage + i * kImage, a.images + chunk_of(i) * kImage, kImage, &load_full[i]);
      }
    for (uint32_t i = 0; i < n && ok; ++i) {
      const uint32_t b = i & 1, s = i % kStages;
      ok = mbar_wait(&load_full[s], (i / kStages) & 1);
      if (ok && i >= 2) ok = mbar_wait(&d_full[b], ((i - 2) / 2) & 1);  // MMA1(i-2) released A1[b]
      if (!ok) break;
      const float *cen = reinterpret_cast<const float *>(stage + s * kImage + kB1Bytes + kB2Bytes + kXXBytes);
      for (int r = lane; r < kChunk; r += 32) {  // A1[b]: seeds centred on the chunk, BF16
        __align__(16) __nv_bfloat16 h[16];
        for (int k = 0; k < 16; ++k)
          h[k] = __float2bfloat16_rn(k < 6 ? seeds[r * 8 + k] - cen[k] : 0.f);
        uint8_t *dst = A1 + b * 4096;
        *reinterpret_cast<uint4 *>(dst + kmajor_offset(r, 0, 128, 256)) = *reinterpret_cast<uint4 *>(&h[0]);
        *reinterpret_cast<uint4 *>(dst + kmajor_offset(r, 8, 128, 256)) = *reinterpret_cast<uint4 *>(&h[8]);
      }
      fence_async_smem();
      __syncwarp();
      if (i >= 2) ok = mbar_wait(&d_free[b], ((i - 2) / 2) & 1);  // epilogue read D[b]
      if (!ok) break;
      tc_fence_after();
      if (lane == 0) {
        mma_bf16(tmem + 128 * b, smem_desc(A1 + b * 4096, 128, 256),
                 smem_desc(stage + s * kImage, 128, 256), idesc_bf16(128, 128), 0);
        mma_commit(&d_full[b]);
      }
      if (i >= 1) {  // MMA2 of the previous chunk, then refill its stage
        const uint32_t j = i - 1, bj = j & 1, sj = j % kStages;
        ok = mbar_wait(&a2_full[bj], (j / 2) & 1);
        if (!ok) break;
        tc_fence_after();
        if (lane == 0) {
          for (uint32_t q = 0; q < 8; ++q)
            mma_bf16(tmem + kT2ColAcc, smem_desc(A2 + bj * 32768 + q * 256, 128, 2048),
                     smem_desc(stage + sj * kImage + kB1Bytes + q * 256, 128, 2048),
                     idesc_bf16(128, 32), (j > 0 || q > 0) ? 1u : 0u);
          mma_commit(&a2_free[bj]);
          mma_commit(&stage_free[sj]);
        }
        if (j + kStages < n) {
          ok = mbar_wait(&stage_free[sj], (j / kStages) & 1);
          if (!ok) break;
          if (lane == 0) {
            mbar_expect_tx(&load_full[sj], kImage);
            tma_bulk_load(stage + sj * kImage, a.images + chunk_of(j + kStages) * kImage, kImage,
                          &load_full[sj]);
          }
        }
      }
    }
    if (ok && n) {  // last MMA2
      const uint32_t j = n - 1, bj = j & 1, sj = j % kStages;
      ok = mbar_wait(&a2_full[bj], (j / 2) & 1);
      tc_fence_after();
      if (ok && lane == 0) {
        for (uint32_t q = 0; q < 8; ++q)
          mma_bf16(tmem + kT2ColAcc, smem_desc(A2 + bj * 32768 + q * 256, 128, 2048),
                   smem_desc(stage + sj * kImage + kB1Bytes + q * 256, 128, 2048),
                   idesc_bf16(128, 32), (j > 0 || q > 0) ? 1u : 0u);
        mma_commit(acc_done);
      }
    }
    if (!ok && lane == 0) {
      atomicExch(a.status, DS_SPIN_LIMIT);
      mbar_arrive(acc_done);  // release the epilogue
    }
  } else {
    // ------------------------------------------------------- epilogue
    // warpgroup g owns D columns 32g..32g+31; the weights are
    // w = max(0, 1 - (|s'|^2 + |x'|^2 - 2 s'.x') / h^2)
    const int quad = warp & 3, g = warp >> 2, row = quad * 32 + lane;
    float m[6];
    for (int d = 0; d < 6; ++d) m[d] = seeds[row * 8 + d];
    const float2 two_inv_h2 = make_float2(2.f * a.inv_h2, 2.f * a.inv_h2);
    const float2 neg_inv_h2 = make_float2(-a.inv_h2, -a.inv_h2);
    for (uint32_t i = 0; i < n; ++i) {
      const uint32_t b = i & 1, s = i % kStages;
      if (!mbar_wait(&load_full[s], (i / kStages) & 1) || !mbar_wait(&d_full[b], (i / 2) & 1)) {
        ok = false;
        break;
      }
      tc_fence_after();
      float dot[32];
      tmem_ld32(tmem + (uint32_t(quad * 32) << 16) + 128 * b + 32 * g, dot);
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(&d_free[b]);
      const uint8_t *st_s = stage + s * kImage;
      const float *cen = reinterpret_cast<const float *>(st_s + kB1Bytes + kB2Bytes + kXXBytes);
      float ss = 0;
      for (int d = 0; d < 6; ++d) {
        float r = __bfloat162float(__float2bfloat16_rn(m[d] - cen[d]));
        ss = fmaf(r, r, ss);
      }
      const float rowc = 1.f - ss * a.inv_h2;
      const float2 rowc2 = make_float2(rowc, rowc);
      const float4 *xx4 = reinterpret_cast<const float4 *>(st_s + kB1Bytes + kB2Bytes) + 8 * g;
      __align__(16) __nv_bfloat162 w[16];
      for (int j4 = 0; j4 < 8; ++j4) {
        float4 x = xx4[j4];
        float2 t0 = fma2(make_float2(dot[4 * j4], dot[4 * j4 + 1]), two_inv_h2,
                         fma2(make_float2(x.x, x.y), neg_inv_h2, rowc2));
        float2 t1 = fma2(make_float2(dot[4 * j4 + 2], dot[4 * j4 + 3]), two_inv_h2,
                         fma2(make_float2(x.z, x.w), neg_inv_h2, rowc2));
        w[2 * j4] = __floats2bfloat162_rn(fmaxf(t0.x, 0.f), fmaxf(t0.y, 0.f));
        w[2 * j4 + 1] = __floats2bfloat162_rn(fmaxf(t1.x, 0.f), fmaxf(t1.y, 0.f));
      }
      if (i >= 2 && !mbar_wait(&a2_free[b], ((i - 2) / 2) & 1)) {
        ok = false;
        break;
      }
      uint8_t *dst = A2 + b * 32768;
      for (int kb = 0; kb < 4; ++kb)
        *reinterpret_cast<uint4 *>(dst + kmajor_offset(row, 32 * g + 8 * kb, 128, 2048)) =
            *reinterpret_cast<uint4 *>(&w[4 * kb]);
      fence_async_smem();
      __syncwarp();
      if (lane == 0) mbar_arrive(&a2_full[b]);
    }
    if (!ok && lane == 0) atomicExch(a.status, DS_SPIN_LIMIT);
  }
  __syncthreads();
  if (warp < 4) {  // warpgroup 0 writes the tile's partial sums
    const int quad = warp & 3, row = quad * 32 + lane;
    float acc[32];
    for (int j = 0; j < 32; ++j) acc[j] = 0.f;
    if (n && mbar_wait(acc_done, 0)) {
      tc_fence_after();
      tmem_ld32(tmem + (uint32_t(quad * 32) << 16) + kT2ColAcc, acc);
    }
    float *out = a.partial + (split * slots + tile * kChunk + row) * 8;
    for (int d = 0; d < 6; ++d) out[d] = acc[d] + acc[16 + d];  // BF16 x + its residue
    out[6] = acc[6];
    out[7] = 0.f;
  }
  if (tid == 0 && n && a.evals) atomicAdd(a.evals, uint64_t(n) * uint64_t(kChunk * kChunk));
  tc_fence_before();
  __syncthreads();
  if (warp == 0 && n) tmem_dealloc(tmem, kT2Cols);
}

// ------------------------------------------------------ tensor self-test
// One tile: D = A1 . B1^T (128 x 128 x 16) and ACC = A2 . B2^T (128 x 16 x
// 128) from row-major BF16 inputs, through the same layouts, TMA, MMA and
// TMEM path as ms_tile_tc.
__global__ void __launch_bounds__(256, 1) tc_selftest(const __nv_bfloat16 *a1, const __nv_bfloat16 *b1,
                                                      const __nv_bfloat16 *a2, const __nv_bfloat16 *b2,
                                                      uint8_t *scratch, float *d_out, float *acc_out,
                                                      int *status) {
  extern __shared__ __align__(1024) uint8_t smem[];
  uint8_t *A1 = smem + kOffA1, *A2 = smem + kOffA2, *S = smem + kOffStage;
  uint64_t *bar = reinterpret_cast<uint64_t *>(smem + kOffBars);
  uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(smem + kOffMisc);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31, quad = warp & 3, wg = warp >> 2;
  const int row = quad * 32 + lane;
  // stage B1 | B2 in global scratch in the canonical layout, then TMA it in
  if (tid < 128) {
    __nv_bfloat16 *g1 = reinterpret_cast<__nv_bfloat16 *>(scratch);
    __nv_bfloat16 *g2 = reinterpret_cast<__nv_bfloat16 *>(scratch + kB1Bytes);
    for (int k = 0; k < 16; ++k) {
      g1[kmajor_offset(tid, k, 128, 256) / 2] = b1[tid * 16 + k];
      g2[kmajor_offset(k, tid, 128, 2048) / 2] = b2[k * 128 + tid];
    }
    __nv_bfloat16 *s1 = reinterpret_cast<__nv_bfloat16 *>(A1);
    __nv_bfloat16 *s2 = reinterpret_cast<__nv_bfloat16 *>(A2);
    for (int k = 0; k < 16; ++k) s1[kmajor_offset(tid, k, 128, 256) / 2] = a1[tid * 16 + k];
    for (int k = 0; k < 128; ++k) s2[kmajor_offset(tid, k, 128, 2048) / 2] = a2[tid * 128 + k];
    asm volatile("fence.proxy.async.global;" ::: "memory");
  }
  if (tid == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    fence_mbar_init();
  }
  if (warp == 0) tmem_alloc(tmem_slot, kTmemCols);
  __threadfence();
  fence_async_smem();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;
  bool ok = true;
  if (tid == 0) {
    asm volatile("fence.proxy.async.global;" ::: "memory");
    mbar_expect_tx(&bar[0], kB1Bytes + kSelfB2);
    tma_bulk_load(S, scratch, kB1Bytes + kSelfB2, &bar[0]);
  }
  ok = __syncthreads_and(mbar_wait(&bar[0], 0));
  if (ok && tid == 0) {
    mma_bf16(tmem + kColD, smem_desc(A1, 128, 256), smem_desc(S, 128, 256), idesc_bf16(128, 128), 0);
    for (uint32_t s = 0; s < 8; ++s)
      mma_bf16(tmem + kColAcc, smem_desc(A2 + s * 256, 128, 2048),
               smem_desc(S + kB1Bytes + s * 256, 128, 2048), idesc_bf16(128, 16), s > 0);
    mma_commit(&bar[1]);
  }
  if (ok) ok = __syncthreads_and(mbar_wait(&bar[1], 0));
  tc_fence_after();
  if (ok) {
    for (int half = 0; half < 2; ++half) {
      float v[32];
      uint32_t col = 64 * wg + 32 * half;
      tmem_ld32(tmem + (uint32_t(quad * 32) << 16) + kColD + col, v);
      for (int j = 0; j < 32; ++j) d_out[row * 128 + col + j] = v[j];
    }
    if (wg == 0) {
      float v[32];
      tmem_ld32(tmem + (uint32_t(quad * 32) << 16) + kColAcc, v);
      for (int j = 0; j < 16; ++j) acc_out[row * 16 + j] = v[j];
    }
  }
  if (!ok && tid == 0) atomicExch(status, DS_SPIN_LIMIT);
  tc_fence_before();
  __syncthreads();
  if (warp == 0) tmem_dealloc(tmem, kTmemCols);
}

__global__ void ms_update_bulk(float *means, const float *partial, uint64_t splits, uint64_t slots,
                               const int32_t *ids, uint64_t nactive, float h2, float stop,
                               uint8_t *state) {
  uint64_t slot = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (slot >= nactive) return;
  int32_t s = ids[slot];
  float acc[7] = {0, 0, 0, 0, 0, 0, 0};
  for (uint64_t p = 0; p < splits; ++p)
    for (int d = 0; d < 7; ++d) acc[d] += partial[(p * slots + slot) * 8 + d];
  if (acc[6] <= 1e-14f) {
    state[s] = 2;
    return;
  }
  float move = 0;
  for (int d = 0; d < 6; ++d) {
    float nx = acc[d] / acc[6];
    float e = means[uint64_t(s) * 8 + d] - nx;
    move += e * e;
    means[uint64_t(s) * 8 + d] = nx;
  }
  if (move < stop * h2) state[s] = 1;
}

}  // namespace

// Active-seed list as in the SIMT path (meanshift_fast.cu).
unsigned active_seeds(Call &call, const VoteSet &v, const float *means, const uint8_t *state,
                      uint64_t k, int32_t *ids);

bool meanshift_bf16_bulk(Call &call, const VoteSet &v, float *means, uint8_t *state, uint64_t k,
                         double h2, int max_iter, int *iterations, double *evaluations,
                         uint32_t *trace, int trace_len) {
  *iterations = 0;
  *evaluations = 0;
  if (!k || !v.q) return false;
  const uint64_t max_tiles = (k + kChunk - 1) / kChunk;
  if (max_tiles * v.nchunks >= (uint64_t(1) << 31)) return false;  // list entries are int32
  cudaStream_t st = call.stream();
  static bool configured = false;
  if (!configured) {
    SYM_CUDA(cudaFuncSetAttribute(ms_tile_tc2, cudaFuncAttributeMaxDynamicSharedMemorySize, kT2Smem));
    configured = true;
  }
  uint8_t *images = call.alloc<uint8_t>(v.nchunks * kImage);
  build_images<<<unsigned(v.nchunks), kChunk, 0, st>>>(v.desc, v.q, v.nchunks, v.cbox, images);
  check_launch();
  int32_t *ids = call.alloc<int32_t>(k);
  float *boxes = call.alloc<float>(max_tiles * 12);
  uint8_t *need = call.alloc<uint8_t>(max_tiles * v.nchunks);
  int32_t *list = call.alloc<int32_t>(max_tiles * v.nchunks);
  uint64_t *count = call.alloc<uint64_t>(1), *offsets = call.alloc<uint64_t>(max_tiles + 1);
  const uint64_t max_splits = 152;
  float *partial = call.alloc<float>(max_splits * max_tiles * kChunk * 8);
  unsigned long long *evals = call.alloc<unsigned long long>(1);
  SYM_CUDA(cudaMemsetAsync(evals, 0, 8, st));
  float gap = float(std::sqrt(h2)) + 1e-6f;
  call.launched();
  int it = 0;
  for (; it < max_iter; ++it) {
    unsigned n = active_seeds(call, v, means, state, k, ids);
    if (!n) break;
    if (trace && it < trace_len) trace[it] = n;
    const uint64_t tiles = (n + kChunk - 1) / kChunk;
    const uint64_t splits = std::max<uint64_t>(1, max_splits / tiles);
    auto mark = call.ctx->arena.mark();
    tile_boxes<<<unsigned(tiles), kChunk, 0, st>>>(means, ids, n, boxes);
    check_launch();
    tile_needs<<<dim3(blocks_for(v.nchunks), unsigned(tiles)), kThreads, 0, st>>>(
        boxes, v.cbox, v.nchunks, gap * gap, need);
    check_launch();
    compact_indices(call, need, tiles * v.nchunks, list, count);
    tile_offsets<<<blocks_for(tiles + 1), kThreads, 0, st>>>(list, count, tiles, v.nchunks, offsets);
    check_launch();
    Tc2Args args{images, v.nchunks, list, offsets, splits, means, ids, n,
                 float(1.0 / h2), partial, evals, call.status()};
    ms_tile_tc2<<<dim3(unsigned(tiles), unsigned(splits)), kThreads2, kT2Smem, st>>>(args);
    check_launch();
    ms_update_bulk<<<blocks_for(n), kThreads, 0, st>>>(means, partial, splits, tiles * kChunk, ids,
                                                       n, float(h2), 1e-5f, state);
    check_launch();
    call.launched(5);
    call.ctx->arena.rewind(mark);
  }
  call.check_status("mean_shift (tensor)");
  unsigned long long ev = 0;
  call.d2h(&ev, evals, 8);
  call.sync();
  *iterations = it;
  *evaluations = double(ev);
  return true;
}

void tc_selftest_host(Call &call, const uint16_t *a1, const uint16_t *b1, const uint16_t *a2,
                      const uint16_t *b2, float *d_out, float *acc_out) {
  static bool configured = false;
  if (!configured) {
    SYM_CUDA(cudaFuncSetAttribute(tc_selftest, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  kSmemRequest));
    configured = true;
  }
  auto up = [&](const uint16_t *p, size_t n) {
    return reinterpret_cast<const __nv_bfloat16 *>(call.upload(p, n));
  };
  const __nv_bfloat16 *da1 = up(a1, 128 * 16), *db1 = up(b1, 128 * 16), *da2 = up(a2, 128 * 128),
                      *db2 = up(b2, 16 * 128);
  uint8_t *scratch = call.alloc<uint8_t>(kB1Bytes + kSelfB2);
  float *dd = call.alloc<float>(128 * 128), *dacc = call.alloc<float>(128 * 16);
  tc_selftest<<<1, 256, kSmemRequest, call.stream()>>>(da1, db1, da2, db2, scratch, dd, dacc,
                                                       call.status());
  check_launch();
  call.launched();
  call.d2h(d_out, dd, 128 * 128 * 4);
  call.d2h(acc_out, dacc, 128 * 16 * 4);
  call.check_status("tensor self-test");
}

}  // namespace sym
