// SPDX-License-Identifier: MPL-2.0
// BF16 tensor-core mean-shift bulk iterations on sm_103a (tcgen05 + TMEM).
//
// Flash-style, per (tile of 128 seeds, chunk of 128 votes), in units of the
// bandwidth h with the vote set's centre c_g and the chunk centre c_c:
//   u = (s - c_g)/h per seed, as a BF16 value + residue (once per tile)
//   E = (c_c - c_g)/h per chunk, v = (x - c_c)/h per vote, and the per-vote
//       constant f = -2 E.v as a BF16 value + residue (the chunk image)
//   MMA1  D[128x128] = [2u_hi, 1, 1 | 2u_lo, 1, 1] . [v, -|v|^2 | v, f]^T
//                    = 2 (u - E).v - |v|^2                 (tcgen05.mma K=16)
//   epilogue: w = relu(D + 1 - |u - E|^2) = max(0, 1 - |s - x|^2/h^2),
//           one packed FP32 add and one cvt.rn.relu.bf16x2 per two weights,
//           written as BF16 into shared memory
//   MMA2  ACC[128x16] += W[128x128] . [x_hi, 1, 0, x_lo]  (sum w x, sum w)
// The seed offsets are represented to ~2^-17 by their BF16 pairs and the
// epilogue uses the same represented values, so the large offsets cancel
// exactly; v is chunk-relative (small) and rounds once.  MMA2 uses the
// uncentred x split into BF16 value and residue plus a ones column, so sum
// w x and sum w come out of TMEM directly.
// The chunk image is laid out in the canonical no-swizzle K-major
// core-matrix order (8 rows x 16 bytes per core matrix), so one TMA bulk copy
// (cp.async.bulk + mbarrier complete_tx) stages a chunk.  Every mbarrier wait
// is bounded; on timeout the CTA records a status, drains its copies and
// MMAs, and frees its TMEM.
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

// A waiting thread is suspended by the hardware until the phase completes
// (or kSuspendNs pass), so waiting warps take no issue slots from the
// working ones.
constexpr uint32_t kSuspendNs = 20000;
constexpr uint64_t kWaitLimitNs = 2000000000ull;  // a wait gives up after 2 s

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity), "r"(kSuspendNs)
      : "memory");
  return ok != 0;
}

__device__ __forceinline__ uint64_t global_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Bounded wait: false when the barrier phase did not complete within
// limit_ns.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity,
                                          uint64_t limit_ns = kWaitLimitNs) {
  if (mbar_try_wait(bar, parity)) return true;
  const uint64_t t0 = global_ns();
  do {
    if (mbar_try_wait(bar, parity)) return true;
  } while (global_ns() - t0 < limit_ns);
  return false;
}

// Bounded wait whose outcome is the same in every lane of the warp (each
// lane polls, so each performs the acquire; all agree on success).
__device__ __forceinline__ bool warp_wait(uint64_t *bar, uint32_t parity) {
  return __all_sync(0xffffffffu, mbar_wait(bar, parity));
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

// Same, with the A operand (M x 16 BF16) read from TMEM at column a_tmem:
// row m in lane m, two K-consecutive elements per 32-bit column (the lower
// K index in the low half).
__device__ __forceinline__ void mma_bf16_ts(uint32_t d_tmem, uint32_t a_tmem, uint64_t b,
                                            uint32_t idesc, uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], [%1], %2, %3, p;\n\t}" ::"r"(d_tmem),
      "r"(a_tmem), "l"(b), "r"(idesc), "r"(accumulate)
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

// This thread's TMEM lane, 32 (or 8) consecutive 32-bit columns from
// registers; tmem_wait_st makes them visible before the next handshake.
__device__ __forceinline__ void tmem_st32(uint32_t taddr, const uint32_t (&r)[32]) {
  asm volatile(
      "tcgen05.st.sync.aligned.32x32b.x32.b32 [%0], "
      "{%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,"
      "%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31,%32};" ::"r"(taddr),
      "r"(r[0]), "r"(r[1]), "r"(r[2]), "r"(r[3]), "r"(r[4]), "r"(r[5]), "r"(r[6]), "r"(r[7]),
      "r"(r[8]), "r"(r[9]), "r"(r[10]), "r"(r[11]), "r"(r[12]), "r"(r[13]), "r"(r[14]),
      "r"(r[15]), "r"(r[16]), "r"(r[17]), "r"(r[18]), "r"(r[19]), "r"(r[20]), "r"(r[21]),
      "r"(r[22]), "r"(r[23]), "r"(r[24]), "r"(r[25]), "r"(r[26]), "r"(r[27]), "r"(r[28]),
      "r"(r[29]), "r"(r[30]), "r"(r[31])
      : "memory");
}
__device__ __forceinline__ void tmem_st16(uint32_t taddr, const uint32_t (&r)[16]) {
  asm volatile(
      "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], "
      "{%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16};" ::"r"(taddr),
      "r"(r[0]), "r"(r[1]), "r"(r[2]), "r"(r[3]), "r"(r[4]), "r"(r[5]), "r"(r[6]), "r"(r[7]),
      "r"(r[8]), "r"(r[9]), "r"(r[10]), "r"(r[11]), "r"(r[12]), "r"(r[13]), "r"(r[14]),
      "r"(r[15])
      : "memory");
}
__device__ __forceinline__ void tmem_st8(uint32_t taddr, const uint32_t (&r)[8]) {
  asm volatile("tcgen05.st.sync.aligned.32x32b.x8.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8};" ::"r"(
                   taddr),
               "r"(r[0]), "r"(r[1]), "r"(r[2]), "r"(r[3]), "r"(r[4]), "r"(r[5]), "r"(r[6]),
               "r"(r[7])
               : "memory");
}
__device__ __forceinline__ void tmem_wait_st() {
  asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
}

// tcgen05.ld of 32 columns without the wait (pair with tmem_wait_ld).
__device__ __forceinline__ void tmem_ld32_async(uint32_t taddr, uint32_t (&r)[32]) {
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
}
__device__ __forceinline__ void tmem_wait_ld() {
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

// ------------------------------------------------------------- layouts
// Canonical no-swizzle K-major tile of 16-bit elements: core matrices of 8
// rows x 8 elements (16 bytes per row), `lbo` bytes between K-adjacent core
// matrices, `sbo` bytes between row groups.
__host__ __device__ constexpr uint32_t kmajor_offset(uint32_t row, uint32_t k, uint32_t lbo,
                                                     uint32_t sbo) {
  return (row / 8) * sbo + (k / 8) * lbo + (row % 8) * 16 + (k % 8) * 2;
}

// Chunk image (one TMA bulk copy), built per mean-shift call for 1/h:
//   B1   128 votes x 16, K-major (LBO 128, SBO 256): v = (x - c_c)/h in k
//        0..5 and again in k 8..13; -|v|^2 of the rounded v as a BF16 value
//        and residue in k 6, 7 (-1e30 for padding votes, which then get
//        w = 0); f = -2 E.v as a BF16 value and residue in k 14, 15
//   B2   16 features x 128 votes, K-major (LBO 128, SBO 2048): BF16(x) in
//        features 0..5, ones in 6, the BF16 residue x - BF16(x) in 8..13
//   CEN  E = (c_c - c_g)/h (8 floats)
constexpr uint32_t kB1Bytes = 4096, kB2Bytes = 4096, kCenBytes = 32;
constexpr uint32_t kImage = kB1Bytes + kB2Bytes + kCenBytes;  // 8224
static_assert(kImage % 16 == 0, "TMA bulk copies move multiples of 16 bytes");

__device__ __forceinline__ void split_bf16(float x, __nv_bfloat16 &hi, __nv_bfloat16 &lo) {
  hi = __float2bfloat16_rn(x);
  lo = __float2bfloat16_rn(x - __bfloat162float(hi));
}

// Two consecutive BF16 values as one 32-bit TMEM column (first in the low half).
__device__ __forceinline__ uint32_t bf16_pair(const __nv_bfloat16 *p) {
  return uint32_t(__bfloat16_as_ushort(p[0])) | (uint32_t(__bfloat16_as_ushort(p[1])) << 16);
}

__global__ void build_images(const float *desc, uint64_t q, uint64_t nchunks, const float *cbox,
                             const float *gbox, float inv_h, uint8_t *images) {
  // the image is assembled in shared memory (its 2-byte entries lie 16 or
  // 128 bytes apart for neighbouring votes) and written out in 16-byte words
  __shared__ __align__(16) uint8_t img[kImage];
  uint64_t c = blockIdx.x;
  int t = threadIdx.x;  // vote in chunk
  if (c >= nchunks) return;
  const float *b = cbox + c * 12;
  float cen[6], e[6];
  for (int d = 0; d < 6; ++d) {
    cen[d] = 0.5f * (b[d] + b[6 + d]);
    e[d] = (cen[d] - 0.5f * (gbox[d] + gbox[6 + d])) * inv_h;
  }
  uint64_t v = c * kChunk + t;
  bool live = v < q;
  __nv_bfloat16 *b1 = reinterpret_cast<__nv_bfloat16 *>(img);
  __nv_bfloat16 *b2 = reinterpret_cast<__nv_bfloat16 *>(img + kB1Bytes);
  float *ce = reinterpret_cast<float *>(img + kB1Bytes + kB2Bytes);
  if (t < 8) ce[t] = t < 6 ? e[t] : 0.f;
  const __nv_bfloat16 zero = __float2bfloat16_rn(0.f);
  float n2 = 0, f = 0;
  for (int d = 0; d < 6; ++d) {
    float x = live ? desc[v * 8 + d] : 0.f;
    __nv_bfloat16 h = __float2bfloat16_rn(live ? (x - cen[d]) * inv_h : 0.f);
    float r = __bfloat162float(h);
    n2 = fmaf(r, r, n2);
    f = fmaf(-2.f * e[d], r, f);
    b1[kmajor_offset(t, d, 128, 256) / 2] = h;
    b1[kmajor_offset(t, 8 + d, 128, 256) / 2] = h;
    __nv_bfloat16 xh, xl;
    split_bf16(x, xh, xl);
    b2[kmajor_offset(d, t, 128, 2048) / 2] = xh;
    b2[kmajor_offset(8 + d, t, 128, 2048) / 2] = xl;
  }
  __nv_bfloat16 nh, nl, fh, fl;
  split_bf16(live ? -n2 : -1e30f, nh, nl);
  split_bf16(f, fh, fl);
  b1[kmajor_offset(t, 6, 128, 256) / 2] = nh;
  b1[kmajor_offset(t, 7, 128, 256) / 2] = nl;
  b1[kmajor_offset(t, 14, 128, 256) / 2] = fh;
  b1[kmajor_offset(t, 15, 128, 256) / 2] = fl;
  b2[kmajor_offset(6, t, 128, 2048) / 2] = __float2bfloat16_rn(live ? 1.f : 0.f);
  for (int k : {7, 14, 15}) b2[kmajor_offset(k, t, 128, 2048) / 2] = zero;
  __syncthreads();
  const uint4 *src = reinterpret_cast<const uint4 *>(img);
  uint4 *dst = reinterpret_cast<uint4 *>(images + c * kImage);
  for (int w = t; w < int(kImage / 16); w += kChunk) dst[w] = src[w];
}

__device__ __forceinline__ float box_gap2_tc(const float *lo, const float *hi, const float *b) {
  float g = 0;
  for (int k = 0; k < 6; ++k) {
    float d = fmaxf(fmaxf(b[k] - hi[k], lo[k] - b[6 + k]), 0.f);
    g += d * d;
  }
  return g;
}

// ------------------------------------------------- work lists per tile
// The number of active seeds n = nact[0] is read on the device by every
// kernel of an iteration, so the host never waits for it: grids are sized
// for all k seeds and blocks past the active tiles return at once.
__device__ __forceinline__ uint32_t active_tiles(const unsigned *nact) {
  return (nact[0] + kChunk - 1) / kChunk;
}

// boxes[t * kBoxFloats ..]: the box of tile t's active seeds (12 floats:
// lo, hi), then the boxes of its eight groups of 16 seeds (one block per
// tile).  Then the block cull: sblk[t * nblk ..] lists, in ascending order,
// the blocks of kBlockChunks chunks whose box lies within the bandwidth of
// the tile's box and of some group's box (exact, as the chunk tests), and
// nsurv[t] counts them; their counts bcount[t * nblk + j] are zeroed.
constexpr int kGroupSeeds = 16, kBoxFloats = 12 * (1 + kChunk / kGroupSeeds);
constexpr int kCullThreads = 512;  // threads of tile_boxes (the first kChunk hold the seeds)
__global__ void __launch_bounds__(kCullThreads) tile_boxes(const float *means, const int32_t *ids,
                                                           const unsigned *nact, const float *bbox,
                                                           uint32_t nblk, float skip_gap2,
                                                           float *boxes, uint32_t *sblk,
                                                           uint32_t *nsurv, uint32_t *bcount) {
  __shared__ float part[kChunk / kGroupSeeds][12];
  __shared__ float tb[kBoxFloats];
  __shared__ uint32_t warp_cnt[kCullThreads / 32], base_s;
  if (blockIdx.x >= active_tiles(nact)) return;
  if (threadIdx.x < kChunk) {  // whole warps
    const uint64_t slot = uint64_t(blockIdx.x) * kChunk + threadIdx.x;
    const bool live = slot < nact[0];
    float lo[6], hi[6];
    for (int d = 0; d < 6; ++d) {
      float m = live ? means[uint64_t(ids[slot]) * 8 + d] : 0.f;
      lo[d] = live ? m : INFINITY, hi[d] = live ? m : -INFINITY;
    }
    for (int o = kGroupSeeds / 2; o; o >>= 1)  // within each group of 16 lanes
      for (int d = 0; d < 6; ++d) {
        lo[d] = fminf(lo[d], __shfl_xor_sync(0xffffffffu, lo[d], o));
        hi[d] = fmaxf(hi[d], __shfl_xor_sync(0xffffffffu, hi[d], o));
      }
    const int group = threadIdx.x / kGroupSeeds;
    if (threadIdx.x % kGroupSeeds == 0)
      for (int d = 0; d < 6; ++d) part[group][d] = lo[d], part[group][6 + d] = hi[d];
  }
  if (threadIdx.x == 0) base_s = 0;
  __syncthreads();
  float *out = boxes + uint64_t(blockIdx.x) * kBoxFloats;
  constexpr int kGroups = kChunk / kGroupSeeds;
  if (threadIdx.x < 12) {
    float v = part[0][threadIdx.x];
    for (int w = 1; w < kGroups; ++w)
      v = threadIdx.x < 6 ? fminf(v, part[w][threadIdx.x]) : fmaxf(v, part[w][threadIdx.x]);
    out[threadIdx.x] = v, tb[threadIdx.x] = v;
  } else if (threadIdx.x < kBoxFloats) {
    const float v = part[(threadIdx.x - 12) / 12][(threadIdx.x - 12) % 12];
    out[threadIdx.x] = v, tb[threadIdx.x] = v;
  }
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t *mine = sblk + uint64_t(blockIdx.x) * nblk;
  for (uint32_t b0 = 0; b0 < nblk; b0 += kCullThreads) {
    const uint32_t b = b0 + threadIdx.x;
    bool keep = false;
    if (b < nblk) {
      float bb[12];
      for (int d = 0; d < 12; ++d) bb[d] = bbox[uint64_t(b) * 12 + d];
      if (box_gap2_tc(tb, tb + 6, bb) <= skip_gap2)
        for (int g = 0; g < kGroups && !keep; ++g)
          keep = box_gap2_tc(tb + 12 + 12 * g, tb + 18 + 12 * g, bb) <= skip_gap2;
    }
    const uint32_t bal = __ballot_sync(0xffffffffu, keep);
    if (lane == 0) warp_cnt[warp] = __popc(bal);
    __syncthreads();
    uint32_t before = base_s, total = 0;
    for (int w = 0; w < kCullThreads / 32; ++w) {
      if (w < warp) before += warp_cnt[w];
      total += warp_cnt[w];
    }
    if (keep) {
      const uint32_t at = before + __popc(bal & ((1u << lane) - 1u));
      mine[at] = b;
      bcount[uint64_t(blockIdx.x) * nblk + at] = 0;  // tile_count adds the block's kept chunks
    }
    __syncthreads();
    if (threadIdx.x == 0) base_s += total;
    __syncthreads();
  }
  if (threadIdx.x == 0) nsurv[blockIdx.x] = base_s;
}

// The CTAs of a list kernel's grid shared among the active tiles: CTA i
// serves tile i % tiles and takes every per-th of its surviving blocks,
// starting at i / tiles (per = CTAs / tiles); false for a CTA left over.
__device__ __forceinline__ bool list_share(const unsigned *nact, uint32_t &t, uint32_t &sub,
                                           uint32_t &per) {
  const uint32_t tiles = active_tiles(nact), i = blockIdx.x;
  if (!tiles) return false;
  per = gridDim.x / tiles;
  if (!per || i >= per * tiles) return false;
  t = i % tiles, sub = i / tiles;
  return true;
}

constexpr int kListThreads = 256;  // chunks per block of the list kernels
static_assert(kListThreads == kBlockChunks, "one thread per chunk of a block box");

// need[t * nchunks + c]: some seed of tile t lies within the bandwidth of
// chunk c's box, for the chunks of tile t's surviving blocks: tested
// against the tile's box, each group's box (16 seeds), each quad's box (4
// consecutive seeds), then the quad's seeds, among the seeds within the
// bandwidth of the block's box only (a mask per block).  Exact for Epanechnikov
// weights: every vote of a skipped chunk is farther than the bandwidth from
// every seed of the tile; and a box holds its seeds' coordinates, so in
// FP32 too its gap (monotone in every operation) is never above a seed's.
// bcount[t * nblk + j] (zeroed by tile_boxes) gains the kept chunks of the
// tile's j-th surviving block, one integer atomic per warp: no barrier
// between blocks, and the counts do not depend on the order.
constexpr int kQuads = kChunk / 4;
__global__ void __launch_bounds__(kListThreads) tile_count(const float *boxes, const float *means,
                                                           const int32_t *ids, const unsigned *nact,
                                                           const float *cbox, const float *bbox,
                                                           uint64_t nchunks, const uint32_t *sblk,
                                                           const uint32_t *nsurv, uint32_t nblk,
                                                           float skip_gap2, uint8_t *need,
                                                           uint32_t *bcount) {
  __shared__ float seed[kChunk * 6];
  __shared__ float gb[kBoxFloats];
  __shared__ float qb[kQuads * 12];
  __shared__ bool alive[kChunk];
  __shared__ uint32_t reach[kChunk / 32];  // seeds within the bandwidth of the block's box
  uint32_t t, sub, per;
  if (!list_share(nact, t, sub, per)) return;
  const unsigned nactive = nact[0];
  const uint32_t ns = nsurv[t];
  if (sub >= ns) return;
  for (int i = threadIdx.x; i < kChunk; i += blockDim.x) {
    const uint64_t slot = uint64_t(t) * kChunk + i;
    const bool live = slot < nactive;
    alive[i] = live;
    for (int d = 0; d < 6; ++d) seed[i * 6 + d] = live ? means[uint64_t(ids[slot]) * 8 + d] : 1e30f;
  }
  if (threadIdx.x < kBoxFloats) gb[threadIdx.x] = boxes[uint64_t(t) * kBoxFloats + threadIdx.x];
  __syncthreads();
  if (threadIdx.x < kQuads) {  // a quad without live seeds gets an empty box (gap infinite)
    float lo[6], hi[6];
    for (int d = 0; d < 6; ++d) lo[d] = INFINITY, hi[d] = -INFINITY;
    for (int i = 4 * threadIdx.x; i < 4 * threadIdx.x + 4; ++i)
      if (alive[i])
        for (int d = 0; d < 6; ++d) lo[d] = fminf(lo[d], seed[i * 6 + d]), hi[d] = fmaxf(hi[d], seed[i * 6 + d]);
    for (int d = 0; d < 6; ++d) qb[threadIdx.x * 12 + d] = lo[d], qb[threadIdx.x * 12 + 6 + d] = hi[d];
  }
  __syncthreads();
  const int lane = threadIdx.x & 31;
  uint32_t *bc = bcount + uint64_t(t) * nblk;
  for (uint32_t j = sub; j < ns; j += per) {
    const uint32_t blk = sblk[uint64_t(t) * nblk + j];
    // the seeds that can reach the block at all: a seed beyond the
    // bandwidth of the block's box is beyond it for each of its chunks
    // (their boxes lie inside it), so the chunk tests skip it
    __syncthreads();  // the previous block's mask is no longer read
    if (threadIdx.x < kChunk) {  // whole warps
      bool ok = false;
      if (alive[threadIdx.x]) {
        const float *bb = bbox + uint64_t(blk) * 12;
        float q = 0;
        for (int d = 0; d < 6; ++d) {
          const float x = seed[threadIdx.x * 6 + d];
          const float e = fmaxf(fmaxf(bb[d] - x, x - bb[6 + d]), 0.f);
          q += e * e;
        }
        ok = q <= skip_gap2;
      }
      const unsigned bal = __ballot_sync(0xffffffffu, ok);
      if (lane == 0) reach[threadIdx.x >> 5] = bal;
    }
    __syncthreads();
    const uint64_t c = uint64_t(blk) * kBlockChunks + threadIdx.x;
    bool keep = false;
    if (c < nchunks) {
      float cb[12];
      for (int d = 0; d < 12; ++d) cb[d] = cbox[c * 12 + d];
      if (box_gap2_tc(gb, gb + 6, cb) <= skip_gap2)
        for (int g = 0; g < kChunk / kGroupSeeds && !keep; ++g) {
          const uint32_t gm = (reach[g >> 1] >> ((g & 1) * kGroupSeeds)) & 0xffffu;
          if (!gm) continue;
          const float *b = gb + 12 + 12 * g;
          if (box_gap2_tc(b, b + 6, cb) > skip_gap2) continue;
          for (int qd = 4 * g; qd < 4 * g + 4 && !keep; ++qd) {
            const uint32_t qm = (gm >> (4 * (qd - 4 * g))) & 0xfu;
            if (!qm) continue;
            if (box_gap2_tc(qb + 12 * qd, qb + 12 * qd + 6, cb) > skip_gap2) continue;
            for (int i = 4 * qd; i < 4 * qd + 4 && !keep; ++i) {
              if (!((qm >> (i - 4 * qd)) & 1u)) continue;
              float q = 0;
              for (int d = 0; d < 6; ++d) {
                const float x = seed[i * 6 + d];
                const float e = fmaxf(fmaxf(cb[d] - x, x - cb[6 + d]), 0.f);
                q += e * e;
              }
              keep = q <= skip_gap2;
            }
          }
        }
      need[uint64_t(t) * nchunks + c] = keep;
    }
    const unsigned bal = __ballot_sync(0xffffffffu, keep);
    if (lane == 0 && bal) atomicAdd(&bc[j], unsigned(__popc(bal)));
  }
}

// Inclusive scan of one value per thread over a block of 1024 threads;
// `total` receives the block's sum.  Uses warp_sum[32] (shared).
__device__ __forceinline__ uint32_t block_scan_1024(uint32_t v, uint32_t *warp_sum, uint32_t &total) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t x = v;
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) warp_sum[warp] = x;
  __syncthreads();
  if (warp == 0) {
    uint32_t w = warp_sum[lane];
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += y;
    }
    warp_sum[lane] = w;  // inclusive over warps
  }
  __syncthreads();
  const uint32_t r = (warp ? warp_sum[warp - 1] : 0u) + x;
  total = warp_sum[31];
  __syncthreads();
  return r;
}

// One block of 1024 threads.  The surviving (tile, block) entries, tile by
// tile and in block order within a tile, form the list's order: seg[t] =
// exclusive scan of nsurv over the active tiles; boff[t * nblk + j] = the
// list position of entry (t, j)'s first kept chunk (exclusive scan of the
// counts over all entries in that order); offsets[t] = the first list
// entry of tile t (offsets[tiles] = the list length); and the work plan:
// tile t gets pieces[t+1] - pieces[t] CTAs, about len_t * budget / total
// of them (at least one), so every CTA streams a similar number of chunks;
// budget = sms - tiles (at least tiles), so the pieces fill one wave of the
// GPU.  seg holds max_tiles + 1 entries.  A list longer than `cap` (which
// the counts never give) records DS_CAPACITY and leaves an empty plan.
__global__ void __launch_bounds__(1024) scan_lists(const uint32_t *bcount, const uint32_t *nsurv,
                                                   const unsigned *nact, uint32_t nblk, uint32_t sms,
                                                   uint64_t cap, uint32_t *seg, uint32_t *boff,
                                                   uint64_t *offsets, uint32_t *pieces,
                                                   int *status) {
  __shared__ uint32_t warp_sum[32];
  __shared__ uint32_t carry_s;
  const uint32_t tiles = active_tiles(nact);
  if (threadIdx.x == 0) carry_s = 0;
  __syncthreads();
  for (uint32_t base = 0; base < tiles; base += blockDim.x) {  // segment starts
    const uint32_t t = base + threadIdx.x;
    const uint32_t v = t < tiles ? nsurv[t] : 0u;
    uint32_t total;
    const uint32_t incl = block_scan_1024(v, warp_sum, total);
    if (t < tiles) seg[t] = carry_s + incl - v;
    __syncthreads();
    if (threadIdx.x == 0) carry_s += total;
    __syncthreads();
  }
  const uint32_t entries = carry_s;
  __syncthreads();  // every thread has read carry_s before it is reset
  if (threadIdx.x == 0) seg[tiles] = entries, carry_s = 0;
  __syncthreads();
  for (uint32_t base = 0; base < entries; base += blockDim.x) {  // list positions
    const uint32_t e = base + threadIdx.x;
    uint32_t t = 0, v = 0;
    if (e < entries) {  // the tile of entry e: the last t with seg[t] <= e
      uint32_t lo = 0, hi = tiles;  // seg[lo] <= e < seg[hi]
      while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (seg[mid] <= e) lo = mid;
        else hi = mid;
      }
      t = lo;
      v = bcount[uint64_t(t) * nblk + (e - seg[t])];
    }
    uint32_t total;
    const uint32_t incl = block_scan_1024(v, warp_sum, total);
    if (e < entries) boff[uint64_t(t) * nblk + (e - seg[t])] = carry_s + incl - v;
    __syncthreads();
    if (threadIdx.x == 0) carry_s += total;
    __syncthreads();
  }
  const uint32_t list_len = carry_s;
  for (uint32_t t = threadIdx.x; t < tiles; t += blockDim.x)  // a tile with no entry starts
    offsets[t] = seg[t] < seg[t + 1] ? boff[uint64_t(t) * nblk] : 0u;  // fixed below
  __syncthreads();
  if (threadIdx.x == 0 && list_len > cap) {
    atomicExch(status, DS_CAPACITY);
    for (uint32_t t = 0; t <= tiles; ++t) offsets[t] = 0, pieces[t] = 0;
    return;
  }
  if (threadIdx.x == 0) {
    // empty tiles take the position where the next entries start
    uint64_t next = list_len;
    for (uint32_t t = tiles; t-- > 0;) {
      if (seg[t] < seg[t + 1]) next = offsets[t];
      else offsets[t] = next;
    }
    offsets[tiles] = list_len;
    const uint32_t budget = tiles < sms ? sms - tiles : tiles;
    uint32_t at = 0;
    for (uint32_t t = 0; t < tiles; ++t) {
      pieces[t] = at;
      const uint64_t len = offsets[t + 1] - offsets[t];
      const uint64_t want = list_len ? (len * budget + list_len - 1) / list_len : 1;
      at += uint32_t(want ? want : 1);
    }
    pieces[tiles] = at;
  }
}

// list[boff[t * nblk + j] + r] = t * nchunks + c for the r-th kept chunk c
// (ascending) of tile t's j-th surviving block: per tile, the kept chunks in
// ascending order.  CTAs shared among tiles as tile_count's.
__global__ void __launch_bounds__(kListThreads) scatter_lists(const uint8_t *need,
                                                              const uint32_t *boff,
                                                              const uint32_t *bcount,
                                                              const uint32_t *sblk,
                                                              const uint32_t *nsurv, uint32_t nblk,
                                                              const unsigned *nact,
                                                              uint64_t nchunks, uint64_t cap,
                                                              int32_t *list, int *status) {
  __shared__ uint32_t warp_cnt[kListThreads / 32];
  uint32_t t, sub, per;
  if (!list_share(nact, t, sub, per)) return;
  const uint32_t ns = nsurv[t];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (uint32_t j = sub; j < ns; j += per) {
    const uint64_t e = uint64_t(t) * nblk + j;
    if (!bcount[e]) continue;  // the same for the whole CTA
    const uint64_t c = uint64_t(sblk[e]) * kBlockChunks + threadIdx.x;
    const bool keep = c < nchunks && need[uint64_t(t) * nchunks + c];
    const uint32_t bal = __ballot_sync(0xffffffffu, keep);
    if (lane == 0) warp_cnt[warp] = __popc(bal);
    __syncthreads();
    uint64_t before = boff[e];
    for (int w = 0; w < warp; ++w) before += warp_cnt[w];
    before += __popc(bal & ((1u << lane) - 1u));
    if (keep && before < cap) list[before] = int32_t(uint64_t(t) * nchunks + c);
    else if (keep) atomicExch(status, DS_CAPACITY);
    __syncthreads();
  }
}

// --------------------------------------------- pipelined tensor kernel
// Warp roles (19 warps):
//   warps 0..15  the epilogue, two pairs of warpgroups taking alternate
//                chunks (pair p = warp / 8 owns the chunks i with
//                i % 2 == p); in a pair, warp w reads TMEM lanes 32(w%4)..
//                and D columns 64((w/4)%2)..+63
//   warp 16      TMA: streams the chunk images through the stage ring
//   warps 17, 18 MMA issue for pair 0 / pair 1 (one lane each): MMA1 of
//                the pair's chunk k + 1 once it landed and D[p] was read,
//                then MMA2 of chunk k once W[p] was written.
//                A single thread issues one tcgen05.mma per ~85 cycles
//                whatever its N, while the tensor pipe takes an N = 16 MMA
//                every ~40 cycles from two issuers (measured on GB300), so
//                each pair drives its own stream of MMAs
//   shared memory  kStagesTc TMA buffers of one chunk image each, ATILE
//                  (A operand of MMA1, once per tile), U
//   TMEM columns   D[p] = 128p (MMA1 accumulators), W[p] = 256 + 64p (the
//                  BF16 weights, A operand of MMA2), ACC[p][q] = 384 + 64p
//                  + 16q for q = 0..3 (pair p's accumulators, K-step q of
//                  MMA2 into ACC[p][q % 4]; zeroed at the start, summed in
//                  a fixed order at the end)
// mbarriers: load_full[s] (TMA bytes), stage_free[s] (MMA2 of the chunk in
// stage s done; arrived at by the pair once its wait for that MMA2 passed), d_full[p] (MMA1 done), d_free[p] (pair p read D[p]),
// w_full[p] (pair p wrote W[p]), w_free[p] (MMA2 done), acc_done[p].  Every
// wait is bounded; on timeout a warp records the status and stops, an MMA
// warp drains its MMAs into acc_done[p], the TMA warp its copies.
constexpr int kStagesTc = 12;
constexpr int kPairWarps = 8, kTmaWarp = 16, kMmaWarp = 17;  // warps 0..15: the two pairs
constexpr int kThreadsTc = 19 * 32;
constexpr uint32_t kTcStage = 0;                                     // kStagesTc x kImage
constexpr uint32_t kTcU = (kStagesTc * kImage + 1023) / 1024 * 1024; // 128 x 8 floats
constexpr uint32_t kTcATile = kTcU + 128 * 8 * 4;                    // 4096, K-major
constexpr uint32_t kTcBars = kTcATile + 4096;                        // 2 kStagesTc + 10
constexpr uint32_t kTcMisc = kTcBars + 48 * 8;                      // TMEM address, K-step masks
constexpr uint32_t kTcSmem = kTcMisc + 64;
static_assert(kImage % 16 == 0, "TMA alignment");
static_assert(kTcATile % 1024 == 0, "descriptor alignment");
static_assert(2 * kStagesTc + 10 <= 48, "barrier slots");
static_assert(kTcSmem <= 227 * 1024, "shared memory per CTA");
constexpr uint32_t kTcCols = 512, kTcColW = 256, kTcColAcc = 384;

struct TcArgs {
  const uint8_t *images;
  uint64_t nchunks;
  const int32_t *list;      // needed (tile, chunk) entries, t * nchunks + c
  const uint64_t *offsets;  // tiles + 1: first list entry of each tile
  const uint32_t *pieces;   // tiles + 1: first piece (CTA) of each tile
  const unsigned *nact;     // nact[0] = active seeds (tiles of kChunk)
  const float *means;
  const int32_t *ids;
  const float *gbox;        // box of all votes; its centre is c_g
  float inv_h;
  float gauss_k2;           // 0: Epanechnikov; k > 0 (a power of 2): 2^(-k d^2/h^2) - 2^-k
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

// {relu(lo), relu(hi)} rounded to BF16 and packed, lo in the low half.
__device__ __forceinline__ uint32_t relu_bf16x2(float lo, float hi) {
  uint32_t r;
  asm("cvt.rn.relu.bf16x2.f32 %0, %1, %2;" : "=r"(r) : "f"(hi), "f"(lo));
  return r;
}

// Shifted Gaussian weights 2^a - 2^-k from the exponents a = -k d^2 / h^2
// (the MMA's D with the seed operand scaled by k, plus -k |u - E|^2), two at
// a time: the exponents rounded to BF16, one MUFU BF16x2 base-2
// exponential, one BF16x2 FMA with relu (votes past the cut, a < -k, get 0).
__device__ __forceinline__ uint32_t gauss_bf16x2(float lo, float hi, uint32_t neg_floor2) {
  uint32_t x, e, w;
  asm("cvt.rn.bf16x2.f32 %0, %1, %2;" : "=r"(x) : "f"(hi), "f"(lo));
  asm("ex2.approx.ftz.bf16x2 %0, %1;" : "=r"(e) : "r"(x));
  asm("fma.rn.relu.bf16x2 %0, %1, %2, %3;" : "=r"(w) : "r"(e), "r"(0x3F803F80u), "r"(neg_floor2));
  return w;
}

// ACC[q % 4] += W[:, 16q..16q+15] . B2[:, 16q..16q+15]^T for the eight
// K-steps q of the chunk (16 votes each); W in TMEM, the accumulators start
// at zero.  Unrolled with constant descriptor offsets: the issuing thread
// waits ~50 cycles per tcgen05.mma, and every instruction between two MMAs
// adds to that (a branch per K-step nearly doubled the cost on GB300).
// Skipping all-zero K-steps saves nothing once the tile's chunk list is
// culled per seed: under 1% of the 16-vote x 128-seed blocks are zero.
__device__ __forceinline__ void mma2_chunk(uint32_t acc, uint32_t w_tmem, const uint8_t *b2) {
  const uint64_t b = smem_desc(b2, 128, 2048);
#pragma unroll
  for (uint32_t q = 0; q < 8; ++q)
    mma_bf16_ts(acc + 16 * (q & 3u), w_tmem + 8 * q, b + 16 * q, idesc_bf16(128, 16), 1u);
}

__global__ void __launch_bounds__(kThreadsTc, 1) ms_tile_tc(TcArgs a) {
  extern __shared__ __align__(1024) uint8_t smem[];
  uint8_t *stage = smem + kTcStage;
  float *U = reinterpret_cast<float *>(smem + kTcU);
  uint8_t *ATILE = smem + kTcATile;
  uint64_t *bars = reinterpret_cast<uint64_t *>(smem + kTcBars);
  uint64_t *load_full = bars, *stage_free = bars + kStagesTc;
  uint64_t *d_full = bars + 2 * kStagesTc, *d_free = d_full + 2, *w_full = d_full + 4;
  uint64_t *w_free = d_full + 6, *acc_done = d_full + 8;  // acc_done[2]
  uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(smem + kTcMisc);

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  // piece -> (tile, share of the tile's list)
  const uint32_t piece = blockIdx.x;
  const uint32_t ntiles = active_tiles(a.nact);
  if (piece >= a.pieces[ntiles]) return;
  const uint64_t nactive = a.nact[0];
  uint64_t lo_t = 0, hi_t = ntiles;  // last tile whose first piece is <= piece
  while (hi_t - lo_t > 1) {
    uint64_t mid = (lo_t + hi_t) / 2;
    if (a.pieces[mid] <= piece) lo_t = mid;
    else hi_t = mid;
  }
  const uint64_t tile = lo_t;
  const uint64_t k = piece - a.pieces[tile], np = a.pieces[tile + 1] - a.pieces[tile];
  const uint64_t lt0 = a.offsets[tile], len = a.offsets[tile + 1] - lt0;
  const uint64_t e0 = lt0 + len * k / np, e1 = lt0 + len * (k + 1) / np;
  const uint32_t n = uint32_t(e1 - e0);
  const uint64_t tbase = tile * a.nchunks;

  // u = (s - c_g)/h of this tile's seeds: U (FP32 sums of the BF16 pairs)
  // and ATILE rows [2u_hi, 1, 1 | 2u_lo, 1, 1] in shared memory
  if (tid < kChunk) {
    uint64_t slot = tile * kChunk + tid;
    bool live = slot < nactive;
    int32_t sd = live ? a.ids[slot] : 0;
    __align__(16) __nv_bfloat16 k0[8], k1[8];
    // Gaussian weights: the whole operand scaled by the power of two k
    // (exact in BF16), so D comes out as k times the Epanechnikov D
    const float kscale = a.gauss_k2 > 0.f ? a.gauss_k2 : 1.f;
    const __nv_bfloat16 kone = __float2bfloat16_rn(kscale);
    for (int d = 0; d < 6; ++d) {
      float cg = 0.5f * (a.gbox[d] + a.gbox[6 + d]);
      float u = live ? (a.means[uint64_t(sd) * 8 + d] - cg) * a.inv_h : 0.f;
      __nv_bfloat16 hi, lo;
      split_bf16(u, hi, lo);
      U[tid * 8 + d] = __bfloat162float(hi) + __bfloat162float(lo);
      k0[d] = __float2bfloat16_rn(2.f * kscale * __bfloat162float(hi));  // exact
      k1[d] = __float2bfloat16_rn(2.f * kscale * __bfloat162float(lo));
    }
    k0[6] = k0[7] = k1[6] = k1[7] = kone;
    *reinterpret_cast<uint4 *>(ATILE + kmajor_offset(tid, 0, 128, 256)) = *reinterpret_cast<uint4 *>(k0);
    *reinterpret_cast<uint4 *>(ATILE + kmajor_offset(tid, 8, 128, 256)) = *reinterpret_cast<uint4 *>(k1);
  }
  if (tid == 0) {
    for (int s = 0; s < kStagesTc; ++s) mbar_init(&load_full[s], 1), mbar_init(&stage_free[s], 1);
    for (int p = 0; p < 2; ++p) {
      mbar_init(&d_full[p], 1), mbar_init(&w_free[p], 1);
      mbar_init(&d_free[p], kPairWarps), mbar_init(&w_full[p], kPairWarps);
    }
    mbar_init(&acc_done[0], 1), mbar_init(&acc_done[1], 1);
    fence_mbar_init();
  }
  if (warp == 0 && n) tmem_alloc(tmem_slot, kTcCols);
  fence_async_smem();  // ATILE written by the generic proxy, read by the MMA
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = n ? *tmem_slot : 0;
  auto stage_of = [&](uint32_t i) { return stage + (i % kStagesTc) * kImage; };
  if (n && warp < 4) {  // ACC starts at zero (MMA2 always accumulates)
    uint32_t z[32];
    for (int j = 0; j < 32; ++j) z[j] = 0u;
    for (int q2 = 0; q2 < 4; ++q2) tmem_st32(tmem + (uint32_t(warp * 32) << 16) + kTcColAcc + 32 * q2, z);
    tmem_wait_st();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();

  if (warp == kTmaWarp) {
    // ------------------------------------------------ TMA producer
    // chunk ids of the work list, 32 per batch, lane l holding entry
    // 32 * batch + l; the next batch is loaded one batch ahead, so no
    // global-load latency sits on the issue path.  chunk_of is called by the
    // whole warp with non-decreasing i.
    auto load_batch = [&](uint32_t batch) -> uint32_t {
      uint32_t idx = batch * 32 + lane;
      return idx < n ? uint32_t(uint64_t(a.list[e0 + idx]) - tbase) : 0u;
    };
    uint32_t cur = load_batch(0), nxt = load_batch(1), cur_batch = 0;
    auto chunk_of = [&](uint32_t i) -> uint64_t {
      while (i / 32 != cur_batch) {
        cur = nxt;
        nxt = load_batch(++cur_batch + 1);
      }
      return __shfl_sync(0xffffffffu, cur, i % 32);
    };
    bool ok = true;
    uint32_t issued = 0;
    for (; issued < n && issued < uint32_t(kStagesTc); ++issued) {
      const uint64_t c = chunk_of(issued);
      if (lane == 0) {
        mbar_expect_tx(&load_full[issued], kImage);
        tma_bulk_load(stage + issued * kImage, a.images + c * kImage, kImage, &load_full[issued]);
      }
    }
    // chunk j + kStagesTc reuses the stage of chunk j once MMA2(j) is done
    for (uint32_t j = 0; j + kStagesTc < n; ++j) {
      const uint64_t c = chunk_of(j + kStagesTc);
      ok = warp_wait(&stage_free[j % kStagesTc], (j / kStagesTc) & 1);
      if (!ok) break;
      if (lane == 0) {
        mbar_expect_tx(&load_full[j % kStagesTc], kImage);
        tma_bulk_load(stage_of(j), a.images + c * kImage, kImage, &load_full[j % kStagesTc]);
      }
      ++issued;
    }
    if (!ok && lane == 0) {
      atomicExch(a.status, DS_SPIN_LIMIT);
      // drain: wait (bounded) for every copy issued, so none lands after exit
      for (uint32_t c = 0; c < issued; ++c) mbar_wait(&load_full[c % kStagesTc], (c / kStagesTc) & 1);
    }
  } else if (warp >= kMmaWarp) {
    // ------------------------------------------------ MMA issue, pair p
    const uint32_t p = uint32_t(warp - kMmaWarp);
    const uint32_t np = n > p ? (n - p + 1) / 2 : 0;  // chunks 2k + p of the pair
    if (lane == 0 && n) {
      bool ok = true;
      const uint32_t dcol = tmem + 128 * p, wcol = tmem + kTcColW + 64 * p;
      const uint32_t acc = tmem + kTcColAcc + 64 * p;
      // MMA1 of the pair's chunk k (chunk 2k + p) once it landed and the
      // pair read D[p] for chunk k - 1
      auto mma1 = [&](uint32_t k) -> bool {
        const uint32_t i = 2 * k + p;
        if (!mbar_wait(&load_full[i % kStagesTc], (i / kStagesTc) & 1)) return false;
        if (k > 0 && !mbar_wait(&d_free[p], (k - 1) & 1)) return false;
        tc_fence_after();
        mma_bf16(dcol, smem_desc(ATILE, 128, 256), smem_desc(stage_of(i), 128, 256),
                 idesc_bf16(128, 128), 0);
        mma_commit(&d_full[p]);
        return true;
      };
      // the pair reads D for chunk k before it writes W for chunk k, so
      // MMA1(k + 1) is always ready before MMA2(k): the issuer takes them in
      // that order, sleeping in each wait
      if (np) ok = mma1(0);
      for (uint32_t k = 0; ok && k < np; ++k) {
        if (k + 1 < np && !(ok = mma1(k + 1))) break;
        if (!(ok = mbar_wait(&w_full[p], k & 1))) break;  // the pair wrote W[p]
        tc_fence_after();
        mma2_chunk(acc, wcol, stage_of(2 * k + p) + kB1Bytes);
        mma_commit(&w_free[p]);  // W[p] and the chunk's stage are free again
      }
      if (!ok) atomicExch(a.status, DS_SPIN_LIMIT);
      mma_commit(&acc_done[p]);  // once every MMA issued has completed
    }
    __syncwarp();
  } else {
    // ------------------------------------------------ pair p
    // row `row`, D columns 64h..64h+63:  w = relu(D + 1 - |u - E|^2)
    const int p = warp / kPairWarps, quad = warp & 3, h = (warp >> 2) & 1, row = quad * 32 + lane;
    const float *u = U + row * 8;
    const float2 one2 = make_float2(1.f, 1.f);
    const uint32_t lane_base = uint32_t(quad * 32) << 16;
    const uint32_t dcol = tmem + 128 * p + 64 * h, wcol = tmem + kTcColW + 64 * p + 32 * h;
    const bool gauss = a.gauss_k2 > 0.f;
    uint32_t neg_floor2 = 0;  // -2^-k in both BF16 halves
    if (gauss) {
      const uint32_t h16 = __bfloat16_as_ushort(__float2bfloat16_rn(-exp2f(-a.gauss_k2)));
      neg_floor2 = h16 | (h16 << 16);
    }
    bool ok = true;
    uint32_t kth = 0;  // index of chunk i among the pair's chunks
    for (uint32_t i = p; i < n; i += 2, ++kth) {
      if (!warp_wait(&d_full[p], kth & 1) ||
          !warp_wait(&load_full[i % kStagesTc], (i / kStagesTc) & 1)) {
        ok = false;
        break;
      }
      tc_fence_after();
      const float *E = reinterpret_cast<const float *>(stage_of(i) + kB1Bytes + kB2Bytes);
      float rowc = 1.f;
      for (int d = 0; d < 6; ++d) {
        float r = u[d] - E[d];
        rowc = fmaf(-r, r, rowc);
      }
      uint32_t w[16], w2[16];
      {
        uint32_t d0[32], d1[32];
        tmem_ld32_async(lane_base + dcol, d0);
        tmem_ld32_async(lane_base + dcol + 32, d1);
        tmem_wait_ld();
        tc_fence_before();
        __syncwarp();
        if (lane == 0) mbar_arrive(&d_free[p]);  // D[p] may be overwritten
        if (gauss) {  // a = k D - k |u - E|^2 = -k d^2 / h^2
          const float rowg = a.gauss_k2 * (rowc - 1.f);
          const float2 rowg2 = make_float2(rowg, rowg);
          for (int j = 0; j < 16; ++j) {
            float2 t = fma2(make_float2(__uint_as_float(d0[2 * j]), __uint_as_float(d0[2 * j + 1])),
                            one2, rowg2);
            w[j] = gauss_bf16x2(t.x, t.y, neg_floor2);
          }
          for (int j = 0; j < 16; ++j) {
            float2 t = fma2(make_float2(__uint_as_float(d1[2 * j]), __uint_as_float(d1[2 * j + 1])),
                            one2, rowg2);
            w2[j] = gauss_bf16x2(t.x, t.y, neg_floor2);
          }
        } else {
          const float2 rowc2 = make_float2(rowc, rowc);
          for (int j = 0; j < 16; ++j) {
            float2 t = fma2(make_float2(__uint_as_float(d0[2 * j]), __uint_as_float(d0[2 * j + 1])),
                            one2, rowc2);
            w[j] = relu_bf16x2(t.x, t.y);
          }
          for (int j = 0; j < 16; ++j) {
            float2 t = fma2(make_float2(__uint_as_float(d1[2 * j]), __uint_as_float(d1[2 * j + 1])),
                            one2, rowc2);
            w2[j] = relu_bf16x2(t.x, t.y);
          }
        }
      }
      if (kth > 0) {
        if (!warp_wait(&w_free[p], (kth - 1) & 1)) {  // MMA2(i-2) read W[p]
          ok = false;
          break;
        }
        // MMA2(i-2) also finished reading chunk i-2's stage, and the pair
        // read its centre before w_full: the TMA warp may refill it (the
        // last two chunks of a pair are never refilled)
        if (quad == 0 && h == 0 && lane == 0) mbar_arrive(&stage_free[(i - 2) % kStagesTc]);
      }
      tc_fence_after();
      tmem_st16(lane_base + wcol, w);
      tmem_st16(lane_base + wcol + 16, w2);
      tmem_wait_st();
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(&w_full[p]);
    }
    if (!ok && lane == 0) atomicExch(a.status, DS_SPIN_LIMIT);
  }
  __syncthreads();
  if (warp < 4) {  // warpgroup 0 writes the tile's partial sums
    const int quad = warp & 3, row = quad * 32 + lane;
    float acc[16];
    for (int j = 0; j < 16; ++j) acc[j] = 0.f;
    if (n && warp_wait(&acc_done[0], 0) && warp_wait(&acc_done[1], 0)) {
      tc_fence_after();
      for (int q2 = 0; q2 < 4; ++q2) {  // ACC[0][0..3], ACC[1][0..3], two per load
        float v[32];
        tmem_ld32(tmem + (uint32_t(quad * 32) << 16) + kTcColAcc + 32 * q2, v);
        for (int j = 0; j < 16; ++j) acc[j] += v[j];
        for (int j = 0; j < 16; ++j) acc[j] += v[16 + j];
      }
    }
    // piece-major: value d of row r of piece p at (p * 8 + d) * 128 + r
    float *out = a.partial + uint64_t(piece) * 8 * kChunk + row;
    for (int d = 0; d < 6; ++d) out[d * kChunk] = acc[d] + acc[8 + d];  // BF16 x + its residue
    out[6 * kChunk] = acc[6];
  }
  if (tid == 0 && n && a.evals) atomicAdd(a.evals, uint64_t(n) * uint64_t(kChunk * kChunk));
  tc_fence_before();
  __syncthreads();
  if (warp == 0 && n) tmem_dealloc(tmem, kTcCols);
}

// ------------------------------------------------------ tensor self-test
// One tile: D = A1 . B1^T (128 x 128 x 16) and ACC = A2 . B2^T (128 x 16 x
// 128) from row-major BF16 inputs, through the same paths as ms_tile_tc: B
// operands in the canonical shared-memory layout staged by one TMA bulk
// copy, A operands written to TMEM with tcgen05.st, tcgen05.mma with A from
// TMEM, results read with tcgen05.ld.
constexpr uint32_t kSelfB2 = 4096;
constexpr uint32_t kOffStage = 0, kOffBars = 8192, kOffMisc = kOffBars + 64;
constexpr uint32_t kSmemRequest = 16 * 1024;
constexpr uint32_t kTmemCols = 256, kColD = 0, kColAcc = 128, kColA1 = 160, kColA2 = 192;

__global__ void __launch_bounds__(256, 1) tc_selftest(const __nv_bfloat16 *a1, const __nv_bfloat16 *b1,
                                                      const __nv_bfloat16 *a2, const __nv_bfloat16 *b2,
                                                      uint8_t *scratch, float *d_out, float *acc_out,
                                                      int *status) {
  extern __shared__ __align__(1024) uint8_t smem[];
  uint8_t *S = smem + kOffStage;
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
    asm volatile("fence.proxy.async.global;" ::: "memory");
  }
  if (tid == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    fence_mbar_init();
  }
  if (warp == 0) tmem_alloc(tmem_slot, kTmemCols);
  __threadfence();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;
  if (wg == 0) {  // A1 and A2 rows into TMEM, lane = row
    const uint32_t lane_base = uint32_t(quad * 32) << 16;
    uint32_t r8[8], r32[32];
    for (int c = 0; c < 8; ++c) r8[c] = bf16_pair(a1 + row * 16 + 2 * c);
    tmem_st8(tmem + lane_base + kColA1, r8);
    for (int half = 0; half < 2; ++half) {
      for (int c = 0; c < 32; ++c) r32[c] = bf16_pair(a2 + row * 128 + 64 * half + 2 * c);
      tmem_st32(tmem + lane_base + kColA2 + 32 * half, r32);
    }
    tmem_wait_st();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  bool ok = true;
  if (tid == 0) {
    asm volatile("fence.proxy.async.global;" ::: "memory");
    mbar_expect_tx(&bar[0], kB1Bytes + kSelfB2);
    tma_bulk_load(S, scratch, kB1Bytes + kSelfB2, &bar[0]);
  }
  ok = __syncthreads_and(mbar_wait(&bar[0], 0));
  if (ok && tid == 0) {
    tc_fence_after();
    mma_bf16_ts(tmem + kColD, tmem + kColA1, smem_desc(S, 128, 256), idesc_bf16(128, 128), 0);
    for (uint32_t s = 0; s < 8; ++s)
      mma_bf16_ts(tmem + kColAcc, tmem + kColA2 + 8 * s, smem_desc(S + kB1Bytes + s * 256, 128, 2048),
                  idesc_bf16(128, 16), s > 0);
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

// The kernels' bounded wait made to run out: one warp holds TMEM as the
// mean-shift kernel does, waits with mbar_wait on a barrier nothing arrives
// at, with a limit of limit_ns instead of 2 s, then records DS_SPIN_LIMIT,
// frees its TMEM and returns -- the path a real kernel takes when a copy or
// an MMA never completes.  No copy or MMA is issued.
__global__ void __launch_bounds__(32, 1) wait_selftest(uint64_t limit_ns, int *status) {
  __shared__ __align__(8) uint64_t bar;
  __shared__ uint32_t tmem_slot;
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    fence_mbar_init();
  }
  tmem_alloc(&tmem_slot, 32);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_slot;
  const bool ok = __all_sync(0xffffffffu, mbar_wait(&bar, 0, limit_ns));
  if (!ok && threadIdx.x == 0) atomicExch(status, DS_SPIN_LIMIT);
  tc_fence_before();
  __syncthreads();
  tmem_dealloc(tmem, 32);
}

// Sum of a seed's pieces (fixed order), then the mean-shift step; a seed
// leaves the bulk (kNear: the FP32 polish takes it on with Newton steps)
// when its squared move falls under kSwitch2 h^2.
__global__ void __launch_bounds__(256) ms_update_bulk(float *means, const float *partial,
                                                       const uint32_t *pieces, const int32_t *ids,
                                                       const unsigned *nact, float h2,
                                                       uint8_t *state) {
  // one warp per seed: the lanes stride over the tile's pieces, a fixed
  // butterfly sums them, lane 0 takes the step
  const uint64_t slot = uint64_t(blockIdx.x) * 8 + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (slot >= nact[0]) return;  // whole warp
  const int32_t s = ids[slot];
  const uint64_t tile = slot / kChunk, row = slot % kChunk;
  float acc[7] = {0, 0, 0, 0, 0, 0, 0};
  for (uint32_t p = pieces[tile] + lane; p < pieces[tile + 1]; p += 32)
    for (int d = 0; d < 7; ++d) acc[d] += partial[(uint64_t(p) * 8 + d) * kChunk + row];
  for (int d = 0; d < 7; ++d)
    for (int o = 16; o; o >>= 1) acc[d] += __shfl_xor_sync(0xffffffffu, acc[d], o);
  if (lane != 0) return;
  if (acc[6] <= 1e-14f) {
    state[s] = kExhausted;
    return;
  }
  float move = 0;
  for (int d = 0; d < 6; ++d) {
    float nx = acc[d] / acc[6];
    float e = means[uint64_t(s) * 8 + d] - nx;
    move += e * e;
    means[uint64_t(s) * 8 + d] = nx;
  }
  if (move < float(kSwitch2) * h2) state[s] = kNear;
}

}  // namespace

bool meanshift_bf16_bulk(Call &call, const VoteSet &v, float *means, uint8_t *state, uint64_t k,
                         double h2, int max_iter, int *iterations, double *evaluations,
                         uint32_t *trace, int trace_len, double *kernel_ms,
                         uint64_t *kernel_launches, double *seed_iterations) {
  *iterations = 0;
  *evaluations = 0;
  if (kernel_ms) *kernel_ms = 0;
  if (kernel_launches) *kernel_launches = 0;
  if (!k || !v.q) return false;
  const uint64_t max_tiles = (k + kChunk - 1) / kChunk;
  if (max_tiles * v.nchunks >= (uint64_t(1) << 31)) return false;  // list entries are int32
  cudaStream_t st = call.stream();
  // once per process (thread-safe: calls from several host threads may race)
  static const bool configured = [] {
    SYM_CUDA(cudaFuncSetAttribute(ms_tile_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, kTcSmem));
    return true;
  }();
  (void)configured;
  uint8_t *images = call.alloc<uint8_t>(v.nchunks * kImage);
  build_images<<<unsigned(v.nchunks), kChunk, 0, st>>>(v.desc, v.q, v.nchunks, v.cbox, v.gbox,
                                                       float(1.0 / std::sqrt(h2)), images);
  check_launch();
  int32_t *ids = call.alloc<int32_t>(k);
  float *boxes = call.alloc<float>(max_tiles * kBoxFloats);
  const uint32_t nblk = uint32_t(v.nblocks);
  uint8_t *need = call.alloc<uint8_t>(max_tiles * v.nchunks);
  uint32_t *bcount = call.alloc<uint32_t>(max_tiles * nblk), *boff = call.alloc<uint32_t>(max_tiles * nblk);
  uint32_t *sblk = call.alloc<uint32_t>(max_tiles * nblk), *nsurv = call.alloc<uint32_t>(max_tiles);
  uint32_t *seg = call.alloc<uint32_t>(max_tiles + 1);
  const uint64_t list_cap = max_tiles * v.nchunks;
  int32_t *list = call.alloc<int32_t>(list_cap);
  // CTAs of the list kernels, shared among the active tiles at run time:
  // one full wave of the GPU at their occupancy
  static const int list_per_sm = [] {
    int a = 0, b = 0;
    SYM_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&a, tile_count, kListThreads, 0));
    SYM_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, scatter_lists, kListThreads, 0));
    return std::max(1, std::min(a, b));
  }();
  const unsigned list_ctas = unsigned(std::max<uint64_t>(max_tiles, uint64_t(152) * list_per_sm));
  uint64_t *offsets = call.alloc<uint64_t>(max_tiles + 1);
  uint32_t *pieces = call.alloc<uint32_t>(max_tiles + 1);
  // budget + tiles CTAs: tc_ctas_per_sm waves of the 152 SMs
  const uint32_t sms = 152 * uint32_t(v.tuning.tc_ctas_per_sm);
  const uint64_t max_grid = std::max<uint64_t>(sms, 2 * max_tiles);
  float *partial = call.alloc<float>(max_grid * kChunk * 8);
  unsigned *nact = call.alloc<unsigned>(2), *iter = call.alloc<unsigned>(1);
  const unsigned trace_cap = unsigned(std::max(max_iter, 1));
  uint32_t *trace_dev = call.alloc<uint32_t>(trace_cap);
  unsigned long long *evals = call.alloc<unsigned long long>(1);
  SYM_CUDA(cudaMemsetAsync(evals, 0, 8, st));
  SYM_CUDA(cudaMemsetAsync(iter, 0, 4, st));
  const float gap = float(std::sqrt(h2)) + 1e-6f;
  call.launched();
  TcArgs args{images, v.nchunks, list, offsets, pieces, nact, means, ids, v.gbox,
              float(1.0 / std::sqrt(h2)), float(v.kernel_k), partial, evals, call.status()};
  // CUDA events around every launch of the tensor kernel (its own time)
  std::vector<cudaEvent_t> marks;
  auto mark_event = [&]() {
    cudaEvent_t e;
    SYM_CUDA(cudaEventCreate(&e));
    SYM_CUDA(cudaEventRecord(e, st));
    marks.push_back(e);
  };
  // Iterations are launched back to back: each reads the active-seed count
  // that the previous one left on the device, and one whose count is zero
  // returns at once.  The host looks at the count every kCheck iterations.
  const int kCheck = v.tuning.check_interval;
  int it = 0;
  for (; it < max_iter; ++it) {
    active_seeds_async(call, v, means, state, k, ids, nact, iter, trace_dev, trace_cap);
    tile_boxes<<<unsigned(max_tiles), kCullThreads, 0, st>>>(means, ids, nact, v.bbox, nblk,
                                                              gap * gap, boxes, sblk, nsurv, bcount);
    check_launch();
    tile_count<<<list_ctas, kListThreads, 0, st>>>(boxes, means, ids, nact, v.cbox, v.bbox,
                                                   v.nchunks, sblk, nsurv, nblk, gap * gap, need,
                                                   bcount);
    check_launch();
    scan_lists<<<1, 1024, 0, st>>>(bcount, nsurv, nact, nblk, sms, list_cap, seg, boff, offsets,
                                   pieces, call.status());
    check_launch();
    scatter_lists<<<list_ctas, kListThreads, 0, st>>>(need, boff, bcount, sblk, nsurv, nblk, nact,
                                                      v.nchunks, list_cap, list, call.status());
    check_launch();
    if (kernel_ms) mark_event();
    ms_tile_tc<<<unsigned(max_grid), kThreadsTc, kTcSmem, st>>>(args);
    check_launch();
    if (kernel_ms) mark_event();
    ms_update_bulk<<<unsigned((k + 7) / 8), 256, 0, st>>>(means, partial, pieces, ids, nact,
                                                          float(h2), state);
    check_launch();
    call.launched(6);
    if (it % kCheck == kCheck - 1) {
      unsigned n = 0;
      call.d2h(&n, nact, sizeof(unsigned));
      call.sync();
      if (!n) {
        ++it;
        break;
      }
    }
  }
  call.check_status("mean_shift (tensor)");
  unsigned long long ev = 0;
  unsigned active_iterations = 0;
  call.d2h(&ev, evals, 8);
  call.d2h(&active_iterations, iter, sizeof(unsigned));
  call.sync();
  *iterations = int(active_iterations);
  *evaluations = double(ev);
  if ((trace && trace_len > 0) || seed_iterations) {
    std::vector<uint32_t> tr(trace_cap);
    call.d2h(tr.data(), trace_dev, trace_cap * sizeof(uint32_t));
    call.sync();
    for (int i = 0; trace && i < trace_len && i < int(active_iterations) && i < int(trace_cap); ++i)
      trace[i] = tr[i];
    // every iteration with active seeds is recorded (trace_cap = max_iter)
    for (unsigned i = 0; seed_iterations && i < active_iterations && i < trace_cap; ++i)
      *seed_iterations += tr[i];
  }
  // launches after the last iteration with active seeds found none and
  // returned at once: only the active ones are timed
  for (size_t i = 0; i + 1 < marks.size() && i / 2 < active_iterations; i += 2) {
    float ms = 0;
    SYM_CUDA(cudaEventElapsedTime(&ms, marks[i], marks[i + 1]));
    *kernel_ms += ms;
  }
  if (kernel_launches) *kernel_launches = std::min<uint64_t>(marks.size() / 2, active_iterations);
  for (auto e : marks) cudaEventDestroy(e);
  return true;
}

void wait_selftest_host(Call &call, uint64_t limit_ns) {
  wait_selftest<<<1, 32, 0, call.stream()>>>(limit_ns, call.status());
  check_launch();
  call.launched();
  call.check_status("tensor-kernel wait self-test");
}

void tc_selftest_host(Call &call, const uint16_t *a1, const uint16_t *b1, const uint16_t *a2,
                      const uint16_t *b2, float *d_out, float *acc_out) {
  static const bool configured = [] {
    SYM_CUDA(cudaFuncSetAttribute(tc_selftest, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  kSmemRequest));
    return true;
  }();
  (void)configured;
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
