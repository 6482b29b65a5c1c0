// Exhaustive k-NN with a tensor-core pre-selection: the precision path of the
// linear search over float objects.
//
// The reference's exhaustive search (ObjectSpaceRepository::linearSearch,
// lib/NGT/ObjectSpaceRepository.h:860-922) compares the query with every
// object and keeps the `size` smallest (distance, id) keys.  Here the bulk of
// that work is a dense product Q x X^T on the tensor cores:
//
//   1. every row x gets a bf16 copy (K padded to a multiple of 64) and an
//      affine pair (a, b) so that score = a * (q . x) + b orders rows like the
//      metric does (larger score = closer):
//        L2, normalized L2, inner product (L2 over the augmented rows):
//            a = 1, b = -|x|^2 / 2          (|q - x|^2 = |q|^2 - 2 (q.x - |x|^2/2))
//        cosine, angle:                     a = 1 / |x|, b = 0
//        normalized cosine, normalized angle: a = 1, b = 0 (rows are unit length)
//   2. tc_score_kernel: bf16 x bf16 -> fp32 GEMM with tcgen05.mma (M = 128 rows,
//      N = 256 queries, K = 16 per instruction), operands staged by TMA
//      (cp.async.bulk.tensor, 128-byte swizzle) through a 4-stage mbarrier
//      pipeline, accumulators double-buffered in TMEM (2 x 256 columns) and
//      read back with tcgen05.ld by sixteen epilogue warps (four per TMEM lane
//      quadrant).  The first `first_rows` rows are written out densely; on the
//      remaining rows, taken in parts that double in size, the epilogue keeps
//      only scores that beat the query's threshold, and tc_compact_kernel cuts
//      each list back to the C best and raises the threshold between two parts.
//      A two-SM form (cta_group::2, M = 256 over a pair of CTAs, each staging
//      its own rows and half of the query tile) gives the same scores.
//   3. tc_first_select_kernel: per query, the C best scores of the dense part
//      (exact radix select on 64-bit (score key, row) keys); the C-th becomes
//      the threshold, and the C keys the first candidates.  Every row past the
//      dense part has a larger id, so a row whose score key equals the
//      threshold's can never displace it: the filter keeps strictly better keys.
//   4. tc_final_kernel: per query, the C best approximate keys among the
//      candidates (the global top C by approximate score, ties by id), their
//      exact distances with the index's comparator on the fp32 rows (the same
//      lane grouping as the plain linear search, hence the same rounding), a
//      bitonic sort by (distance, id), optionally the FP64 order of the
//      candidates tied at the cut, and the first `size` of them.
//
// The result equals the plain linear search whenever the true `size` nearest
// rows are among the C best approximate scores; the candidate oversampling C
// is the caller's choice.  A query whose candidate list overflowed reports
// status bit 1.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>
#include <cuda_fp8.h>
#include <algorithm>
#include <array>
#include <cfloat>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>
#include "engine.h"
#include "distance.cuh"
#include "kernels.h"

namespace ngtg {

#define TC_CUDA(x)                                                                                  \
  do {                                                                                              \
    cudaError_t e_ = (x);                                                                           \
    if (e_ != cudaSuccess)                                                                          \
      throw std::runtime_error(std::string("CUDA error ") + cudaGetErrorString(e_) + " in " #x);     \
  } while (0)

namespace tc {

constexpr uint32_t BM = 128;            // rows per tile (TMEM lanes)
constexpr uint32_t BN = 256;            // queries per tile (TMEM columns per accumulator)
constexpr uint32_t BK = 64;             // bf16 elements per k-block: one 128-byte swizzle row
constexpr uint32_t STAGES = 4;
constexpr uint32_t A_BYTES = BM * BK * 2;
constexpr uint32_t B_BYTES = BN * BK * 2;
constexpr uint32_t STAGE_BYTES = A_BYTES + B_BYTES;
constexpr uint32_t SMEM_BYTES = STAGES * STAGE_BYTES + 1024;   // + slack for 1024-byte alignment
// The two-SM form (cta_group::2): each CTA of a pair stages its own 128 rows and
// one half (128 queries) of the query tile, 32 KB per k-block, in 6 stages.
constexpr uint32_t STAGES2 = 6;
constexpr uint32_t STAGE2_BYTES = A_BYTES + B_BYTES / 2;
constexpr uint32_t MAX_STAGES = STAGES2 > STAGES ? STAGES2 : STAGES;
static_assert(STAGES2 * STAGE2_BYTES + 1024 <= SMEM_BYTES, "two-SM stages fit the same shared memory");
constexpr uint32_t EPI_WARPS = 16;      // four per TMEM lane quadrant, each a quarter of the columns
constexpr uint32_t EPI_PARTS = EPI_WARPS / 4;
constexpr uint32_t THREADS = 64 + 32 * EPI_WARPS;   // warp 0 TMA, warp 1 MMA, warps 2.. epilogue
constexpr uint32_t TMEM_COLS = 2 * BN;
constexpr uint32_t kInvalidKey = 0xff800000u;   // score key of -inf; valid keys are smaller
constexpr uint64_t kWaitNs = 2000000000ull;     // bound of every wait (2 s)
constexpr int kDeferQueries = 8;                // filter epilogue: see tc_score_kernel

// Instruction descriptor of tcgen05.mma kind::f16: D fp32 (bits 4-5 = 1), A and
// B bf16 (bits 7-9, 10-12 = 1), both K-major (bits 15, 16 = 0), N >> 3 at bits
// 17-22, M >> 4 at bits 24-28.
constexpr uint32_t kIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((BN >> 3) << 17) | ((BM >> 4) << 24);
// kind::f8f6f4 with A and B E4M3 (format 0 at bits 7-9 and 10-12), D fp32.  One MMA
// consumes K = 32 one-byte elements, the same 32 bytes of each 128-byte swizzle
// row as a bf16 MMA's K = 16, so staging, descriptors and k-steps are shared.
constexpr uint32_t kIdescF8 = (1u << 4) | ((BN >> 3) << 17) | ((BM >> 4) << 24);
// The same with M = 256 for a pair of CTAs (cta_group::2): rows 0-127 from the
// first CTA's A tile, 128-255 from the second's; each accumulates its own 128 rows.
constexpr uint32_t kIdesc2 = (kIdesc & ~(0x1Fu << 24)) | (((2 * BM) >> 4) << 24);
constexpr uint32_t kIdescF8_2 = (kIdescF8 & ~(0x1Fu << 24)) | (((2 * BM) >> 4) << 24);
constexpr float kE4M3Max = 448.f;       // largest finite E4M3 value

struct ScoreArgs {
  uint32_t row_begin, row_end;          // rows [row_begin, row_end); row_begin % BM == 0
  uint32_t nq, kblocks;
  const float* row_scale;
  const float* row_bias;
  const uint8_t* present;
  float* dense;                         // dense mode: dense[q * dense_ld + (row - row_begin)]
  uint32_t dense_ld;
  const float* thr;                     // filter mode: keep scores > thr[q]
  unsigned long long* cand;             // [nq][cap] (key << 32 | row)
  uint32_t* cand_count;
  uint32_t cap;
  uint32_t* status;                     // bit 1: candidate list overflow
  uint32_t* error;                      // bit 1: producer wait, 2: MMA wait, 4: epilogue wait ran out
  const float* qscale;                  // fp8 scores: per-query dequantisation scale (bf16: unused)
};

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ uint64_t global_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}
__device__ __forceinline__ bool mbar_try(uint32_t bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ bool mbar_try_cluster(uint32_t bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.acquire.cluster.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}
// Waits until the phase of parity `parity` completed; false when the wait ran
// out (kWaitNs) or another role aborted (abort may be null: no abort check).
__device__ __noinline__ bool mbar_wait(uint32_t bar, uint32_t parity, const volatile uint32_t* abort) {
  if (mbar_try(bar, parity)) return true;
  const uint64_t t0 = global_ns();
  while (true) {
    if (mbar_try(bar, parity)) return true;
    if (abort && *abort) return false;
    if (global_ns() - t0 > kWaitNs) return false;
  }
}
// The same with acquire at cluster scope (arrivals from the other CTA of a pair).
__device__ __noinline__ bool mbar_wait_cluster(uint32_t bar, uint32_t parity, const volatile uint32_t* abort) {
  if (mbar_try_cluster(bar, parity)) return true;
  const uint64_t t0 = global_ns();
  while (true) {
    if (mbar_try_cluster(bar, parity)) return true;
    if (abort && *abort) return false;
    if (global_ns() - t0 > kWaitNs) return false;
  }
}

__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap* map, uint32_t bar, int x, int y) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4}], [%2];"
      ::"r"(dst), "l"(reinterpret_cast<uint64_t>(map)), "r"(bar), "r"(x), "r"(y)
      : "memory");
}

// The same load for a CTA pair (cta_group::2): the box lands in this CTA's shared
// memory and completes on `bar`, a shared::cluster address that may name the
// mbarrier of the other CTA of the pair.
__device__ __forceinline__ void tma_load_2d_pair(uint32_t dst, const CUtensorMap* map, uint32_t bar, int x, int y) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes.cta_group::2"
      " [%0], [%1, {%3, %4}], [%2];"
      ::"r"(dst), "l"(reinterpret_cast<uint64_t>(map)), "r"(bar), "r"(x), "r"(y)
      : "memory");
}
// shared::cluster address of this CTA's shared-memory address `addr` in CTA `rank`.
__device__ __forceinline__ uint32_t map_to_rank(uint32_t addr, uint32_t rank) {
  uint32_t r;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(addr), "r"(rank));
  return r;
}
// Arrive on an mbarrier of any CTA of the cluster (release at cluster scope).
__device__ __forceinline__ void mbar_arrive_cluster(uint32_t bar_cluster) {
  asm volatile("mbarrier.arrive.release.cluster.shared::cluster.b64 _, [%0];" ::"r"(bar_cluster) : "memory");
}
__device__ __forceinline__ uint32_t cluster_ctarank() {
  uint32_t r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}
// Every thread of every CTA of the cluster (all of them execute it, converged).
__device__ __forceinline__ void cluster_sync() {
  asm volatile("barrier.cluster.arrive.release.aligned;\nbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// Shared-memory matrix descriptor of a K-major tile with 128-byte swizzle:
// start address >> 4 (bits 0-13), leading offset 16 B (ignored for swizzled
// K-major), stride 1024 B between 8-row groups (bits 32-45), descriptor version
// 1 (bits 46-47), layout SWIZZLE_128B = 2 (bits 61-63).
__device__ __forceinline__ uint64_t sw128_desc(uint32_t saddr) {
  return (uint64_t)((saddr >> 4) & 0x3FFFu) | ((uint64_t)1 << 16) | ((uint64_t)(1024 >> 4) << 32) |
         ((uint64_t)1 << 46) | ((uint64_t)2 << 61);
}

__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}"
      ::"r"(d_tmem), "l"(adesc), "l"(bdesc), "r"(kIdesc), "r"(accumulate)
      : "memory");
}
__device__ __forceinline__ void mma_f8(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::f8f6f4 [%0], %1, %2, %3, p;\n}"
      ::"r"(d_tmem), "l"(adesc), "l"(bdesc), "r"(kIdescF8), "r"(accumulate)
      : "memory");
}
__device__ __forceinline__ void mma_commit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}

// The CTA-pair forms (every tcgen05 instruction of a kernel has the same
// cta_group): one thread of the pair's first CTA issues the M = 256 MMA, whose
// A and B descriptors name the same shared-memory offsets in both CTAs.
__device__ __forceinline__ void mma_bf16_pair(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::2.kind::f16 [%0], %1, %2, %3, p;\n}"
      ::"r"(d_tmem), "l"(adesc), "l"(bdesc), "r"(kIdesc2), "r"(accumulate)
      : "memory");
}
__device__ __forceinline__ void mma_f8_pair(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::2.kind::f8f6f4 [%0], %1, %2, %3, p;\n}"
      ::"r"(d_tmem), "l"(adesc), "l"(bdesc), "r"(kIdescF8_2), "r"(accumulate)
      : "memory");
}
// Arrive on the mbarrier at offset `bar` of both CTAs of the pair when the
// pair's MMAs issued so far have completed.
__device__ __forceinline__ void mma_commit_pair_both(uint32_t bar) {
  asm volatile(
      "tcgen05.commit.cta_group::2.mbarrier::arrive::one.shared::cluster.multicast::cluster.b64 [%0], %1;"
      ::"r"(bar), "h"((uint16_t)3)
      : "memory");
}
__device__ __forceinline__ void mma_commit_pair_local(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::2.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}

// 32 consecutive fp32 columns of this warp's 32 TMEM lanes, one lane per thread.
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t (&v)[32]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
      "%15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
      : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
        "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15]),
        "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]), "=r"(v[22]), "=r"(v[23]),
        "=r"(v[24]), "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
      : "r"(taddr));
}
// Waits for the loads above; the registers are operands so that no use of them
// is scheduled before the wait.
__device__ __forceinline__ void tmem_ld_wait(uint32_t (&v)[32]) {
  asm volatile("tcgen05.wait::ld.sync.aligned;"
               : "+r"(v[0]), "+r"(v[1]), "+r"(v[2]), "+r"(v[3]), "+r"(v[4]), "+r"(v[5]), "+r"(v[6]), "+r"(v[7]),
                 "+r"(v[8]), "+r"(v[9]), "+r"(v[10]), "+r"(v[11]), "+r"(v[12]), "+r"(v[13]), "+r"(v[14]),
                 "+r"(v[15]), "+r"(v[16]), "+r"(v[17]), "+r"(v[18]), "+r"(v[19]), "+r"(v[20]), "+r"(v[21]),
                 "+r"(v[22]), "+r"(v[23]), "+r"(v[24]), "+r"(v[25]), "+r"(v[26]), "+r"(v[27]), "+r"(v[28]),
                 "+r"(v[29]), "+r"(v[30]), "+r"(v[31])
               :
               : "memory");
}

// One fp32 column of this warp's 32 TMEM lanes, one lane per thread, loaded and waited for.
__device__ __forceinline__ uint32_t tmem_ld1(uint32_t taddr) {
  uint32_t r;
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x1.b32 {%0}, [%1];\n\ttcgen05.wait::ld.sync.aligned;"
               : "=r"(r)
               : "r"(taddr)
               : "memory");
  return r;
}

// Larger score -> smaller key (unsigned order); NaN and -inf -> kInvalidKey or
// above.  -0 is folded to +0, so that "key < key(t)" and "s > t" agree.
__device__ __forceinline__ uint32_t score_key(float s) {
  if (s != s) return 0xffffffffu;
  uint32_t f = __float_as_uint(s + 0.0f);
  uint32_t asc = (f & 0x80000000u) ? ~f : (f | 0x80000000u);
  return ~asc;
}
// The score of a key (inverse of score_key on valid keys).
__device__ __forceinline__ float key_score(uint32_t key) {
  const uint32_t asc = ~key;
  return __uint_as_float((asc & 0x80000000u) ? (asc & 0x7fffffffu) : ~asc);
}

// kFp8: A (rows) and B (queries) hold per-row / per-query scaled E4M3 values; the
// accumulator is multiplied by the query's scale in the epilogue (the row's scale
// is folded into row_scale).
// kPair: the CTAs run in pairs (clusters of two) on the two-SM MMA: a work unit is
// row tiles 2i and 2i+1 of one query tile.  Each CTA stages its own row tile and
// one half of the query tile (128 queries); the first CTA's MMA thread issues
// M = 256 x N = 256 MMAs over both CTAs' shared memory, each CTA's TMEM holding
// its own rows' accumulator.  Both CTAs' copies complete on the first CTA's
// stage barrier; the MMA commits arrive on both CTAs' stage-empty and
// accumulator-full barriers; both CTAs' epilogue warps arrive on the first
// CTA's accumulator-empty barrier.
template <bool kDense, bool kFp8, bool kPair>
__global__ void __launch_bounds__(THREADS, 1)
tc_score_kernel(const __grid_constant__ CUtensorMap mapA, const __grid_constant__ CUtensorMap mapB, ScoreArgs a) {
  constexpr uint32_t NST = kPair ? STAGES2 : STAGES;
  constexpr uint32_t SBYTES = kPair ? STAGE2_BYTES : STAGE_BYTES;
  extern __shared__ __align__(1024) unsigned char dsmem[];
  __shared__ __align__(8) uint64_t bar_full[MAX_STAGES], bar_empty[MAX_STAGES], bar_tfull[2], bar_tempty[2], bar_drain;
  __shared__ uint32_t tmem_base_sh;
  __shared__ volatile uint32_t abort_sh;
  const uint32_t base = (smem_u32(dsmem) + 1023u) & ~1023u;
  const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint32_t mtiles = (a.row_end - a.row_begin + BM - 1) / BM;
  const uint32_t ntiles = (a.nq + BN - 1) / BN;
  // work units: tiles, or (kPair) pairs of row tiles of one query tile per CTA pair
  const uint32_t rank = kPair ? cluster_ctarank() : 0u;
  const uint32_t unit0 = kPair ? blockIdx.x >> 1 : blockIdx.x;
  const uint32_t ustep = kPair ? gridDim.x >> 1 : gridDim.x;
  const uint32_t units = kPair ? (mtiles + 1) / 2 * ntiles : mtiles * ntiles;
  // row tile of work unit u (the query tile is u % ntiles)
  auto row_tile = [&](uint32_t u) { return kPair ? 2 * (u / ntiles) + rank : u / ntiles; };

  if (threadIdx.x == 0) {
    for (uint32_t s = 0; s < NST; s++) {
      mbar_init(smem_u32(&bar_full[s]), 1);
      mbar_init(smem_u32(&bar_empty[s]), 1);
    }
    for (uint32_t b = 0; b < 2; b++) {
      mbar_init(smem_u32(&bar_tfull[b]), 1);
      // one arrival per epilogue thread, or (kPair) per epilogue warp of both CTAs
      mbar_init(smem_u32(&bar_tempty[b]), kPair ? 2 * EPI_WARPS : 32 * EPI_WARPS);
    }
    mbar_init(smem_u32(&bar_drain), 1);
    abort_sh = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    if constexpr (kPair) {
      // one warp of each CTA of the pair allocates collectively: the same columns in both
      asm volatile("tcgen05.alloc.cta_group::2.sync.aligned.shared::cta.b32 [%0], %1;"
                   ::"r"(smem_u32(&tmem_base_sh)), "r"(TMEM_COLS)
                   : "memory");
      asm volatile("tcgen05.relinquish_alloc_permit.cta_group::2.sync.aligned;" ::: "memory");
    } else {
      asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                   ::"r"(smem_u32(&tmem_base_sh)), "r"(TMEM_COLS)
                   : "memory");
      asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if constexpr (kPair) cluster_sync();        // both CTAs' barriers exist before any remote arrive
  const uint32_t tmem = tmem_base_sh;

  if (warp == 0) {
    if (lane == 0) {
      // TMA producer
      uint32_t stage = 0, phase = 0;
      uint32_t pending = 0, last_parity = 0;     // per stage: a load in flight, parity of its phase
      for (uint32_t t = unit0; t < units && !abort_sh; t += ustep) {
        const int row0 = (int)(a.row_begin + row_tile(t) * BM);
        const int q0 = (int)((t % ntiles) * BN);
        for (uint32_t kb = 0; kb < a.kblocks; kb++) {
          if (!mbar_wait(smem_u32(&bar_empty[stage]), phase ^ 1u, &abort_sh)) {
            atomicOr(a.error, 1u);
            abort_sh = 1;
            break;
          }
          const uint32_t sA = base + stage * SBYTES, sB = sA + A_BYTES;
          const uint32_t fb = smem_u32(&bar_full[stage]);
          if constexpr (kPair) {
            // both CTAs' copies complete on the first CTA's stage barrier
            if (rank == 0) mbar_expect_tx(fb, 2 * STAGE2_BYTES);
            const uint32_t fb0 = map_to_rank(fb, 0);
            tma_load_2d_pair(sA, &mapA, fb0, (int)(kb * BK), row0);
            tma_load_2d_pair(sB, &mapB, fb0, (int)(kb * BK), q0 + (int)(rank * (BN / 2)));
          } else {
            mbar_expect_tx(fb, STAGE_BYTES);
            tma_load_2d(sA, &mapA, fb, (int)(kb * BK), row0);
            tma_load_2d(sB, &mapB, fb, (int)(kb * BK), q0);
          }
          pending |= 1u << stage;
          last_parity = (last_parity & ~(1u << stage)) | (phase << stage);
          if (++stage == NST) {
            stage = 0;
            phase ^= 1u;
          }
        }
      }
      // no copy may land in shared memory after the CTA exits: wait for the last
      // phase of each stage used (kPair: its consumption, which follows the copies)
      for (uint32_t s = 0; s < NST; s++) {
        if (!(pending & (1u << s))) continue;
        if constexpr (kPair)
          mbar_wait(smem_u32(&bar_empty[s]), (last_parity >> s) & 1u, nullptr);
        else
          mbar_wait(smem_u32(&bar_full[s]), (last_parity >> s) & 1u, nullptr);
      }
    }
  } else if (warp == 1) {
    if (lane == 0 && rank == 0) {
      // MMA issuer (kPair: the first CTA's, for both)
      uint32_t stage = 0, phase = 0, local = 0;
      for (uint32_t t = unit0; t < units && !abort_sh; t += ustep, local++) {
        const uint32_t buf = local & 1u, tphase = (local >> 1) & 1u;
        const bool ready = kPair ? mbar_wait_cluster(smem_u32(&bar_tempty[buf]), tphase ^ 1u, &abort_sh)
                                 : mbar_wait(smem_u32(&bar_tempty[buf]), tphase ^ 1u, &abort_sh);
        if (!ready) {
          atomicOr(a.error, 2u);
          abort_sh = 1;
          break;
        }
        tc_fence_after();
        const uint32_t d = tmem + buf * BN;
        bool ok = true;
        for (uint32_t kb = 0; kb < a.kblocks; kb++) {
          if (!mbar_wait(smem_u32(&bar_full[stage]), phase, &abort_sh)) {
            atomicOr(a.error, 2u);
            abort_sh = 1;
            ok = false;
            break;
          }
          tc_fence_after();
          const uint32_t sA = base + stage * SBYTES, sB = sA + A_BYTES;
#pragma unroll
          for (uint32_t k = 0; k < BK / 16; k++) {
            const uint64_t da = sw128_desc(sA + k * 32), db = sw128_desc(sB + k * 32);
            const uint32_t acc = (kb | k) != 0 ? 1u : 0u;
            if constexpr (kPair && kFp8) mma_f8_pair(d, da, db, acc);
            else if constexpr (kPair) mma_bf16_pair(d, da, db, acc);
            else if constexpr (kFp8) mma_f8(d, da, db, acc);
            else mma_bf16(d, da, db, acc);
          }
          if constexpr (kPair) mma_commit_pair_both(smem_u32(&bar_empty[stage]));
          else mma_commit(smem_u32(&bar_empty[stage]));
          if (++stage == NST) {
            stage = 0;
            phase ^= 1u;
          }
        }
        if (!ok) break;
        if constexpr (kPair) mma_commit_pair_both(smem_u32(&bar_tfull[buf]));
        else mma_commit(smem_u32(&bar_tfull[buf]));
      }
      // every MMA issued has completed before TMEM is released
      if constexpr (kPair) mma_commit_pair_local(smem_u32(&bar_drain));
      else mma_commit(smem_u32(&bar_drain));
      mbar_wait(smem_u32(&bar_drain), 0, nullptr);
    }
  } else {
    // epilogue: warp w reads TMEM lanes 32 * (w % 4) .. + 31 (one row per
    // thread) and one of EPI_PARTS column ranges of the 256 columns
    const uint32_t quad = warp & 3u;
    const uint32_t part = (warp - 2u) >> 2;
    uint32_t local = 0;
    for (uint32_t t = unit0; t < units; t += ustep, local++) {
      const uint32_t buf = local & 1u, tphase = (local >> 1) & 1u;
      // what does not depend on the accumulator is loaded before the wait
      const uint32_t row0 = a.row_begin + row_tile(t) * BM;
      const uint32_t q0 = (t % ntiles) * BN;
      const uint32_t row = row0 + quad * 32 + lane;
      const bool in_range = row < a.row_end;
      const bool rvalid = in_range && row != 0 && a.present[row];
      const float sc = rvalid ? a.row_scale[row] : 0.f;
      const float bi = rvalid ? a.row_bias[row] : 0.f;
      // per chunk of 32 queries of this warp's columns: lane j holds the
      // threshold (+inf past the last query) and the scale of query qb + j
      constexpr uint32_t CH = BN / (32 * EPI_PARTS);
      static_assert(CH * 32 * EPI_PARTS == BN, "whole chunks of 32 queries per epilogue warp");
      float thr_c[CH], qs_c[CH];
#pragma unroll
      for (uint32_t i = 0; i < CH; i++) {
        const uint32_t qj = q0 + (part * CH + i) * 32 + lane;
        thr_c[i] = (!kDense && qj < a.nq) ? __ldg(a.thr + qj) : INFINITY;
        qs_c[i] = (kFp8 && qj < a.nq) ? __ldg(a.qscale + qj) : 1.f;
      }
      uint32_t ok = 1;
      if (lane == 0) ok = mbar_wait(smem_u32(&bar_tfull[buf]), tphase, &abort_sh) ? 1u : 0u;
      ok = __shfl_sync(0xffffffffu, ok, 0);     // the warp stays converged for tcgen05.ld
      if (!ok) {
        if (lane == 0) atomicOr(a.error, 4u);
        abort_sh = 1;
        break;
      }
      tc_fence_after();
      // this warp's first TMEM column: lanes 32 * quad.., its column range
      const uint32_t tcol = tmem + ((quad * 32u) << 16) + buf * BN + part * CH * 32;
      // rolled loops over the chunks keep the epilogue's code small (per-chunk
      // values shift down into index 0 of their arrays)
      if constexpr (kDense) {
#pragma unroll 1
        for (uint32_t i = 0; i < CH; i++) {
          const uint32_t qb = q0 + (part * CH + i) * 32;
          if (qb >= a.nq) break;                 // warp-uniform
          const float qs = qs_c[0];
#pragma unroll
          for (uint32_t c = 0; c + 1 < CH; c++) qs_c[c] = qs_c[c + 1];
          uint32_t v[32];
          tmem_ld32(tcol + i * 32, v);
          tmem_ld_wait(v);
#pragma unroll
          for (uint32_t j = 0; j < 32; j++) {
            const uint32_t q = qb + j;
            // the shuffle runs on every lane of the warp, whatever its row
            const float scj = kFp8 ? sc * __shfl_sync(0xffffffffu, qs, j) : sc;
            const float s = fmaf(__uint_as_float(v[j]), scj, bi) + 0.0f;
            if (in_range && q < a.nq) a.dense[(size_t)q * a.dense_ld + (row - a.row_begin)] = rvalid ? s : -INFINITY;
          }
        }
      } else {
        // Pass 1 over the chunks: the filter.  A chunk where more than
        // kDeferQueries queries have passing rows stores its entries at once (one
        // atomic per query, all 32 queries in one warp-wide step).  Otherwise each
        // such query gets one atomic that reserves its rows' slots, issued without
        // waiting for its result, and pass 2 reads that query's score column again
        // from TMEM and stores the (key, row) entries: the tile's atomics are in
        // flight together instead of one round trip per chunk.
        float qs_k[CH];
        uint32_t pass_c[CH] = {}, base_c[CH] = {}, any_c[CH] = {};
#pragma unroll
        for (uint32_t c = 0; c < CH; c++) qs_k[c] = qs_c[c];
#pragma unroll 1
        for (uint32_t i = 0; i < CH; i++) {
          const uint32_t qb = q0 + (part * CH + i) * 32;
          const float thr = thr_c[0], qs = qs_c[0];
#pragma unroll
          for (uint32_t c = 0; c + 1 < CH; c++) {
            thr_c[c] = thr_c[c + 1];
            qs_c[c] = qs_c[c + 1];
          }
          uint32_t v[32];
          tmem_ld32(tcol + i * 32, v);
          tmem_ld_wait(v);
          // passed: the queries of the chunk whose threshold this lane's row
          // passes (none past the last query: its threshold is +inf)
          uint32_t passed = 0;
#pragma unroll
          for (uint32_t j = 0; j < 32; j++) {
            const float t = __shfl_sync(0xffffffffu, thr, j);
            const float scj = kFp8 ? sc * __shfl_sync(0xffffffffu, qs, j) : sc;
            const float s = fmaf(__uint_as_float(v[j]), scj, bi);
            passed |= (rvalid && s > t) ? 1u << j : 0u;
          }
          uint32_t qany = __reduce_or_sync(0xffffffffu, passed);
          uint32_t base = 0;                     // lane j: first reserved slot of query qb + j
          if (__popc(qany) > kDeferQueries) {
            // many queries pass (the first parts): all 32 served at once, now.
            // mine (lane j): the rows that pass query qb + j; one atomic per lane
            uint32_t mine = 0;
#pragma unroll
            for (uint32_t j = 0; j < 32; j++) {
              const uint32_t m = __ballot_sync(0xffffffffu, (passed >> j) & 1u);
              mine = lane == j ? m : mine;
            }
            if (mine != 0u) base = atomicAdd(a.cand_count + qb + lane, (uint32_t)__popc(mine));
            const uint32_t below = (1u << lane) - 1u;
#pragma unroll
            for (uint32_t j = 0; j < 32; j++) {
              const uint32_t mj = __shfl_sync(0xffffffffu, mine, j);
              const uint32_t bj = __shfl_sync(0xffffffffu, base, j);
              const float scj = kFp8 ? sc * __shfl_sync(0xffffffffu, qs, j) : sc;
              if ((passed >> j) & 1u) {
                const uint32_t q = qb + j;
                const uint32_t slot = bj + (uint32_t)__popc(mj & below);
                const float s = fmaf(__uint_as_float(v[j]), scj, bi);
                if (slot < a.cap)
                  a.cand[(size_t)q * a.cap + slot] = ((unsigned long long)score_key(s) << 32) | row;
                else
                  atomicOr(a.status + q, 1u);
              }
            }
            qany = 0;                            // nothing left for pass 2
          } else {
            for (uint32_t bits = qany; bits != 0u; bits &= bits - 1u) {
              const uint32_t j = (uint32_t)__ffs(bits) - 1u;
              const uint32_t m = __ballot_sync(0xffffffffu, (passed >> j) & 1u);
              if (lane == j) base = atomicAdd(a.cand_count + qb + j, (uint32_t)__popc(m));
            }
          }
#pragma unroll
          for (uint32_t c = 0; c + 1 < CH; c++) {
            pass_c[c] = pass_c[c + 1];
            base_c[c] = base_c[c + 1];
            any_c[c] = any_c[c + 1];
          }
          pass_c[CH - 1] = passed;
          base_c[CH - 1] = base;
          any_c[CH - 1] = qany;
        }
        const uint32_t below = (1u << lane) - 1u;
#pragma unroll 1
        for (uint32_t i = 0; i < CH; i++) {
          const uint32_t passed = pass_c[0], base = base_c[0], qany = any_c[0];
          const float qs = qs_k[0];
#pragma unroll
          for (uint32_t c = 0; c + 1 < CH; c++) {
            pass_c[c] = pass_c[c + 1];
            base_c[c] = base_c[c + 1];
            any_c[c] = any_c[c + 1];
            qs_k[c] = qs_k[c + 1];
          }
          const uint32_t qb = q0 + (part * CH + i) * 32;
          for (uint32_t bits = qany; bits != 0u; bits &= bits - 1u) {
            const uint32_t j = (uint32_t)__ffs(bits) - 1u;
            const uint32_t m = __ballot_sync(0xffffffffu, (passed >> j) & 1u);
            const uint32_t bj = __shfl_sync(0xffffffffu, base, j);
            const float scj = kFp8 ? sc * __shfl_sync(0xffffffffu, qs, j) : sc;
            const uint32_t raw = tmem_ld1(tcol + i * 32 + j);
            if ((passed >> j) & 1u) {
              const uint32_t q = qb + j;
              const uint32_t slot = bj + (uint32_t)__popc(m & below);
              const float s = fmaf(__uint_as_float(raw), scj, bi);
              if (slot < a.cap)
                a.cand[(size_t)q * a.cap + slot] = ((unsigned long long)score_key(s) << 32) | row;
              else
                atomicOr(a.status + q, 1u);
            }
          }
        }
      }
      tc_fence_before();
      if constexpr (kPair) {
        // the warp's TMEM loads are complete (tcgen05.wait::ld); lane 0 tells the MMA CTA
        __syncwarp();
        if (lane == 0) mbar_arrive_cluster(map_to_rank(smem_u32(&bar_tempty[buf]), 0));
      } else {
        mbar_arrive(smem_u32(&bar_tempty[buf]));
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  // kPair: the first CTA's MMAs into this CTA's TMEM, its commits on this CTA's
  // barriers and this CTA's arrivals on its barriers are over before either leaves
  if constexpr (kPair) cluster_sync();
  if (warp == 1) {
    tc_fence_after();
    if constexpr (kPair)
      asm volatile("tcgen05.dealloc.cta_group::2.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS) : "memory");
    else
      asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS) : "memory");
  }
}

// The k-th smallest (1-based, 1 <= k <= n) of n distinct 64-bit keys in shared
// memory: up to eight 8-bit radix passes (warp 0 scans the 256-bin histogram),
// ended early once the k-th key is the only key with the prefix found so far.
__device__ unsigned long long block_select_u64(const unsigned long long* keys, uint32_t n, uint32_t k,
                                               uint32_t* hist) {
  __shared__ unsigned long long sh_prefix;
  __shared__ uint32_t sh_need, sh_single;
  const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  unsigned long long prefix = 0, mask = 0;
  uint32_t need = k;
  for (int shift = 56; shift >= 0; shift -= 8) {
    for (uint32_t i = threadIdx.x; i < 256; i += blockDim.x) hist[i] = 0;
    __syncthreads();
    for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) {
      const unsigned long long x = keys[i];
      if ((x & mask) == prefix) atomicAdd(&hist[(uint32_t)(x >> shift) & 255u], 1u);
    }
    __syncthreads();
    if (warp == 0) {
      uint32_t c[8], sum = 0;
#pragma unroll
      for (int j = 0; j < 8; j++) {
        c[j] = hist[lane * 8 + j];
        sum += c[j];
      }
      uint32_t incl = sum;
#pragma unroll
      for (int off = 1; off < 32; off <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, incl, off);
        if (lane >= (uint32_t)off) incl += y;
      }
      const uint32_t excl = incl - sum;
      const unsigned here = __ballot_sync(0xffffffffu, excl < need && incl >= need);
      if (lane == (uint32_t)(__ffs(here) - 1)) {
        uint32_t acc = excl, j = 0;
        for (j = 0; j < 7; j++) {
          if (acc + c[j] >= need) break;
          acc += c[j];
        }
        sh_prefix = prefix | ((unsigned long long)(lane * 8 + j) << shift);
        sh_need = need - acc;
        sh_single = c[j] == 1u ? 1u : 0u;
      }
    }
    __syncthreads();
    prefix = sh_prefix;
    need = sh_need;
    mask |= 255ull << shift;
    const bool single = sh_single != 0u && shift > 0;
    __syncthreads();
    if (single) {
      // one key has this prefix: it is the k-th
      for (uint32_t i = threadIdx.x; i < n; i += blockDim.x)
        if ((keys[i] & mask) == prefix) sh_prefix = keys[i];
      __syncthreads();
      const unsigned long long r = sh_prefix;
      __syncthreads();
      return r;
    }
  }
  return prefix;
}

// Per query: the C best keys of the dense part -> first candidates and threshold.
__global__ void __launch_bounds__(512)
tc_first_select_kernel(const float* __restrict__ dense, uint32_t ld, uint32_t nrows, uint32_t C,
                       float* __restrict__ thr, unsigned long long* __restrict__ cand,
                       uint32_t* __restrict__ cand_count, uint32_t cap, uint32_t row_offset) {
  extern __shared__ __align__(16) unsigned char smem[];
  unsigned long long* keys = reinterpret_cast<unsigned long long*>(smem);   // ld
  __shared__ uint32_t hist[256];
  __shared__ uint32_t sh_n, sh_m;
  const uint32_t q = blockIdx.x;
  if (threadIdx.x == 0) sh_n = sh_m = 0;
  __syncthreads();
  const float* S = dense + (size_t)q * ld;
  for (uint32_t r = threadIdx.x; r < nrows; r += blockDim.x) {
    const uint32_t key = score_key(S[r]);
    if (key < kInvalidKey) keys[atomicAdd(&sh_n, 1u)] = ((unsigned long long)key << 32) | (r + row_offset);
  }
  __syncthreads();
  const uint32_t n = sh_n;
  unsigned long long kth = ~0ull;
  if (n > C) kth = block_select_u64(keys, n, C, hist);
  unsigned long long* out = cand + (size_t)q * cap;
  for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) {
    const unsigned long long x = keys[i];
    if (x <= kth) out[atomicAdd(&sh_m, 1u)] = x;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    cand_count[q] = sh_m;
    thr[q] = n > C ? key_score((uint32_t)(kth >> 32)) : -INFINITY;
  }
}

// Per query, between two parts of the filtered rows: the C best candidate keys
// are kept (written back in place) and the threshold moves up to the C-th.  The
// rows still to come have larger ids, so the strict filter stays exact.
__global__ void __launch_bounds__(512)
tc_compact_kernel(unsigned long long* __restrict__ cand, uint32_t* __restrict__ cand_count, uint32_t cap, uint32_t C,
                  float* __restrict__ thr, uint32_t* __restrict__ status) {
  extern __shared__ __align__(16) unsigned char smem[];
  unsigned long long* keys = reinterpret_cast<unsigned long long*>(smem);   // cap
  __shared__ uint32_t hist[256];
  __shared__ uint32_t sh_m;
  const uint32_t q = blockIdx.x;
  uint32_t n = cand_count[q];
  if (n <= C) return;                                   // uniform over the CTA
  if (n > cap) {
    if (threadIdx.x == 0) status[q] |= 1u;
    n = cap;
  }
  unsigned long long* list = cand + (size_t)q * cap;
  for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) keys[i] = list[i];
  if (threadIdx.x == 0) sh_m = 0;
  __syncthreads();
  const unsigned long long kth = block_select_u64(keys, n, C, hist);
  for (uint32_t i = threadIdx.x; i < n; i += blockDim.x)
    if (keys[i] <= kth) list[atomicAdd(&sh_m, 1u)] = keys[i];
  __syncthreads();
  if (threadIdx.x == 0) {
    cand_count[q] = C;
    thr[q] = key_score((uint32_t)(kth >> 32));
  }
}

// Distance between the query row q (shared memory) and object row x in FP64,
// computed by one warp (lanes over the elements; every lane returns the value).
template <Metric M>
__device__ double fp64_distance(const float* q, const float* x, uint32_t n, uint32_t lane) {
  double a = 0.0, b = 0.0, c = 0.0;
  for (uint32_t i = lane; i < n; i += 32) {
    const double u = q[i], v = x[i];
    if constexpr (M == Metric::L2) {
      a += (u - v) * (u - v);
    } else {
      a += u * v;
      b += u * u;
      c += v * v;
    }
  }
  for (int off = 16; off > 0; off >>= 1) {
    a += __shfl_xor_sync(0xffffffffu, a, off);
    b += __shfl_xor_sync(0xffffffffu, b, off);
    c += __shfl_xor_sync(0xffffffffu, c, off);
  }
  if constexpr (M == Metric::L2) return sqrt(a);
  if constexpr (M == Metric::NormalizedL2) return sqrt(fmax(0.0, 2.0 - 2.0 * a));
  if constexpr (M == Metric::NormalizedCosine) return fabs(1.0 - a);
  if constexpr (M == Metric::Cosine) return fabs(1.0 - a / sqrt(b * c));
  const double cs = M == Metric::Angle ? a / sqrt(b * c) : a;
  return cs >= 1.0 ? 0.0 : cs <= -1.0 ? acos(-1.0) : acos(cs);
}

constexpr uint32_t kTieWindow = 64;     // largest tie window the FP64 check resolves

// Per query: top C approximate candidates, exact distances, sorted, first `size`.
// kTies: the FP64 check at the cut.  The fp32 distances of the candidates next to
// the size-th one (within 1e-4 x max(d, 1), well above the fp32 evaluation error
// of these sums) are recomputed in FP64, and the ones that belong to the FP64 top
// `size` are returned in those places (in fp32 (distance, id) order): the returned
// set is then the FP64 ground truth's among the candidates.  A window wider than
// kTieWindow entries keeps the fp32 result and sets status bit 4.
template <Metric M, bool kTies>
__global__ void __launch_bounds__(256)
tc_final_kernel(DevGraph g, const uint4* __restrict__ queries, uint32_t q0, const unsigned long long* __restrict__ cand,
                const uint32_t* __restrict__ cand_count, uint32_t cap, uint32_t C, uint32_t P, uint32_t size,
                uint32_t group, ObjDist* __restrict__ out, uint32_t kmax, uint32_t* __restrict__ out_count,
                uint32_t* __restrict__ status) {
  extern __shared__ __align__(16) unsigned char smem[];
  uint4* qv = reinterpret_cast<uint4*>(smem);                                        // row_chunks
  unsigned long long* keys = reinterpret_cast<unsigned long long*>(qv + g.row_chunks);  // cap
  unsigned long long* sel = keys + cap;                                               // P
  __shared__ uint32_t hist[256];
  __shared__ uint32_t sh_m;
  const uint32_t qi = blockIdx.x, q = q0 + qi;
  const uint32_t rc = g.row_chunks;
  for (uint32_t i = threadIdx.x; i < rc; i += blockDim.x) qv[i] = queries[(size_t)q * rc + i];
  uint32_t n = cand_count[qi];
  if (n > cap) n = cap;
  const unsigned long long* src = cand + (size_t)qi * cap;
  for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) keys[i] = src[i];
  if (threadIdx.x == 0) sh_m = 0;
  __syncthreads();
  unsigned long long kth = ~0ull;
  if (n > C) kth = block_select_u64(keys, n, C, hist);
  for (uint32_t i = threadIdx.x; i < n; i += blockDim.x)
    if (keys[i] <= kth) sel[atomicAdd(&sh_m, 1u)] = keys[i];
  __syncthreads();
  const uint32_t m = sh_m;
  for (uint32_t i = m + threadIdx.x; i < P; i += blockDim.x) sel[i] = ~0ull;
  // exact distances: groups of `group` lanes per row, as the plain linear search
  const int G = (int)group;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int gl = lane & (G - 1);
  const uint32_t gpw = 32 / G, ngroups = blockDim.x / G;
  // each group computes kRows rows at once (their loads in flight together);
  // every row's lanes and summation order are those of group_distance
  constexpr uint32_t kRows = 4;
  for (uint32_t b = warp * gpw * kRows; b < m; b += ngroups * kRows) {
    uint32_t idx[kRows], row[kRows];
    Acc<ObjType::Float, M> acc[kRows];
#pragma unroll
    for (uint32_t r = 0; r < kRows; r++) {
      idx[r] = b + r * gpw + (uint32_t)(lane / G);
      row[r] = idx[r] < m ? (uint32_t)sel[idx[r]] : 0u;
    }
    for (int c = gl; c < (int)rc; c += G) {
      const uint4 qc = qv[c];
#pragma unroll
      for (uint32_t r = 0; r < kRows; r++) acc[r].add(qc, __ldg(g.objects + (size_t)row[r] * rc + c), c);
    }
#pragma unroll
    for (uint32_t r = 0; r < kRows; r++) {
      acc[r].reduce(G);
      const float d = acc[r].finish();
      if (idx[r] < m && gl == 0) sel[idx[r]] = pack_key(d, row[r]);
    }
  }
  __syncthreads();
  // bitonic sort of P keys (P a power of two)
  for (uint32_t k2 = 2; k2 <= P; k2 <<= 1) {
    for (uint32_t j = k2 >> 1; j > 0; j >>= 1) {
      for (uint32_t i = threadIdx.x; i < P; i += blockDim.x) {
        const uint32_t l = i ^ j;
        if (l > i) {
          const unsigned long long x = sel[i], y = sel[l];
          const bool up = (i & k2) == 0;
          if ((x > y) == up) {
            sel[i] = y;
            sel[l] = x;
          }
        }
      }
      __syncthreads();
    }
  }
  const uint32_t kk = min(size, m);
  if constexpr (kTies) {
    __shared__ uint32_t sh_lo, sh_hi;
    __shared__ double wd[kTieWindow];
    __shared__ unsigned long long wk[kTieWindow];
    if (threadIdx.x == 0) {
      sh_lo = sh_hi = kk;
      if (kk > 0 && kk < m) {
        const float dk = key_dist(sel[kk - 1]);
        const float tol = 1e-4f * fmaxf(dk, 1.f);
        uint32_t lo = kk - 1, hi = kk;
        while (lo > 0 && key_dist(sel[lo - 1]) >= dk - tol) lo--;
        while (hi < m && key_dist(sel[hi]) <= dk + tol) hi++;
        if (hi > kk) {                       // the window crosses the cut
          if (hi - lo <= kTieWindow) {
            sh_lo = lo;
            sh_hi = hi;
          } else if (status) {
            status[q] |= 4u;
          }
        }
      }
    }
    __syncthreads();
    const uint32_t lo = sh_lo, hi = sh_hi;
    if (hi > kk) {
      const float* qf = reinterpret_cast<const float*>(qv);
      const uint32_t n = rc * 4;
      for (uint32_t i = lo + warp; i < hi; i += blockDim.x / 32) {
        const uint32_t row = key_id(sel[i]);
        const double d = fp64_distance<M>(qf, reinterpret_cast<const float*>(g.objects + (size_t)row * rc), n,
                                          (uint32_t)lane);
        if (lane == 0) {
          wd[i - lo] = d;
          wk[i - lo] = sel[i];
        }
      }
      __syncthreads();
      if (threadIdx.x == 0) {
        // the (kk - lo) best of the window by (FP64 distance, id) take places lo..kk-1,
        // in their fp32 (distance, id) order
        const uint32_t w = hi - lo, need = kk - lo;
        uint32_t put = lo;
        for (uint32_t i = 0; i < w && put < kk; i++) {
          uint32_t rank = 0;
          for (uint32_t j = 0; j < w; j++)
            rank += (wd[j] < wd[i] || (wd[j] == wd[i] && key_id(wk[j]) < key_id(wk[i]))) ? 1u : 0u;
          if (rank < need) sel[put++] = wk[i];
        }
      }
      __syncthreads();
    }
  }
  for (uint32_t i = threadIdx.x; i < kk; i += blockDim.x)
    out[(size_t)q * kmax + i] = ObjDist{key_id(sel[i]), key_dist(sel[i])};
  if (threadIdx.x == 0) {
    out_count[q] = kk;
    if (status && cand_count[qi] > cap) status[q] |= 1u;
  }
}

// bf16 rows (K padded to kpad) and the affine pair of each row.
__global__ void tc_rows_kernel(const float* __restrict__ x, uint32_t nrows, uint32_t dpad, uint32_t kpad, int mode,
                               __nv_bfloat16* __restrict__ out, float* __restrict__ scale, float* __restrict__ bias) {
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t row = blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5);
  if (row >= nrows) return;
  const float* xr = x + (size_t)row * dpad;
  __nv_bfloat16* o = out + (size_t)row * kpad;
  float n2 = 0.f;
  for (uint32_t c = lane; c < kpad; c += 32) {
    const float v = c < dpad ? xr[c] : 0.f;
    n2 = fmaf(v, v, n2);
    o[c] = __float2bfloat16_rn(v);
  }
  for (int off = 16; off > 0; off >>= 1) n2 += __shfl_xor_sync(0xffffffffu, n2, off);
  if (lane == 0) {
    if (mode == 0) {            // L2 family
      scale[row] = 1.f;
      bias[row] = -0.5f * n2;
    } else if (mode == 1) {     // cosine, angle
      scale[row] = n2 > 0.f ? rsqrtf(n2) : 0.f;
      bias[row] = 0.f;
    } else {                    // rows of unit length
      scale[row] = 1.f;
      bias[row] = 0.f;
    }
  }
}

// Per-row scaled E4M3 rows (K padded to kpad8): row r holds x / s_r with
// s_r = max|x| / 448 (1 for a zero row), rounded to nearest E4M3; scale8[r] = the
// row's affine scale (as in tc_rows_kernel) times s_r, so that the accumulated
// sum times scale8[r] times the query's own scale is the bf16 path's a (q . x).
__global__ void tc_rows8_kernel(const float* __restrict__ x, uint32_t nrows, uint32_t dpad, uint32_t kpad8,
                                const float* __restrict__ scale, uint8_t* __restrict__ out,
                                float* __restrict__ scale8) {
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t row = blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5);
  if (row >= nrows) return;
  const float* xr = x + (size_t)row * dpad;
  float mx = 0.f;
  for (uint32_t c = lane; c < dpad; c += 32) mx = fmaxf(mx, fabsf(xr[c]));
  for (int off = 16; off > 0; off >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, off));
  const float sr = mx > 0.f ? mx / kE4M3Max : 1.f;
  uint8_t* o = out + (size_t)row * kpad8;
  for (uint32_t c = lane; c < kpad8; c += 32)
    o[c] = c < dpad ? (uint8_t)__nv_cvt_float_to_fp8(xr[c] / sr, __NV_SATFINITE, __NV_E4M3) : (uint8_t)0;
  if (lane == 0) scale8[row] = scale[row] * sr;
}

// Per-query scaled E4M3 query rows [nq_pad][kpad8] and their scales (one warp per
// query; rows past nq and columns past dpad are zero).
__global__ void tc_queries8_kernel(const float* __restrict__ rows, uint32_t dpad, uint32_t nq, uint32_t nq_pad,
                                   uint32_t kpad8, uint8_t* __restrict__ out, float* __restrict__ qscale) {
  const uint32_t lane = threadIdx.x & 31;
  for (uint32_t q = blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5); q < nq_pad;
       q += gridDim.x * (blockDim.x / 32)) {
    const float* xr = rows + (size_t)q * dpad;
    float mx = 0.f;
    if (q < nq)
      for (uint32_t c = lane; c < dpad; c += 32) mx = fmaxf(mx, fabsf(xr[c]));
    for (int off = 16; off > 0; off >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, off));
    const float t = mx > 0.f ? mx / kE4M3Max : 1.f;
    uint8_t* o = out + (size_t)q * kpad8;
    for (uint32_t c = lane; c < kpad8; c += 32)
      o[c] = (q < nq && c < dpad) ? (uint8_t)__nv_cvt_float_to_fp8(xr[c] / t, __NV_SATFINITE, __NV_E4M3)
                                  : (uint8_t)0;
    if (lane == 0) qscale[q] = t;
  }
}

// bf16 query rows [nq_pad][kpad]; rows past nq and columns past dpad are zero.
__global__ void tc_queries_kernel(const float* __restrict__ rows, uint32_t dpad, uint32_t nq, uint32_t nq_pad,
                                  uint32_t kpad, __nv_bfloat16* __restrict__ out) {
  const size_t n = (size_t)nq_pad * kpad;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const uint32_t q = (uint32_t)(i / kpad), c = (uint32_t)(i % kpad);
    out[i] = __float2bfloat16_rn(q < nq && c < dpad ? rows[(size_t)q * dpad + c] : 0.f);
  }
}

typedef void (*FinalFn)(DevGraph, const uint4*, uint32_t, const unsigned long long*, const uint32_t*, uint32_t,
                        uint32_t, uint32_t, uint32_t, uint32_t, ObjDist*, uint32_t, uint32_t*, uint32_t*);

template <bool kTies>
FinalFn final_kernel_t(Metric m) {
  switch (m) {
    case Metric::L2: return &tc_final_kernel<Metric::L2, kTies>;
    case Metric::NormalizedL2: return &tc_final_kernel<Metric::NormalizedL2, kTies>;
    case Metric::Cosine: return &tc_final_kernel<Metric::Cosine, kTies>;
    case Metric::Angle: return &tc_final_kernel<Metric::Angle, kTies>;
    case Metric::NormalizedCosine: return &tc_final_kernel<Metric::NormalizedCosine, kTies>;
    case Metric::NormalizedAngle: return &tc_final_kernel<Metric::NormalizedAngle, kTies>;
    default: return nullptr;
  }
}
FinalFn final_kernel(Metric m, bool ties) { return ties ? final_kernel_t<true>(m) : final_kernel_t<false>(m); }

int row_mode(Metric m) {
  switch (m) {
    case Metric::L2:
    case Metric::NormalizedL2:
    case Metric::InnerProduct: return 0;
    case Metric::Cosine:
    case Metric::Angle: return 1;
    case Metric::NormalizedCosine:
    case Metric::NormalizedAngle: return 2;
    default: return -1;
  }
}

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    cudaError_t e = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q);
    if (e != cudaSuccess || q != cudaDriverEntryPointSuccess || p == nullptr)
      throw std::runtime_error("cuTensorMapEncodeTiled is not available from the driver");
    return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  }();
  return fn;
}

// 2-D bf16 tensor map over rows x kpad (row stride kpad * 2 bytes), box
// BK x box_rows, 128-byte swizzle; reads past the last row return zeros.
CUtensorMap make_map(const void* base, uint64_t rows, uint64_t kpad, uint32_t box_rows) {
  CUtensorMap m;
  cuuint64_t dims[2] = {kpad, rows};
  cuuint64_t strides[1] = {kpad * 2};
  cuuint32_t box[2] = {BK, box_rows};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = encode_fn()(&m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(base), dims, strides, box, estr,
                           CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                           CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) throw std::runtime_error("cuTensorMapEncodeTiled failed: " + std::to_string((int)r));
  return m;
}

// The same over E4M3 rows: rows x kpad8 bytes, box 128 x box_rows.
CUtensorMap make_map8(const void* base, uint64_t rows, uint64_t kpad8, uint32_t box_rows) {
  CUtensorMap m;
  cuuint64_t dims[2] = {kpad8, rows};
  cuuint64_t strides[1] = {kpad8};
  cuuint32_t box[2] = {128, box_rows};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = encode_fn()(&m, CU_TENSOR_MAP_DATA_TYPE_UINT8, 2, const_cast<void*>(base), dims, strides, box, estr,
                           CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                           CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) throw std::runtime_error("cuTensorMapEncodeTiled failed: " + std::to_string((int)r));
  return m;
}

uint32_t pow2_at_least(uint32_t v) {
  uint32_t p = 1;
  while (p < v) p <<= 1;
  return p;
}

}  // namespace tc

// Device state of the tensor-core linear search (built on first use).
struct TcState {
  __nv_bfloat16* rows = nullptr;   // [nrows][kpad]
  float* scale = nullptr;
  float* bias = nullptr;
  uint32_t kpad = 0;
  CUtensorMap mapA;
  // per-row scaled E4M3 rows (built on the first fp8 search)
  uint8_t* rows8 = nullptr;        // [nrows][kpad8]
  float* scale8 = nullptr;         // affine scale x the row's E4M3 scale
  uint32_t kpad8 = 0;
  CUtensorMap mapA8;
  // scratch, grown on demand
  void* scratch = nullptr;
  size_t scratch_bytes = 0;
  uint32_t* error = nullptr;
  // phase timing of the last query batch: dense part + selection, filtered
  // part (the score kernel over the remaining rows), final re-rank
  cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
  float phase_ms[3] = {0.f, 0.f, 0.f};
  // captured launch sequences (opt-in): one per shape, buffers and scratch
  struct Graph {
    std::array<uint64_t, 16> key;
    cudaGraphExec_t exec;
    uint64_t launches;
  };
  std::vector<Graph> graphs;
};

void tc_drop_graphs(TcState* s) {
  for (auto& g : s->graphs) cudaGraphExecDestroy(g.exec);
  s->graphs.clear();
}

void tc_release(TcState* s) {
  if (!s) return;
  cudaFree(s->rows);
  cudaFree(s->rows8);
  cudaFree(s->scale8);
  cudaFree(s->scale);
  cudaFree(s->bias);
  cudaFree(s->scratch);
  cudaFree(s->error);
  for (cudaEvent_t e : s->ev)
    if (e) cudaEventDestroy(e);
  tc_drop_graphs(s);
  delete s;
}

bool GraphEngine::tc_supported() const {
  return host_.prop.otype == ObjType::Float && tc::row_mode(host_.prop.metric) >= 0;
}

void GraphEngine::ensure_tc_rows() {
  if (tc_) return;
  if (!tc_supported())
    throw std::runtime_error("the tensor-core linear search needs float objects and an L2, inner-product, cosine or "
                             "angle distance");
  std::unique_ptr<TcState> s(new TcState());
  const uint32_t dpad = host_.dpad;
  s->kpad = (dpad + tc::BK - 1) / tc::BK * tc::BK;
  const size_t nrows = host_.nrows;
  TC_CUDA(cudaMalloc(&s->rows, nrows * s->kpad * 2));
  TC_CUDA(cudaMalloc(&s->scale, nrows * 4));
  TC_CUDA(cudaMalloc(&s->bias, nrows * 4));
  TC_CUDA(cudaMalloc(&s->error, 4));
  for (cudaEvent_t& e : s->ev) TC_CUDA(cudaEventCreate(&e));
  TC_CUDA(cudaMemsetAsync(s->error, 0, 4, stream_));
  const unsigned blocks = (unsigned)((nrows + 7) / 8);
  tc::tc_rows_kernel<<<blocks, 256, 0, stream_>>>(static_cast<const float*>(d_objects_), (uint32_t)nrows, dpad,
                                                  s->kpad, tc::row_mode(host_.prop.metric), s->rows, s->scale,
                                                  s->bias);
  TC_CUDA(cudaGetLastError());
  launches_++;
  s->mapA = tc::make_map(s->rows, nrows, s->kpad, tc::BM);
  TC_CUDA(cudaStreamSynchronize(stream_));
  tc_ = s.release();
}

void GraphEngine::ensure_tc_rows8() {
  ensure_tc_rows();
  TcState& s = *tc_;
  if (s.rows8) return;
  const uint32_t dpad = host_.dpad;
  const uint32_t kpad8 = (dpad + 127) / 128 * 128;
  const size_t nrows = host_.nrows;
  TC_CUDA(cudaMalloc(&s.rows8, nrows * kpad8));
  TC_CUDA(cudaMalloc(&s.scale8, nrows * 4));
  s.kpad8 = kpad8;
  const unsigned blocks = (unsigned)((nrows + 7) / 8);
  tc::tc_rows8_kernel<<<blocks, 256, 0, stream_>>>(static_cast<const float*>(d_objects_), (uint32_t)nrows, dpad,
                                                   kpad8, s.scale, s.rows8, s.scale8);
  TC_CUDA(cudaGetLastError());
  launches_++;
  s.mapA8 = tc::make_map8(s.rows8, nrows, kpad8, tc::BM);
  TC_CUDA(cudaStreamSynchronize(stream_));
}

namespace {

template <bool kFp8, bool kPair>
void launch_scores_t(const CUtensorMap& mapA, const CUtensorMap& mapB, const tc::ScoreArgs& a, bool dense,
                     cudaStream_t s, unsigned grid) {
  auto fn = dense ? tc::tc_score_kernel<true, kFp8, kPair> : tc::tc_score_kernel<false, kFp8, kPair>;
  if constexpr (kPair) {
    // clusters of two CTAs (grid even)
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(tc::THREADS);
    cfg.dynamicSmemBytes = tc::SMEM_BYTES;
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = 2;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    TC_CUDA(cudaLaunchKernelEx(&cfg, fn, mapA, mapB, a));
  } else {
    fn<<<grid, tc::THREADS, tc::SMEM_BYTES, s>>>(mapA, mapB, a);
  }
}

// The shared-memory size of every form of the score kernel on the current device
// (set before the launches, so that a launch sequence can be captured into a graph).
void prepare_score_kernels() {
  {
    const void* fns[] = {(const void*)tc::tc_score_kernel<true, false, false>,
                         (const void*)tc::tc_score_kernel<false, false, false>,
                         (const void*)tc::tc_score_kernel<true, true, false>,
                         (const void*)tc::tc_score_kernel<false, true, false>,
                         (const void*)tc::tc_score_kernel<true, false, true>,
                         (const void*)tc::tc_score_kernel<false, false, true>,
                         (const void*)tc::tc_score_kernel<true, true, true>,
                         (const void*)tc::tc_score_kernel<false, true, true>};
    for (const void* f : fns)
      TC_CUDA(cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tc::SMEM_BYTES));
  }
}

// mapB: the query tiles (256-row boxes); mapBh: the same with 128-row boxes, for
// the two-CTA (pair) kernel, which runs when `pair` is set.
void launch_scores(const TcState& st, const CUtensorMap& mapB, const CUtensorMap* mapBh, tc::ScoreArgs a, bool dense,
                   cudaStream_t s, int sms, bool fp8 = false) {
  const uint32_t mtiles = (a.row_end - a.row_begin + tc::BM - 1) / tc::BM;
  const uint32_t ntiles = (a.nq + tc::BN - 1) / tc::BN;
  const uint32_t tiles = mtiles * ntiles;
  if (tiles == 0) return;
  const bool pair = mapBh != nullptr;
  const unsigned grid = pair ? 2u * (unsigned)std::min<uint32_t>((mtiles + 1) / 2 * ntiles, (uint32_t)sms / 2)
                             : (unsigned)std::min<uint32_t>(tiles, (uint32_t)sms);
  if (fp8) {
    a.row_scale = st.scale8;
    a.kblocks = st.kpad8 / 128;
    if (pair) launch_scores_t<true, true>(st.mapA8, *mapBh, a, dense, s, grid);
    else launch_scores_t<true, false>(st.mapA8, mapB, a, dense, s, grid);
  } else {
    if (pair) launch_scores_t<false, true>(st.mapA, *mapBh, a, dense, s, grid);
    else launch_scores_t<false, false>(st.mapA, mapB, a, dense, s, grid);
  }
  TC_CUDA(cudaGetLastError());
}

void check_error(const TcState& st, cudaStream_t s) {
  uint32_t err = 0;
  TC_CUDA(cudaMemcpyAsync(&err, st.error, 4, cudaMemcpyDeviceToHost, s));
  TC_CUDA(cudaStreamSynchronize(s));
  if (err) {
    TC_CUDA(cudaMemsetAsync(st.error, 0, 4, s));
    throw std::runtime_error("tensor-core score kernel: a pipeline wait ran out (code " + std::to_string(err) + ")");
  }
}

}  // namespace

void GraphEngine::tc_scores_device(const uint4* d_rows, size_t nq, float* d_scores, size_t ld, cudaStream_t stream) {
  std::lock_guard<std::mutex> lock(mu_);
  TC_CUDA(cudaSetDevice(device_));
  ensure_tc_rows();
  if (nq == 0) return;
  if (ld < host_.nrows) throw std::runtime_error("score stride smaller than the number of rows");
  if (nq > (1u << 20)) throw std::runtime_error("at most 2^20 queries per call");
  const TcState& st = *tc_;
  int sms = 0;
  TC_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device_));
  __nv_bfloat16* qb = nullptr;
  const size_t nq_pad = (nq + tc::BN - 1) / tc::BN * tc::BN;
  TC_CUDA(cudaMallocAsync(&qb, nq_pad * st.kpad * 2, stream));
  tc::tc_queries_kernel<<<1024, 256, 0, stream>>>(reinterpret_cast<const float*>(d_rows), host_.dpad, (uint32_t)nq,
                                                  (uint32_t)nq_pad, st.kpad, qb);
  TC_CUDA(cudaGetLastError());
  CUtensorMap mapB = tc::make_map(qb, nq_pad, st.kpad, tc::BN);
  tc::ScoreArgs a{};
  a.row_begin = 0;
  a.row_end = (uint32_t)host_.nrows;
  a.nq = (uint32_t)nq;
  a.kblocks = st.kpad / tc::BK;
  a.row_scale = st.scale;
  a.row_bias = st.bias;
  a.present = d_present_;
  a.dense = d_scores;
  a.dense_ld = (uint32_t)ld;
  a.error = st.error;
  prepare_score_kernels();
  launch_scores(st, mapB, nullptr, a, true, stream, sms);
  launches_ += 2;
  TC_CUDA(cudaFreeAsync(qb, stream));
  check_error(st, stream);
}

void GraphEngine::linear_search_tc_device(const uint4* d_rows, size_t nq, size_t size, size_t candidates,
                                          ObjDist* d_out, size_t kmax, uint32_t* d_counts, uint32_t* d_status,
                                          cudaStream_t stream, bool fp8, bool fp64_ties, bool pair) {
  std::lock_guard<std::mutex> lock(mu_);
  TC_CUDA(cudaSetDevice(device_));
  ensure_tc_rows();
  if (fp8) ensure_tc_rows8();
  if (nq == 0) return;
  if (size == 0) throw std::runtime_error("result size must be at least 1");
  if (kmax < size) throw std::runtime_error("kmax smaller than the result size");
  if (!d_status) throw std::runtime_error("a status buffer is required");
  size_t C = candidates ? candidates : std::max<size_t>(4 * size, 64);
  if (C < size) C = size;
  if (C > 4096) throw std::runtime_error("at most 4096 candidates per query (and results <= candidates)");
  const tc::FinalFn fin = tc::final_kernel(kernel_metric(host_.prop.metric), fp64_ties);
  if (!fin) throw std::runtime_error("unsupported distance for the tensor-core linear search");
  const TcState& st = *tc_;
  // the rows searched: the whole index, or the shard [tc_row_begin_, tc_row_end_)
  const uint32_t rb = std::min<uint32_t>(tc_row_begin_, (uint32_t)host_.nrows);
  const uint32_t nrows = tc_row_end_ ? std::min<uint32_t>(tc_row_end_, (uint32_t)host_.nrows) : (uint32_t)host_.nrows;
  if (rb >= nrows) {
    TC_CUDA(cudaMemsetAsync(d_counts, 0, nq * 4, stream));
    TC_CUDA(cudaMemsetAsync(d_status, 0, nq * 4, stream));
    TC_CUDA(cudaStreamSynchronize(stream));
    return;
  }
  // rows of the dense first part: >= C, a multiple of the tile height, <= 16384
  // (automatic: 8192; the threshold then tightens between the doubling parts)
  size_t first = tc_first_rows_ ? tc_first_rows_ : 8192;
  first = std::max<size_t>(first, C);
  first = std::min<size_t>((first + tc::BM - 1) / tc::BM * tc::BM, 16384);
  if (first < C) throw std::runtime_error("too many candidates for the dense first part");
  const uint32_t r0 = (uint32_t)std::min<size_t>((size_t)rb + first, nrows);
  const uint32_t cap = std::min<uint32_t>(16384, std::max<uint32_t>(8192, tc::pow2_at_least((uint32_t)(4 * C))));
  const uint32_t P = tc::pow2_at_least((uint32_t)C);
  int sms = 0;
  TC_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device_));
  const size_t qbmax = std::min<size_t>(nq, 16384);
  // scratch: bf16 or E4M3 queries | dense scores | candidates | counts | thresholds | query scales
  const size_t qbpad = (qbmax + tc::BN - 1) / tc::BN * tc::BN;
  const size_t b_q = (qbpad * std::max<size_t>(st.kpad * 2, st.kpad8) + 255) / 256 * 256;
  const size_t b_d = (qbmax * (size_t)first * 4 + 255) / 256 * 256;
  const size_t b_c = qbmax * (size_t)cap * 8;
  const size_t need = b_q + b_d + b_c + 2 * qbmax * 4 + qbpad * 4 + 512;
  if (tc_->scratch_bytes < need) {
    TC_CUDA(cudaStreamSynchronize(stream));
    tc_drop_graphs(tc_);                       // they name the old scratch
    TC_CUDA(cudaFree(tc_->scratch));
    tc_->scratch = nullptr;
    tc_->scratch_bytes = 0;
    TC_CUDA(cudaMalloc(&tc_->scratch, need));
    tc_->scratch_bytes = need;
  }
  uint8_t* sp = static_cast<uint8_t*>(tc_->scratch);
  __nv_bfloat16* qbuf = reinterpret_cast<__nv_bfloat16*>(sp);
  float* dense = reinterpret_cast<float*>(sp + b_q);
  unsigned long long* cand = reinterpret_cast<unsigned long long*>(sp + b_q + b_d);
  uint32_t* ccount = reinterpret_cast<uint32_t*>(sp + b_q + b_d + b_c);
  float* thr = reinterpret_cast<float*>(ccount + qbmax);
  float* qscale = thr + qbmax;
  uint8_t* qbuf8 = reinterpret_cast<uint8_t*>(sp);
  const uint32_t rc = dev_.row_chunks;
  uint32_t group = 1;
  while (group < rc && group < 32) group <<= 1;
  const size_t fin_smem = (size_t)rc * 16 + (size_t)cap * 8 + (size_t)P * 8;
  TC_CUDA(cudaFuncSetAttribute((const void*)fin, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)fin_smem));
  TC_CUDA(cudaFuncSetAttribute((const void*)tc::tc_first_select_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)(first * 8)));
  TC_CUDA(cudaFuncSetAttribute((const void*)tc::tc_compact_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)(cap * 8)));
  prepare_score_kernels();
  // the launch sequence (timing: phase events between its parts)
  auto enqueue = [&](bool timing) {
  TC_CUDA(cudaMemsetAsync(d_status, 0, nq * 4, stream));
  for (size_t q0 = 0; q0 < nq; q0 += qbmax) {
    const uint32_t nb = (uint32_t)std::min(qbmax, nq - q0);
    const uint32_t nbpad = (nb + tc::BN - 1) / tc::BN * tc::BN;
    if (timing) TC_CUDA(cudaEventRecord(st.ev[0], stream));
    const float* qrows = reinterpret_cast<const float*>(d_rows) + q0 * host_.dpad;
    CUtensorMap mapB, mapBh;
    if (fp8) {
      tc::tc_queries8_kernel<<<1024, 256, 0, stream>>>(qrows, host_.dpad, nb, nbpad, st.kpad8, qbuf8, qscale);
      mapB = tc::make_map8(qbuf8, nbpad, st.kpad8, tc::BN);
      if (pair) mapBh = tc::make_map8(qbuf8, nbpad, st.kpad8, tc::BN / 2);
    } else {
      tc::tc_queries_kernel<<<1024, 256, 0, stream>>>(qrows, host_.dpad, nb, nbpad, st.kpad, qbuf);
      mapB = tc::make_map(qbuf, nbpad, st.kpad, tc::BN);
      if (pair) mapBh = tc::make_map(qbuf, nbpad, st.kpad, tc::BN / 2);
    }
    const CUtensorMap* half = pair ? &mapBh : nullptr;
    TC_CUDA(cudaGetLastError());
    tc::ScoreArgs a{};
    a.nq = nb;
    a.kblocks = st.kpad / tc::BK;
    a.qscale = qscale;
    a.row_scale = st.scale;
    a.row_bias = st.bias;
    a.present = d_present_;
    a.error = st.error;
    // dense first part
    a.row_begin = rb;
    a.row_end = r0;
    a.dense = dense;
    a.dense_ld = (uint32_t)first;
    launch_scores(st, mapB, half, a, true, stream, sms, fp8);
    tc::tc_first_select_kernel<<<nb, 512, first * 8, stream>>>(dense, (uint32_t)first, r0 - rb, (uint32_t)C, thr,
                                                               cand, ccount, cap, rb);
    TC_CUDA(cudaGetLastError());
    launches_ += 3;
    if (timing) TC_CUDA(cudaEventRecord(st.ev[1], stream));
    // filtered rest, in parts that double in size; between two parts the
    // candidate lists are cut back to C and the thresholds move up
    a.dense = nullptr;
    a.thr = thr;
    a.cand = cand;
    a.cand_count = ccount;
    a.cap = cap;
    a.status = d_status + q0;
    // Valid (present) rows seen so far.  While fewer than C, every query's threshold
    // is still -inf and each valid row of the next part is appended on top of them,
    // so such a part ends before it could pass the list capacity (an index with
    // most low ids removed); the presence flags are the same for every query.
    size_t valid = 0;
    for (uint32_t i = std::max<uint32_t>(rb, 1); i < r0; i++) valid += host_.present[i] ? 1 : 0;
    for (uint32_t row = r0, part = std::max<uint32_t>(r0 - rb, tc::BM); row < nrows; part *= 2) {
      uint32_t end = (uint32_t)std::min<uint64_t>(nrows, (uint64_t)row + part);
      if (valid < C) {
        const size_t room = cap - valid;          // >= 3 C and >= 6144: cap >= max(8192, 4 C), C <= 2048 there
        size_t v = 0;
        uint32_t e = row;
        while (e < end && v + (host_.present[e] ? 1 : 0) <= room) v += host_.present[e++] ? 1 : 0;
        if (e < end) {
          e = std::max<uint32_t>(row + tc::BM, e / tc::BM * tc::BM);   // whole tiles; room >= one tile
          v = 0;
          for (uint32_t i = row; i < e; i++) v += host_.present[i] ? 1 : 0;
        }
        end = e;
        valid += v;
      }
      a.row_begin = row;
      a.row_end = end;
      launch_scores(st, mapB, half, a, false, stream, sms, fp8);
      launches_++;
      if (end < nrows) {
        tc::tc_compact_kernel<<<nb, 512, cap * 8, stream>>>(cand, ccount, cap, (uint32_t)C, thr, d_status + q0);
        TC_CUDA(cudaGetLastError());
        launches_++;
      }
      row = end;
    }
    if (timing) TC_CUDA(cudaEventRecord(st.ev[2], stream));
    fin<<<nb, 256, fin_smem, stream>>>(dev_, d_rows, (uint32_t)q0, cand, ccount, cap, (uint32_t)C, P,
                                       (uint32_t)size, group, d_out, (uint32_t)kmax, d_counts, d_status);
    TC_CUDA(cudaGetLastError());
    if (timing) TC_CUDA(cudaEventRecord(st.ev[3], stream));
    launches_++;
  }
  };
  cudaStreamCaptureStatus capture = cudaStreamCaptureStatusNone;
  TC_CUDA(cudaStreamIsCapturing(stream, &capture));
  if (!tc_graphs_ || capture != cudaStreamCaptureStatusNone) {
    // launched directly (also into a capture the caller runs on this stream)
    enqueue(capture == cudaStreamCaptureStatusNone);
    if (capture != cudaStreamCaptureStatusNone) return;
    check_error(st, stream);
    for (int i = 0; i < 3; i++) TC_CUDA(cudaEventElapsedTime(&tc_->phase_ms[i], st.ev[i], st.ev[i + 1]));
    return;
  }
  // graph replay: the sequence is captured once per shape, buffers, scratch, row range
  // and options, and replayed on later calls that match
  const std::array<uint64_t, 16> key = {(uint64_t)(uintptr_t)d_rows, nq, size, C,
                                        (uint64_t)(uintptr_t)d_out, kmax, (uint64_t)(uintptr_t)d_counts,
                                        (uint64_t)(uintptr_t)d_status,
                                        (uint64_t)fp8 | (uint64_t)fp64_ties << 1 | (uint64_t)pair << 2, rb, nrows,
                                        first, (uint64_t)(uintptr_t)tc_->scratch, tc_->scratch_bytes, 0, 0};
  TcState::Graph* g = nullptr;
  for (auto& x : tc_->graphs)
    if (x.key == key) g = &x;
  if (!g) {
    if (tc_->graphs.size() >= 8) {
      TC_CUDA(cudaStreamSynchronize(stream));
      cudaGraphExecDestroy(tc_->graphs.front().exec);
      tc_->graphs.erase(tc_->graphs.begin());
    }
    const uint64_t l0 = launches_;
    TC_CUDA(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
    cudaGraph_t graph = nullptr;
    try {
      enqueue(false);
    } catch (...) {
      cudaStreamEndCapture(stream, &graph);
      if (graph) cudaGraphDestroy(graph);
      throw;
    }
    TC_CUDA(cudaStreamEndCapture(stream, &graph));
    cudaGraphExec_t exec = nullptr;
    const cudaError_t ie = cudaGraphInstantiate(&exec, graph, 0);
    cudaGraphDestroy(graph);
    TC_CUDA(ie);
    tc_->graphs.push_back(TcState::Graph{key, exec, launches_ - l0});
    g = &tc_->graphs.back();
    launches_ = l0;
  }
  TC_CUDA(cudaEventRecord(st.ev[0], stream));
  TC_CUDA(cudaGraphLaunch(g->exec, stream));
  TC_CUDA(cudaEventRecord(st.ev[3], stream));
  launches_ += g->launches;
  check_error(st, stream);
  // one replay: its whole time is reported as the middle phase
  float total = 0.f;
  TC_CUDA(cudaEventElapsedTime(&total, st.ev[0], st.ev[3]));
  tc_->phase_ms[0] = 0.f;
  tc_->phase_ms[1] = total;
  tc_->phase_ms[2] = 0.f;
}

void GraphEngine::set_tc_graphs(bool on) {
  std::lock_guard<std::mutex> lock(mu_);
  tc_graphs_ = on;
  if (!on && tc_) {
    TC_CUDA(cudaSetDevice(device_));
    TC_CUDA(cudaDeviceSynchronize());
    tc_drop_graphs(tc_);
  }
}

void GraphEngine::tc_phase_ms(float* out) const {
  for (int i = 0; i < 3; i++) out[i] = tc_ ? tc_->phase_ms[i] : 0.f;
}

}  // namespace ngtg
