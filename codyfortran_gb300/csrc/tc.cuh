// tc.cuh -- tcgen05 GEMM entry points shared by the mixed-precision kernels.
#pragma once
#include <cuda.h>
#include <cuda_bf16.h>

#include <utility>
#include <vector>

#include "common.cuh"

// The three contractions of the mixed form; their per-trajectory sizes come
// from the TrajShape table (M rows of A, N rows of B, K tiles per segment).
enum { TC_GEMM_W = 0, TC_GEMM_Z = 1, TC_GEMM_H2 = 2 };

// Picks the K-split count that fills ~one wave of 152 SMs (each split keeps >= 2 K tiles).
int tc_split_count(int M, int N, int BN, int kTiles, int nb);
// N-tile width used for an output of N columns (64, 128 or 256).
int tc_tile_n(int N);
// 3D TMA map over a bf16 operand of the context: [nb][rowsMax][pitch] (pitch
// elements per row, trajectories bs bytes apart); box = 64 x boxRows x 1.
CUtensorMap tc_make_map(const cgpu_ctx* c, const __nv_bfloat16* base, int rowsMax, int pitch, int boxRows);
// P[traj][split][M][N] (fp32) = A[M,K] B[N,K]^T over `terms` K segments of
// segPitch elements each (the valid K of a segment is the trajectory's padded K).
void tc_gemm(cgpu_ctx* c, int gemmId, const CUtensorMap& ta, const CUtensorMap& tb, int bn, float* P, int terms,
             int segPitch, int nSplit, int Mmax, int Nmax, int* err);

// Fixed-point slice GEMM (k_fx.cu): out[traj][split][M][N] (FP64) = A B^T (the
// B map with 16-row boxes, the A map with 128-row boxes) for
// operands carried as L base-2^digitBits digit slices (K segments of
// segPitchA / segPitch elements) with row exponents expA / expB; maxRow /
// maxCol (unsplit K only) receive the largest biased exponent of |C| per row /
// column.  compact: the two-CTAs-per-SM configuration (small K).  aShared: A
// is one matrix shared by the trajectories, read at each trajectory's vRow.
// nSplit: K splits of the longest contraction (segPitch / 64 K blocks, kPer
// blocks per split); a trajectory of fewer K blocks takes only the splits its
// own K needs, balanced, and its remaining partials are written as zeros.
void fx_gemm(cgpu_ctx* c, int L, int digitBits, bool compact, int gemmId, const CUtensorMap& ta,
             const CUtensorMap& tb, int bn, double* out, const int* expA, const int* expB, unsigned* maxRow,
             unsigned* maxCol, int segPitchA, int segPitch, int aShared, int nSplit, const void* tiles, int nTiles,
             int* err);
// Device list of the fixed-point GEMM's tiles (trajectory, row, column, K split) of the
// context for an N tile of bn columns: only tiles inside a trajectory's output.
void* fx_build_tiles(cgpu_ctx* c, int gemmId, int bn, int nSplit, int* nTiles);
// 3D TMA map over an explicit [planes][rowsMax][pitch] bf16 tensor (planes planeBytes apart).
CUtensorMap tc_make_map_planes(const __nv_bfloat16* base, int rowsMax, int pitch, int boxRows, int planes,
                               size_t planeBytes);
// Digit width (6..8 bits) and slice count carrying at least targetBits
// fractional bits for a contraction of kTiles 64-wide K blocks: the widest
// digits whose two leading level sums stay exact in FP32 over the whole K
// (K <= 2^(24-2b)) and whose epilogue sum of the levels stays inside int64
// (b (L-1) <= 38).
void fx_plan(int kTiles, int targetBits, int* digitBits, int* slices);
// N-tile width for N output columns and L slices (wide: L * BN <= 512, compact: <= 256).
int fx_tile_n(int N, int L, bool compact);
// Whether a compact configuration exists for L slices.
bool fx_compact_ok(int L);
// The instantiated (N tile width, compact) configurations for L slices.
void fx_tile_configs(int L, std::vector<std::pair<int, bool>>& out);
bool fx_tile_supported(int bn, int L, bool compact);
// Fewest K splits that keep every split inside the exact range of the digits.
int fx_min_splits(int kTiles, int digitBits);
// The split count fx_gemm runs for a request of s splits (balanced K blocks per split).
int fx_normalize_splits(int kTiles, int s);
// K splits of the fixed-point GEMM: about one wave of 152 SMs, and every split
// inside the exact range of the level sums at digitBits (2^(24-2b) K).
int fx_split_count(int M, int N, int BN, int kTiles, int nb, int digitBits);

// ---- device helpers shared by the tcgen05 kernels (TMA, mbarriers, MMA, TMEM) ----
namespace tcdev {

constexpr int TC_BM = 128;
constexpr int TC_BK = 64;  // bf16 elements per 128-byte swizzle row
constexpr long long TC_WAIT_CYCLES = 4000000000LL;

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

__device__ __forceinline__ bool mbar_test(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

// mbarrier.try_wait: suspends the thread in hardware for a bounded, implementation-defined
// time while the phase is incomplete; true once it completed.
__device__ __forceinline__ bool mbar_try(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Bounded wait: false when the limit expires or another role aborted.
__device__ inline bool mbar_wait(uint64_t* bar, uint32_t parity, volatile int* abortFlag) {
  if (mbar_try(bar, parity)) return true;
  long long t0 = clock64();
  while (!mbar_try(bar, parity)) {
    if (*abortFlag) return false;
    if (clock64() - t0 > TC_WAIT_CYCLES) return false;
  }
  return true;
}

__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, uint64_t* bar, int c0, int c1,
                                            int c2) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];" ::
          "r"(smem_u32(dst)),
      "l"((uint64_t)map), "r"(c0), "r"(c1), "r"(c2), "r"(smem_u32(bar))
      : "memory");
}

// Shared-memory matrix descriptor: K-major, 128-byte swizzle, 8-row atoms of 1024 bytes.
__device__ __forceinline__ uint64_t sw128_desc(uint32_t saddr) {
  return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((uint64_t)1 << 16) | ((uint64_t)(1024 >> 4) << 32) |
         ((uint64_t)1 << 46) | ((uint64_t)2 << 61);
}

__device__ __forceinline__ void umma_bf16(uint32_t tmemD, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                          uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(
          tmemD),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}

// The same MMA with the A operand's collector buffer: coll 1 reads A from
// shared memory and keeps it (fill), 2 reuses the kept A (use), 3 reuses it a
// last time (lastuse); 0 = umma_bf16.  A run fill, use..., lastuse carries
// the same A descriptor and is issued back to back by one thread.  Callers
// pass coll from unrolled loops, so the branches fold away.
__device__ __forceinline__ void umma_bf16_coll(int coll, uint32_t tmemD, uint64_t adesc, uint64_t bdesc,
                                               uint32_t idesc, uint32_t accumulate) {
  if (coll == 1)
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16.collector::a::fill [%0], %1, %2, %3, p;\n}\n" ::"r"(tmemD),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
  else if (coll == 2)
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16.collector::a::use [%0], %1, %2, %3, p;\n}\n" ::"r"(tmemD),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
  else if (coll == 3)
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16.collector::a::lastuse [%0], %1, %2, %3, p;\n}\n" ::"r"(tmemD),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
  else
    umma_bf16(tmemD, adesc, bdesc, idesc, accumulate);
}

__device__ __forceinline__ void umma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}

#define TMEM_LD_X8(taddr, r)                                                                            \
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"                    \
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]) \
               : "r"(taddr))

#define TMEM_LD_X16(taddr, r)                                                                                  \
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, " \
               "[%16];"                                                                                        \
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),            \
                 "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),        \
                 "=r"(r[14]), "=r"(r[15])                                                                      \
               : "r"(taddr))

// Per-trajectory sizes of a contraction: M rows of A, N rows of B, K tiles per segment.
__device__ __forceinline__ void tc_dims(const TrajShape& S, int gemmId, int& M, int& N, int& segTiles) {
  int P2 = 2 * S.nPairs, Q2 = 2 * S.nOS * S.nOS;
  if (gemmId == TC_GEMM_W) { M = S.nG; N = P2; segTiles = S.Kg / TC_BK; }
  else if (gemmId == TC_GEMM_Z) { M = S.nG; N = Q2; segTiles = S.Kp / TC_BK; }
  else { M = P2; N = P2; segTiles = S.Kg / TC_BK; }
}


}  // namespace tcdev
