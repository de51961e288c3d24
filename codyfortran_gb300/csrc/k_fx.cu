// k_fx.cu -- fixed-point split GEMM on tcgen05 tensor cores (the mixed_fx form
// of the contractions of ApplyCorrelationOp,
// src/Method/Mb/OrbBased/S_Method_Mb_OrbBased.f90:647-872).
//
// An FP64 operand row x[0..K) is carried as L slices of base-2^b digits under
// one power of two per row:
//     x[k] ~= 2^e sum_{i<L} d_i[k] 2^(-b(i+1)),   max_k |x[k]| < 2^e,
//     |d_0| <= 2^b, d_i in [-2^(b-1), 2^(b-1)) for i > 0 (bf16 holds them exactly, b <= 8),
// i.e. x rounded to bL fractional bits of its row maximum.  The product of an
// A row and a B row splits into levels l = i + j:
//     C = 2^(ea + eb) sum_l 2^(-b(l+2)) D_l,   D_l = sum_{i+j=l} sum_k a_i[k] b_j[k].
// Each level has its own FP32 accumulator in tensor memory (L accumulators of
// BN columns), fed by the slice products of that level.  A slice product is
// an integer of magnitude <= 2^2b, so D_0 and D_1 stay below 2^24 -- exact in
// FP32 -- for K <= 2^(24-2b) (b = 6: K <= 4096, 7: 1024, 8: 256; longer
// contractions are split in K and the FP64 partials summed) and D_2 for
// K <= 0.8 2^(24-2b); a higher level that passes 2^24 rounds by 2^-24 of a
// term at least 2^-2b below the result's scale.  The epilogue combines the
// levels in 64-bit integers (Horner in base 2^b), converts once to FP64 and
// applies the power-of-two scale, so C is the product of the truncated
// operands whatever the summation order.  Levels l >= L are not formed; with
// the operand truncation (2^-(bL+1) of each row maximum) they bound the error
// at about 2^-bL max|a| max|b| K.
//
// Pipeline: one TMA producer thread, one MMA issuer thread, eight epilogue
// warps (the tile's accumulators fill the tensor memory, so the epilogue of
// one tile cannot overlap the MMAs of the next; two warps per lane quarter
// halve its latency-bound duration).  Per 64-wide K block the producer loads the L slices of the B tile
// (in 16-row boxes, only the rows of the trajectory's own columns) into one
// ring stage and the L slices of the A tile into L stages of a second ring; the issuer runs the L(L+1)/2 slice products of the block from
// shared memory with the MMA width cut to the trajectory's own N, the L - i
// products of A slice i back to back per 16-wide K step so that A comes from
// the tensor core's collector buffer after its first read.  The
// epilogue stages the FP64 tile in shared memory for coalesced stores.  The
// wide configuration (two B stages, deep A ring) holds one CTA per SM; the
// compact one (one B stage, L A stages, <= 256 TMEM columns) two.  Every wait
// is bounded: on expiry the kernel sets an error flag, drains its copies,
// frees its tensor memory and returns.
#include <cuda.h>
#include <cuda_bf16.h>

#include <algorithm>

#include "common.cuh"
#include "tc.cuh"

namespace {

using namespace tcdev;

constexpr int FX_SMEM_MAX = 232448;

template <int BN, int L, int NA_, int NB_>
struct FxCfg {
  static constexpr int A_BYTES = TC_BM * TC_BK * 2;
  static constexpr int B_BYTES = BN * TC_BK * 2;
  static constexpr int BG_BYTES = L * B_BYTES;
  static constexpr int NB = NB_;
  // NA_ == 0: as many A stages as fit (at most 8)
  static constexpr int NA = NA_ > 0 ? NA_ : std::min(8, (FX_SMEM_MAX - 2048 - NB * BG_BYTES) / A_BYTES);
  static constexpr int RING = NA * A_BYTES + NB * BG_BYTES;
  static constexpr int SMEM = RING + 1024;
  static constexpr int SP = BN + 1;  // staged output row pitch (doubles)
  static constexpr uint32_t TMEM_COLS = (L * BN) <= 32 ? 32 : (L * BN) <= 64 ? 64 : (L * BN) <= 128 ? 128
                                        : (L * BN) <= 256 ? 256 : 512;
  static_assert(L * BN <= 512, "tensor memory holds 512 columns");
  static_assert(BN % 16 == 0 && BN >= 16, "N tile: multiple of 16");
  static_assert(NA >= 2 || NA >= L, "A ring");
  static_assert(SMEM + 2048 <= FX_SMEM_MAX, "shared memory");
  static_assert(TC_BM * SP * 8 <= RING, "output staging fits the ring");
};

// T 2^e as a double by integer operations (the FP64 pipes are the scarce
// resource): round-to-nearest-even when |T| needs more than 53 bits; results
// outside the normal range go through ldexp.
__device__ __forceinline__ double ll_scaled(long long T, int e) {
  if (T == 0) return 0.0;
  const unsigned long long sign = T < 0 ? 0x8000000000000000ull : 0ull;
  unsigned long long a = T < 0 ? (unsigned long long)(-T) : (unsigned long long)T;
  const int msb = 63 - __clzll((long long)a);
  int ee;  // value = a 2^ee with a in [2^52, 2^53)
  if (msb > 52) {
    const int sh = msb - 52;
    const unsigned long long rem = a & ((1ull << sh) - 1), half = 1ull << (sh - 1);
    a >>= sh;
    if (rem > half || (rem == half && (a & 1ull))) a++;
    ee = e + sh;
    if (a >> 53) {
      a >>= 1;
      ee++;
    }
  } else {
    a <<= (52 - msb);
    ee = e - (52 - msb);
  }
  const int be = ee + 52 + 1023;
  if (be <= 0 || be >= 2047) return ldexp((double)T, e);
  return __longlong_as_double((long long)(sign | ((unsigned long long)be << 52) | (a & 0xFFFFFFFFFFFFFull)));
}

// One work item of a persistent CTA: trajectory, first output row, first
// output column, K split.
struct FxTile {
  int traj, m0, n0, split;
};

// out[traj][split][M][N] = C (FP64) over the tile list; a persistent CTA takes
// tiles blockIdx.x, blockIdx.x + gridDim.x, ...  Warps 0..EW-1: epilogue (TMEM
// lanes 32(w%4)..32(w%4)+31, column batches of CB); warp EW: TMA producer;
// warp EW+1: MMA issuer.  The rings and their
// phases run on across tiles; the accumulator hand-off uses accFull (MMA ->
// epilogue) and accEmpty (epilogue -> MMA), so the producer loads the next
// tile while the epilogue drains the current one.  K splits: a trajectory of
// segTiles K blocks takes ceil(segTiles / kPer) balanced splits; the tiles of
// the list beyond them write zero partials.  maxRow/maxCol (unsplit K only):
// the largest biased exponent of |C| per output row / column.
// aShared: A is shared by the trajectories (3D map with one plane per root
// grid); the trajectory's rows start at vRow of plane vRoot, its K range at
// vRow - gShift, its row exponents at expA[vExp].
template <int BN, int L, int NA_, int NB_, int EW, int CB>
__global__ void __launch_bounds__(32 * (EW + 2), NA_ > 0 ? 2 : 1)
    k_fx_gemm(const __grid_constant__ CUtensorMap tA, const __grid_constant__ CUtensorMap tB, double* __restrict__ out,
              const int* __restrict__ expA, const int* __restrict__ expB, unsigned* __restrict__ maxRow,
              unsigned* __restrict__ maxCol, TRAJ_ARGS, int gemmId, int segPitchA, int segPitch, int aShared,
              int kPer, int digitBits, const FxTile* __restrict__ tiles, int nTiles, int* __restrict__ err) {
  using C = FxCfg<BN, L, NA_, NB_>;
  constexpr int NA = C::NA, NB = C::NB;
  static_assert(EW % 4 == 0 && (CB == 8 || CB == 16) && BN % CB == 0, "epilogue warps / column batch");
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  uint8_t* ringA = smem;
  uint8_t* ringB = smem + NA * C::A_BYTES;
  __shared__ __align__(8) uint64_t aFull[NA], aEmpty[NA], bFull[NB], bEmpty[NB], accFull, accEmpty, finalBar;
  __shared__ uint32_t tmemSlot;
  __shared__ volatile int abortFlag;
  __shared__ int consumedA, consumedB, issuedA, issuedB;

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x == 0) {
    abortFlag = 0;
    consumedA = consumedB = issuedA = issuedB = 0;
    for (int s = 0; s < NA; s++) {
      mbar_init(&aFull[s], 1);
      mbar_init(&aEmpty[s], 1);
    }
    for (int s = 0; s < NB; s++) {
      mbar_init(&bFull[s], 1);
      mbar_init(&bEmpty[s], 1);
    }
    mbar_init(&accFull, 1);
    mbar_init(&accEmpty, EW);
    mbar_init(&finalBar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmemSlot)),
                 "r"(C::TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = tmemSlot;

  // per-tile geometry (every role derives the same values)
  auto geometry = [&](const FxTile& tl, int& M, int& N, int& nT, int& kt0, int& nk) {
    int segTiles;
    tc_dims(shp[tl.traj], gemmId, M, N, segTiles);
    nT = min(BN, (N - tl.n0 + 15) / 16 * 16);
    const int sT = max(1, (segTiles + kPer - 1) / kPer);  // this trajectory's splits
    const int per = (segTiles + sT - 1) / sT;              // <= kPer
    kt0 = tl.split * per;
    nk = tl.split < sT ? max(0, min(segTiles, kt0 + per) - kt0) : 0;
  };

  if (warp == EW) {
    if (lane == 0) {
      // TMA producer: per K block the L B slices (16-row boxes of the tile's rows), then the L A slices
      int ta = 0, tb = 0;
      for (int t = blockIdx.x; t < nTiles && !abortFlag; t += gridDim.x) {
        const FxTile tl = tiles[t];
        int M, N, nT, kt0, nk;
        geometry(tl, M, N, nT, kt0, nk);
        const TrajShape& T = shp[tl.traj];
        const int aRow0 = aShared ? T.vRow : 0, aCol0 = aShared ? T.vRow - T.gShift : 0;
        const int aZ = aShared ? T.vRoot : tl.traj;
        for (int kb = 0; kb < nk && !abortFlag; kb++) {
          const int sb = tb % NB, rb = tb / NB;
          if (!mbar_wait(&bEmpty[sb], (rb & 1) ^ 1, &abortFlag)) {
            abortFlag = 1;
            atomicExch(err, 11);
            break;
          }
          const int x0 = (kt0 + kb) * TC_BK;
          mbar_expect_tx(&bFull[sb], (uint32_t)(L * nT * TC_BK * 2));
          for (int j = 0; j < L; j++)
            for (int r = 0; r < nT; r += 16)
              tma_load_3d(ringB + sb * C::BG_BYTES + j * C::B_BYTES + r * TC_BK * 2, &tB, &bFull[sb],
                          j * segPitch + x0, tl.n0 + r, tl.traj);
          tb++;
          issuedB = tb;
          for (int i = 0; i < L; i++) {
            const int sa = ta % NA, ra = ta / NA;
            if (!mbar_wait(&aEmpty[sa], (ra & 1) ^ 1, &abortFlag)) {
              abortFlag = 1;
              atomicExch(err, 12);
              break;
            }
            mbar_expect_tx(&aFull[sa], C::A_BYTES);
            tma_load_3d(ringA + sa * C::A_BYTES, &tA, &aFull[sa], i * segPitchA + aCol0 + x0, aRow0 + tl.m0, aZ);
            ta++;
            issuedA = ta;
          }
        }
      }
    }
  } else if (warp == EW + 1) {
    if (lane == 0) {
      // MMA issuer: kind::f16, D=F32, A=B=BF16, K-major, M=128; descriptors
      // advance by address / 16: +2 per 16-wide K step, +B_BYTES/16 per B slice
      const uint64_t bdesc0 = sw128_desc(smem_u32(ringB));
      const uint64_t adesc0 = sw128_desc(smem_u32(ringA));
      int ca = 0, cb = 0, ph = 0;  // ph: accumulator phases (tiles with K work)
      for (int t = blockIdx.x; t < nTiles && !abortFlag; t += gridDim.x) {
        const FxTile tl = tiles[t];
        int M, N, nT, kt0, nk;
        geometry(tl, M, N, nT, kt0, nk);
        if (nk == 0) continue;  // the epilogue writes the empty split's zeros
        const uint32_t idesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(nT >> 3) << 17) |
                               ((uint32_t)(TC_BM >> 4) << 24);
        if (ph > 0 && !mbar_wait(&accEmpty, (ph - 1) & 1, &abortFlag)) {  // the epilogue drained TMEM
          abortFlag = 1;
          atomicExch(err, 16);
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        bool ok = true;
        for (int kb = 0; kb < nk && ok; kb++) {
          const int sb = cb % NB, rb = cb / NB;
          if (!mbar_wait(&bFull[sb], rb & 1, &abortFlag)) {
            abortFlag = 1;
            atomicExch(err, 13);
            ok = false;
            break;
          }
          cb++;
          consumedB = cb;
          asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
          const uint64_t bd = bdesc0 + (uint64_t)((sb * C::BG_BYTES) >> 4);
#pragma unroll
          for (int i = 0; i < L; i++) {
            const int sa = ca % NA, ra = ca / NA;
            if (!mbar_wait(&aFull[sa], ra & 1, &abortFlag)) {
              abortFlag = 1;
              atomicExch(err, 14);
              ok = false;
              break;
            }
            ca++;
            consumedA = ca;
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint64_t ad = adesc0 + (uint64_t)((sa * C::A_BYTES) >> 4);
            // the L - i products of A slice i share each 16-wide K step of A:
            // issued back to back, A is read from shared memory once per step
            // and reused from the collector buffer
#pragma unroll
            for (int k = 0; k < TC_BK / 16; k++) {
#pragma unroll
              for (int j = 0; j < L - i; j++) {
                const int last = L - i - 1;
                const int coll = last == 0 ? 0 : (j == 0 ? 1 : (j == last ? 3 : 2));
                umma_bf16_coll(coll, tmem + (uint32_t)((i + j) * BN), ad + 2 * k,
                               bd + (uint64_t)((j * C::B_BYTES) >> 4) + 2 * k, idesc,
                               (kb > 0 || i > 0 || k > 0) ? 1u : 0u);
              }
            }
            umma_commit(&aEmpty[sa]);
          }
          if (ok) umma_commit(&bEmpty[sb]);
        }
        if (!ok) break;
        umma_commit(&accFull);
        ph++;
      }
      umma_commit(&finalBar);  // arrives when every issued MMA has completed
    }
  } else {
    // epilogue: warp w owns TMEM lanes [32q, 32q+32) = tile rows, q = w % 4
    // (the lane quarter a warp may access), and every (EW/4)-th batch of CB
    // columns starting at batch w / 4
    const long long base = 1LL << digitBits;
    const int q = warp & 3, cg = warp >> 2;
    int ph = 0;
    for (int t = blockIdx.x; t < nTiles; t += gridDim.x) {
      const FxTile tl = tiles[t];
      int M, N, nT, kt0, nk;
      geometry(tl, M, N, nT, kt0, nk);
      double* Oz = batn(out, bs, tl.traj) + (size_t)tl.split * (size_t)M * N;
      const int r = q * 32 + lane, row = tl.m0 + r;
      const bool rowOk = row < M;
      if (nk == 0) {  // empty split: its partial is zero
        if (rowOk && cg == 0)
          for (int col = tl.n0; col < min(N, tl.n0 + BN); col++) Oz[(size_t)row * N + col] = 0.0;
        continue;
      }
      const bool waited = mbar_wait(&accFull, ph & 1, &abortFlag);
      if (__any_sync(0xffffffffu, !waited)) {
        if (lane == 0) atomicExch(err, 15);
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const TrajShape& T = shp[tl.traj];
      const int* eA = aShared ? expA + T.vExp : batn(expA, bs, tl.traj);
      const int* eB = batn(expB, bs, tl.traj);
      const int ea = rowOk ? eA[row] - digitBits * (L + 1) : 0;
      unsigned rowMaxEx = 0;
#pragma unroll 1
      for (int c = cg * CB; c < nT; c += (EW / 4) * CB) {
        uint32_t acc[L][CB];
#pragma unroll
        for (int l = 0; l < L; l++) {
          if (CB == 16)
            TMEM_LD_X16(tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(l * BN + c), acc[l]);
          else
            TMEM_LD_X8(tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(l * BN + c), acc[l]);
        }
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
        double v[CB];
#pragma unroll
        for (int j = 0; j < CB; j++) {
          const int col = tl.n0 + c + j;
          unsigned ex = 0;
          v[j] = 0.0;
          if (rowOk && col < N) {
            long long Tv = 0;
#pragma unroll
            for (int l = 0; l < L; l++) Tv = Tv * base + (long long)__float2int_rn(__uint_as_float(acc[l][j]));
            v[j] = ll_scaled(Tv, ea + eB[col]);
            ex = (unsigned)(__double2hiint(v[j]) >> 20) & 0x7FFu;
          }
          if (maxCol) {
            unsigned m = __reduce_max_sync(0xffffffffu, ex);
            if (lane == 0 && m) atomicMax(batn(maxCol, bs, tl.traj) + col, m);
          }
          rowMaxEx = max(rowMaxEx, ex);
        }
        if (rowOk) {
          double* dst = Oz + (size_t)row * N + tl.n0 + c;
#pragma unroll
          for (int j = 0; j < CB; j += 2)
            if (tl.n0 + c + j < N) *reinterpret_cast<double2*>(dst + j) = make_double2(v[j], v[j + 1]);
        }
      }
      if (maxRow && rowOk && rowMaxEx) atomicMax(batn(maxRow, bs, tl.traj) + row, rowMaxEx);
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      __syncwarp();
      if (lane == 0) mbar_arrive(&accEmpty);
      ph++;
    }
  }
  __syncthreads();
  // every issued MMA has completed before the tensor memory is freed; after an
  // abort also the TMA copies that were issued but never consumed (bounded waits)
  if (warp == EW && lane == 0) {
    volatile int dummy = 0;
    mbar_wait(&finalBar, 0, &dummy);
    if (abortFlag) {
      for (int t = consumedA; t < issuedA; t++) mbar_wait(&aFull[t % NA], (t / NA) & 1, &dummy);
      for (int t = consumedB; t < issuedB; t++) mbar_wait(&bFull[t % NB], (t / NB) & 1, &dummy);
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(C::TMEM_COLS) : "memory");
}

template <int BN, int L, int NA_, int NB_>
void launch_fx_t(cgpu_ctx* c, const CUtensorMap& ta, const CUtensorMap& tb, double* out, const int* expA,
                 const int* expB, unsigned* maxRow, unsigned* maxCol, int gemmId, int segPitchA, int segPitch,
                 int aShared, int kPer, int digitBits, const FxTile* tiles, int nTiles, int ctasPerSm, int* err) {
  using C = FxCfg<BN, L, NA_, NB_>;
  // eight epilogue warps (two per tensor-memory lane quarter); the compact
  // configuration (two CTAs per SM) loads eight columns per batch to stay
  // inside half the register file
  constexpr int EW = 8, CB = NA_ > 0 ? 8 : 16;
  auto kern = k_fx_gemm<BN, L, NA_, NB_, EW, CB>;
  static bool attr = false;
  if (!attr) {
    CODY_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, C::SMEM));
    attr = true;
  }
  if (nTiles <= 0) return;
  const int grid = std::min(nTiles, c->numSms * ctasPerSm);
  kern<<<grid, 32 * (EW + 2), C::SMEM, c->stream>>>(ta, tb, out, expA, expB, maxRow, maxCol, TRAJ_PASS(c), gemmId,
                                                    segPitchA, segPitch, aShared, kPer, digitBits, tiles, nTiles, err);
  CODY_LAUNCHED(c);
}

}  // namespace

// 64-wide K blocks per split within which the two leading level sums stay
// exact in FP32: K <= 2^(24-2b).
static int fx_exact_tiles(int b) { return (1 << (24 - 2 * b)) / TC_BK; }

void fx_plan(int kTiles, int targetBits, int* digitBits, int* slices) {
  // the widest digits whose exact range holds the whole contraction (an extra
  // K split costs more in tile epilogues and partial sums than a slice)
  int b = 8;
  while (b > 6 && kTiles > fx_exact_tiles(b)) b--;
  int L = (targetBits + b - 1) / b;
  // |Horner sum| < K 2^(b(L+1)+1) <= 2^(25+b(L-1)) must stay inside int64
  while (b > 6 && b * (L - 1) > 38) {
    b--;
    L = (targetBits + b - 1) / b;
  }
  if (L > 6 || b * (L - 1) > 38) throw std::string("fx_plan: no digit width carries the target bits");
  *digitBits = b;
  *slices = L;
}

// The instantiated N tiles (fx_gemm's cases): L accumulators of BN columns in
// 512 (wide) or 256 (compact, two CTAs per SM) tensor-memory columns.
struct FxTileCfg {
  int bn, L;
  bool compact;
};
static const FxTileCfg kFxTiles[] = {
    {32, 4, false}, {64, 4, false}, {80, 4, false}, {96, 4, false}, {128, 4, false}, {32, 5, false},
    {64, 5, false}, {80, 5, false}, {96, 5, false}, {32, 6, false}, {64, 6, false},  {80, 6, false},
    {32, 4, true},  {64, 4, true},  {32, 5, true},  {48, 5, true}};

static int fx_max_bn(int L, bool compact) {
  int m = 0;
  for (const FxTileCfg& t : kFxTiles)
    if (t.L == L && t.compact == compact) m = std::max(m, t.bn);
  return m;
}

bool fx_compact_ok(int L) { return fx_max_bn(L, true) > 0; }

void fx_tile_configs(int L, std::vector<std::pair<int, bool>>& out) {
  out.clear();
  for (const FxTileCfg& t : kFxTiles)
    if (t.L == L) out.push_back({t.bn, t.compact});
}

bool fx_tile_supported(int bn, int L, bool compact) {
  for (const FxTileCfg& t : kFxTiles)
    if (t.bn == bn && t.L == L && t.compact == compact) return true;
  return false;
}

int fx_min_splits(int kTiles, int digitBits) {
  const int exact = fx_exact_tiles(digitBits);
  return std::max(1, (kTiles + exact - 1) / exact);
}

int fx_normalize_splits(int kTiles, int s) {
  s = std::max(1, std::min(s, kTiles));
  const int per = (kTiles + s - 1) / s;
  return (kTiles + per - 1) / per;
}

int fx_tile_n(int N, int L, bool compact) {
  const int maxBn = fx_max_bn(L, compact);
  if (maxBn == 0) throw std::string("fx_tile_n: no configuration for this slice count");
  const int tiles = (N + maxBn - 1) / maxBn;
  const int want = ((N + tiles - 1) / tiles + 15) / 16 * 16;  // balanced tiles
  int best = maxBn;
  for (const FxTileCfg& t : kFxTiles)
    if (t.L == L && t.compact == compact && t.bn >= want && t.bn < best) best = t.bn;
  return best;
}

int fx_split_count(int M, int N, int BN, int kTiles, int nb, int digitBits) {
  long tiles = (long)((M + TC_BM - 1) / TC_BM) * ((N + BN - 1) / BN) * nb;
  int s = (int)std::max<long>(1, (152 + tiles - 1) / tiles);
  s = std::min(s, std::max(1, kTiles / 2));
  const int exact = fx_exact_tiles(digitBits);
  s = std::max(s, (kTiles + exact - 1) / exact);  // every split inside the exact range of the level sums
  int per = (kTiles + s - 1) / s;
  return (kTiles + per - 1) / per;
}

void* fx_build_tiles(cgpu_ctx* c, int gemmId, int bn, int nSplit, int* nTiles) {
  std::vector<FxTile> v;
  for (int b = 0; b < c->nb; b++) {
    const TrajShape& S = c->shape_h[b];
    int P2 = 2 * S.nPairs, Q2 = 2 * S.nOS * S.nOS, M, N;
    if (gemmId == TC_GEMM_W) { M = S.nG; N = P2; }
    else if (gemmId == TC_GEMM_Z) { M = S.nG; N = Q2; }
    else { M = P2; N = P2; }
    for (int m0 = 0; m0 < M; m0 += TC_BM)
      for (int n0 = 0; n0 < N; n0 += bn)
        for (int z = 0; z < nSplit; z++) v.push_back(FxTile{b, m0, n0, z});
  }
  *nTiles = (int)v.size();
  void* d = nullptr;
  CODY_CUDA(cudaMalloc(&d, sizeof(FxTile) * std::max<size_t>(v.size(), 1)));
  if (!v.empty()) CODY_CUDA(cudaMemcpy(d, v.data(), sizeof(FxTile) * v.size(), cudaMemcpyHostToDevice));
  return d;
}

void fx_gemm(cgpu_ctx* c, int L, int digitBits, bool compact, int gemmId, const CUtensorMap& ta,
             const CUtensorMap& tb, int bn, double* out, const int* expA, const int* expB, unsigned* maxRow,
             unsigned* maxCol, int segPitchA, int segPitch, int aShared, int nSplit, const void* tiles, int nTiles,
             int* err) {
  if (segPitch % TC_BK != 0 || segPitchA % TC_BK != 0)
    throw std::string("fx_gemm: segment pitch must be a multiple of 64");
  if (nSplit > 1 && (maxRow || maxCol)) throw std::string("fx_gemm: output maxima need an unsplit K");
  const int kTiles = segPitch / TC_BK, kPer = (kTiles + nSplit - 1) / nSplit;  // K blocks per split
  if (digitBits < 6 || digitBits > 8 || digitBits * (L - 1) > 38) throw std::string("fx_gemm: digit width");
  if (kPer > fx_exact_tiles(digitBits)) throw std::string("fx_gemm: K split beyond the exact range of the digits");
  const FxTile* tl = (const FxTile*)tiles;
#define FX_CASE(BN_, L_, NA_, NB_, CMP_)                                                                        \
  if (bn == BN_ && L == L_ && compact == CMP_) {                                                                \
    launch_fx_t<BN_, L_, NA_, NB_>(c, ta, tb, out, expA, expB, maxRow, maxCol, gemmId, segPitchA, segPitch,    \
                                   aShared, kPer, digitBits, tl, nTiles, CMP_ ? 2 : 1, err);                   \
    return;                                                                                                     \
  }
  FX_CASE(32, 4, 0, 2, false) FX_CASE(64, 4, 0, 2, false) FX_CASE(80, 4, 0, 2, false) FX_CASE(96, 4, 0, 2, false)
  FX_CASE(128, 4, 0, 2, false)
  FX_CASE(32, 5, 0, 2, false) FX_CASE(64, 5, 0, 2, false) FX_CASE(80, 5, 0, 2, false) FX_CASE(96, 5, 0, 2, false)
  FX_CASE(32, 6, 0, 2, false) FX_CASE(64, 6, 0, 2, false) FX_CASE(80, 6, 0, 2, false)
  FX_CASE(32, 4, 4, 1, true) FX_CASE(64, 4, 4, 1, true)
  FX_CASE(32, 5, 5, 1, true) FX_CASE(48, 5, 5, 1, true)
#undef FX_CASE
  throw std::string("fx_gemm: unsupported tile");
}
