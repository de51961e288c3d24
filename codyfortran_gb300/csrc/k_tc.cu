// k_tc.cu -- tcgen05 tensor-core contractions of the mixed-precision form.
//
// One GEMM kernel, C[M,N] (+)= A[M,K] B[N,K]^T with A and B bf16, both
// K-major, accumulated in FP32 in tensor memory (TMEM):
//   * operands are staged by TMA (cp.async.bulk.tensor, 128B swizzle) into a
//     STAGES-deep shared-memory ring guarded by mbarriers;
//   * one thread issues tcgen05.mma (kind::f16, M=128, N=BN, K=16 per
//     instruction) and commits each stage back to the producer;
//   * four warps read the accumulator with tcgen05.ld and store FP32 partial
//     tiles; split-K partials are summed in FP64 by the consumer kernels.
// Split precision is expressed in the operands: a value x is carried as
// hi = bf16(x), lo = bf16(x - hi) (bf16x3: products hi*hi + hi*lo + lo*hi),
// or as hi/mid/lo (bf16x6: all products of total order <= 2), laid out as
// consecutive K segments so one accumulation sums all products.
//
// Every mbarrier wait is bounded (clock64 limit).  On expiry the kernel sets
// an error flag, drains its own TMA copies with bounded waits, frees its
// TMEM and returns; the host reports the flag as an error.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <cstring>

#include "common.cuh"
#include "tc.cuh"

namespace {

using namespace tcdev;

// P[traj][z][m][n] = sum_{k in split z} A[m][k] B[n][k]; A rows m0.., B rows n0.., bf16 K-major.
// blockIdx.z = trajectory * nSplit + split.  K tile i of the trajectory lies in
// segment i / segTiles at element (segment * segPitch + (i % segTiles) * 64).
template <int BN, int STAGES>
__global__ void __launch_bounds__(128, 1)
    k_tc_gemm(const __grid_constant__ CUtensorMap tA, const __grid_constant__ CUtensorMap tB, float* __restrict__ P,
              TRAJ_ARGS, int gemmId, int terms, int segPitch, int nSplit, int* __restrict__ err) {
  constexpr int A_BYTES = TC_BM * TC_BK * 2;
  constexpr int B_BYTES = BN * TC_BK * 2;
  constexpr int STAGE_BYTES = A_BYTES + B_BYTES;
  constexpr uint32_t TMEM_COLS = BN <= 32 ? 32 : (BN <= 64 ? 64 : (BN <= 128 ? 128 : 256));
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  __shared__ __align__(8) uint64_t fullBar[STAGES];
  __shared__ __align__(8) uint64_t emptyBar[STAGES];
  __shared__ __align__(8) uint64_t doneBar;
  __shared__ uint32_t tmemSlot;
  __shared__ volatile int abortFlag;
  __shared__ int consumed;

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int traj = blockIdx.z / nSplit, split = blockIdx.z % nSplit;
  int M, N, segTiles;
  tc_dims(shp[traj], gemmId, M, N, segTiles);
  const int m0 = blockIdx.x * TC_BM, n0 = blockIdx.y * BN;
  if (m0 >= M || n0 >= N) return;  // tile outside this trajectory's output
  const int ldp = N;
  const int kTiles = terms * segTiles;
  const int per = (kTiles + nSplit - 1) / nSplit;
  const int kt0 = split * per;
  const int kt1 = min(kTiles, kt0 + per);
  const int nk = max(0, kt1 - kt0);
  float* Pz = batn(P, bs, traj) + (size_t)split * (size_t)M * ldp;
  if (nk == 0) {  // empty split: its partial is zero
    for (int e = threadIdx.x; e < TC_BM * BN; e += blockDim.x) {
      int r = m0 + e / BN, col = n0 + e % BN;
      if (r < M && col < N) Pz[(size_t)r * ldp + col] = 0.0f;
    }
    return;
  }

  if (threadIdx.x == 0) {
    abortFlag = 0;
    consumed = 0;
    for (int s = 0; s < STAGES; s++) {
      mbar_init(&fullBar[s], 1);
      mbar_init(&emptyBar[s], 1);
    }
    mbar_init(&doneBar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmemSlot)),
                 "r"(TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = tmemSlot;

  int issued = 0;
  if (nk > 0 && warp == 0 && lane == 0) {
    // TMA producer
    for (int i = 0; i < nk; i++) {
      int s = i % STAGES, r = i / STAGES;
      if (!mbar_wait(&emptyBar[s], (r & 1) ^ 1, &abortFlag)) {
        abortFlag = 1;
        atomicExch(err, 1);
        break;
      }
      mbar_expect_tx(&fullBar[s], STAGE_BYTES);
      int kt = kt0 + i;
      int x = (kt / segTiles) * segPitch + (kt % segTiles) * TC_BK;
      tma_load_3d(smem + s * STAGE_BYTES, &tA, &fullBar[s], x, m0, traj);
      tma_load_3d(smem + s * STAGE_BYTES + A_BYTES, &tB, &fullBar[s], x, n0, traj);
      issued = i + 1;
    }
  } else if (nk > 0 && warp == 1 && lane == 0) {
    // MMA issuer: instruction descriptor kind::f16, D=F32, A=B=BF16, K-major, N=BN, M=128
    const uint32_t idesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(BN >> 3) << 17) |
                           ((uint32_t)(TC_BM >> 4) << 24);
    int i = 0;
    for (; i < nk; i++) {
      int s = i % STAGES, r = i / STAGES;
      if (!mbar_wait(&fullBar[s], r & 1, &abortFlag)) {
        abortFlag = 1;
        atomicExch(err, 2);
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      uint32_t a = smem_u32(smem + s * STAGE_BYTES);
      uint32_t b = a + A_BYTES;
#pragma unroll
      for (int k = 0; k < TC_BK / 16; k++)
        umma_bf16(tmem, sw128_desc(a + k * 32), sw128_desc(b + k * 32), idesc, (i > 0 || k > 0) ? 1u : 0u);
      umma_commit(&emptyBar[s]);
    }
    consumed = i;
    umma_commit(&doneBar);
  }
  __syncwarp();
  bool ok = (nk > 0) && mbar_wait(&doneBar, 0, &abortFlag);
  if (!ok && nk > 0) atomicExch(err, 3);
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  __syncwarp();
  // epilogue: warp w owns TMEM lanes [32w, 32w+32) = tile rows
  const int row = m0 + warp * 32 + lane;
#pragma unroll 1
  for (int c = 0; c < BN; c += 16) {
    uint32_t r[16];
    TMEM_LD_X16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c, r);
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
    if (ok && !abortFlag && row < M) {
#pragma unroll
      for (int j = 0; j < 16; j++) {
        int col = n0 + c + j;
        if (col < N) Pz[(size_t)row * ldp + col] = __uint_as_float(r[j]);
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  // drain TMA copies that were issued but never consumed (only after an abort)
  if (warp == 0 && lane == 0 && abortFlag) {
    volatile int dummy = 0;
    mbar_wait(&doneBar, 0, &dummy);  // the issued MMAs finish before the tensor memory is freed
    for (int i = consumed; i < issued; i++) {
      int s = i % STAGES, r = i / STAGES;
      mbar_wait(&fullBar[s], r & 1, &dummy);
    }
  }
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS) : "memory");
}

PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;

void ensure_encode() {
  if (g_encode) return;
  cudaDriverEntryPointQueryResult q;
  void* fn = nullptr;
  CODY_CUDA(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q));
  if (q != cudaDriverEntryPointSuccess || !fn) throw std::string("cuda: cuTensorMapEncodeTiled unavailable");
  g_encode = (PFN_cuTensorMapEncodeTiled_v12000)fn;
}

template <int BN, int STAGES>
void launch_gemm_t(cgpu_ctx* c, const CUtensorMap& ta, const CUtensorMap& tb, float* P, int gemmId, int terms,
                   int segPitch, int nSplit, int Mmax, int Nmax, int* err) {
  constexpr int smem = STAGES * (TC_BM * TC_BK * 2 + BN * TC_BK * 2) + 1024;
  static bool attr = false;
  if (!attr) {
    CODY_CUDA(cudaFuncSetAttribute(k_tc_gemm<BN, STAGES>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
    attr = true;
  }
  dim3 grid(ceil_div(Mmax, TC_BM), ceil_div(Nmax, BN), (unsigned)(c->nb * nSplit));
  k_tc_gemm<BN, STAGES><<<grid, 128, smem, c->stream>>>(ta, tb, P, TRAJ_PASS(c), gemmId, terms, segPitch, nSplit,
                                                        err);
  CODY_LAUNCHED(c);
}

}  // namespace

int tc_tile_n(int N) {
  int best = 64, bestCols = ((N + 63) / 64) * 64;
  for (int bn : {128, 256}) {
    int cols = ((N + bn - 1) / bn) * bn;
    if (cols <= bestCols) { best = bn; bestCols = cols; }
  }
  return best;
}

int tc_split_count(int M, int N, int BN, int kTiles, int nb) {
  long tiles = (long)((M + TC_BM - 1) / TC_BM) * ((N + BN - 1) / BN) * nb;
  int s = (int)std::max<long>(1, (152 + tiles - 1) / tiles);
  s = std::min(s, std::max(1, kTiles / 2));
  int per = (kTiles + s - 1) / s;
  return (kTiles + per - 1) / per;
}

// 3D bf16 tensor [nb][rowsMax][pitch] (pitch contiguous, multiple of 64, trajectories bs bytes apart).
CUtensorMap tc_make_map(const cgpu_ctx* c, const __nv_bfloat16* base, int rowsMax, int pitch, int boxRows) {
  return tc_make_map_planes(base, rowsMax, pitch, boxRows, c->nb, c->bs);
}

CUtensorMap tc_make_map_planes(const __nv_bfloat16* base, int rowsMax, int pitch, int boxRows, int planes,
                               size_t planeBytes) {
  ensure_encode();
  if (planes > 1 && planeBytes % 16 != 0) throw std::string("tensor map: bad alignment");
  if (planes == 1) planeBytes = (size_t)pitch * 2 * (size_t)rowsMax;
  if ((uintptr_t)base % 16 != 0 || pitch % TC_BK != 0 || planeBytes % 16 != 0)
    throw std::string("tensor map: bad alignment");
  CUtensorMap m;
  std::memset(&m, 0, sizeof(m));
  cuuint64_t dims[3] = {(cuuint64_t)pitch, (cuuint64_t)rowsMax, (cuuint64_t)planes};
  cuuint64_t strides[2] = {(cuuint64_t)pitch * 2, (cuuint64_t)planeBytes};
  cuuint32_t box[3] = {(cuuint32_t)TC_BK, (cuuint32_t)boxRows, 1};
  cuuint32_t es[3] = {1, 1, 1};
  CUresult r = g_encode(&m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, const_cast<__nv_bfloat16*>(base), dims, strides, box,
                        es, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                        CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) throw std::string("cuda: cuTensorMapEncodeTiled failed");
  return m;
}

void tc_gemm(cgpu_ctx* c, int gemmId, const CUtensorMap& ta, const CUtensorMap& tb, int bn, float* P, int terms,
             int segPitch, int nSplit, int Mmax, int Nmax, int* err) {
  if (segPitch % TC_BK != 0) throw std::string("tc_gemm: segment pitch must be a multiple of 64");
  if (bn == 64) launch_gemm_t<64, 6>(c, ta, tb, P, gemmId, terms, segPitch, nSplit, Mmax, Nmax, err);
  else if (bn == 128) launch_gemm_t<128, 5>(c, ta, tb, P, gemmId, terms, segPitch, nSplit, Mmax, Nmax, err);
  else launch_gemm_t<256, 4>(c, ta, tb, P, gemmId, terms, segPitch, nSplit, Mmax, Nmax, err);
}
