// tc.cuh -- tcgen05 GEMM entry points shared by the mixed-precision kernels.
#pragma once
#include <cuda.h>
#include <cuda_bf16.h>

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
