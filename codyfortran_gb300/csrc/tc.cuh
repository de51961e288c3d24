// tc.cuh -- tcgen05 GEMM entry points shared by the mixed-precision kernels.
#pragma once
#include <cuda_bf16.h>

#include "common.cuh"

// Picks the K-split count that fills ~one wave of 152 SMs (each split keeps >= 2 K tiles).
int tc_split_count(int M, int N, int BN, int kTiles);
// N-tile width used for an output of N columns (64, 128 or 256).
int tc_tile_n(int N);
// P[split][M][N] (fp32) = A[M,K] B[N,K]^T; A and B bf16 K-major, K a multiple of 64.
// Returns the number of splits written.
int tc_gemm(cgpu_ctx* c, const __nv_bfloat16* A, int M, const __nv_bfloat16* B, int N, int K, float* P, int nSplit,
            int* err);
