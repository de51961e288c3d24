// k_ci.cu -- CI vector kernels over determinant bitstrings.
//
//   * ConfigList tables generated on the device (SetupSinglesData /
//     SetupDoublesData, src/ConfigList/AllActive/S_ConfigList_AllActive.f90:141-349):
//     candidate excitations in the reference loop order, validity and fermion
//     sign from popcounts (ExciteConfiguration,
//     src/ConfigList/AllActive/Fermions/S_ConfigList_AllActive_Fermions.f90:232-334),
//     target index from the lexicographic rank (Combinatorics_IndexOfCombiNoRepeat,
//     src/Utils/M_Utils_Combinatorics.f90:43-73) written as an additive table;
//     warp ballots compact the valid candidates so the tables are bit-exact.
//   * H1/H2 application and RDM accumulation (ApplyH1FillRdm1 / ApplyH2FillRdm2,
//     src/Coeffs/Generic/S_Coeffs_Generic.f90:103-319), one warp per global
//     configuration.
//   * h1/h2 folding and RDM unfolding (FillH1Lin :440-464, FillH2Lin :478-542,
//     FillRdm1FromRdm1Lin :325-349, FillRdm2FromRdm2Lin :362-434).
#include <algorithm>
#include <type_traits>

#include "common.cuh"

namespace {

// threads of an RDM pair-gather block (one pair of singles codes per thread):
// the staged CI vector (up to 72 KB) allows three blocks per SM and the
// registers two of 512 threads, so the block size sets the warps in flight for
// these latency-bound gathers
constexpr int CI_PAIR_THREADS = 512;
// threads of an RDM code-gather block (one code per warp)
constexpr int CI_RDM_THREADS = 512;
// threads of an H.C block (one configuration per warp): with 55 registers per
// thread two 512-thread blocks fit an SM, 32 warps sharing two staged CI vectors
constexpr int CI_APPLY_THREADS = 512;

__device__ __forceinline__ unsigned long long bitmask_below(int p) {  // bits [0, p)
  return p >= 64 ? ~0ULL : ((1ULL << p) - 1ULL);
}

// Apply a_j (1-based orbital) to code; returns false if unoccupied.
__device__ __forceinline__ bool destroy(unsigned long long& code, int j, int& sgn) {
  unsigned long long b = 1ULL << (j - 1);
  if (!(code & b)) return false;
  sgn ^= __popcll(code & bitmask_below(j - 1)) & 1;
  code &= ~b;
  return true;
}

__device__ __forceinline__ bool create(unsigned long long& code, int i, int& sgn) {
  unsigned long long b = 1ULL << (i - 1);
  if (code & b) return false;
  sgn ^= __popcll(code & bitmask_below(i - 1)) & 1;
  code |= b;
  return true;
}

// rank = 1 + C(M,N) + sum over occupied orbitals of rankTab[pos][orb]
__device__ __forceinline__ int rank_of(unsigned long long code, const int* __restrict__ rankTab, int M, int base) {
  int r = base;
  int pos = 1;
  while (code) {
    int b = __ffsll((long long)code);  // 1-based orbital
    r += rankTab[pos * (M + 1) + b];
    pos++;
    code &= code - 1ULL;
  }
  return r;
}

__device__ __forceinline__ void decode_tri(int a, int& hi, int& lo) {  // a = hi(hi-1)/2 + (lo-1), lo <= hi, 1-based
  int h = (int)((1.0 + sqrt(1.0 + 8.0 * (double)a)) * 0.5);
  while (h * (h - 1) / 2 > a) h--;
  while ((h + 1) * h / 2 <= a) h++;
  hi = h;
  lo = a - h * (h - 1) / 2 + 1;
}

// kind 0: singles, 1: doubles.  fill == 0: count into nConn; fill == 1: write tables.
__global__ void k_build_tables(int kind, int fill, const int64_t* __restrict__ codes, int nConf, int M, int nO,
                               int shift, const int* __restrict__ rankTab, int rankBase, int* __restrict__ nConn,
                               int maxConn, int* __restrict__ exc, int* __restrict__ ocode, int8_t* __restrict__ fac) {
  int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  int lane = threadIdx.x & 31;
  if (warp >= nConf) return;
  unsigned long long code0 = (unsigned long long)codes[warp];
  int P = M * (M + 1) / 2;
  long nCand = (kind == 0) ? (long)M * M : (long)P * P;
  int count = 0;
  for (long base = 0; base < nCand; base += 32) {
    long idx = base + lane;
    bool ok = false;
    int sgn = 0, newIdx = 0, oc = 0;
    if (idx < nCand) {
      unsigned long long code = code0;
      if (kind == 0) {
        int j1 = (int)(idx / M) + 1, i1 = (int)(idx % M) + 1;
        ok = destroy(code, j1, sgn) && create(code, i1, sgn);
        if (ok) oc = (i1 + shift - 1) * nO + (j1 + shift);
      } else {
        int a = (int)(idx / P), b = (int)(idx % P);
        int j2, j1, i2, i1;
        decode_tri(a, j2, j1);
        decode_tri(b, i2, i1);
        // destroys left to right (j1 then j2), creates reversed (i2 then i1)
        ok = destroy(code, j1, sgn) && destroy(code, j2, sgn) && create(code, i2, sgn) && create(code, i1, sgn);
        if (ok) oc = (((i1 + shift - 1) * nO + (j1 + shift) - 1) * nO + (i2 + shift) - 1) * nO + (j2 + shift);
      }
      if (ok) newIdx = rank_of(code, rankTab, M, rankBase);
    }
    unsigned int bal = __ballot_sync(0xffffffffu, ok);
    if (fill && ok) {
      int k = count + __popc(bal & ((1u << lane) - 1u));
      size_t at = (size_t)k + (size_t)maxConn * warp;
      exc[at] = newIdx;
      ocode[at] = oc;
      fac[at] = sgn ? -1 : 1;
    }
    count += __popc(bal);
  }
  if (lane == 0 && !fill) nConn[warp] = count;
}

// ---------------------------------------------------------------------------
// Traversal kernels: one warp per global configuration I (1-based iCoeff).
// ---------------------------------------------------------------------------
__device__ __forceinline__ void conf_from_index(const CiView& v, int I, int* conf) {
  int t = I - 1;
  for (int b = 0; b < v.nBt; b++) {
    conf[b] = t % v.nConf[b] + 1;
    t /= v.nConf[b];
  }
}

__device__ __forceinline__ z_t warp_sum(z_t a) {
  for (int o = 16; o > 0; o >>= 1) {
    a.x += __shfl_xor_sync(0xffffffffu, a.x, o);
    a.y += __shfl_xor_sync(0xffffffffu, a.y, o);
  }
  return a;
}

// The CI vector of the block's trajectory: staged in shared memory when it fits
// (random gathers of C then hit shared memory), else read from global memory.
__device__ __forceinline__ const z_t* stage_coeffs(const z_t* __restrict__ Cg, int nC, z_t* sm, int useSmem) {
  if (!useSmem) return Cg;
  for (int i = threadIdx.x; i < nC; i += blockDim.x) sm[i] = Cg[i];
  __syncthreads();
  return sm;
}

// H.C: one warp per configuration, the configurations of one trajectory in a
// block (work[blockIdx.x] = trajectory and range, balanced by the number of terms).
__global__ void k_ci_apply(const z_t* __restrict__ C0, z_t* __restrict__ dC0, const z_t* __restrict__ h1Lin0,
                           const z_t* __restrict__ h2Lin0, TRAJ_ARGS, const CiWork* __restrict__ work, int useSmem,
                           int useH1, int useH2) {
  extern __shared__ z_t csm[];
  const CiWork wk = work[blockIdx.x];
  const int tb = wk.traj;
  const CiView& v = shp[tb].view;
  const z_t* C = stage_coeffs(batn(C0, bs, tb), v.nC, csm, useSmem);
  z_t* dC = batn(dC0, bs, tb);
  const z_t* h1Lin = batn(h1Lin0, bs, tb);
  const z_t* h2Lin = batn(h2Lin0, bs, tb);
  const int lane = threadIdx.x & 31;
  const int nw = blockDim.x >> 5;
  for (int warp = wk.t0 + (threadIdx.x >> 5); warp < wk.t1; warp += nw) {
  int I = warp + 1;
  int conf[CODY_MAX_BT];
  conf_from_index(v, I, conf);
  z_t acc = zmk(0.0, 0.0);
  int nO2 = v.nO * v.nO;
  for (int b = 0; b < v.nBt; b++) {
    int c = conf[b];
    int st = v.stride[b];
    if (useH1) {
      int n = v.sN[b][c - 1];
      size_t col = (size_t)v.maxS[b] * (c - 1);
      for (int k = lane; k < n; k += 32) {
        int oc = v.sCode[b][col + k];
        int jG = I + (v.sExc[b][col + k] - c) * st;
        zfma(acc, h1Lin[oc], zsign(C[jG - 1], v.sFac[b][col + k] < 0));
      }
    }
    if (useH2) {
      int n = v.dN[b][c - 1];
      size_t col = (size_t)v.maxD[b] * (c - 1);
      for (int k = lane; k < n; k += 32) {
        int oc = v.dCode[b][col + k];
        int jG = I + (v.dExc[b][col + k] - c) * st;
        zfma(acc, h2Lin[oc], zsign(C[jG - 1], v.dFac[b][col + k] < 0));
      }
      // inter-body-type terms: products of singles on b and b2 > b (Generic :266-300).
      // Lane k2 holds an edge of b2, the edges of b are broadcast one by one.
      int n1 = v.sN[b][c - 1];
      size_t col1 = (size_t)v.maxS[b] * (c - 1);
      for (int b2 = b + 1; b2 < v.nBt; b2++) {
        int c2 = conf[b2];
        int n2 = v.sN[b2][c2 - 1];
        size_t col2 = (size_t)v.maxS[b2] * (c2 - 1);
        int st2 = v.stride[b2];
        for (int k2b = 0; k2b < n2; k2b += 32) {
          int k2 = k2b + lane;
          bool has2 = k2 < n2;
          int oc2 = has2 ? v.sCode[b2][col2 + k2] : 0;
          int d2 = has2 ? (v.sExc[b2][col2 + k2] - c2) * st2 : 0;
          int f2 = has2 ? v.sFac[b2][col2 + k2] : 0;
          for (int k1b = 0; k1b < n1; k1b += 32) {
            int k1 = k1b + lane;
            int oc1 = 0, d1 = 0, f1 = 0;
            if (k1 < n1) {
              oc1 = v.sCode[b][col1 + k1];
              d1 = (v.sExc[b][col1 + k1] - c) * st;
              f1 = v.sFac[b][col1 + k1];
            }
            int cnt = min(32, n1 - k1b);
#pragma unroll 4
            for (int u = 0; u < cnt; u++) {
              int o1 = __shfl_sync(0xffffffffu, oc1, u);
              int e1 = __shfl_sync(0xffffffffu, d1, u);
              int g1 = __shfl_sync(0xffffffffu, f1, u);
              if (has2) {
                zfma(acc, h2Lin[(o1 - 1) * nO2 + oc2], zsign(C[I - 1 + e1 + d2], g1 * f2 < 0));
              }
            }
          }
        }
      }
    }
  }
  acc = warp_sum(acc);
  if (lane == 0) dC[warp] = zadd(dC[warp], acc);
  }
}

// H.C in double-float arithmetic (the fixed-point forms): the same traversal as
// k_ci_apply with C staged in shared memory as double-floats, the integrals read
// from their double-float copies and every term an FP32 error-free product
// with two-sum accumulation (~47 bits); one conversion to FP64 per configuration.
__global__ void k_ci_apply_df(const z_t* __restrict__ C0, z_t* __restrict__ dC0, const float4* __restrict__ h1Df0,
                              const float4* __restrict__ h2Df0, TRAJ_ARGS, const CiWork* __restrict__ work, int useH1,
                              int useH2) {
  extern __shared__ float4 cdf[];
  const CiWork wk = work[blockIdx.x];
  const int tb = wk.traj;
  const CiView& v = shp[tb].view;
  const z_t* Cg = batn(C0, bs, tb);
  for (int i = threadIdx.x; i < v.nC; i += blockDim.x) cdf[i] = zdf_from(Cg[i]);
  __syncthreads();
  const float4* C = cdf;
  z_t* dC = batn(dC0, bs, tb);
  const float4* h1 = batn(h1Df0, bs, tb);
  const float4* h2 = batn(h2Df0, bs, tb);
  const int lane = threadIdx.x & 31;
  const int nw = blockDim.x >> 5;
  for (int warp = wk.t0 + (threadIdx.x >> 5); warp < wk.t1; warp += nw) {
    int I = warp + 1;
    int conf[CODY_MAX_BT];
    conf_from_index(v, I, conf);
    zdf_acc acc = {0.0f, 0.0f, 0.0f, 0.0f};
    int nO2 = v.nO * v.nO;
    for (int b = 0; b < v.nBt; b++) {
      int c = conf[b];
      int st = v.stride[b];
      if (useH1) {
        int n = v.sN[b][c - 1];
        size_t col = (size_t)v.maxS[b] * (c - 1);
        for (int k = lane; k < n; k += 32) {
          int oc = v.sCode[b][col + k];
          int jG = I + (v.sExc[b][col + k] - c) * st;
          zdf_fma(acc, h1[oc], C[jG - 1], v.sFac[b][col + k] < 0);
        }
      }
      if (useH2) {
        int n = v.dN[b][c - 1];
        size_t col = (size_t)v.maxD[b] * (c - 1);
        for (int k = lane; k < n; k += 32) {
          int oc = v.dCode[b][col + k];
          int jG = I + (v.dExc[b][col + k] - c) * st;
          zdf_fma(acc, h2[oc], C[jG - 1], v.dFac[b][col + k] < 0);
        }
        int n1 = v.sN[b][c - 1];
        size_t col1 = (size_t)v.maxS[b] * (c - 1);
        for (int b2 = b + 1; b2 < v.nBt; b2++) {
          int c2 = conf[b2];
          int n2 = v.sN[b2][c2 - 1];
          size_t col2 = (size_t)v.maxS[b2] * (c2 - 1);
          int st2 = v.stride[b2];
          if (n1 <= 32 && n2 <= 32) {
            // the n1 x n2 pairs of singles spread over all lanes: lane k holds
            // entry k of both tables (integral row / column, configuration
            // offset, sign in bit 0 of the packed code), pair t = (t / n2, t % n2)
            int p1 = 0, e1 = 0, p2 = 0, e2 = 0;
            if (lane < n1) {
              p1 = ((v.sCode[b][col1 + lane] - 1) * nO2) * 2 + (v.sFac[b][col1 + lane] < 0);
              e1 = (v.sExc[b][col1 + lane] - c) * st;
            }
            if (lane < n2) {
              p2 = v.sCode[b2][col2 + lane] * 2 + (v.sFac[b2][col2 + lane] < 0);
              e2 = (v.sExc[b2][col2 + lane] - c2) * st2;
            }
            const int total = n1 * n2, q = 32 / n2, r = 32 - q * n2;
            int k1 = lane / n2, k2 = lane - k1 * n2;
            for (int base = 0; base < total; base += 32) {
              const int a1 = __shfl_sync(0xffffffffu, p1, k1 & 31), x1 = __shfl_sync(0xffffffffu, e1, k1 & 31);
              const int a2 = __shfl_sync(0xffffffffu, p2, k2), x2 = __shfl_sync(0xffffffffu, e2, k2);
              if (base + lane < total)
                zdf_fma(acc, h2[(a1 >> 1) + (a2 >> 1)], C[I - 1 + x1 + x2], ((a1 ^ a2) & 1) != 0);
              k1 += q;
              k2 += r;
              if (k2 >= n2) {
                k2 -= n2;
                k1++;
              }
            }
          } else
          for (int k2b = 0; k2b < n2; k2b += 32) {
            int k2 = k2b + lane;
            bool has2 = k2 < n2;
            int oc2 = has2 ? v.sCode[b2][col2 + k2] : 0;
            int d2 = has2 ? (v.sExc[b2][col2 + k2] - c2) * st2 : 0;
            int f2 = has2 ? v.sFac[b2][col2 + k2] : 0;
            for (int k1b = 0; k1b < n1; k1b += 32) {
              int k1 = k1b + lane;
              int oc1 = 0, d1 = 0, f1 = 0;
              if (k1 < n1) {
                oc1 = v.sCode[b][col1 + k1];
                d1 = (v.sExc[b][col1 + k1] - c) * st;
                f1 = v.sFac[b][col1 + k1];
              }
              int cnt = min(32, n1 - k1b);
#pragma unroll 4
              for (int u = 0; u < cnt; u++) {
                int o1 = __shfl_sync(0xffffffffu, oc1, u);
                int e1 = __shfl_sync(0xffffffffu, d1, u);
                int g1 = __shfl_sync(0xffffffffu, f1, u);
                if (has2) zdf_fma(acc, h2[(o1 - 1) * nO2 + oc2], C[I - 1 + e1 + d2], g1 * f2 < 0);
              }
            }
          }
        }
      }
    }
    acc = zdf_warp_sum(acc);
    if (lane == 0) dC[warp] = zadd(dC[warp], zdf_to_z(acc));
  }
}

// Configuration index (0-based) of the body types other than b1 and b2 (b2 < 0:
// only b1 excluded), from r in mixed radix over those body types.
__device__ __forceinline__ int rest_base(const CiView& v, int r, int b1, int b2) {
  int I = 0;
  for (int b = 0; b < v.nBt; b++) {
    if (b == b1 || b == b2) continue;
    int n = v.nConf[b];
    I += (r % n) * v.stride[b];
    r /= n;
  }
  return I;
}

// RDMs (ApplyH1FillRdm1 / ApplyH2FillRdm2, S_Coeffs_Generic.f90:103-319) as
// gathers: rdmLin(oc) = sum over the excitations (I -> J) with orbital code
// oc of f conj(C_J) C_I.  Every entry has exactly one writer, so there are no
// atomics.  k_ci_rdm_codes: one warp per code of one body type (singles ->
// rdm1, doubles -> rdm2), lanes over the code's excitations (and over the
// configurations of the other body types); k_ci_rdm_pairs: one thread per pair
// of singles codes of two body types (the inter-body-type part of rdm2).
__global__ void k_ci_rdm_codes(const z_t* __restrict__ C0, z_t* __restrict__ r1Lin0, z_t* __restrict__ r2Lin0,
                               TRAJ_ARGS, const CiWork* __restrict__ work, int useSmem, int want1, int want2) {
  extern __shared__ z_t csm[];
  const CiWork wk = work[blockIdx.x];
  const int tb = wk.traj;
  const CiView& v = shp[tb].view;
  const z_t* C = stage_coeffs(batn(C0, bs, tb), v.nC, csm, useSmem);
  z_t* r1Lin = batn(r1Lin0, bs, tb);
  z_t* r2Lin = batn(r2Lin0, bs, tb);
  int nS = 0;
  for (int b = 0; b < v.nBt; b++) nS += v.nSc[b];
  const int lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  for (int task = wk.t0 + (threadIdx.x >> 5); task < wk.t1; task += nw) {
    int q = task;
    const int kind = q < nS ? 0 : 1;
    if (kind == 1) q -= nS;
    if ((kind == 0 && !want1) || (kind == 1 && !want2)) continue;
    int b = 0;
    const int* cnt = kind == 0 ? v.nSc : v.nDc;
    while (q >= cnt[b]) q -= cnt[b++];
    const int* start = kind == 0 ? v.sxStart[b] : v.dxStart[b];
    const int* src = kind == 0 ? v.sxSrc[b] : v.dxSrc[b];
    const int* dst = kind == 0 ? v.sxDst[b] : v.dxDst[b];
    const int8_t* fac = kind == 0 ? v.sxFac[b] : v.dxFac[b];
    const int e0 = start[q], e1 = start[q + 1];
    const int nRest = v.nC / v.nConf[b], st = v.stride[b];
    z_t acc = zmk(0.0, 0.0);
    if (nRest == 1) {
      for (int e = e0 + lane; e < e1; e += 32) zcfma(acc, C[dst[e] * st], zsign(C[src[e] * st], fac[e] < 0));
    } else if (v.nBt == 2) {  // as in k_ci_rdm_codes_df: (e, r) advanced without divisions
      const int sto = v.stride[1 - b], q = 32 / nRest, rr = 32 - q * nRest;
      int e = e0 + lane / nRest, r = lane % nRest;
      for (int t = lane; t < (e1 - e0) * nRest; t += 32) {
        const int base = r * sto;
        zcfma(acc, C[base + dst[e] * st], zsign(C[base + src[e] * st], fac[e] < 0));
        e += q;
        r += rr;
        if (r >= nRest) {
          r -= nRest;
          e++;
        }
      }
    } else {
      for (int t = lane; t < (e1 - e0) * nRest; t += 32) {
        int e = e0 + t / nRest, r = t % nRest;
        int base = rest_base(v, r, b, -1);
        zcfma(acc, C[base + dst[e] * st], zsign(C[base + src[e] * st], fac[e] < 0));
      }
    }
    acc = warp_sum(acc);
    if (lane == 0) (kind == 0 ? r1Lin : r2Lin)[kind == 0 ? v.sxCode[b][q] : v.dxCode[b][q]] = acc;
  }
}

__global__ void k_ci_rdm_pairs(const z_t* __restrict__ C0, z_t* __restrict__ r2Lin0, TRAJ_ARGS,
                               const CiWork* __restrict__ work, int useSmem) {
  extern __shared__ z_t csm[];
  const CiWork wk = work[blockIdx.x];
  const int tb = wk.traj;
  const CiView& v = shp[tb].view;
  const z_t* C = stage_coeffs(batn(C0, bs, tb), v.nC, csm, useSmem);
  z_t* r2Lin = batn(r2Lin0, bs, tb);
  const int nO2 = v.nO * v.nO;
  for (int task = wk.t0 + threadIdx.x; task < wk.t1; task += blockDim.x) {
    int q = task, b1 = 0, b2 = 1;
    for (;;) {
      int seg = v.nSc[b1] * v.nSc[b2];
      if (q < seg) break;
      q -= seg;
      if (++b2 >= v.nBt) { b1++; b2 = b1 + 1; }
    }
    int q1 = q / v.nSc[b2], q2 = q % v.nSc[b2];
    int s1 = v.sxStart[b1][q1], n1 = v.sxStart[b1][q1 + 1] - s1;
    int s2 = v.sxStart[b2][q2], n2 = v.sxStart[b2][q2 + 1] - s2;
    int st1 = v.stride[b1], st2 = v.stride[b2];
    int nRest = v.nC / (v.nConf[b1] * v.nConf[b2]);
    const int *src1 = v.sxSrc[b1], *dst1 = v.sxDst[b1], *src2 = v.sxSrc[b2], *dst2 = v.sxDst[b2];
    const int8_t *fac1 = v.sxFac[b1], *fac2 = v.sxFac[b2];
    z_t acc = zmk(0.0, 0.0);
    for (int e1 = s1; e1 < s1 + n1; e1++) {
      int i1 = src1[e1] * st1, j1 = dst1[e1] * st1;
      bool g1 = fac1[e1] < 0;
#pragma unroll 4
      for (int e2 = s2; e2 < s2 + n2; e2++) {
        int i2 = src2[e2] * st2, j2 = dst2[e2] * st2;
        bool neg = g1 != (fac2[e2] < 0);
        for (int r = 0; r < nRest; r++) {
          int base = nRest == 1 ? 0 : rest_base(v, r, b1, b2);
          zcfma(acc, C[base + j1 + j2], zsign(C[base + i1 + i2], neg));
        }
      }
    }
    r2Lin[(v.sxCode[b1][q1] - 1) * nO2 + v.sxCode[b2][q2]] = acc;
  }
}

// The RDM gathers in double-float arithmetic (the fixed-point forms): as
// k_ci_rdm_codes / k_ci_rdm_pairs with C staged as double-floats and every
// product conj(C_J) C_I an FP32 error-free product with two-sum accumulation.
__global__ void __launch_bounds__(CI_RDM_THREADS, 2) k_ci_rdm_codes_df(const z_t* __restrict__ C0, z_t* __restrict__ r1Lin0, z_t* __restrict__ r2Lin0,
                                  TRAJ_ARGS, const CiWork* __restrict__ work, int want1, int want2) {
  extern __shared__ float4 cdf[];
  const CiWork wk = work[blockIdx.x];
  const int tb = wk.traj;
  const CiView& v = shp[tb].view;
  const z_t* Cg = batn(C0, bs, tb);
  for (int i = threadIdx.x; i < v.nC; i += blockDim.x) cdf[i] = zdf_from(Cg[i]);
  __syncthreads();
  const float4* C = cdf;
  z_t* r1Lin = batn(r1Lin0, bs, tb);
  z_t* r2Lin = batn(r2Lin0, bs, tb);
  int nS = 0;
  for (int b = 0; b < v.nBt; b++) nS += v.nSc[b];
  const int lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  for (int task = wk.t0 + (threadIdx.x >> 5); task < wk.t1; task += nw) {
    int q = task;
    const int kind = q < nS ? 0 : 1;
    if (kind == 1) q -= nS;
    if ((kind == 0 && !want1) || (kind == 1 && !want2)) continue;
    int b = 0;
    const int* cnt = kind == 0 ? v.nSc : v.nDc;
    while (q >= cnt[b]) q -= cnt[b++];
    const int* start = kind == 0 ? v.sxStart[b] : v.dxStart[b];
    const int* src = kind == 0 ? v.sxSrc[b] : v.dxSrc[b];
    const int* dst = kind == 0 ? v.sxDst[b] : v.dxDst[b];
    const int8_t* fac = kind == 0 ? v.sxFac[b] : v.dxFac[b];
    const int e0 = start[q], e1 = start[q + 1];
    const int nRest = v.nC / v.nConf[b], st = v.stride[b];
    zdf_acc acc = {0.0f, 0.0f, 0.0f, 0.0f};
    if (nRest == 1) {
      for (int e = e0 + lane; e < e1; e += 32) zdf_cfma(acc, C[dst[e] * st], C[src[e] * st], fac[e] < 0);
    } else if (v.nBt == 2) {
      // term t = (excitation e0 + t / nRest, configuration r = t % nRest of the
      // other body type), advanced by 32 terms per step without divisions
      const int sto = v.stride[1 - b], q = 32 / nRest, rr = 32 - q * nRest;
      int e = e0 + lane / nRest, r = lane % nRest;
      for (int t = lane; t < (e1 - e0) * nRest; t += 32) {
        const int base = r * sto;
        zdf_cfma(acc, C[base + dst[e] * st], C[base + src[e] * st], fac[e] < 0);
        e += q;
        r += rr;
        if (r >= nRest) {
          r -= nRest;
          e++;
        }
      }
    } else {
      for (int t = lane; t < (e1 - e0) * nRest; t += 32) {
        int e = e0 + t / nRest, r = t % nRest;
        int base = rest_base(v, r, b, -1);
        zdf_cfma(acc, C[base + dst[e] * st], C[base + src[e] * st], fac[e] < 0);
      }
    }
    acc = zdf_warp_sum(acc);
    if (lane == 0) (kind == 0 ? r1Lin : r2Lin)[kind == 0 ? v.sxCode[b][q] : v.dxCode[b][q]] = zdf_to_z(acc);
  }
}

__global__ void __launch_bounds__(CI_PAIR_THREADS, 2) k_ci_rdm_pairs_df(const z_t* __restrict__ C0, z_t* __restrict__ r2Lin0, TRAJ_ARGS,
                                  const CiWork* __restrict__ work) {
  extern __shared__ float4 cdf[];
  const CiWork wk = work[blockIdx.x];
  const int tb = wk.traj;
  const CiView& v = shp[tb].view;
  const z_t* Cg = batn(C0, bs, tb);
  for (int i = threadIdx.x; i < v.nC; i += blockDim.x) cdf[i] = zdf_from(Cg[i]);
  __syncthreads();
  const float4* C = cdf;
  z_t* r2Lin = batn(r2Lin0, bs, tb);
  const int nO2 = v.nO * v.nO;
  for (int task = wk.t0 + threadIdx.x; task < wk.t1; task += blockDim.x) {
    int q = task, b1 = 0, b2 = 1;
    for (;;) {
      int seg = v.nSc[b1] * v.nSc[b2];
      if (q < seg) break;
      q -= seg;
      if (++b2 >= v.nBt) { b1++; b2 = b1 + 1; }
    }
    int q1 = q / v.nSc[b2], q2 = q % v.nSc[b2];
    int s1 = v.sxStart[b1][q1], n1 = v.sxStart[b1][q1 + 1] - s1;
    int s2 = v.sxStart[b2][q2], n2 = v.sxStart[b2][q2 + 1] - s2;
    int st1 = v.stride[b1], st2 = v.stride[b2];
    int nRest = v.nC / (v.nConf[b1] * v.nConf[b2]);
    const int *src1 = v.sxSrc[b1], *dst1 = v.sxDst[b1], *src2 = v.sxSrc[b2], *dst2 = v.sxDst[b2];
    const int8_t *fac1 = v.sxFac[b1], *fac2 = v.sxFac[b2];
    zdf_acc acc = {0.0f, 0.0f, 0.0f, 0.0f};
    for (int e1 = s1; e1 < s1 + n1; e1++) {
      int i1 = src1[e1] * st1, j1 = dst1[e1] * st1;
      bool g1 = fac1[e1] < 0;
#pragma unroll 4
      for (int e2 = s2; e2 < s2 + n2; e2++) {
        int i2 = src2[e2] * st2, j2 = dst2[e2] * st2;
        bool neg = g1 != (fac2[e2] < 0);
        for (int r = 0; r < nRest; r++) {
          int base = nRest == 1 ? 0 : rest_base(v, r, b1, b2);
          zdf_cfma(acc, C[base + j1 + j2], C[base + i1 + i2], neg);
        }
      }
    }
    r2Lin[(v.sxCode[b1][q1] - 1) * nO2 + v.sxCode[b2][q2]] = zdf_to_z(acc);
  }
}

// FillH1Lin: h1Lin((i1-1)*nO + j1) = h1(i1, j1)
__global__ void k_fold_h1(z_t* __restrict__ h1Lin, float4* __restrict__ h1Df, const z_t* __restrict__ h1,
                          TRAJ_ARGS) {
  const int nO = shp[blockIdx.z].nO;
  h1Lin = bat(h1Lin, bs);
  h1Df = bat(h1Df, bs);
  h1 = bat(h1, bs);
  GRID_STRIDE(e, nO * nO) {
    int i1 = (int)(e % nO), j1 = (int)(e / nO);  // 0-based
    h1Lin[i1 * nO + j1 + 1] = h1[e];
    if (h1Df) h1Df[i1 * nO + j1 + 1] = zdf_from(h1[e]);
  }
}

// FillH2Lin (fermions; inter-body-type pairs use the same antisymmetric form)
__global__ void k_fold_h2(z_t* __restrict__ h2Lin, float4* __restrict__ h2Df, const z_t* __restrict__ h2,
                          const int* __restrict__ btOf, TRAJ_ARGS) {
  const int nO = shp[blockIdx.z].nO;
  size_t n4 = (size_t)nO * nO * nO * nO;
  h2Lin = bat(h2Lin, bs);
  h2Df = bat(h2Df, bs);
  h2 = bat(h2, bs);
  btOf = bat(btOf, bs);
  GRID_STRIDE(e, n4) {
    // e = orbCode - 1 with orbCode = (((i1-1) nO + j1 - 1) nO + i2 - 1) nO + j2
    int j2 = (int)(e % nO), i2 = (int)((e / nO) % nO), j1 = (int)((e / nO / nO) % nO), i1 = (int)(e / nO / nO / nO);
    const size_t n = nO;
    const z_t v = h2lin_value(btOf, i1, j1, i2, j2,
                              [&](int a, int b, int c, int d) { return h2[a + n * (b + n * (c + n * d))]; });
    h2Lin[e + 1] = v;
    if (h2Df) h2Df[e + 1] = zdf_from(v);
  }
}

// FillH2Lin straight from the spatial H2s (inside the NonLin derivative: the
// nO^4 h2 is not formed); the same values as k_h2_layout + k_fold_h2.  h2Lin
// (FP64) is written when non-null, h2Df when non-null.  Only the codes of
// FillH2Lin's rule are written: the CI apply reads no other code, and the
// others keep the zeros of the set-up.
// The valid entries i1 < i2, j1 < j2 as pairs p1 = (i1, i2), p2 = (j1, j2) in
// the triangle order (a shared-memory table of P = nO (nO - 1) / 2 pairs): each
// block takes FOLD_CHUNK consecutive p1, its threads all p2; entry
// e = ((i1 nO + j1) nO + i2) nO + j2.
constexpr int FOLD_CHUNK = 8;
constexpr int FOLD_MAX_NO = 64;
__global__ void k_fold_h2s(z_t* __restrict__ h2Lin, float4* __restrict__ h2Df, const z_t* __restrict__ H2s,
                           const int* __restrict__ btOf, TRAJ_ARGS) {
  const TrajShape& T = shp[blockIdx.z];
  const int nO = T.nO, n = T.nOS, restricted = T.restricted, P = nO * (nO - 1) / 2;
  const int p1a = blockIdx.x * FOLD_CHUNK;
  if (p1a >= P) return;
  h2Lin = bat(h2Lin, bs);
  h2Df = bat(h2Df, bs);
  H2s = bat(H2s, bs);
  btOf = bat(btOf, bs);
  __shared__ unsigned char pa[FOLD_MAX_NO * (FOLD_MAX_NO - 1) / 2], pb[FOLD_MAX_NO * (FOLD_MAX_NO - 1) / 2];
  for (int u = 0, base = 0; u < nO - 1; base += nO - 1 - u, u++)
    for (int v = u + 1 + (int)threadIdx.x; v < nO; v += blockDim.x) {
      pa[base + v - u - 1] = (unsigned char)u;
      pb[base + v - u - 1] = (unsigned char)v;
    }
  __syncthreads();
  for (int p1 = p1a; p1 < min(P, p1a + FOLD_CHUNK); p1++) {
    const int i1 = pa[p1], i2 = pb[p1];
    for (int p2 = threadIdx.x; p2 < P; p2 += blockDim.x) {
      const int j1 = pa[p2], j2 = pb[p2];
      if (!bt_rule_ok(btOf, i1, i2, j1, j2)) continue;
      const z_t v = h2lin_value(btOf, i1, j1, i2, j2, [&](int a, int b, int c, int d) {
        return h2_from_h2s(H2s, btOf, restricted, n, a, b, c, d);
      });
      const size_t e = (((size_t)i1 * nO + j1) * nO + i2) * nO + j2;
      if (h2Lin) h2Lin[e + 1] = v;
      if (h2Df) h2Df[e + 1] = zdf_from(v);
    }
  }
}

__global__ void k_unfold_rdm1(z_t* __restrict__ rdm1, const z_t* __restrict__ lin, TRAJ_ARGS) {
  const int nO = shp[blockIdx.z].nO;
  rdm1 = bat(rdm1, bs);
  lin = bat(lin, bs);
  GRID_STRIDE(e, nO * nO) {
    int i1 = (int)(e % nO), j1 = (int)(e / nO);
    rdm1[e] = lin[i1 * nO + j1 + 1];
  }
}

// FillRdm2FromRdm2Lin written per output element: rdm2(a,b,c,d) gathers the
// (up to four) signed lin entries the reference scatters into it.
__global__ void k_unfold_rdm2(z_t* __restrict__ rdm2, const z_t* __restrict__ lin, const int* __restrict__ btOf,
                              TRAJ_ARGS) {
  size_t n = shp[blockIdx.z].nO;
  rdm2 = bat(rdm2, bs);
  lin = bat(lin, bs);
  btOf = bat(btOf, bs);
  GRID_STRIDE(e, n * n * n * n) {
    int a = (int)(e % n), b = (int)((e / n) % n), c = (int)((e / n / n) % n), d = (int)(e / n / n / n);
    rdm2[e] = rdm2_from_lin(lin, btOf, n, a, b, c, d);
  }
}

// Groups an excitation table (maxConn x nConf, on the device) by orbital code:
// distinct codes ascending, edges of one code in table order.
void group_by_code(int nConf, int maxConn, const int* nConn_d, const int* exc_d, const int* code_d,
                   const int8_t* fac_d, int& nCodes, int*& xCode, int*& xStart, int*& xSrc, int*& xDst,
                   int8_t*& xFac, std::vector<int>& nHost, std::vector<int>& startHost) {
  std::vector<int> n(nConf), exc((size_t)maxConn * nConf), code((size_t)maxConn * nConf);
  std::vector<int8_t> fac((size_t)maxConn * nConf);
  CODY_CUDA(cudaMemcpy(n.data(), nConn_d, sizeof(int) * nConf, cudaMemcpyDeviceToHost));
  CODY_CUDA(cudaMemcpy(exc.data(), exc_d, sizeof(int) * exc.size(), cudaMemcpyDeviceToHost));
  CODY_CUDA(cudaMemcpy(code.data(), code_d, sizeof(int) * code.size(), cudaMemcpyDeviceToHost));
  CODY_CUDA(cudaMemcpy(fac.data(), fac_d, fac.size(), cudaMemcpyDeviceToHost));
  std::vector<int> codes;
  size_t E = 0;
  for (int c = 0; c < nConf; c++) E += n[c];
  codes.reserve(E);
  for (int c = 0; c < nConf; c++)
    for (int k = 0; k < n[c]; k++) codes.push_back(code[(size_t)maxConn * c + k]);
  std::sort(codes.begin(), codes.end());
  codes.erase(std::unique(codes.begin(), codes.end()), codes.end());
  nCodes = (int)codes.size();
  std::vector<int> start(nCodes + 1, 0), src(std::max<size_t>(E, 1)), dst(std::max<size_t>(E, 1));
  std::vector<int8_t> f(std::max<size_t>(E, 1));
  auto slot = [&](int oc) { return (int)(std::lower_bound(codes.begin(), codes.end(), oc) - codes.begin()); };
  for (int c = 0; c < nConf; c++)
    for (int k = 0; k < n[c]; k++) start[slot(code[(size_t)maxConn * c + k]) + 1]++;
  for (int q = 0; q < nCodes; q++) start[q + 1] += start[q];
  std::vector<int> fill(start.begin(), start.end() - 1);
  for (int c = 0; c < nConf; c++)
    for (int k = 0; k < n[c]; k++) {
      size_t at = (size_t)maxConn * c + k;
      int e = fill[slot(code[at])]++;
      src[e] = c;
      dst[e] = exc[at] - 1;
      f[e] = fac[at];
    }
  auto upload = [](auto& dptr, const auto& v) {
    using T = typename std::remove_reference<decltype(v)>::type::value_type;
    CODY_CUDA(cudaMalloc(&dptr, sizeof(T) * std::max<size_t>(v.size(), 1)));
    if (!v.empty()) CODY_CUDA(cudaMemcpy(dptr, v.data(), sizeof(T) * v.size(), cudaMemcpyHostToDevice));
  };
  if (codes.empty()) codes.push_back(0);
  upload(xCode, codes);
  upload(xStart, start);
  upload(xSrc, src);
  upload(xDst, dst);
  upload(xFac, f);
  nHost = n;
  startHost = start;
}

long long binom_h(int n, int k) {
  if (k < 0 || n < 0 || k > n) return (n == k) ? 1 : 0;
  long double r = 1.0;
  for (int i = 1; i <= k; i++) r = r * (n - k + i) / i;
  return (long long)llroundl(r);
}

}  // namespace

// ConfigList_Setup for one system: codes in GSL lexicographic order on the
// host, tables on the device (separate allocations, referenced by s.view).
void ci_build_tables(cgpu_ctx* c, SysHost& s) {
  s.view.nBt = c->nBt;
  s.view.nO = s.nO;
  int stride = 1;
  for (int b = 0; b < c->nBt; b++) {
    CiTables& t = s.tab[b];
    int M = s.nOrbs[b], N = s.nBodies[b];
    t.nOrbs = M;
    t.nBodies = N;
    t.shift = s.orbStart[b];
    if (M > 63 || N > M) throw std::string("ConfigList: unsupported orbital/body counts");
    long long nconf = 0;
    for (int k = 0; k <= N; k++) nconf += binom_h(M - N, k) * binom_h(N, k);
    if (nconf > (1LL << 30)) throw std::string("ConfigList: too many configurations");
    t.nConf = (int)nconf;
    std::vector<int64_t> codes(t.nConf);
    std::vector<int> comb(N);
    for (int i = 0; i < N; i++) comb[i] = i;
    for (int iC = 0; iC < t.nConf; iC++) {
      int64_t code = 0;
      for (int j = 0; j < N; j++) code |= (int64_t)1 << comb[j];
      codes[iC] = code;
      int i = N - 1;
      while (i >= 0 && comb[i] == M - N + i) i--;
      if (i < 0) break;
      comb[i]++;
      for (int j = i + 1; j < N; j++) comb[j] = comb[j - 1] + 1;
    }
    // additive rank table: rankTab[i][c] = (i<N ? C(M-c, N-i) : 0) - C(M-c+1, N-i+1)
    std::vector<int> rt((size_t)(N + 1) * (M + 1), 0);
    for (int i = 1; i <= N; i++)
      for (int cc = 1; cc <= M; cc++)
        rt[(size_t)i * (M + 1) + cc] =
            (int)((i < N ? binom_h(M - cc, N - i) : 0) - binom_h(M - cc + 1, N - i + 1));
    int rankBase = 1 + (int)binom_h(M, N);
    CODY_CUDA(cudaMalloc(&t.codes, sizeof(int64_t) * t.nConf));
    CODY_CUDA(cudaMalloc(&t.rankTab, sizeof(int) * rt.size()));
    CODY_CUDA(cudaMemcpy(t.codes, codes.data(), sizeof(int64_t) * t.nConf, cudaMemcpyHostToDevice));
    CODY_CUDA(cudaMemcpy(t.rankTab, rt.data(), sizeof(int) * rt.size(), cudaMemcpyHostToDevice));
    CODY_CUDA(cudaMalloc(&t.sN, sizeof(int) * t.nConf));
    CODY_CUDA(cudaMalloc(&t.dN, sizeof(int) * t.nConf));
    int threads = 256;
    int blocks = (t.nConf * 32 + threads - 1) / threads;
    for (int kind = 0; kind < 2; kind++) {
      int* nConn = kind == 0 ? t.sN : t.dN;
      k_build_tables<<<blocks, threads, 0, c->stream>>>(kind, 0, t.codes, t.nConf, M, s.nO, t.shift, t.rankTab,
                                                         rankBase, nConn, 0, nullptr, nullptr, nullptr);
      CODY_LAUNCHED(c);
      std::vector<int> h(t.nConf);
      CODY_CUDA(cudaMemcpyAsync(h.data(), nConn, sizeof(int) * t.nConf, cudaMemcpyDeviceToHost, c->stream));
      CODY_CUDA(cudaStreamSynchronize(c->stream));
      int mx = *std::max_element(h.begin(), h.end());
      int mxa = std::max(mx, 1);
      int **exc = kind == 0 ? &t.sExc : &t.dExc, **oc = kind == 0 ? &t.sCode : &t.dCode;
      int8_t** fac = kind == 0 ? &t.sFac : &t.dFac;
      CODY_CUDA(cudaMalloc(exc, sizeof(int) * (size_t)mxa * t.nConf));
      CODY_CUDA(cudaMalloc(oc, sizeof(int) * (size_t)mxa * t.nConf));
      CODY_CUDA(cudaMalloc(fac, sizeof(int8_t) * (size_t)mxa * t.nConf));
      CODY_CUDA(cudaMemsetAsync(*exc, 0, sizeof(int) * (size_t)mxa * t.nConf, c->stream));
      CODY_CUDA(cudaMemsetAsync(*oc, 0, sizeof(int) * (size_t)mxa * t.nConf, c->stream));
      CODY_CUDA(cudaMemsetAsync(*fac, 0, sizeof(int8_t) * (size_t)mxa * t.nConf, c->stream));
      k_build_tables<<<blocks, threads, 0, c->stream>>>(kind, 1, t.codes, t.nConf, M, s.nO, t.shift, t.rankTab,
                                                         rankBase, nConn, mxa, *exc, *oc, *fac);
      CODY_LAUNCHED(c);
      if (kind == 0) t.maxS = mx; else t.maxD = mx;
    }
    CODY_CUDA(cudaStreamSynchronize(c->stream));  // the tables are written on the context stream
    group_by_code(t.nConf, std::max(t.maxS, 1), t.sN, t.sExc, t.sCode, t.sFac, t.nSc, t.sxCode, t.sxStart, t.sxSrc,
                  t.sxDst, t.sxFac, s.hsN[b], s.hsxStart[b]);
    group_by_code(t.nConf, std::max(t.maxD, 1), t.dN, t.dExc, t.dCode, t.dFac, t.nDc, t.dxCode, t.dxStart, t.dxSrc,
                  t.dxDst, t.dxFac, s.hdN[b], s.hdxStart[b]);
    CiView& v = s.view;
    v.nSc[b] = t.nSc;
    v.nDc[b] = t.nDc;
    v.sxCode[b] = t.sxCode; v.sxStart[b] = t.sxStart; v.sxSrc[b] = t.sxSrc; v.sxDst[b] = t.sxDst; v.sxFac[b] = t.sxFac;
    v.dxCode[b] = t.dxCode; v.dxStart[b] = t.dxStart; v.dxSrc[b] = t.dxSrc; v.dxDst[b] = t.dxDst; v.dxFac[b] = t.dxFac;
    v.stride[b] = stride;
    v.nConf[b] = t.nConf;
    v.maxS[b] = std::max(t.maxS, 1);
    v.maxD[b] = std::max(t.maxD, 1);
    v.sN[b] = t.sN; v.sExc[b] = t.sExc; v.sCode[b] = t.sCode; v.sFac[b] = t.sFac;
    v.dN[b] = t.dN; v.dExc[b] = t.dExc; v.dCode[b] = t.dCode; v.dFac[b] = t.dFac;
    stride *= t.nConf;
  }
  s.view.nC = stride;
  CODY_CUDA(cudaStreamSynchronize(c->stream));
}

// Work lists of the CI kernels: per trajectory, the configurations (H.C) and the
// RDM tasks, cut into blocks of about the same number of terms.
void ci_build_work(cgpu_ctx* c) {
  std::vector<CiWork> apply, rdm, pairs;
  std::vector<std::vector<long>> aw(c->nb), rw(c->nb), pw(c->nb);
  long aTot = 0, rTot = 0, pTot = 0;
  for (int t = 0; t < c->nb; t++) {
    const SysHost& s = c->sys[t];
    const CiView& v = s.view;
    aw[t].resize(s.nC);
    for (int I = 0; I < s.nC; I++) {
      int conf[CODY_MAX_BT], r = I;
      for (int b = 0; b < v.nBt; b++) {
        conf[b] = r % v.nConf[b];
        r /= v.nConf[b];
      }
      long w = 1;
      for (int b = 0; b < v.nBt; b++) {
        w += s.hsN[b][conf[b]] + s.hdN[b][conf[b]];
        for (int b2 = b + 1; b2 < v.nBt; b2++) w += (long)s.hsN[b][conf[b]] * s.hsN[b2][conf[b2]];
      }
      aw[t][I] = w;
      aTot += w;
    }
    for (int b = 0; b < v.nBt; b++)
      for (int q = 0; q < v.nSc[b]; q++)
        rw[t].push_back(1 + (long)(s.hsxStart[b][q + 1] - s.hsxStart[b][q]) * (v.nC / v.nConf[b]));
    for (int b = 0; b < v.nBt; b++)
      for (int q = 0; q < v.nDc[b]; q++)
        rw[t].push_back(1 + (long)(s.hdxStart[b][q + 1] - s.hdxStart[b][q]) * (v.nC / v.nConf[b]));
    for (int b1 = 0; b1 < v.nBt; b1++)
      for (int b2 = b1 + 1; b2 < v.nBt; b2++) {
        long nRest = v.nC / ((long)v.nConf[b1] * v.nConf[b2]);
        for (int q1 = 0; q1 < v.nSc[b1]; q1++)
          for (int q2 = 0; q2 < v.nSc[b2]; q2++)
            pw[t].push_back(1 + (long)(s.hsxStart[b1][q1 + 1] - s.hsxStart[b1][q1]) *
                                    (s.hsxStart[b2][q2 + 1] - s.hsxStart[b2][q2]) * nRest);
      }
    for (long w : rw[t]) rTot += w;
    for (long w : pw[t]) pTot += w;
  }
  // about 8 blocks per SM in total; a block never spans two trajectories
  auto cut = [](const std::vector<std::vector<long>>& wts, long target, int maxItems, std::vector<CiWork>& out) {
    for (int t = 0; t < (int)wts.size(); t++) {
      int n = (int)wts[t].size(), t0 = 0;
      long acc = 0;
      for (int i = 0; i < n; i++) {
        acc += wts[t][i];
        if (acc >= target || i + 1 - t0 >= maxItems || i == n - 1) {
          out.push_back(CiWork{t, t0, i + 1});
          t0 = i + 1;
          acc = 0;
        }
      }
    }
  };
  // a block holds at least ~8 configurations (one per warp) / ~CI_PAIR_THREADS RDM pair tasks (one per
  // thread) on average
  long nConfTot = 0, nTaskTot = 0, nPairTot = 0;
  for (int t = 0; t < c->nb; t++) {
    nConfTot += (long)aw[t].size();
    nTaskTot += (long)rw[t].size();
    nPairTot += (long)pw[t].size();
  }
  cut(aw, std::max({64L, aTot / (8 * 152), (long)(CI_APPLY_THREADS / 32) * aTot / std::max(1L, nConfTot)}), 1 << 20,
      apply);
  cut(rw, std::max({64L, rTot / (8 * 152), (long)(CI_RDM_THREADS / 32) * rTot / std::max(1L, nTaskTot)}), 1 << 20,
      rdm);
  cut(pw, std::max({64L, pTot / (8 * 152), (long)CI_PAIR_THREADS * pTot / std::max(1L, nPairTot)}), 1 << 20, pairs);
  c->nApplyWork = (int)apply.size();
  c->nRdmWork = (int)rdm.size();
  c->nPairWork = (int)pairs.size();
  auto put = [](CiWork*& d, const std::vector<CiWork>& h) {
    CODY_CUDA(cudaMalloc(&d, sizeof(CiWork) * std::max<size_t>(h.size(), 1)));
    if (!h.empty()) CODY_CUDA(cudaMemcpy(d, h.data(), sizeof(CiWork) * h.size(), cudaMemcpyHostToDevice));
  };
  put(c->applyWork_d, apply);
  put(c->rdmWork_d, rdm);
  put(c->pairWork_d, pairs);
  // the CI vector of one trajectory in shared memory when it fits
  size_t need = sizeof(z_t) * (size_t)c->nC;
  c->ciSmem = need <= 72 * 1024 ? (int)need : 0;  // leaves room for three blocks per SM
  if (c->ciSmem > 48 * 1024) {
    CODY_CUDA(cudaFuncSetAttribute(k_ci_apply, cudaFuncAttributeMaxDynamicSharedMemorySize, c->ciSmem));
    CODY_CUDA(cudaFuncSetAttribute(k_ci_apply_df, cudaFuncAttributeMaxDynamicSharedMemorySize, c->ciSmem));
    CODY_CUDA(cudaFuncSetAttribute(k_ci_rdm_codes_df, cudaFuncAttributeMaxDynamicSharedMemorySize, c->ciSmem));
    CODY_CUDA(cudaFuncSetAttribute(k_ci_rdm_pairs_df, cudaFuncAttributeMaxDynamicSharedMemorySize, c->ciSmem));
    CODY_CUDA(cudaFuncSetAttribute(k_ci_rdm_codes, cudaFuncAttributeMaxDynamicSharedMemorySize, c->ciSmem));
    CODY_CUDA(cudaFuncSetAttribute(k_ci_rdm_pairs, cudaFuncAttributeMaxDynamicSharedMemorySize, c->ciSmem));
  }
}

void launch_ci_apply(cgpu_ctx* c, const z_t* C, z_t* dC, int useH1, int useH2) {
  ProfScope prof(c, CGPU_KERNEL_CI_APPLY);
  if (c->ciDf && c->ciSmem > 0)
    k_ci_apply_df<<<c->nApplyWork, CI_APPLY_THREADS, c->ciSmem, c->stream>>>(C, dC, c->h1Df_d, c->h2Df_d,
                                                                            TRAJ_PASS(c), c->applyWork_d, useH1,
                                                                            useH2);
  else
    k_ci_apply<<<c->nApplyWork, 256, c->ciSmem, c->stream>>>(C, dC, c->h1Lin_d, c->h2Lin_d, TRAJ_PASS(c),
                                                            c->applyWork_d, c->ciSmem > 0, useH1, useH2);
  CODY_LAUNCHED(c);
}

void launch_ci_rdm(cgpu_ctx* c, const z_t* C, int want1, int want2) {
  ProfScope prof(c, CGPU_KERNEL_CI_RDM);
  size_t n2 = (size_t)c->nO * c->nO, n4 = n2 * n2;
  // every code present is written; the other entries of the Lin arrays stay zero
  const bool df = c->ciDf && c->ciSmem > 0;
  if (c->nRdmWork > 0) {
    if (df)
      k_ci_rdm_codes_df<<<c->nRdmWork, CI_RDM_THREADS, c->ciSmem, c->stream>>>(C, c->rdm1Lin_d, c->rdm2Lin_d, TRAJ_PASS(c),
                                                                    c->rdmWork_d, want1, want2);
    else
      k_ci_rdm_codes<<<c->nRdmWork, 256, c->ciSmem, c->stream>>>(C, c->rdm1Lin_d, c->rdm2Lin_d, TRAJ_PASS(c),
                                                                 c->rdmWork_d, c->ciSmem > 0, want1, want2);
    CODY_LAUNCHED(c);
  }
  if (want2 && c->nPairWork > 0) {
    if (df)
      k_ci_rdm_pairs_df<<<c->nPairWork, CI_PAIR_THREADS, c->ciSmem, c->stream>>>(C, c->rdm2Lin_d, TRAJ_PASS(c),
                                                                              c->pairWork_d);
    else
      k_ci_rdm_pairs<<<c->nPairWork, CI_PAIR_THREADS, c->ciSmem, c->stream>>>(C, c->rdm2Lin_d, TRAJ_PASS(c),
                                                                              c->pairWork_d, c->ciSmem > 0);
    CODY_LAUNCHED(c);
  }
  if (want1) {
    k_unfold_rdm1<<<bgrid(c, ew_blocks(c, n2)), 256, 0, c->stream>>>(c->rdm1_d, c->rdm1Lin_d, TRAJ_PASS(c));
    CODY_LAUNCHED(c);
  }
  if (want2 && !c->fuseLayouts) {
    k_unfold_rdm2<<<bgrid(c, ew_blocks(c, n4)), 256, 0, c->stream>>>(c->rdm2_d, c->rdm2Lin_d, c->btOfOrb_d,
                                                                       TRAJ_PASS(c));
    CODY_LAUNCHED(c);
  }
}

void launch_fold_h1(cgpu_ctx* c) {
  ProfScope prof(c, CGPU_KERNEL_FOLD);
  size_t n2 = (size_t)c->nO * c->nO;
  k_fold_h1<<<bgrid(c, ew_blocks(c, n2)), 256, 0, c->stream>>>(c->h1Lin_d, c->ciDf ? c->h1Df_d : nullptr, c->h1_d,
                                                               TRAJ_PASS(c));
  CODY_LAUNCHED(c);
}

void launch_fold_h2(cgpu_ctx* c) {
  ProfScope prof(c, CGPU_KERNEL_FOLD);
  size_t n4 = (size_t)c->nO * c->nO * c->nO * c->nO;
  if (c->fuseLayouts) {
    // h2Lin from the spatial H2s; the FP64 copy only when the FP64 CI apply reads it
    const bool dfOnly = c->ciDf && c->ciSmem > 0;
    if (c->nO > FOLD_MAX_NO) throw std::string("FillH2Lin: more than 64 spin orbitals is not supported");
    const int P = c->nO * (c->nO - 1) / 2;
    k_fold_h2s<<<dim3((unsigned)ceil_div(P, FOLD_CHUNK), 1, c->nb), 128, 0, c->stream>>>(
        dfOnly ? nullptr : c->h2Lin_d, c->ciDf ? c->h2Df_d : nullptr, c->h2s_d, c->btOfOrb_d, TRAJ_PASS(c));
  } else {
    k_fold_h2<<<bgrid(c, ew_blocks(c, n4)), 256, 0, c->stream>>>(c->h2Lin_d, c->ciDf ? c->h2Df_d : nullptr, c->h2_d,
                                                                 c->btOfOrb_d, TRAJ_PASS(c));
  }
  CODY_LAUNCHED(c);
}
