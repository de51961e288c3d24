// k_mixed.cu -- mixed-precision form of ApplyCorrelationOp
// (src/Method/Mb/OrbBased/S_Method_Mb_OrbBased.f90:647-872).
//
// The three contractions run on the tcgen05 GEMM (k_tc.cu) with split-bf16
// operands and FP32 accumulation; split-K partials, the correlation
// epilogue, the RDMs, rho^-1 and everything else stay FP64.
//
//   GEMM1  W[g][2p+s]   = sum_g' V[g][g'] S_s(p, g')            (M=nG, N=2P, K=nG)
//   GEMM2  Z[g][2q+s]   = sum_k  W[g][k] R''[2q+s][k]           (M=nG, N=2Q, K=2P)
//   GEMM3  G[2p+s][2p'+t] = sum_g S_s(p,g) W_t(p',g)            (M=N=2P, K=nG)
// with p, p' unordered orbital pairs (l <= k), s,t in {re, im}, q = (k1, j)
// an ordered pair.  The conjugate symmetry W_(k,l) = conj(W_(l,k)) folds the
// ordered-pair sums into real GEMMs over unordered pairs:
//   sum_(l2,k2) W_(l2k2) R'[(l2,k2), q] = sum_p a_p X_p[q] + b_p Y_p[q],
//   W_p = a_p + i b_p,  X_p = R1 + R2,  Y_p = i (R1 - R2),
//   R1 = R'[(l,k), q], R2 = R'[(k,l), q] (0 when l = k).
//
// The fixed-point form (precision mixed_fx / mixed_fx6) carries every operand
// row as L base-2^b digit slices under one power of two per row (k_fx.cu) and
// returns FP64 results whose only error is the operand truncation (at least
// 30 / 36 bits of each row's maximum): S and V rows for GEMM1, W rows for
// GEMM2, R'' rows, W columns for GEMM3.  fx_plan picks the digit width b of
// each contraction length (GEMM1/3: K = nG, GEMM2: K = 2P) and the slice
// count L = ceil(bits / b).  S carries LS = max(L1, L3) slices: GEMM1 reads
// the first L1 (dropping balanced digits costs at most half a unit of the
// last digit kept), GEMM3 L3.  The row exponents of W come from the GEMM1
// epilogue, or from the reduction of its K splits.
#include <cuda_bf16.h>

#include <array>

#include <algorithm>

#include "common.cuh"
#include "tc.cuh"

struct MixedBufs {
  int terms = 3;            // 3: bf16x3, 6: bf16x6
  int KgMax = 0, KpMax = 0; // segment pitches: the largest padded K of the grid / pair contractions
  int bn1 = 64, bn2 = 64, bn3 = 64;
  int s1 = 1, s2 = 1, s3 = 1;  // K splits of the three GEMMs
  __nv_bfloat16 *VxB = nullptr, *SxA = nullptr, *WxA = nullptr, *WTxB = nullptr, *RxB = nullptr;
  float *P1 = nullptr, *P2 = nullptr, *P3 = nullptr;
  int* err = nullptr;
  double* Zd = nullptr;     // (nG, Q) complex
  CUtensorMap mV, mS, mSasB, mW, mWT, mR;  // TMA maps (A operands box 128 rows, B operands box BN rows)
  // fixed-point form (fxBits > 0): digit width / slices of the K = nG
  // contractions (GEMM1, GEMM3) and of the K = 2P one (GEMM2)
  int fxBits = 0, b1 = 0, L1 = 0, b2 = 0, L2 = 0;
  int fxBits3 = 0, L3 = 0, LS = 0;  // GEMM3 target and slices; S carries LS = max(L1, L3) slices
  bool compact1 = false, compact2 = false, compact3 = false;  // two-CTAs-per-SM configuration per GEMM
  int sCap1 = 1, sCap2 = 1, sCap3 = 1;  // K splits the FP64 partial buffers hold (the tuner stays within them)
  // one interaction matrix per root grid (cgpu_ctx::fxShared): slices [root][c->nG][L1 KgBig]
  // and row exponents [root][c->nG], outside the per-trajectory arena
  // tile lists of the persistent fixed-point GEMMs (device) and their lengths
  void *tiles1 = nullptr, *tiles2 = nullptr, *tiles3 = nullptr;
  int nTiles1 = 0, nTiles2 = 0, nTiles3 = 0;
  int KgBig = 0;
  __nv_bfloat16* Vsh = nullptr;
  int* eVsh = nullptr;
  CUtensorMap mVsh;
  int *eV = nullptr, *eS = nullptr, *eWr = nullptr, *eWc = nullptr, *eR = nullptr;  // row exponents
  unsigned *mWr = nullptr, *mWc = nullptr;  // largest biased exponent of |W| per row g / column n
  double *Wd = nullptr, *Zp = nullptr, *Gd = nullptr;  // FP64 results [split][M][N]
};

namespace {

// Segment patterns: A operands [hi,hi,lo] / [hi,hi,mid,hi,mid,lo],
// B operands [hi,lo,hi] / [hi,mid,hi,lo,mid,hi]; part index 0=hi, 1=mid, 2=lo.
__device__ __forceinline__ int seg_part(int terms, int isB, int seg) {
  if (terms == 3) {
    const int a[3] = {0, 0, 2}, b[3] = {0, 2, 0};
    return isB ? b[seg] : a[seg];
  }
  const int a[6] = {0, 0, 1, 0, 1, 2}, b[6] = {0, 1, 0, 2, 1, 0};
  return isB ? b[seg] : a[seg];
}

// x = hi + mid + lo in bf16 (for terms == 3 the low part is bf16(x - hi)).
__device__ __forceinline__ __nv_bfloat16 split_part(double x, int terms, int part) {
  __nv_bfloat16 hi = __double2bfloat16(x);
  if (part == 0) return hi;
  double r1 = x - (double)__bfloat162float(hi);
  __nv_bfloat16 mid = __double2bfloat16(r1);
  if (terms == 3) return mid;  // the "lo" part of the two-term split
  if (part == 1) return mid;
  return __double2bfloat16(r1 - (double)__bfloat162float(mid));
}

// out[row][seg*pitch + k] = part(value(row,k)), zero for k >= K.
__device__ __forceinline__ void write_split(__nv_bfloat16* out, int row, int k, int K, int pitch, int terms, int isB,
                                            double v) {
  size_t base = (size_t)row * terms * pitch;
  for (int seg = 0; seg < terms; seg++) {
    __nv_bfloat16 h = (k < K) ? split_part(v, terms, seg_part(terms, isB, seg)) : __double2bfloat16(0.0);
    out[base + (size_t)seg * pitch + k] = h;
  }
}

// FP64 -> FP32 by truncating the significand (integer operations only: the FP64
// pipes are the scarce resource).  |x| below the FP32 normal range flushes to
// zero; relative error < 2^-23, below the bf16x3 form's ~2^-16.
__device__ __forceinline__ float f64_to_f32(double x) {
  unsigned long long u = (unsigned long long)__double_as_longlong(x);
  unsigned hi = (unsigned)(u >> 32);
  unsigned sign = hi & 0x80000000u;
  int e = (int)((hi >> 20) & 0x7FFu) - 1023 + 127;
  if (e <= 0) return __int_as_float((int)sign);
  if (e >= 255) return __int_as_float((int)(sign | 0x7F800000u));
  unsigned mant = ((hi & 0xFFFFFu) << 3) | (unsigned)((u >> 29) & 7u);
  return __int_as_float((int)(sign | ((unsigned)e << 23) | mant));
}

// bf16x3 split in FP32: hi = bf16(v), lo = bf16(v - hi); A rows [hi,hi,lo], B rows [hi,lo,hi].
__device__ __forceinline__ void write_split3(__nv_bfloat16* out, int row, int k, int K, int pitch, int isB, float v) {
  size_t base = (size_t)row * 3 * pitch + k;
  __nv_bfloat16 hi = __float2bfloat16_rn(0.0f), lo = hi;
  if (k < K) {
    hi = __float2bfloat16_rn(v);
    lo = __float2bfloat16_rn(v - __bfloat162float(hi));
  }
  out[base] = hi;
  out[base + pitch] = isB ? lo : hi;
  out[base + 2 * (size_t)pitch] = isB ? hi : lo;
}

__global__ void k_split_V(__nv_bfloat16* __restrict__ out, const double* __restrict__ V, int pitch, int terms,
                          TRAJ_ARGS) {
  const TrajShape& T = shp[blockIdx.z];
  const int nG = T.nG, Kpad = T.Kg;
  out = bat(out, bs);
  V = bat(V, bs);
  GRID_STRIDE(e, (size_t)nG * Kpad) {
    int row = (int)(e / Kpad), k = (int)(e % Kpad);
    double v = (k < nG) ? V[(size_t)row * nG + k] : 0.0;
    write_split(out, row, k, nG, pitch, terms, 1, v);
  }
}

// S_s(p, g) = (re, im)[conj(phi_l) phi_k w] for pair p = (l, k), A pattern.
__global__ void k_split_S(__nv_bfloat16* __restrict__ outA, const z_t* __restrict__ orbs, const double* __restrict__ w,
                          const int* __restrict__ pl, const int* __restrict__ pk, int pitch, int terms, TRAJ_ARGS) {
  const TrajShape& T = shp[blockIdx.z];
  const int nG = T.nG, nP = T.nPairs, Kpad = T.Kg;
  outA = bat(outA, bs);
  orbs = bat(orbs, bs);
  w = bat(w, bs);
  pl = bat(pl, bs);
  pk = bat(pk, bs);
  GRID_STRIDE(e, (size_t)2 * nP * Kpad) {
    int row = (int)(e / Kpad), g = (int)(e % Kpad);
    int p = row >> 1, s = row & 1;
    if (terms == 3) {
      float v = 0.0f;
      if (g < nG) {
        z_t a = orbs[(size_t)nG * pl[p] + g], b = orbs[(size_t)nG * pk[p] + g];
        float ar = f64_to_f32(a.x), ai = f64_to_f32(a.y), br = f64_to_f32(b.x), bi = f64_to_f32(b.y);
        float wg = f64_to_f32(w[g]);
        v = s ? (ar * bi - ai * br) * wg : (ar * br + ai * bi) * wg;
      }
      write_split3(outA, row, g, nG, pitch, 0, v);
    } else {
      double v = 0.0;
      if (g < nG) {
        z_t a = orbs[(size_t)nG * pl[p] + g], b = orbs[(size_t)nG * pk[p] + g];
        z_t sv = zscale(zcmul(a, b), w[g]);
        v = s ? sv.y : sv.x;
      }
      write_split(outA, row, g, nG, pitch, terms, 0, v);
    }
  }
}

// W[g][n] = sum_z P1[z][g][n] (FP64), split to WxA (g-major, K = 2P, zero for
// n >= 2P) and WTxB (pair-major, K = nG, zero for g >= nG).  A 32 x 32 tile of
// (g, n) per block: read along n, transposed through shared memory, written
// along n (WxA) and along g (WTxB).
constexpr int SW_T = 32;

__global__ void __launch_bounds__(256) k_split_W(__nv_bfloat16* __restrict__ WxA, __nv_bfloat16* __restrict__ WTxB,
                                                 const float* __restrict__ P1, int nSplit, int pitchP, int pitchG,
                                                 int terms, TRAJ_ARGS) {
  __shared__ double tile[SW_T][SW_T + 1];
  const TrajShape& T = shp[blockIdx.z];
  const int nG = T.nG, N2P = 2 * T.nPairs, KpP = T.Kp, KpG = T.Kg;
  const int g0 = blockIdx.x * SW_T, n0 = blockIdx.y * SW_T;
  if (g0 >= KpG || n0 >= KpP) return;
  WxA = bat(WxA, bs);
  WTxB = bat(WTxB, bs);
  P1 = bat(P1, bs);
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;  // 32 x 8
  for (int r = ty; r < SW_T; r += 8) {
    int g = g0 + r, n = n0 + tx;
    double v = 0.0;
    if (g < nG && n < N2P)
      for (int z = 0; z < nSplit; z++) v += (double)P1[((size_t)z * nG + g) * N2P + n];
    tile[r][tx] = v;
    if (g < nG && n < KpP) {
      if (terms == 3) write_split3(WxA, g, n, N2P, pitchP, 0, (float)v);
      else write_split(WxA, g, n, N2P, pitchP, terms, 0, v);
    }
  }
  __syncthreads();
  for (int r = ty; r < SW_T; r += 8) {
    int n = n0 + r, g = g0 + tx;
    if (n < N2P && g < KpG) {
      if (terms == 3) write_split3(WTxB, n, g, nG, pitchG, 1, (float)tile[tx][r]);
      else write_split(WTxB, n, g, nG, pitchG, terms, 1, tile[tx][r]);
    }
  }
}

// R'' rows n = 2q + s (s: re/im of the output), K = 2p + t (t: a or b of W_p).
__global__ void k_split_R(__nv_bfloat16* __restrict__ RxB, const z_t* __restrict__ Rp, const int* __restrict__ pl,
                          const int* __restrict__ pk, int pitchP, int terms, TRAJ_ARGS) {
  const TrajShape& T = shp[blockIdx.z];
  const int n = T.nOS, nP = T.nPairs, KpP = T.Kp;
  int Q = n * n;
  RxB = bat(RxB, bs);
  Rp = bat(Rp, bs);
  pl = bat(pl, bs);
  pk = bat(pk, bs);
  GRID_STRIDE(e, (size_t)2 * Q * KpP) {
    int row = (int)(e / KpP), k = (int)(e % KpP);
    int q = row >> 1, s = row & 1;
    double v = 0.0;
    if (k < 2 * nP) {
      int p = k >> 1, t = k & 1;
      int l = pl[p], kk = pk[p];
      z_t R1 = Rp[(size_t)(l * n + kk) * Q + q];
      z_t R2 = (l < kk) ? Rp[(size_t)(kk * n + l) * Q + q] : zmk(0.0, 0.0);
      // X = R1 + R2, Y = i (R1 - R2): re/im parts of the selected one
      double r1 = s ? (t ? R1.x : R1.y) : (t ? -R1.y : R1.x);
      double r2 = s ? (t ? R2.x : R2.y) : (t ? -R2.y : R2.x);
      v = t ? r1 - r2 : r1 + r2;
    }
    if (terms == 3) write_split3(RxB, row, k, 2 * nP, pitchP, 1, f64_to_f32(v));
    else write_split(RxB, row, k, 2 * nP, pitchP, terms, 1, v);
  }
}

// Z[g][q] (complex) = sum_z P2[z][g][2q+s]
template <class PT>
__global__ void k_reduce_Z(z_t* __restrict__ Z, const PT* __restrict__ P2, int nSplit, TRAJ_ARGS) {
  const TrajShape& T = shp[blockIdx.z];
  const int nG = T.nG, Q = T.nOS * T.nOS;
  Z = bat(Z, bs);
  P2 = bat(P2, bs);
  GRID_STRIDE(e, (size_t)nG * Q) {
  int g = (int)(e / Q), q = (int)(e % Q);
  double re = 0.0, im = 0.0;
  for (int z = 0; z < nSplit; z++) {
    const PT* r = P2 + ((size_t)z * nG + g) * 2 * Q + 2 * q;
    re += (double)r[0];
    im += (double)r[1];
  }
  Z[e] = zmk(re, im);
  }
}

// H2s[(i1*n+j1)][(l2*n+k2)] = 1/2 sum_g S_(i1j1) W_(l2k2) from the unordered-pair products.
template <class PT>
__global__ void k_reduce_H2(z_t* __restrict__ H2s, const PT* __restrict__ P3, int nSplit,
                            const int* __restrict__ pidx, TRAJ_ARGS) {
  const TrajShape& T = shp[blockIdx.z];
  const int n = T.nOS, nP = T.nPairs;
  int Q = n * n;
  H2s = bat(H2s, bs);
  P3 = bat(P3, bs);
  pidx = bat(pidx, bs);
  GRID_STRIDE(e, (size_t)Q * Q) {
  int row = (int)(e / Q), col = (int)(e % Q);
  int i1 = row / n, j1 = row % n, l2 = col / n, k2 = col % n;
  bool c1 = i1 > j1, c2 = l2 > k2;
  int p = c1 ? pidx[j1 * n + i1] : pidx[i1 * n + j1];
  int pp = c2 ? pidx[k2 * n + l2] : pidx[l2 * n + k2];
  z_t v = zmk(0.0, 0.0);
  if (p >= 0 && pp >= 0) {
    int N2 = 2 * nP;
    double rr = 0, ii = 0, ri = 0, ir = 0;
    for (int z = 0; z < nSplit; z++) {
      const PT* G = P3 + (size_t)z * N2 * N2;
      rr += G[(size_t)(2 * p) * N2 + 2 * pp];
      ii += G[(size_t)(2 * p + 1) * N2 + 2 * pp + 1];
      ri += G[(size_t)(2 * p) * N2 + 2 * pp + 1];
      ir += G[(size_t)(2 * p + 1) * N2 + 2 * pp];
    }
    z_t G1 = zmk(rr - ii, ri + ir);   // sum S_p W_p'
    z_t G2 = zmk(rr + ii, ir - ri);   // sum S_p conj(W_p')
    if (!c1 && !c2) v = G1;
    else if (!c1 && c2) v = G2;
    else if (c1 && !c2) v = zconj(G2);
    else v = zconj(G1);
    v = zscale(v, 0.5);
  }
  H2s[e] = v;
  }
}


// ---- fixed-point digit slices -------------------------------------------------

constexpr int FX_LMAX = 8;

// Signed base-2^b digits of x relative to 2^e (|x| < 2^e): X = round(x 2^(bL-e))
// = sum_i d_i 2^(b(L-1-i)), d_i in [-2^(b-1), 2^(b-1)) for i > 0, |d_0| <= 2^b.
// Integer operations only (bL <= 52; 32-bit arithmetic when bL <= 30).  With
// H = 2^(b-1) sum_{k<L-1} 2^(bk), the digits of Y = X + H below the top one
// are the plain base-2^b digits d_i + 2^(b-1), so every digit is an
// independent bit field of Y: d_i = field_i(Y) - 2^(b-1), d_0 = Y >> b(L-1)
// (arithmetic shift).  The balanced representation is unique, so this gives
// the digits of the carry-by-carry division.
// BT / LT > 0 fix the digit width / slice count at compile time (constant
// shifts); 0 takes them from bRt / LRt.
template <int BT, int LT>
__device__ __forceinline__ void fx_digits_t(double x, int e, int bRt, int LRt, int (&d)[FX_LMAX]) {
  const int b = BT > 0 ? BT : bRt, L = LT > 0 ? LT : LRt;
  const unsigned long long u = (unsigned long long)__double_as_longlong(x);
  const int ex = (int)((u >> 52) & 0x7FF);
  long long X = 0;
  if (ex != 0) {
    const unsigned long long mant = (u & 0xFFFFFFFFFFFFFull) | (1ull << 52);
    const int sh = 1075 - ex - b * L + e;  // >= 53 - bL > 0 because |x| < 2^e
    if (sh < 63) X = (long long)((mant + (1ull << (sh - 1))) >> sh);
    if (u >> 63) X = -X;
  }
  const int mask = (1 << b) - 1, half = 1 << (b - 1);
  if (b * L <= 30) {  // |X| <= 2^30, H < 2^30
    int H = 0;
#pragma unroll
    for (int i = 1; i < FX_LMAX; i++)
      if (i < L) H = (H << b) | half;
    const int Y = (int)X + H;
#pragma unroll
    for (int i = 1; i < FX_LMAX; i++)
      if (i < L) d[i] = ((int)((unsigned)Y >> (b * (L - 1 - i))) & mask) - half;
    d[0] = Y >> (b * (L - 1));
    return;
  }
  long long H = 0;
#pragma unroll
  for (int i = 1; i < FX_LMAX; i++)
    if (i < L) H = (H << b) | half;
  const long long Y = X + H;
#pragma unroll
  for (int i = 1; i < FX_LMAX; i++)
    if (i < L) d[i] = ((int)((unsigned long long)Y >> (b * (L - 1 - i))) & mask) - half;
  d[0] = (int)(Y >> (b * (L - 1)));
}

// bf16 of an integer |d| <= 256 without a conversion instruction: the FP32
// magic-number sum 1.5 2^23 + d is exact, subtracting 1.5 2^23 leaves d as an
// FP32 with at most 9 significant bits, whose upper half is its bf16.
__device__ __forceinline__ __nv_bfloat16 fx_bf16(int d) {
  const float f = __int_as_float(0x4B400000 + d) - 12582912.0f;
  return __ushort_as_bfloat16((unsigned short)(__float_as_uint(f) >> 16));
}

__device__ __forceinline__ unsigned fx_biased_exp(double v) { return (unsigned)(__double2hiint(v) >> 20) & 0x7FFu; }
// smallest e with |x| < 2^e for the largest biased exponent m of a row (0: all zero)
__device__ __forceinline__ int fx_exp(unsigned m) { return m ? (int)m - 1022 : 0; }

__device__ __forceinline__ void fx_digits(double x, int e, int b, int L, int (&d)[FX_LMAX]) {
  fx_digits_t<0, 0>(x, e, b, L, d);
}

template <int BT, int LT>
__device__ __forceinline__ void fx_store_t(__nv_bfloat16* rowBase, size_t pitch, int k, bool valid, double v, int e,
                                           int bRt, int LRt) {
  const int L = LT > 0 ? LT : LRt;
  int d[FX_LMAX];
#pragma unroll
  for (int l = 0; l < FX_LMAX; l++) d[l] = 0;
  if (valid) fx_digits_t<BT, LT>(v, e, bRt, LRt, d);
#pragma unroll
  for (int l = 0; l < FX_LMAX; l++)
    if (l < L) rowBase[(size_t)l * pitch + k] = fx_bf16(d[l]);
}

__device__ __forceinline__ void fx_store(__nv_bfloat16* rowBase, size_t pitch, int k, bool valid, double v, int e,
                                         int b, int L) {
  fx_store_t<0, 0>(rowBase, pitch, k, valid, v, e, b, L);
}

__device__ unsigned fx_block_max(unsigned m) {
  __shared__ unsigned red[32];
  m = __reduce_max_sync(0xffffffffu, m);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) red[wid] = m;
  __syncthreads();
  const int nw = (blockDim.x + 31) >> 5;
  unsigned r = 0;
  for (int i = 0; i < nw; i++) r = max(r, red[i]);
  return r;
}

// One block per row: the row's values in dynamic shared memory, the exponent
// of its maximum, then the L digit planes: value k at column shift + k, zero
// elsewhere in [0, Kpad).
template <int BT = 0, int LT = 0, class F>
__device__ void fx_row(__nv_bfloat16* rowBase, int* expOut, int K, int Kpad, int pitch, int b, int L, int shift,
                       F value) {
  extern __shared__ double fxbuf[];
  unsigned m = 0;
  for (int k = threadIdx.x; k < K; k += blockDim.x) {
    const double v = value(k);
    fxbuf[k] = v;
    m = max(m, fx_biased_exp(v));
  }
  const int e = fx_exp(fx_block_max(m));
  if (threadIdx.x == 0) *expOut = e;
  for (int k = threadIdx.x; k < Kpad; k += blockDim.x) {
    const int src = k - shift;
    const bool valid = src >= 0 && src < K;
    fx_store_t<BT, LT>(rowBase, pitch, k, valid, valid ? fxbuf[src] : 0.0, e, b, L);
  }
}

__global__ void __launch_bounds__(256) k_fx_split_V(__nv_bfloat16* __restrict__ out, int* __restrict__ eV,
                                                     const double* __restrict__ V, int pitch, int b, int L,
                                                     TRAJ_ARGS) {
  const TrajShape& T = shp[blockIdx.z];
  const int g = blockIdx.x, nG = T.nG;
  if (g >= nG) return;
  out = bat(out, bs);
  eV = bat(eV, bs);
  V = bat(V, bs);
  const double* row = V + (size_t)g * nG;
  fx_row(out + (size_t)g * L * pitch, eV + g, nG, T.Kg, pitch, b, L, 0, [&](int k) { return row[k]; });
}

// Rows 2p (real part) and 2p + 1 (imaginary part) of S = conj(phi_l) phi_k w
// over the grid (p = (l, k)), one block per pair: the complex product and the
// weight in double-float arithmetic (FP32 pipe; ~2^-44 relative, far below the
// digits' 2^-36 of the row maximum), both rows staged in shared memory, each
// with the exponent of its own maximum.  Block 0 of a trajectory also clears
// the W exponent maxima for GEMM1.
template <int BT, int LT>
__global__ void __launch_bounds__(256) k_fx_split_S(__nv_bfloat16* __restrict__ out, int* __restrict__ eS,
                                                     unsigned* __restrict__ mWr, unsigned* __restrict__ mWc,
                                                     const z_t* __restrict__ orbs, const double* __restrict__ w,
                                                     const int* __restrict__ pl, const int* __restrict__ pk, int pitch,
                                                     int b, int L, TRAJ_ARGS) {
  const TrajShape& T = shp[blockIdx.z];
  const int p = blockIdx.x, nG = T.nG, nP = T.nPairs;
  if (p >= nP) return;
  out = bat(out, bs);
  eS = bat(eS, bs);
  orbs = bat(orbs, bs);
  w = bat(w, bs);
  pl = bat(pl, bs);
  pk = bat(pk, bs);
  if (p == 0) {
    mWr = bat(mWr, bs);
    mWc = bat(mWc, bs);
    for (int i = threadIdx.x; i < nG; i += blockDim.x) mWr[i] = 0u;
    for (int i = threadIdx.x; i < 2 * nP; i += blockDim.x) mWc[i] = 0u;
  }
  extern __shared__ double fxbuf[];  // [2][pitch]: the real and the imaginary row
  const z_t* a = orbs + (size_t)nG * pl[p];
  const z_t* bo = orbs + (size_t)nG * pk[p];
  unsigned mr = 0, mi = 0;
  for (int g = threadIdx.x; g < nG; g += blockDim.x) {
    const z_t av = a[g], bv = bo[g];
    const float2 ar = df_split(av.x), ai = df_split(av.y), br = df_split(bv.x), bi = df_split(bv.y);
    const float2 wg = df_split(w[g]);
    // conj(a) b = (ar br + ai bi) + i (ar bi - ai br)
    const float2 re = df_dot2(ar, br, ai, bi);
    const float2 im = df_dot2(ar, bi, make_float2(-ai.x, -ai.y), br);
    float s0 = 0.0f, c0 = 0.0f, s1 = 0.0f, c1 = 0.0f;
    df_mul_acc(s0, c0, re.x, re.y, wg.x, wg.y);
    df_mul_acc(s1, c1, im.x, im.y, wg.x, wg.y);
    const double vr = df_to_d(make_float2(s0, c0)), vi = df_to_d(make_float2(s1, c1));
    fxbuf[g] = vr;
    fxbuf[pitch + g] = vi;
    mr = max(mr, fx_biased_exp(vr));
    mi = max(mi, fx_biased_exp(vi));
  }
  const int er = fx_exp(fx_block_max(mr));
  const int ei = fx_exp(fx_block_max(mi));
  if (threadIdx.x == 0) {
    eS[2 * p] = er;
    eS[2 * p + 1] = ei;
  }
  __nv_bfloat16* rowR = out + (size_t)(2 * p) * L * pitch;
  __nv_bfloat16* rowI = out + (size_t)(2 * p + 1) * L * pitch;
  const int Kpad = T.Kg, shift = T.gShift;
  for (int k = threadIdx.x; k < Kpad; k += blockDim.x) {
    const int src = k - shift;
    const bool valid = src >= 0 && src < nG;
    fx_store_t<BT, LT>(rowR, pitch, k, valid, valid ? fxbuf[src] : 0.0, er, b, L);
    fx_store_t<BT, LT>(rowI, pitch, k, valid, valid ? fxbuf[pitch + src] : 0.0, ei, b, L);
  }
}

// Row n = 2q + s of R'' (K = 2p + t), as k_split_R.
template <int BT, int LT>
__global__ void k_fx_split_R(__nv_bfloat16* __restrict__ out, int* __restrict__ eR, const z_t* __restrict__ Rp,
                             const int* __restrict__ pl, const int* __restrict__ pk, int pitch, int b, int L,
                             TRAJ_ARGS) {
  const TrajShape& T = shp[blockIdx.z];
  const int n = T.nOS, nP = T.nPairs, Q = n * n;
  const int row = blockIdx.x;
  if (row >= 2 * Q) return;
  out = bat(out, bs);
  eR = bat(eR, bs);
  Rp = bat(Rp, bs);
  pl = bat(pl, bs);
  pk = bat(pk, bs);
  const int q = row >> 1, s = row & 1;
  fx_row<BT, LT>(out + (size_t)row * L * pitch, eR + row, 2 * nP, T.Kp, pitch, b, L, 0, [&](int k) {
    const int p = k >> 1, t = k & 1;
    const int l = pl[p], kk = pk[p];
    const z_t R1 = Rp[(size_t)(l * n + kk) * Q + q];
    const z_t R2 = (l < kk) ? Rp[(size_t)(kk * n + l) * Q + q] : zmk(0.0, 0.0);
    const double r1 = s ? (t ? R1.x : R1.y) : (t ? -R1.y : R1.x);
    const double r2 = s ? (t ? R2.x : R2.y) : (t ? -R2.y : R2.x);
    return t ? r1 - r2 : r1 + r2;
  });
}

// W = sum of the K-split partials (into slot 0) and the exponent maxima of its
// rows and columns (used when GEMM1 ran with split K).
__global__ void k_fx_reduce_W(double* __restrict__ Wd, unsigned* __restrict__ mWr, unsigned* __restrict__ mWc,
                              int nSplit, TRAJ_ARGS) {
  const TrajShape& T = shp[blockIdx.z];
  const int nG = T.nG, N = 2 * T.nPairs;
  Wd = bat(Wd, bs);
  mWr = bat(mWr, bs);
  mWc = bat(mWc, bs);
  const size_t tot = (size_t)nG * N;
  GRID_STRIDE(e, tot) {
    double v = 0.0;
    for (int z = 0; z < nSplit; z++) v += Wd[(size_t)z * tot + e];
    Wd[e] = v;
    const unsigned ex = fx_biased_exp(v);
    if (ex) {
      atomicMax(mWr + e / N, ex);
      atomicMax(mWc + e % N, ex);
    }
  }
}

// W (FP64 [nG][2P]) to WxA (rows g, K = 2P: b2/L2 digits) and WTxB (rows n,
// K = nG at columns gShift + g: b1/L3 digits) planes, with the row exponents
// eWr[g] / eWc[n].  One block per 32-row strip of W, walking the trajectory's
// own K = 2P columns in 32 x 32 tiles transposed through shared memory.
// B1/L3T, B2/L2T > 0: the digit plans fixed at compile time (0: run-time b1, L3, b2, L2).
template <int B1, int L3T, int B2, int L2T>
__global__ void __launch_bounds__(256) k_fx_split_W(__nv_bfloat16* __restrict__ WxA, __nv_bfloat16* __restrict__ WTxB,
                                                     int* __restrict__ eWr, int* __restrict__ eWc,
                                                     const double* __restrict__ Wd, const unsigned* __restrict__ mWr,
                                                     const unsigned* __restrict__ mWc, int pitchP, int pitchG, int b1,
                                                     int L3rt, int b2, int L2rt, TRAJ_ARGS) {
  const int L3 = L3T > 0 ? L3T : L3rt, L2 = L2T > 0 ? L2T : L2rt;
  __shared__ double tile[SW_T][SW_T + 1];
  const TrajShape& T = shp[blockIdx.z];
  const int nG = T.nG, N2P = 2 * T.nPairs, KpP = T.Kp, KpG = T.Kg;
  const int g0 = blockIdx.x * SW_T;
  if (g0 >= KpG) return;
  WxA = bat(WxA, bs);
  WTxB = bat(WTxB, bs);
  eWr = bat(eWr, bs);
  eWc = bat(eWc, bs);
  Wd = bat(Wd, bs);
  mWr = bat(mWr, bs);
  mWc = bat(mWc, bs);
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;  // 32 x 8
  const int sh = T.gShift;
  for (int n0 = 0; n0 < KpP; n0 += SW_T) {
    if (n0 > 0) __syncthreads();  // the previous tile has been read
    for (int r = ty; r < SW_T; r += 8) {
      const int g = g0 + r, n = n0 + tx;
      const bool valid = g < nG && n < N2P;
      const double v = valid ? Wd[(size_t)g * N2P + n] : 0.0;
      tile[r][tx] = v;
      if (g < nG) {
        const int e = fx_exp(mWr[g]);
        if (n == 0) eWr[g] = e;
        fx_store_t<B2, L2T>(WxA + (size_t)g * L2 * pitchP, pitchP, n, valid, v, e, b2, L2);
      }
    }
    __syncthreads();
    for (int r = ty; r < SW_T; r += 8) {
      const int n = n0 + r, g = g0 + tx, col = g + sh;
      if (n < N2P && col < KpG) {
        const int e = fx_exp(mWc[n]);
        if (g == 0) eWc[n] = e;
        fx_store_t<B1, L3T>(WTxB + (size_t)n * L3 * pitchG, pitchG, col, g < nG, tile[tx][r], e, b1, L3);
      }
      if (n < N2P && g0 == 0)  // columns before the shifted grid
        for (int cz = tx; cz < sh; cz += 32)
          fx_store_t<B1, L3T>(WTxB + (size_t)n * L3 * pitchG, pitchG, cz, false, 0.0, 0, b1, L3);
    }
  }
}

size_t take(size_t& off, size_t bytes) {
  size_t o = (off + 255) & ~(size_t)255;
  off = o + std::max<size_t>(bytes, 1);
  return o;
}

}  // namespace

// Sizes (base == nullptr) or places (base = the arena) the mixed-form buffers of
// one trajectory block starting at byte offset `off`; returns the end offset.
size_t mixed_layout(cgpu_ctx* c, char* base, size_t off) {
  if (c->precision == CGPU_PREC_FP64 || !c->hasInteraction) return off;
  if (!c->mixed) c->mixed = new MixedBufs();
  MixedBufs* m = c->mixed;
  m->fxBits = c->precision == CGPU_PREC_MIXED_FX ? 30 : c->precision == CGPU_PREC_MIXED_FX6 ? 36 : 0;
  m->fxBits3 = m->fxBits;
  m->terms = c->precision == CGPU_PREC_MIXED_X6 ? 6 : 3;
  int nG = c->nG, nP = c->nPairs, Q = c->nOS * c->nOS, T = m->terms;
  m->KgMax = (nG + 63) / 64 * 64;
  m->KpMax = (2 * nP + 63) / 64 * 64;
  typedef __nv_bfloat16 bf;
  if (m->fxBits) {
    m->KgMax = c->fxKgMax;  // includes the K-tile offsets of a shared interaction matrix
    // digit widths from the longest contraction of the batch (K = nG, K = 2P)
    fx_plan(m->KgMax / 64, m->fxBits, &m->b1, &m->L1);
    int b3 = 0;
    fx_plan(m->KgMax / 64, m->fxBits3, &b3, &m->L3);
    if (b3 != m->b1) throw std::string("mixed_fx: GEMM1 and GEMM3 share the S digits");
    m->LS = std::max(m->L1, m->L3);
    fx_plan(m->KpMax / 64, m->fxBits, &m->b2, &m->L2);
    const int L1 = m->L1, L2 = m->L2;
    m->compact2 = c->nb > 1 && fx_compact_ok(L2);
    m->bn1 = fx_tile_n(2 * nP, L1, false);
    m->bn2 = fx_tile_n(2 * Q, L2, m->compact2);
    m->bn3 = fx_tile_n(2 * nP, m->L3, false);
    m->s1 = fx_split_count(nG, 2 * nP, m->bn1, m->KgMax / 64, c->nb, m->b1);
    m->s2 = fx_split_count(nG, 2 * Q, m->bn2, m->KpMax / 64, c->nb, m->b2);
    m->s3 = fx_split_count(2 * nP, 2 * nP, m->bn3, m->KgMax / 64, c->nb, m->b1);
    // partial buffers: a single system holds twice the heuristic's K splits
    // (room for the tile tuner), a batch exactly the heuristic's
    const int grow = c->nb == 1 ? 2 : 1;
    m->sCap1 = std::min(m->s1 * grow, m->KgMax / 64);
    m->sCap2 = std::min(m->s2 * grow, m->KpMax / 64);
    m->sCap3 = std::min(m->s3 * grow, m->KgMax / 64);
    const size_t perTrajV = c->fxShared ? 0 : 1;
    size_t oV = take(off, perTrajV * sizeof(bf) * (size_t)nG * L1 * m->KgMax);
    size_t oS = take(off, sizeof(bf) * (size_t)2 * nP * m->LS * m->KgMax);
    size_t oW = take(off, sizeof(bf) * (size_t)nG * L2 * m->KpMax);
    size_t oWT = take(off, sizeof(bf) * (size_t)2 * nP * m->L3 * m->KgMax);
    size_t oR = take(off, sizeof(bf) * (size_t)2 * Q * L2 * m->KpMax);
    size_t oWd = take(off, sizeof(double) * (size_t)m->sCap1 * nG * 2 * nP);
    size_t oZp = take(off, m->sCap2 > 1 ? sizeof(double) * (size_t)m->sCap2 * nG * 2 * Q : 0);
    size_t oGd = take(off, sizeof(double) * (size_t)m->sCap3 * 2 * nP * 2 * nP);
    size_t oE = take(off, sizeof(int));
    size_t oZ = take(off, sizeof(double) * (size_t)2 * nG * Q);
    size_t oeV = take(off, perTrajV * sizeof(int) * (size_t)nG);
    size_t oeS = take(off, sizeof(int) * (size_t)2 * nP);
    size_t oeWr = take(off, sizeof(int) * (size_t)nG);
    size_t oeWc = take(off, sizeof(int) * (size_t)2 * nP);
    size_t oeR = take(off, sizeof(int) * (size_t)2 * Q);
    size_t omWr = take(off, sizeof(unsigned) * (size_t)nG);
    size_t omWc = take(off, sizeof(unsigned) * (size_t)2 * nP);
    if (base) {
      m->VxB = perTrajV ? (bf*)(base + oV) : nullptr;
      m->SxA = (bf*)(base + oS);
      m->WxA = (bf*)(base + oW);
      m->WTxB = (bf*)(base + oWT);
      m->RxB = (bf*)(base + oR);
      m->Wd = (double*)(base + oWd);
      m->Zp = m->sCap2 > 1 ? (double*)(base + oZp) : nullptr;
      m->Gd = (double*)(base + oGd);
      m->err = (int*)(base + oE);
      m->Zd = (double*)(base + oZ);
      m->eV = perTrajV ? (int*)(base + oeV) : nullptr;
      m->eS = (int*)(base + oeS);
      m->eWr = (int*)(base + oeWr);
      m->eWc = (int*)(base + oeWc);
      m->eR = (int*)(base + oeR);
      m->mWr = (unsigned*)(base + omWr);
      m->mWc = (unsigned*)(base + omWc);
    }
    return off;
  }
  // W = V S: in a batch one N tile of 256 covers all pairs (2P <= 156 for 12
  // orbitals), so the large V operand streams once per trajectory
  m->bn1 = (c->nb > 1 && 2 * nP <= 256) ? 256 : tc_tile_n(2 * nP);
  m->bn2 = tc_tile_n(2 * Q);
  m->bn3 = tc_tile_n(2 * nP);
  m->s1 = tc_split_count(nG, 2 * nP, m->bn1, T * m->KgMax / 64, c->nb);
  m->s2 = tc_split_count(nG, 2 * Q, m->bn2, T * m->KpMax / 64, c->nb);
  m->s3 = tc_split_count(2 * nP, 2 * nP, m->bn3, T * m->KgMax / 64, c->nb);
  size_t oV = take(off, sizeof(bf) * (size_t)nG * T * m->KgMax);
  size_t oS = take(off, sizeof(bf) * (size_t)2 * nP * T * m->KgMax);
  size_t oW = take(off, sizeof(bf) * (size_t)nG * T * m->KpMax);
  size_t oWT = take(off, sizeof(bf) * (size_t)2 * nP * T * m->KgMax);
  size_t oR = take(off, sizeof(bf) * (size_t)2 * Q * T * m->KpMax);
  size_t o1 = take(off, sizeof(float) * (size_t)m->s1 * nG * 2 * nP);
  size_t o2 = take(off, sizeof(float) * (size_t)m->s2 * nG * 2 * Q);
  size_t o3 = take(off, sizeof(float) * (size_t)m->s3 * 2 * nP * 2 * nP);
  size_t oE = take(off, sizeof(int));
  size_t oZ = take(off, sizeof(double) * (size_t)2 * nG * Q);
  if (base) {
    m->VxB = (bf*)(base + oV);
    m->SxA = (bf*)(base + oS);
    m->WxA = (bf*)(base + oW);
    m->WTxB = (bf*)(base + oWT);
    m->RxB = (bf*)(base + oR);
    m->P1 = (float*)(base + o1);
    m->P2 = (float*)(base + o2);
    m->P3 = (float*)(base + o3);
    m->err = (int*)(base + oE);
    m->Zd = (double*)(base + oZ);
  }
  return off;
}

void mixed_free(cgpu_ctx* c) {
  if (c->mixed) {
    if (c->mixed->Vsh) cudaFree(c->mixed->Vsh);
    if (c->mixed->eVsh) cudaFree(c->mixed->eVsh);
    for (void* p : {c->mixed->tiles1, c->mixed->tiles2, c->mixed->tiles3})
      if (p) cudaFree(p);
  }
  delete c->mixed;  // the other buffers belong to the arena
  c->mixed = nullptr;
}

// After the arena holds V: bf16 splits of V (static) and the TMA maps.
void mixed_init(cgpu_ctx* c) {
  MixedBufs* m = c->mixed;
  if (!m) return;
  int T = m->terms, pG = T * m->KgMax, pP = T * m->KpMax, pS = pG, pWT = pG;
  if (m->fxBits) {
    pG = m->L1 * m->KgMax;   // V: K = nG slices
    pS = m->LS * m->KgMax;   // S (GEMM1 reads the first L1 slices, GEMM3 L3)
    pWT = m->L3 * m->KgMax;  // W columns for GEMM3
    pP = m->L2 * m->KpMax;   // W, R: K = 2P slices
  }
  size_t nGK = (size_t)c->nG * m->KgMax;
  if (m->fxBits && c->fxShared) {
    // each root trajectory's interaction matrix, sliced once for the batch
    const int nR = (int)c->fxRoots.size();
    m->KgBig = (c->nG + 63) / 64 * 64;
    const size_t plane = (size_t)c->nG * m->L1 * m->KgBig;  // elements per root
    CODY_CUDA(cudaMalloc(&m->Vsh, sizeof(__nv_bfloat16) * plane * nR));
    CODY_CUDA(cudaMalloc(&m->eVsh, sizeof(int) * (size_t)c->nG * nR));
    CODY_CUDA(cudaMemsetAsync(m->Vsh, 0, sizeof(__nv_bfloat16) * plane * nR, c->stream));
    for (int r = 0; r < nR; r++) {
      const int root = c->fxRoots[r], nGb = c->sys[root].nG;
      const double* Vb = (const double*)((const char*)c->Vint_d + (size_t)root * c->bs);
      k_fx_split_V<<<dim3(nGb, 1, 1), 256, sizeof(double) * m->KgBig, c->stream>>>(
          m->Vsh + plane * r, m->eVsh + (size_t)c->nG * r, Vb, m->KgBig, m->b1, m->L1, c->shape_d + root, 0);
      CODY_LAUNCHED(c);
    }
    m->mVsh = tc_make_map_planes(m->Vsh, c->nG, m->L1 * m->KgBig, 128, nR, sizeof(__nv_bfloat16) * plane);
  } else if (m->fxBits)
    k_fx_split_V<<<dim3(c->nG, 1, c->nb), 256, sizeof(double) * m->KgMax, c->stream>>>(m->VxB, m->eV, c->Vint_d,
                                                                                     m->KgMax, m->b1, m->L1,
                                                                                     TRAJ_PASS(c));
  else
    k_split_V<<<bgrid(c, ew_blocks(c, nGK)), 256, 0, c->stream>>>(m->VxB, c->Vint_d, m->KgMax, T, TRAJ_PASS(c));
  CODY_LAUNCHED(c);
  int P2 = 2 * c->nPairs, Q2 = 2 * c->nOS * c->nOS;
  if (m->VxB) m->mV = tc_make_map(c, m->VxB, c->nG, pG, 128);
  // the fixed-point GEMM loads its B operands in 16-row boxes
  m->mS = tc_make_map(c, m->SxA, P2, pS, m->fxBits ? 16 : m->bn1);
  m->mW = tc_make_map(c, m->WxA, c->nG, pP, 128);
  m->mR = tc_make_map(c, m->RxB, Q2, pP, m->fxBits ? 16 : m->bn2);
  m->mSasB = tc_make_map(c, m->SxA, P2, pS, 128);
  if (m->fxBits) {
    m->tiles1 = fx_build_tiles(c, TC_GEMM_W, m->bn1, m->s1, &m->nTiles1);
    m->tiles2 = fx_build_tiles(c, TC_GEMM_Z, m->bn2, m->s2, &m->nTiles2);
    m->tiles3 = fx_build_tiles(c, TC_GEMM_H2, m->bn3, m->s3, &m->nTiles3);
  }
  m->mWT = tc_make_map(c, m->WTxB, P2, pWT, m->fxBits ? 16 : m->bn3);
  CODY_CUDA(cudaStreamSynchronize(c->stream));
}

int mixed_error(cgpu_ctx* c) {
  if (!c->mixed) return 0;
  int e = 0;
  CODY_CUDA(cudaMemcpy(&e, c->mixed->err, sizeof(int), cudaMemcpyDeviceToHost));
  return e;
}

// The three fixed-point contractions with their K-split reductions, on the
// operands the digit splits left in the arena (one call = one launch of the
// GEMM, plus the reduction when K is split).
// W = V S (pair potentials; row / column exponent maxima for the W split).
static void fx_run_W(cgpu_ctx* c) {
  MixedBufs* m = c->mixed;
  const int nG = c->nG, nP = c->nPairs;
  const bool one = m->s1 == 1;
  if (c->fxShared)
    fx_gemm(c, m->L1, m->b1, m->compact1, TC_GEMM_W, m->mVsh, m->mS, m->bn1, m->Wd, m->eVsh, m->eS,
            one ? m->mWr : nullptr, one ? m->mWc : nullptr, m->KgBig, m->KgMax, 1, m->s1, m->tiles1, m->nTiles1,
            m->err);
  else
    fx_gemm(c, m->L1, m->b1, m->compact1, TC_GEMM_W, m->mV, m->mS, m->bn1, m->Wd, m->eV, m->eS,
            one ? m->mWr : nullptr, one ? m->mWc : nullptr, m->KgMax, m->KgMax, 0, m->s1, m->tiles1, m->nTiles1,
            m->err);
  if (!one) {
    k_fx_reduce_W<<<bgrid(c, ew_blocks(c, (size_t)nG * 2 * nP)), 256, 0, c->stream>>>(m->Wd, m->mWr, m->mWc, m->s1,
                                                                                   TRAJ_PASS(c));
    CODY_LAUNCHED(c);
  }
}

// Z = W R'' (the correlation contraction) into Zd.
static void fx_run_Z(cgpu_ctx* c) {
  MixedBufs* m = c->mixed;
  const int nG = c->nG, Q = c->nOS * c->nOS;
  fx_gemm(c, m->L2, m->b2, m->compact2, TC_GEMM_Z, m->mW, m->mR, m->bn2, m->s2 > 1 ? m->Zp : m->Zd, m->eWr, m->eR,
          nullptr, nullptr, m->KpMax, m->KpMax, 0, m->s2, m->tiles2, m->nTiles2, m->err);
  if (m->s2 > 1) {
    k_reduce_Z<<<bgrid(c, ew_blocks(c, (size_t)nG * Q)), 256, 0, c->stream>>>((z_t*)m->Zd, m->Zp, m->s2,
                                                                        TRAJ_PASS(c));
    CODY_LAUNCHED(c);
  }
}

// G = S^T W (h2) and its reduction into the spatial h2 block.
static void fx_run_H2(cgpu_ctx* c) {
  MixedBufs* m = c->mixed;
  const int Q = c->nOS * c->nOS;
  fx_gemm(c, m->L3, m->b1, m->compact3, TC_GEMM_H2, m->mSasB, m->mWT, m->bn3, m->Gd, m->eS, m->eWc, nullptr, nullptr,
          m->KgMax, m->KgMax, 0, m->s3, m->tiles3, m->nTiles3, m->err);
  k_reduce_H2<<<bgrid(c, ew_blocks(c, (size_t)Q * Q)), 256, 0, c->stream>>>(c->h2s_d, m->Gd, m->s3, c->pidx_d,
                                                                      TRAJ_PASS(c));
  CODY_LAUNCHED(c);
}

// ---- tile tuner hooks ---------------------------------------------------------

bool fx_tiles_get(const cgpu_ctx* c, int* t) {
  const MixedBufs* m = c->mixed;
  if (!m || !m->fxBits) return false;
  const int v[9] = {m->bn1, m->compact1, m->s1, m->bn2, m->compact2, m->s2, m->bn3, m->compact3, m->s3};
  for (int i = 0; i < 9; i++) t[i] = v[i];
  return true;
}

// Slices, digit width, K blocks, split capacity and output columns of GEMM g.
static void fx_gemm_plan(const cgpu_ctx* c, int g, int& L, int& b, int& kTiles, int& cap, int& N) {
  const MixedBufs* m = c->mixed;
  if (g == TC_GEMM_W) { L = m->L1; b = m->b1; kTiles = m->KgMax / 64; cap = m->sCap1; N = 2 * c->nPairs; }
  else if (g == TC_GEMM_Z) { L = m->L2; b = m->b2; kTiles = m->KpMax / 64; cap = m->sCap2; N = 2 * c->nOS * c->nOS; }
  else { L = m->L3; b = m->b1; kTiles = m->KgMax / 64; cap = m->sCap3; N = 2 * c->nPairs; }
}

void fx_tiles_set(cgpu_ctx* c, const int* t) {
  MixedBufs* m = c->mixed;
  if (!m || !m->fxBits) throw std::string("tiles: not a fixed-point context");
  int bn[3], sp[3];
  bool cm[3];
  for (int g = 0; g < 3; g++) {
    int L, b, kTiles, cap, N;
    fx_gemm_plan(c, g, L, b, kTiles, cap, N);
    bn[g] = t[3 * g];
    cm[g] = t[3 * g + 1] != 0;
    if (!fx_tile_supported(bn[g], L, cm[g])) throw std::string("tiles: no fixed-point GEMM configuration for that tile");
    if (t[3 * g + 2] < 1 || t[3 * g + 2] > kTiles) throw std::string("tiles: K split count outside 1..K blocks");
    sp[g] = fx_normalize_splits(kTiles, t[3 * g + 2]);
    // every split keeps at least two K blocks, as the set-up heuristic does
    if (sp[g] < fx_min_splits(kTiles, b) || sp[g] > cap || (sp[g] > 1 && sp[g] > kTiles / 2))
      throw std::string("tiles: K split outside the exact range of the digits or the partial buffers");
  }
  void** lists[3] = {&m->tiles1, &m->tiles2, &m->tiles3};
  int* counts[3] = {&m->nTiles1, &m->nTiles2, &m->nTiles3};
  CODY_CUDA(cudaStreamSynchronize(c->stream));
  for (int g = 0; g < 3; g++) {
    if (*lists[g]) CODY_CUDA(cudaFree(*lists[g]));
    *lists[g] = fx_build_tiles(c, g, bn[g], sp[g], counts[g]);
  }
  m->bn1 = bn[0]; m->compact1 = cm[0]; m->s1 = sp[0];
  m->bn2 = bn[1]; m->compact2 = cm[1]; m->s2 = sp[1];
  m->bn3 = bn[2]; m->compact3 = cm[2]; m->s3 = sp[2];
}

void fx_tile_candidates(const cgpu_ctx* c, int g, std::vector<std::array<int, 3>>& out) {
  out.clear();
  if (!c->mixed || !c->mixed->fxBits) return;
  int L, b, kTiles, cap, N;
  fx_gemm_plan(c, g, L, b, kTiles, cap, N);
  std::vector<std::pair<int, bool>> cfgs;
  fx_tile_configs(L, cfgs);
  std::vector<int> splits;
  for (int s : {1, 2, 3, 4, cap}) {
    int v = fx_normalize_splits(kTiles, s);
    if (v >= fx_min_splits(kTiles, b) && v <= cap && (v == 1 || v <= kTiles / 2) &&
        std::find(splits.begin(), splits.end(), v) == splits.end())
      splits.push_back(v);
  }
  for (const auto& cf : cfgs) {
    if (cf.first >= 2 * ((N + 15) / 16 * 16)) continue;  // wider than twice the output: idle MMA columns only
    for (int v : splits) out.push_back({cf.first, cf.second ? 1 : 0, v});
  }
}

double fx_time_contraction(cgpu_ctx* c, int g, int reps) {
  auto run = [&]() {
    if (g == TC_GEMM_W) fx_run_W(c);
    else if (g == TC_GEMM_Z) fx_run_Z(c);
    else fx_run_H2(c);
  };
  run();
  cudaEvent_t e0, e1;
  CODY_CUDA(cudaEventCreate(&e0));
  CODY_CUDA(cudaEventCreate(&e1));
  CODY_CUDA(cudaEventRecord(e0, c->stream));
  for (int r = 0; r < reps; r++) run();
  CODY_CUDA(cudaEventRecord(e1, c->stream));
  CODY_CUDA(cudaEventSynchronize(e1));
  float ms = 0.f;
  CODY_CUDA(cudaEventElapsedTime(&ms, e0, e1));
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (mixed_error(c)) throw std::string("tiles: a fixed-point GEMM reported a wait timeout while timing");
  return ms / reps;
}

// The fixed-point form of the three contractions.
void correlation_fx(cgpu_ctx* c, z_t* dOrbs, const z_t* orbs, int wantH2) {
  MixedBufs* m = c->mixed;
  const int nG = c->nG, nP = c->nPairs, n = c->nOS, Q = n * n;
  z_t* Z = (z_t*)m->Zd;
  {
    ProfScope prof(c, CGPU_KERNEL_PAIR_POTENTIALS);
    auto split_s = k_fx_split_S<0, 0>;
    if (m->b1 == 6 && m->LS == 6) split_s = k_fx_split_S<6, 6>;
    else if (m->b1 == 6 && m->LS == 5) split_s = k_fx_split_S<6, 5>;
    const size_t shS = 2 * sizeof(double) * m->KgMax;
    if (shS > 48 * 1024)
      CODY_CUDA(cudaFuncSetAttribute(split_s, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shS));
    split_s<<<dim3(nP, 1, c->nb), 256, shS, c->stream>>>(
        m->SxA, m->eS, m->mWr, m->mWc, orbs, c->w_d, c->pairL_d, c->pairK_d, m->KgMax, m->b1, m->LS, TRAJ_PASS(c));
    CODY_LAUNCHED(c);
    fx_run_W(c);
    dim3 gw(ceil_div(m->KgMax, SW_T), 1, c->nb);
    // the digit plans of the two fixed-point forms on long grids, compiled in
    auto split_w = k_fx_split_W<0, 0, 0, 0>;
    if (m->b1 == 6 && m->L3 == 6 && m->b2 == 8 && m->L2 == 5) split_w = k_fx_split_W<6, 6, 8, 5>;
    else if (m->b1 == 6 && m->L3 == 5 && m->b2 == 8 && m->L2 == 4) split_w = k_fx_split_W<6, 5, 8, 4>;
    split_w<<<gw, 256, 0, c->stream>>>(m->WxA, m->WTxB, m->eWr, m->eWc, m->Wd, m->mWr, m->mWc, m->KpMax, m->KgMax,
                                       m->b1, m->L3, m->b2, m->L2, TRAJ_PASS(c));
    CODY_LAUNCHED(c);
  }
  {
    ProfScope prof(c, CGPU_KERNEL_CORRELATION);
    auto split_r = k_fx_split_R<0, 0>;
    if (m->b2 == 8 && m->L2 == 5) split_r = k_fx_split_R<8, 5>;
    else if (m->b2 == 8 && m->L2 == 4) split_r = k_fx_split_R<8, 4>;
    split_r<<<dim3(2 * Q, 1, c->nb), 64, sizeof(double) * m->KpMax, c->stream>>>(
        m->RxB, m->eR, c->Rp_d, c->pairL_d, c->pairK_d, m->KpMax, m->b2, m->L2, TRAJ_PASS(c));
    CODY_LAUNCHED(c);
    fx_run_Z(c);
    launch_corr_epilogue(c, dOrbs, orbs, Z);
  }
  if (wantH2) {
    ProfScope prof(c, CGPU_KERNEL_H2);
    fx_run_H2(c);
    launch_h2_layout(c);
  }
}

// ApplyCorrelationOp in the mixed form: dOrbs += rho^-1 rho2 W phi; h2 (FP64 nO^4) when wantH2.
void launch_correlation_mixed(cgpu_ctx* c, z_t* dOrbs, const z_t* orbs, int wantH2) {
  launch_rdm_inverse(c);
  if (!c->hasInteraction) {
    if (wantH2) {
      batch_zero(c, c->h2_d, sizeof(z_t) * (size_t)c->nO * c->nO * c->nO * c->nO);
      batch_zero(c, c->h2s_d, sizeof(z_t) * (size_t)c->nOS * c->nOS * c->nOS * c->nOS);
    }
    return;
  }
  MixedBufs* m = c->mixed;
  int nG = c->nG, nP = c->nPairs, n = c->nOS, Q = n * n, T = m->terms;
  if (m->fxBits) return correlation_fx(c, dOrbs, orbs, wantH2);
  {
    ProfScope prof(c, CGPU_KERNEL_PAIR_POTENTIALS);
    k_split_S<<<bgrid(c, ew_blocks(c, (size_t)2 * nP * m->KgMax)), 256, 0, c->stream>>>(
        m->SxA, orbs, c->w_d, c->pairL_d, c->pairK_d, m->KgMax, T, TRAJ_PASS(c));
    CODY_LAUNCHED(c);
    // V carries the B split pattern, S the A pattern: hi*hi + lo*hi + hi*lo (x3)
    tc_gemm(c, TC_GEMM_W, m->mV, m->mS, m->bn1, m->P1, T, m->KgMax, m->s1, nG, 2 * nP, m->err);
    dim3 gw(ceil_div(m->KgMax, SW_T), ceil_div(m->KpMax, SW_T), c->nb);
    k_split_W<<<gw, 256, 0, c->stream>>>(m->WxA, m->WTxB, m->P1, m->s1, m->KpMax, m->KgMax, T, TRAJ_PASS(c));
    CODY_LAUNCHED(c);
  }
  {
    ProfScope prof(c, CGPU_KERNEL_CORRELATION);
    k_split_R<<<bgrid(c, ew_blocks(c, (size_t)2 * Q * m->KpMax)), 256, 0, c->stream>>>(m->RxB, c->Rp_d, c->pairL_d,
                                                                                   c->pairK_d, m->KpMax, T,
                                                                                   TRAJ_PASS(c));
    CODY_LAUNCHED(c);
    tc_gemm(c, TC_GEMM_Z, m->mW, m->mR, m->bn2, m->P2, T, m->KpMax, m->s2, nG, 2 * Q, m->err);
    z_t* Z = (z_t*)m->Zd;
    k_reduce_Z<<<bgrid(c, ew_blocks(c, (size_t)nG * Q)), 256, 0, c->stream>>>(Z, m->P2, m->s2, TRAJ_PASS(c));
    CODY_LAUNCHED(c);
    launch_corr_epilogue(c, dOrbs, orbs, Z);
  }
  if (wantH2) {
    ProfScope prof(c, CGPU_KERNEL_H2);
    tc_gemm(c, TC_GEMM_H2, m->mSasB, m->mWT, m->bn3, m->P3, T, m->KgMax, m->s3, 2 * nP, 2 * nP, m->err);
    k_reduce_H2<<<bgrid(c, ew_blocks(c, (size_t)Q * Q)), 256, 0, c->stream>>>(c->h2s_d, m->P3, m->s3, c->pidx_d,
                                                                        TRAJ_PASS(c));
    CODY_LAUNCHED(c);
    launch_h2_layout(c);
  }
}
