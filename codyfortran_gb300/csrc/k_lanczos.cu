// k_lanczos.cu -- short-iterative-Lanczos kernels
// (PerformLanczosStep / EvaluateExpInSubspace / MetricDot,
//  src/IntegratorList/Sil/S_IntegratorList_Sil.f90:184-310).
//
// Per Krylov iteration j the reference does
//   w = H v_j - beta_{j-1} v_{j-1};  alpha_j = Re<v_j,w>;  w -= alpha_j v_j;
//   for k = 1..j: w -= <v_k,w> v_k   (modified Gram-Schmidt);  beta_j = ||w||.
// With the basis orthonormal, the projections it removes are those of H v_j on
// v_1..v_j; the kernels remove them in a classical Gram-Schmidt pass (one
// fused reduction) and a second pass when the first one cancelled most of w,
// which reproduces the reference's vectors and coefficients to rounding.
// With a window k > 1 the passes run against v_{j-k+1}..v_j only (orthogonal
// to the rest in exact arithmetic).  k = 1 is the three-term recurrence
// proper: w = H v_j - beta_{j-1} v_{j-1}, alpha_j = Re<v_j, w>_m,
// w -= alpha_j v_j, with beta_{j-1} known from the previous iteration (no dot
// with v_{j-1}; about 30% fewer FP64 operations per entry than k = 2).  Its
// basis vectors stay unnormalised (v_k = s_k u_k): the operator is linear, so
// the recurrence applies the scales inside its two passes and the separate
// v_{j+1} = w / beta_j pass disappears.  Every reduction is deterministic:
// per-block partials in a fixed order, re-summed identically by every
// consumer block.
//
// Device scalar block lz[] (doubles):
#include <algorithm>

#include "common.cuh"

namespace {

constexpr int LZ_ALPHA = 0;     // alpha_j          [0, 64)
constexpr int LZ_BETA = 64;     // beta_j           [64, 128)
constexpr int LZ_D = 128;       // dots (complex)   [128, 256)
constexpr int LZ_PHI = 256;     // phi (complex)    [256, 384)
constexpr int LZ_NRM = 384;     // state norm
constexpr int LZ_ERR = 385;     // error estimate
constexpr int LZ_MDIM = 386;    // subspace dimension used
constexpr int LZ_DONE = 387;    // breakdown flag (1 = stop growing)
constexpr int LZ_ZERO = 388;    // zero-norm start (output = input)
constexpr int LZ_DT = 389;      // dt of the current sub-step
constexpr int LZ_BREAKJ = 390;  // iteration at which breakdown happened
constexpr int LZ_S = 400;       // scale of basis slot k: v_(k+1) = s_k u_k  [400, 433)
constexpr int LZ_SMAX = 33;
static_assert(LZ_S == CODY_LZ_S && LZ_BETA == CODY_LZ_BETA && LZ_DONE == CODY_LZ_DONE, "Lanczos scalar slots");

constexpr int LZ_THREADS = 256;

__device__ z_t block_sum2(z_t v) {
  __shared__ z_t red[32];
  for (int o = 16; o > 0; o >>= 1) {
    v.x += __shfl_down_sync(0xffffffffu, v.x, o);
    v.y += __shfl_down_sync(0xffffffffu, v.y, o);
  }
  int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) red[wid] = v;
  __syncthreads();
  int nw = (blockDim.x + 31) >> 5;
  v = (threadIdx.x < nw) ? red[threadIdx.x] : zmk(0.0, 0.0);
  if (wid == 0)
    for (int o = 16; o > 0; o >>= 1) {
      v.x += __shfl_down_sync(0xffffffffu, v.x, o);
      v.y += __shfl_down_sync(0xffffffffu, v.y, o);
    }
  return v;
}

constexpr int LZ_WARPS = LZ_THREADS / 32;
constexpr int LZ_EMAX = 4;                         // state entries per thread and chunk (at most)
constexpr int LZ_VPW = 32 / LZ_WARPS;              // Krylov vectors per warp (at most 32 vectors)

// Chunked reductions against the Krylov basis.  A block walks chunks of
// LZ_THREADS * E consecutive state entries; the chunk of m * w is staged in
// shared memory, and warp q forms the dots of the basis vectors q, q + 8, ...
// with it (lanes over the entries, so every basis load is coalesced and a
// thread holds at most four accumulators).
__device__ __forceinline__ void chunk_dots(z_t (&acc)[LZ_VPW], const z_t* __restrict__ V, size_t ldv, int nVec,
                                           const TrajShape& S, size_t c0, int cn, const z_t* sw) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int q = 0; q < LZ_VPW; q++) {
    int k = wid + q * LZ_WARPS;
    if (k >= nVec) break;
    const z_t* Vk = V + ldv * k;
    z_t a = acc[q];
    for (int t = lane; t < cn; t += 32) {
      z_t v = Vk[vidx(S, c0 + t)];
      z_t b = sw[t];
      a.x += v.x * b.x + v.y * b.y;
      a.y += v.x * b.y - v.y * b.x;
    }
    acc[q] = a;
  }
}

// part[blk*stride + k] = warp sums of acc (one warp per vector k)
__device__ __forceinline__ void store_dots(z_t (&acc)[LZ_VPW], int nVec, z_t* __restrict__ part, int stride) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int q = 0; q < LZ_VPW; q++) {
    int k = wid + q * LZ_WARPS;
    if (k >= nVec) break;
    z_t a = acc[q];
    for (int o = 16; o > 0; o >>= 1) {
      a.x += __shfl_xor_sync(0xffffffffu, a.x, o);
      a.y += __shfl_xor_sync(0xffffffffu, a.y, o);
    }
    if (lane == 0) part[(size_t)blockIdx.x * stride + k] = a;
  }
}

// Second Gram-Schmidt pass needed?  True when the first pass cancelled most of
// w: ||w1||^2 <= eta^2 ||w0||^2 (w0 = H v_j before, w1 after the projections),
// the classical criterion for a loss of orthogonality beyond rounding.  Every
// block sums the same partials in the same order, so all blocks agree.
constexpr double LZ_ETA2 = 1.0e-2;
__device__ bool reorth_needed(const z_t* __restrict__ w0n, int stride, int nBlk0, const z_t* __restrict__ w1n,
                              int nBlk1) {
  __shared__ z_t g[2];
  sum_partials(w0n, nBlk0, stride, 1, g);
  sum_partials(w1n, nBlk1, 1, 1, g + 1);
  return g[1].x <= LZ_ETA2 * g[0].x;
}

// part[blk*stride + k] = sum_{i in blk} conj(V_k[i]) m[i] w[i] for k < nVec, in
// one pass over the data; with withNorm also part[blk*stride + nVec] = ||w||_m^2.
// Gated (gate0 != null): only when the reorthogonalisation test says so.
__global__ void __launch_bounds__(LZ_THREADS) k_mdot(z_t* __restrict__ part, int stride, const z_t* __restrict__ V,
                                                      size_t ldv, int nVec, const z_t* __restrict__ w,
                                                      const double* __restrict__ m, TRAJ_ARGS,
                                                      const double* __restrict__ lz, int E, int withNorm,
                                                      const z_t* __restrict__ gate0, int gateStride,
                                                      const z_t* __restrict__ gate1, int nBlkGate, int nBlkGate0) {
  const TrajShape& S = shp[blockIdx.z];
  lz = bat(lz, bs);
  if (lz[LZ_DONE] != 0.0) return;
  if (gate0 && !reorth_needed(bat(gate0, bs), gateStride, nBlkGate0, bat(gate1, bs), nBlkGate)) return;
  part = bat(part, bs);
  V = bat(V, bs);
  w = bat(w, bs);
  m = bat(m, bs);
  __shared__ z_t sw[LZ_THREADS * LZ_EMAX];
  const size_t n = S.nS;
  const int CH = LZ_THREADS * E;
  z_t acc[LZ_VPW];
#pragma unroll
  for (int q = 0; q < LZ_VPW; q++) acc[q] = zmk(0.0, 0.0);
  double nacc = 0.0;
  for (size_t c0 = (size_t)blockIdx.x * CH; c0 < n; c0 += (size_t)gridDim.x * CH) {
    int cn = (int)min((size_t)CH, n - c0);
    __syncthreads();
    for (int t = threadIdx.x; t < cn; t += LZ_THREADS) {
      size_t i = vidx(S, c0 + t);
      z_t wi = w[i];
      z_t b = zscale(wi, m[i]);
      sw[t] = b;
      nacc += wi.x * b.x + wi.y * b.y;
    }
    __syncthreads();
    chunk_dots(acc, V, ldv, nVec, S, c0, cn, sw);
  }
  store_dots(acc, nVec, part, stride);
  if (withNorm) {
    z_t t = block_sum2(zmk(nacc, 0.0));
    if (threadIdx.x == 0) part[(size_t)blockIdx.x * stride + nVec] = t;
  }
}

// Every block re-sums the dot partials (fixed order) into shared coefficients,
// subtracts w -= sum_k coef_k V_k and emits the partials of the metric norm^2
// of the new w.  Block 0 stores coefficient k at lz[LZ_D + 2 (dotBase + k)]
// (dotBase < 0: not stored).  Gated as k_mdot.
__global__ void __launch_bounds__(LZ_THREADS) k_cgs_pass(z_t* __restrict__ w, const z_t* __restrict__ V, size_t ldv,
                                                          int nVec, const z_t* __restrict__ partIn, int inStride,
                                                          int nBlkIn, z_t* __restrict__ partOut,
                                                          const double* __restrict__ m, TRAJ_ARGS,
                                                          double* __restrict__ lz, int dotBase, int E,
                                                          const z_t* __restrict__ gate0, int gateStride,
                                                          const z_t* __restrict__ gate1, int scaleIdx, int nBlkGate,
                                                          int nBlkGate0) {
  const TrajShape& S = shp[blockIdx.z];
  lz = bat(lz, bs);
  if (lz[LZ_DONE] != 0.0) return;
  if (gate0 && !reorth_needed(bat(gate0, bs), gateStride, nBlkGate0, bat(gate1, bs), nBlkGate)) return;
  w = bat(w, bs);
  V = bat(V, bs);
  partIn = bat(partIn, bs);
  partOut = bat(partOut, bs);
  m = bat(m, bs);
  __shared__ z_t coef[32];
  const size_t n = S.nS;
  const int CH = LZ_THREADS * E;
  sum_partials(partIn, nBlkIn, inStride, nVec, coef);
  if (scaleIdx >= 0) {  // unnormalised basis vectors u_k: the projection on u_k is <u_k, w> s_k^2 u_k
    __syncthreads();
    for (int k = threadIdx.x; k < nVec; k += blockDim.x) coef[k] = zscale(coef[k], lz[scaleIdx + k] * lz[scaleIdx + k]);
    __syncthreads();
  }
  if (dotBase >= 0 && blockIdx.x == 0)
    for (int k = threadIdx.x; k < nVec; k += blockDim.x) {
      lz[LZ_D + 2 * (dotBase + k)] = coef[k].x;
      lz[LZ_D + 2 * (dotBase + k) + 1] = coef[k].y;
    }
  double nacc = 0.0;
  for (size_t c0 = (size_t)blockIdx.x * CH; c0 < n; c0 += (size_t)gridDim.x * CH) {
    int cn = (int)min((size_t)CH, n - c0);
    for (int t = threadIdx.x; t < cn; t += LZ_THREADS) {
      size_t i = vidx(S, c0 + t);
      z_t r = w[i];
      for (int k = 0; k < nVec; k++) {
        z_t v = V[ldv * k + i];
        z_t cf = coef[k];
        r.x -= cf.x * v.x - cf.y * v.y;
        r.y -= cf.x * v.y + cf.y * v.x;
      }
      w[i] = r;
      double mi = m[i];
      nacc += (r.x * r.x + r.y * r.y) * mi;
    }
  }
  z_t t = block_sum2(zmk(nacc, 0.0));
  if (threadIdx.x == 0) partOut[blockIdx.x] = t;
}

// beta_j = sqrt(sum partials); alpha_j from the first-pass dot; v_{j+1} = w / beta_j.
// j is 1-based; alpha/beta stored at index j-1.
// The norm partials are those of the first pass (partIn) or, when the
// reorthogonalisation test fired, of the second (partAlt).
__global__ void k_lz_finish(z_t* __restrict__ vNext, const z_t* __restrict__ w, const z_t* __restrict__ partIn,
                            const z_t* __restrict__ partAlt, const z_t* __restrict__ gate0, int gateStride,
                            int nBlkIn, TRAJ_ARGS, double* __restrict__ lz, int j, int maxDim, double zeroThr) {
  const TrajShape& S = shp[blockIdx.z];
  lz = bat(lz, bs);
  if (lz[LZ_DONE] != 0.0) return;
  vNext = bat(vNext, bs);
  w = bat(w, bs);
  partIn = bat(partIn, bs);
  if (reorth_needed(bat(gate0, bs), gateStride, nBlkIn, partIn, nBlkIn)) partIn = bat(partAlt, bs);
  const size_t n = S.nS;
  __shared__ z_t tot[1];
  sum_partials(partIn, nBlkIn, 1, 1, tot);
  double be = sqrt(tot[0].x);
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    lz[LZ_ALPHA + j - 1] = lz[LZ_D + 2 * (j - 1)];
    lz[LZ_BETA + j - 1] = be;
  }
  bool breakdown = be <= zeroThr;
  if (breakdown || j == maxDim) {
    if (blockIdx.x == 0 && threadIdx.x == 0) {
      lz[LZ_MDIM] = j;
      if (breakdown) {
        lz[LZ_BREAKJ] = j;
      }
    }
    return;
  }
  if (vNext == nullptr) return;
  const double inv = 1.0 / be;
  for (size_t l = blockIdx.x * (size_t)blockDim.x + threadIdx.x; l < n; l += (size_t)gridDim.x * blockDim.x) {
    size_t i = vidx(S, l);
    vNext[i] = zscale(w[i], inv);
  }
}

__global__ void k_lz_mark_done(double* lz, int j, size_t bs) {
  // executed after k_lz_finish of iteration j: a breakdown stops the growth
  lz = bat(lz, bs);
  if (lz[LZ_DONE] == 0.0 && lz[LZ_BREAKJ] == (double)j) lz[LZ_DONE] = 1.0;
}

// EvaluateExpInSubspace: phi = exp(-i dt T_m) e1 for the m x m Lanczos
// tridiagonal T_m and the error estimate beta_m |phi_m|.  The reference
// diagonalises T_m (DSYEV) and forms U exp(-i dt L) U^T e1; the same vector is
// computed here without an eigensolver, by the Chebyshev (Jacobi-Anger)
// expansion of the exponential (Tal-Ezer & Kosloff, J. Chem. Phys. 81, 3967 (1984)):
//   T' = (T - c)/R with spectrum in [-1, 1] (Gershgorin bounds),
//   exp(-i z x) = J_0(z) + 2 sum_k (-i)^k J_k(z) T_k(x),  z = dt R,
//   phi = exp(-i dt c) sum_k a_k q_k,  q_0 = e1, q_1 = T' e1, q_{k+1} = 2 T' q_k - q_{k-1}.
// The Bessel values J_k(z) come from Miller's backward recurrence normalised
// by J_0 + 2 sum J_2k = 1.  The series is summed until the coefficients fall
// below 1e-17 relative, i.e. to machine precision.  One warp, lane i = row i (m <= 32).
__global__ void k_lz_expsub(double* __restrict__ lz, int mFixed, double dt, double tol, size_t bs) {
  constexpr int KMAX = 1200;
  lz = bat(lz, bs);
  __shared__ double J[KMAX + 2];
  __shared__ int nTerms;
  int lane = threadIdx.x;
  int m = mFixed > 0 ? mFixed : (int)lz[LZ_MDIM];
  if (m > 32) m = 32;
  if (m < 1) return;
  double a = (lane < m) ? lz[LZ_ALPHA + lane] : 0.0;
  double bl = (lane >= 1 && lane < m) ? lz[LZ_BETA + lane - 1] : 0.0;  // beta_{i-1}: couples i-1, i
  double br = (lane + 1 < m) ? lz[LZ_BETA + lane] : 0.0;               // beta_i:   couples i, i+1
  double lo = (lane < m) ? a - fabs(bl) - fabs(br) : 1e300;
  double hi = (lane < m) ? a + fabs(bl) + fabs(br) : -1e300;
  for (int o = 16; o > 0; o >>= 1) {
    lo = fmin(lo, __shfl_xor_sync(0xffffffffu, lo, o));
    hi = fmax(hi, __shfl_xor_sync(0xffffffffu, hi, o));
  }
  double c = 0.5 * (hi + lo);
  double R = 0.5 * (hi - lo);
  R = R * (1.0 + 1e-12) + 1e-300;
  double z = fabs(dt) * R;
  double sgn = dt >= 0.0 ? 1.0 : -1.0;  // exp(-i dt T) with dt < 0 is the complex conjugate series
  if (lane == 0) {
    int K = (int)(1.5 * z + 40.0);
    if (K > KMAX - 20) K = KMAX - 20;
    if (z < 1e-300) {
      J[0] = 1.0;
      for (int k = 1; k <= K; k++) J[k] = 0.0;
    } else {
      int N = K + 20;
      double jp = 0.0, jc = 1e-280, norm = 0.0;
      for (int k = N; k >= 1; k--) {
        double jm = (2.0 * k / z) * jc - jp;  // J_{k-1}
        jp = jc;
        jc = jm;
        if (k - 1 <= K) J[k - 1] = jc;
        if (k - 1 >= 1 && ((k - 1) & 1) == 0) norm += 2.0 * jc;
        if (fabs(jc) > 1e250) {  // rescale to keep the recurrence finite
          double s = 1e-250;
          jc *= s;
          jp *= s;
          norm *= s;
          for (int q = k - 1; q <= K && q <= N; q++) J[q] *= s;
        }
      }
      norm += jc;  // J_0
      for (int k = 0; k <= K; k++) J[k] /= norm;
    }
    int n = K;  // |J_k(z)| <= 1, so an absolute cut-off is relative to the largest term
    while (n > 1 && fabs(J[n]) < 1e-18 && n > z) n--;
    nTerms = n;
  }
  __syncwarp();
  int K = nTerms;
  double inv = 1.0 / R;
  double ta = (a - c) * inv, tl = bl * inv, tr = br * inv;
  // q_0 = e1, q_1 = T' e1
  double qm = (lane == 0) ? 1.0 : 0.0;
  double qlm = __shfl_up_sync(0xffffffffu, qm, 1);
  double qrm = __shfl_down_sync(0xffffffffu, qm, 1);
  double q = ta * qm + tl * (lane >= 1 ? qlm : 0.0) + tr * (lane + 1 < m ? qrm : 0.0);
  if (lane >= m) q = 0.0;
  double pr = J[0] * qm, pi = 0.0;
  // a_k = 2 (-i)^k J_k: k = 1 -> -2i J_1
  pi += -2.0 * J[1] * q;
  for (int k = 2; k <= K; k++) {
    double ql = __shfl_up_sync(0xffffffffu, q, 1);
    double qr = __shfl_down_sync(0xffffffffu, q, 1);
    double qn = 2.0 * (ta * q + tl * (lane >= 1 ? ql : 0.0) + tr * (lane + 1 < m ? qr : 0.0)) - qm;
    if (lane >= m) qn = 0.0;
    qm = q;
    q = qn;
    double co = 2.0 * J[k];
    switch (k & 3) {
      case 0: pr += co * q; break;   // (-i)^k = 1
      case 1: pi -= co * q; break;   // -i
      case 2: pr -= co * q; break;   // -1
      default: pi += co * q; break;  // +i
    }
  }
  pi *= sgn;
  // phase exp(-i dt c)
  double sn, cs;
  sincos(dt * c, &sn, &cs);
  double fr = cs * pr + sn * pi;
  double fi = cs * pi - sn * pr;
  if (lane < m) {
    lz[LZ_PHI + 2 * lane] = fr;
    lz[LZ_PHI + 2 * lane + 1] = fi;
  }
  if (lane == m - 1) {
    double err = lz[LZ_BETA + m - 1] * sqrt(fr * fr + fi * fi);
    if (lz[LZ_BREAKJ] == (double)m) err = 0.0;
    lz[LZ_ERR] = err;
    (void)tol;
  }
}


// out = nrm * sum_{j < mDim} phi_j s_j V_j   (or out = in when the start vector had zero norm)
// DF: the sum in double-float arithmetic on the orbital entries (the
// fixed-point forms; the FP64 form costs 4 m FP64 FMA per entry on the scarce
// FP64 pipe), rounded once to FP64; the CI coefficients stay FP64.
template <bool DF>
__global__ void k_lz_combine(z_t* __restrict__ out, const z_t* __restrict__ in, const z_t* __restrict__ V,
                             size_t ldv, TRAJ_ARGS, const double* __restrict__ lz) {
  const TrajShape& S = shp[blockIdx.z];
  out = bat(out, bs);
  in = bat(in, bs);
  V = bat(V, bs);
  lz = bat(lz, bs);
  const size_t n = S.nS;
  __shared__ z_t phi[CODY_MAX_KRYLOV];
  __shared__ float4 phiDf[CODY_MAX_KRYLOV];
  int m = (int)lz[LZ_MDIM];
  double nrm = lz[LZ_NRM];
  bool zero = lz[LZ_ZERO] != 0.0;
  for (int k = threadIdx.x; k < m; k += blockDim.x) {
    // the coefficient with the norm folded in (one rounding)
    phi[k] = zscale(zmk(lz[LZ_PHI + 2 * k], lz[LZ_PHI + 2 * k + 1]), lz[LZ_S + k]);
    if (DF) phiDf[k] = zdf_from(zscale(phi[k], nrm));
  }
  __syncthreads();
  for (size_t l = blockIdx.x * (size_t)blockDim.x + threadIdx.x; l < n; l += (size_t)gridDim.x * blockDim.x) {
    size_t i = vidx(S, l);
    if (zero) {
      out[i] = in[i];
      continue;
    }
    if (DF && l >= (size_t)S.nC) {  // orbital entries; the coefficients stay FP64
      zdf_acc acc = {0.0f, 0.0f, 0.0f, 0.0f};
      for (int k = 0; k < m; k++) zdf_fma(acc, phiDf[k], zdf_from(V[ldv * k + i]), false);
      out[i] = zdf_to_z(acc);
    } else {
      z_t acc = zmk(0.0, 0.0);
      for (int k = 0; k < m; k++) zfma(acc, V[ldv * k + i], phi[k]);
      out[i] = zscale(acc, nrm);
    }
  }
}

// nrm = sqrt(<s,s>_m); v1 = s / nrm; resets the per-step flags.
__global__ void k_lz_start(z_t* __restrict__ v1, const z_t* __restrict__ s, const z_t* __restrict__ partIn, int nBlkIn,
                           TRAJ_ARGS, double* __restrict__ lz, double zeroThr) {
  const TrajShape& S = shp[blockIdx.z];
  v1 = bat(v1, bs);
  s = bat(s, bs);
  partIn = bat(partIn, bs);
  lz = bat(lz, bs);
  const size_t n = S.nS;
  __shared__ z_t tot[1];
  sum_partials(partIn, nBlkIn, 1, 1, tot);
  double nr = sqrt(tot[0].x);
  bool zero = nr <= zeroThr;
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    lz[LZ_NRM] = nr;
    lz[LZ_ZERO] = zero ? 1.0 : 0.0;
    lz[LZ_DONE] = zero ? 1.0 : 0.0;
    lz[LZ_BREAKJ] = -1.0;
    lz[LZ_MDIM] = 0.0;
    lz[LZ_ERR] = 0.0;
  }
  if (blockIdx.x == 0)
    for (int k = threadIdx.x; k < LZ_SMAX; k += blockDim.x) lz[LZ_S + k] = 1.0;
  if (zero) return;
  const double inv = 1.0 / nr;
  for (size_t l = blockIdx.x * (size_t)blockDim.x + threadIdx.x; l < n; l += (size_t)gridDim.x * blockDim.x) {
    size_t i = vidx(S, l);
    v1[i] = zscale(s[i], inv);
  }
}

__global__ void k_norm_partial(z_t* __restrict__ part, const z_t* __restrict__ v, const double* __restrict__ m,
                               TRAJ_ARGS) {
  const TrajShape& S = shp[blockIdx.z];
  part = bat(part, bs);
  v = bat(v, bs);
  m = bat(m, bs);
  const size_t n = S.nS;
  z_t s = zmk(0.0, 0.0);
  for (size_t l = blockIdx.x * (size_t)blockDim.x + threadIdx.x; l < n; l += (size_t)gridDim.x * blockDim.x) {
    size_t i = vidx(S, l);
    z_t b = v[i];
    s.x += (b.x * b.x + b.y * b.y) * m[i];
  }
  s = block_sum2(s);
  if (threadIdx.x == 0) part[blockIdx.x] = s;
}

// Three-term recurrence on unnormalised basis vectors u_k (v_k = s_k u_k,
// s_k at lz[LZ_S + k - 1]): the operator is linear, so h = H u_j = H v_j / s_j
// and every pass forms the reference's w from h on the fly; u_(j+1) = w and
// s_(j+1) = 1 / beta_j replace the separate normalisation pass.
//
// Pass 1: part[blk*2] = sum m Re(conj(v_j) w'), part[blk*2+1] = sum m |w'|^2,
// w' = s_j h - beta_{j-1} v_{j-1}.
__global__ void __launch_bounds__(LZ_THREADS) k_lz3_dot(z_t* __restrict__ part, const z_t* __restrict__ vPrev,
                                                         const z_t* __restrict__ vCur, const z_t* __restrict__ w,
                                                         const double* __restrict__ m, TRAJ_ARGS,
                                                         const double* __restrict__ lz, int j) {
  const TrajShape& S = shp[blockIdx.z];
  lz = bat(lz, bs);
  if (lz[LZ_DONE] != 0.0) return;
  vCur = bat(vCur, bs);
  w = bat(w, bs);
  m = bat(m, bs);
  const double sj = lz[LZ_S + j - 1];
  const double bp = (j > 1) ? lz[LZ_BETA + j - 2] * lz[LZ_S + j - 2] : 0.0;  // beta_{j-1} s_{j-1}
  vPrev = (j > 1) ? bat(vPrev, bs) : nullptr;
  const size_t n = S.nS;
  double a = 0.0, q = 0.0;
  for (size_t l = blockIdx.x * (size_t)blockDim.x + threadIdx.x; l < n; l += (size_t)gridDim.x * blockDim.x) {
    const size_t i = vidx(S, l);
    const z_t h = w[i];
    z_t x = zmk(sj * h.x, sj * h.y);
    if (vPrev) {
      const z_t p = vPrev[i];
      x.x = fma(-bp, p.x, x.x);
      x.y = fma(-bp, p.y, x.y);
    }
    const z_t v = vCur[i];
    const double mi = m[i];
    a = fma(mi, fma(v.x, x.x, v.y * x.y), a);
    q = fma(mi, fma(x.x, x.x, x.y * x.y), q);
  }
  const z_t t = block_sum2(zmk(a * sj, q));
  if (threadIdx.x == 0) {
    part[(size_t)blockIdx.x * 2] = zmk(t.x, 0.0);
    part[(size_t)blockIdx.x * 2 + 1] = zmk(t.y, 0.0);
  }
}

// Pass 2: alpha_j from the pass-1 partials (stored at lz[LZ_D + 2 (j-1)]),
// u_(j+1) = s_j h - beta_{j-1} v_{j-1} - alpha_j v_j into dst (the next basis
// slot, or h itself after the last iteration), partials of ||u_(j+1)||_m^2.
// DF: the update and the norm in double-float arithmetic on the orbital
// entries (the fixed-point forms), each new entry rounded once to FP64; the
// CI coefficients (the first nC entries, a small share) stay FP64, so that
// their norm is conserved to FP64 rounding over long runs.
template <bool DF>
__global__ void __launch_bounds__(LZ_THREADS) k_lz3_update(z_t* __restrict__ dst, const z_t* __restrict__ w,
                                                            const z_t* __restrict__ vPrev,
                                                            const z_t* __restrict__ vCur, const z_t* __restrict__ partIn,
                                                            int nBlkIn, z_t* __restrict__ partOut,
                                                            const double* __restrict__ m, TRAJ_ARGS,
                                                            double* __restrict__ lz, int j) {
  const TrajShape& S = shp[blockIdx.z];
  lz = bat(lz, bs);
  if (lz[LZ_DONE] != 0.0) return;
  dst = bat(dst, bs);
  w = bat(w, bs);
  vCur = bat(vCur, bs);
  partIn = bat(partIn, bs);
  partOut = bat(partOut, bs);
  m = bat(m, bs);
  const double sj = lz[LZ_S + j - 1];
  const double bp = (j > 1) ? lz[LZ_BETA + j - 2] * lz[LZ_S + j - 2] : 0.0;
  vPrev = (j > 1) ? bat(vPrev, bs) : nullptr;
  __shared__ z_t al[1];
  sum_partials(partIn, nBlkIn, 2, 1, al);
  const double alpha = al[0].x;
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    lz[LZ_D + 2 * (j - 1)] = alpha;
    lz[LZ_D + 2 * (j - 1) + 1] = 0.0;
  }
  const double as = alpha * sj;
  const size_t n = S.nS;
  double q = 0.0;
  if (DF) {
    const float2 sj2 = df_split(sj), nbp2 = df_split(-bp), nas2 = df_split(-as), zero2 = make_float2(0.0f, 0.0f);
    float qs = 0.0f, qc = 0.0f;
    double qC = 0.0;  // the coefficient entries' norm part, FP64
    for (size_t l = blockIdx.x * (size_t)blockDim.x + threadIdx.x; l < n; l += (size_t)gridDim.x * blockDim.x) {
      const size_t i = vidx(S, l);
      if (l < (size_t)S.nC) {
        const z_t h = w[i];
        z_t x = zmk(sj * h.x, sj * h.y);
        if (vPrev) {
          const z_t p = vPrev[i];
          x.x = fma(-bp, p.x, x.x);
          x.y = fma(-bp, p.y, x.y);
        }
        const z_t v = vCur[i];
        x.x = fma(-as, v.x, x.x);
        x.y = fma(-as, v.y, x.y);
        dst[i] = x;
        qC = fma(m[i], fma(x.x, x.x, x.y * x.y), qC);
        continue;
      }
      const z_t h = w[i], v = vCur[i];
      float2 pr = zero2, pi = zero2;
      if (vPrev) {
        const z_t p = vPrev[i];
        pr = df_split(p.x);
        pi = df_split(p.y);
      }
      const float2 xr = df_dot3(sj2, df_split(h.x), nbp2, pr, nas2, df_split(v.x));
      const float2 xi = df_dot3(sj2, df_split(h.y), nbp2, pi, nas2, df_split(v.y));
      dst[i] = zmk(df_to_d(xr), df_to_d(xi));
      const float2 u = df_dot2(xr, xr, xi, xi), m2 = df_split(m[i]);
      df_mul_acc(qs, qc, m2.x, m2.y, u.x, u.y);
    }
    q = (f2d_exact(qs) + f2d_exact(qc)) + qC;
  } else
  for (size_t l = blockIdx.x * (size_t)blockDim.x + threadIdx.x; l < n; l += (size_t)gridDim.x * blockDim.x) {
    const size_t i = vidx(S, l);
    const z_t h = w[i];
    z_t x = zmk(sj * h.x, sj * h.y);
    if (vPrev) {
      const z_t p = vPrev[i];
      x.x = fma(-bp, p.x, x.x);
      x.y = fma(-bp, p.y, x.y);
    }
    const z_t v = vCur[i];
    x.x = fma(-as, v.x, x.x);
    x.y = fma(-as, v.y, x.y);
    dst[i] = x;
    q = fma(m[i], fma(x.x, x.x, x.y * x.y), q);
  }
  const z_t t = block_sum2(zmk(q, 0.0));
  if (threadIdx.x == 0) partOut[blockIdx.x] = t;
}

// End of a three-term iteration, one block per trajectory: beta_j from the norm
// partials of the first pass (or of the second, when the reorthogonalisation
// test fired), alpha_j and beta_j into the tridiagonal, s_(j+1) = 1 / beta_j;
// a breakdown or the last iteration fixes the subspace dimension, a breakdown
// also stops the growth.
__global__ void __launch_bounds__(LZ_THREADS) k_lz_scalars(const z_t* __restrict__ partIn, int nBlkIn,
                                                            const z_t* __restrict__ partAlt, int nBlkAlt,
                                                            const z_t* __restrict__ gate0, int gateStride,
                                                            int nBlkGate0, TRAJ_ARGS, double* __restrict__ lz, int j,
                                                            int maxDim, double zeroThr) {
  lz = bat(lz, bs);
  if (lz[LZ_DONE] != 0.0) return;
  partIn = bat(partIn, bs);
  int nPart = nBlkIn;
  if (reorth_needed(bat(gate0, bs), gateStride, nBlkGate0, partIn, nBlkIn)) {
    partIn = bat(partAlt, bs);
    nPart = nBlkAlt;
  }
  __shared__ z_t tot[1];
  sum_partials(partIn, nPart, 1, 1, tot);
  if (threadIdx.x != 0) return;
  const double be = sqrt(tot[0].x);
  lz[LZ_ALPHA + j - 1] = lz[LZ_D + 2 * (j - 1)];
  lz[LZ_BETA + j - 1] = be;
  const bool breakdown = be <= zeroThr;
  if (breakdown || j == maxDim) {
    lz[LZ_MDIM] = j;
    if (breakdown) {
      lz[LZ_BREAKJ] = j;
      lz[LZ_DONE] = 1.0;
    }
    return;
  }
  lz[LZ_S + j] = 1.0 / be;
}

}  // namespace

size_t lanczos_partial_need(const cgpu_ctx* c) { return (size_t)c->lzBlocks * (2 * (c->maxKrylov + 1) + 2); }

// Starts a Lanczos pass from the vector v (device, state layout): basis[:,0] = v/|v|.
void launch_lanczos_start(cgpu_ctx* c, const z_t* v) {
  ProfScope prof(c, CGPU_KERNEL_VECTOR);
  int nBlk = c->lzBlocks;
  k_norm_partial<<<bgrid(c, nBlk), LZ_THREADS, 0, c->stream>>>(c->partial_d, v, c->metric_d, TRAJ_PASS(c));
  CODY_LAUNCHED(c);
  k_lz_start<<<bgrid(c, nBlk), LZ_THREADS, 0, c->stream>>>(c->basis_d, v, c->partial_d, nBlk, TRAJ_PASS(c), c->lz_d,
                                                           1.0e-14);
  CODY_LAUNCHED(c);
}

// After lw_d holds H v_j: Gram-Schmidt against v_1..v_j (or the window's last
// vectors), the gated second pass, beta_j, v_{j+1}.
void launch_lanczos_update(cgpu_ctx* c, int j, int maxDim, int pass1Blocks) {
  ProfScope prof(c, CGPU_KERNEL_LANCZOS);
  size_t ld = c->nS;
  int nBlk = c->lzBlocks;
  // p1: pass-1 dots with the nv vectors and ||w0||^2 (stride nv+1); p2: ||w1||^2
  // after pass 1; p3, p4: dots and norm of the gated second pass
  z_t* p1 = c->partial_d;
  z_t* p2 = p1 + (size_t)nBlk * (c->maxKrylov + 1);
  z_t* p3 = p2 + nBlk;
  z_t* p4 = p3 + (size_t)nBlk * (c->maxKrylov + 1);
  if (j > 32) throw std::string("SIL: Krylov order above 32");
  if (c->krylovWindow == 1) {
    // three-term recurrence on unnormalised basis vectors; the gated second
    // pass re-orthogonalises the new vector against u_j
    const z_t* vCur = c->basis_d + ld * (size_t)(j - 1);
    const z_t* vPrev = (j > 1) ? c->basis_d + ld * (size_t)(j - 2) : nullptr;
    z_t* uNext = (j < maxDim) ? c->basis_d + ld * (size_t)j : c->lw_d;
    dim3 g = bgrid(c, nBlk);
    const int E = c->lzElems;
    // pass 1 (alpha and ||w'||^2 partials): here, or already emitted by the
    // fused one-body apply (pass1Blocks partials per trajectory)
    const int n1 = pass1Blocks > 0 ? pass1Blocks : nBlk;
    if (pass1Blocks <= 0) {
      k_lz3_dot<<<g, LZ_THREADS, 0, c->stream>>>(p1, vPrev, vCur, c->lw_d, c->metric_d, TRAJ_PASS(c), c->lz_d, j);
      CODY_LAUNCHED(c);
    }
    auto update = c->ciDf ? k_lz3_update<true> : k_lz3_update<false>;
    update<<<g, LZ_THREADS, 0, c->stream>>>(uNext, c->lw_d, vPrev, vCur, p1, n1, p2, c->metric_d, TRAJ_PASS(c),
                                            c->lz_d, j);
    CODY_LAUNCHED(c);
    // the gated second pass rarely fires: one block per trajectory reads the
    // gate (and, when it fires, walks the whole vector)
    dim3 g1 = bgrid(c, 1);
    k_mdot<<<g1, LZ_THREADS, 0, c->stream>>>(p3, 1, vCur, ld, 1, uNext, c->metric_d, TRAJ_PASS(c), c->lz_d, E, 0,
                                             p1 + 1, 2, p2, nBlk, n1);
    CODY_LAUNCHED(c);
    k_cgs_pass<<<g1, LZ_THREADS, 0, c->stream>>>(uNext, vCur, ld, 1, p3, 1, 1, p4, c->metric_d, TRAJ_PASS(c), c->lz_d,
                                                 -1, E, p1 + 1, 2, p2, LZ_S + j - 1, nBlk, n1);
    CODY_LAUNCHED(c);
    k_lz_scalars<<<g1, LZ_THREADS, 0, c->stream>>>(p2, nBlk, p4, 1, p1 + 1, 2, n1, TRAJ_PASS(c), c->lz_d, j, maxDim,
                                                   1.0e-14);
    CODY_LAUNCHED(c);
    return;
  }
  const int base = (c->krylovWindow > 0) ? std::max(0, j - c->krylovWindow) : 0;
  const int nv = j - base, s1 = nv + 1;
  const z_t* V = c->basis_d + ld * (size_t)base;
  const int E = c->lzElems;
  dim3 g = bgrid(c, nBlk);
  k_mdot<<<g, LZ_THREADS, 0, c->stream>>>(p1, s1, V, ld, nv, c->lw_d, c->metric_d, TRAJ_PASS(c), c->lz_d, E, 1,
                                          nullptr, 0, nullptr, nBlk, nBlk);
  CODY_LAUNCHED(c);
  k_cgs_pass<<<g, LZ_THREADS, 0, c->stream>>>(c->lw_d, V, ld, nv, p1, s1, nBlk, p2, c->metric_d, TRAJ_PASS(c),
                                              c->lz_d, base, E, nullptr, 0, nullptr, -1, nBlk, nBlk);
  CODY_LAUNCHED(c);
  k_mdot<<<g, LZ_THREADS, 0, c->stream>>>(p3, nv, V, ld, nv, c->lw_d, c->metric_d, TRAJ_PASS(c), c->lz_d, E, 0,
                                          p1 + nv, s1, p2, nBlk, nBlk);
  CODY_LAUNCHED(c);
  k_cgs_pass<<<g, LZ_THREADS, 0, c->stream>>>(c->lw_d, V, ld, nv, p3, nv, nBlk, p4, c->metric_d, TRAJ_PASS(c),
                                              c->lz_d, -1, E, p1 + nv, s1, p2, -1, nBlk, nBlk);
  CODY_LAUNCHED(c);
  z_t* vNext = (j < maxDim) ? c->basis_d + ld * (size_t)j : nullptr;
  k_lz_finish<<<g, LZ_THREADS, 0, c->stream>>>(vNext, c->lw_d, p2, p4, p1 + nv, s1, nBlk, TRAJ_PASS(c), c->lz_d, j,
                                               maxDim, 1.0e-14);
  CODY_LAUNCHED(c);
  k_lz_mark_done<<<bgrid(c, 1), 1, 0, c->stream>>>(c->lz_d, j, c->bs);
  CODY_LAUNCHED(c);
}

void launch_lanczos_tail(cgpu_ctx* c, int j, double dt, int evalExp) {
  ProfScope prof(c, CGPU_KERNEL_VECTOR);
  if (!evalExp) return;
  k_lz_expsub<<<bgrid(c, 1), 32, 0, c->stream>>>(c->lz_d, j, dt, 0.0, c->bs);
  CODY_LAUNCHED(c);
}

void launch_lanczos_combine(cgpu_ctx* c, z_t* out, const z_t* start) {
  ProfScope prof(c, CGPU_KERNEL_VECTOR);
  auto comb = c->ciDf ? k_lz_combine<true> : k_lz_combine<false>;
  comb<<<bgrid(c, c->lzBlocks), LZ_THREADS, 0, c->stream>>>(out, start, c->basis_d, c->nS, TRAJ_PASS(c), c->lz_d);
  CODY_LAUNCHED(c);
}

void launch_lz_set(cgpu_ctx* c, int idx, double v) { launch_set_scalar(c, c->lz_d + idx, v); }
