// k_lanczos.cu -- short-iterative-Lanczos kernels
// (PerformLanczosStep / EvaluateExpInSubspace / MetricDot,
//  src/IntegratorList/Sil/S_IntegratorList_Sil.f90:184-310).
//
// Per Krylov iteration j the reference does
//   w = H v_j - beta_{j-1} v_{j-1};  alpha_j = Re<v_j,w>;  w -= alpha_j v_j;
//   for k = 1..j: w -= <v_k,w> v_k   (modified Gram-Schmidt);  beta_j = ||w||.
// With the basis orthonormal, the projections it removes are those of H v_j on
// v_1..v_j; the kernels remove them in two classical Gram-Schmidt passes
// (each pass one fused reduction), which reproduces the reference's vectors
// and coefficients to rounding.  Every reduction is deterministic: per-block
// partials in a fixed order, re-summed identically by every consumer block.
//
// Device scalar block lz[] (doubles):
#include <type_traits>

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

constexpr int LZ_BLOCKS = 148;
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

constexpr int LZ_MAXV = 32;  // Krylov vectors handled per reduction pass

// Block-reduces acc[0..nVec) (register arrays of every thread) into out[0..nVec).
template <int MAXV>
__device__ void block_reduce_many(z_t (&acc)[MAXV], int nVec, z_t* __restrict__ out) {
  __shared__ z_t red[MAXV][LZ_THREADS / 32];
  int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < MAXV; k++) {
    if (k >= nVec) break;
    z_t v = acc[k];
    for (int o = 16; o > 0; o >>= 1) {
      v.x += __shfl_down_sync(0xffffffffu, v.x, o);
      v.y += __shfl_down_sync(0xffffffffu, v.y, o);
    }
    if (lane == 0) red[k][wid] = v;
  }
  __syncthreads();
  for (int k = threadIdx.x; k < nVec; k += blockDim.x) {
    z_t s = zmk(0.0, 0.0);
    for (int q = 0; q < LZ_THREADS / 32; q++) s = zadd(s, red[k][q]);
    out[k] = s;
  }
}

// part[blk*nVec + k] = sum_{i in blk} conj(V_k[i]) m[i] w[i], all k in one pass over the data.
template <int MAXV>
__global__ void __launch_bounds__(LZ_THREADS) k_mdot(z_t* __restrict__ part, const z_t* __restrict__ V, size_t ldv,
                                                      int nVec, const z_t* __restrict__ w,
                                                      const double* __restrict__ m, size_t n,
                                                      const double* __restrict__ lz) {
  if (lz && lz[LZ_DONE] != 0.0) return;
  z_t acc[MAXV];
#pragma unroll
  for (int k = 0; k < MAXV; k++) acc[k] = zmk(0.0, 0.0);
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    z_t b = zscale(w[i], m[i]);
#pragma unroll
    for (int k = 0; k < MAXV; k++) {
      if (k >= nVec) break;
      z_t a = V[ldv * k + i];
      acc[k].x += a.x * b.x + a.y * b.y;
      acc[k].y += a.x * b.y - a.y * b.x;
    }
  }
  block_reduce_many<MAXV>(acc, nVec, part + (size_t)blockIdx.x * nVec);
}

// Every block re-sums the partials (fixed order) into shared coefficients,
// subtracts w -= sum_k coef_k V_k, and in the same pass emits partials for the
// next stage: mode 0: dots of the new w with V_0..V_{nVec-1}; mode 1: the
// metric norm^2 of the new w.  Block 0 stores the first-pass coefficients at lz[LZ_D].
template <int MAXV>
__global__ void __launch_bounds__(LZ_THREADS) k_cgs_pass(z_t* __restrict__ w, const z_t* __restrict__ V, size_t ldv,
                                                          int nVec, const z_t* __restrict__ partIn, int nBlkIn,
                                                          z_t* __restrict__ partOut, const double* __restrict__ m,
                                                          size_t n, double* __restrict__ lz, int mode,
                                                          int storeDots) {
  if (lz[LZ_DONE] != 0.0) return;
  __shared__ z_t coef[MAXV];
  sum_partials(partIn, nBlkIn, nVec, nVec, coef);
  if (storeDots && blockIdx.x == 0)
    for (int k = threadIdx.x; k < nVec; k += blockDim.x) {
      lz[LZ_D + 2 * k] = coef[k].x;
      lz[LZ_D + 2 * k + 1] = coef[k].y;
    }
  z_t acc[MAXV];
#pragma unroll
  for (int k = 0; k < MAXV; k++) acc[k] = zmk(0.0, 0.0);
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    z_t r = w[i];
#pragma unroll
    for (int k = 0; k < MAXV; k++) {
      if (k >= nVec) break;
      z_t v = V[ldv * k + i];
      z_t cf = coef[k];
      r.x -= cf.x * v.x - cf.y * v.y;
      r.y -= cf.x * v.y + cf.y * v.x;
    }
    w[i] = r;
    z_t b = zscale(r, m[i]);
    if (mode == 0) {
#pragma unroll
      for (int k = 0; k < MAXV; k++) {
        if (k >= nVec) break;
        z_t a = V[ldv * k + i];
        acc[k].x += a.x * b.x + a.y * b.y;
        acc[k].y += a.x * b.y - a.y * b.x;
      }
    } else {
      acc[0].x += r.x * b.x + r.y * b.y;
    }
  }
  if (mode == 0) {
    block_reduce_many<MAXV>(acc, nVec, partOut + (size_t)blockIdx.x * nVec);
  } else {
    block_reduce_many<MAXV>(acc, 1, partOut + blockIdx.x);
  }
}

// beta_j = sqrt(sum partials); alpha_j from the first-pass dot; v_{j+1} = w / beta_j.
// j is 1-based; alpha/beta stored at index j-1.
__global__ void k_lz_finish(z_t* __restrict__ vNext, const z_t* __restrict__ w, const z_t* __restrict__ partIn,
                            int nBlkIn, size_t n, double* __restrict__ lz, int j, int maxDim, double zeroThr) {
  if (lz[LZ_DONE] != 0.0) return;
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
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    z_t v = w[i];
    vNext[i] = zmk(v.x / be, v.y / be);
  }
}

__global__ void k_lz_mark_done(double* lz, int j) {
  // executed after k_lz_finish of iteration j: a breakdown stops the growth
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
__global__ void k_lz_expsub(double* __restrict__ lz, int mFixed, double dt, double tol) {
  constexpr int KMAX = 1200;
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


// out = nrm * sum_{j < mDim} phi_j V_j   (or out = in when the start vector had zero norm)
__global__ void k_lz_combine(z_t* __restrict__ out, const z_t* __restrict__ in, const z_t* __restrict__ V,
                             size_t ldv, size_t n, const double* __restrict__ lz) {
  __shared__ z_t phi[CODY_MAX_KRYLOV];
  int m = (int)lz[LZ_MDIM];
  double nrm = lz[LZ_NRM];
  bool zero = lz[LZ_ZERO] != 0.0;
  for (int k = threadIdx.x; k < m; k += blockDim.x) phi[k] = zmk(lz[LZ_PHI + 2 * k], lz[LZ_PHI + 2 * k + 1]);
  __syncthreads();
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    if (zero) {
      out[i] = in[i];
      continue;
    }
    z_t acc = zmk(0.0, 0.0);
    for (int k = 0; k < m; k++) zfma(acc, V[ldv * k + i], phi[k]);
    out[i] = zscale(acc, nrm);
  }
}

// nrm = sqrt(<s,s>_m); v1 = s / nrm; resets the per-step flags.
__global__ void k_lz_start(z_t* __restrict__ v1, const z_t* __restrict__ s, const z_t* __restrict__ partIn, int nBlkIn,
                           size_t n, double* __restrict__ lz, double zeroThr) {
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
  if (zero) return;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    z_t v = s[i];
    v1[i] = zmk(v.x / nr, v.y / nr);
  }
}

__global__ void k_norm_partial(z_t* __restrict__ part, const z_t* __restrict__ v, const double* __restrict__ m, size_t n) {
  z_t s = zmk(0.0, 0.0);
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    z_t b = v[i];
    s.x += (b.x * b.x + b.y * b.y) * m[i];
  }
  s = block_sum2(s);
  if (threadIdx.x == 0) part[blockIdx.x] = s;
}

void ensure_lz_partial(cgpu_ctx* c) {
  size_t need = (size_t)LZ_BLOCKS * (CODY_MAX_KRYLOV + 1) * 2;
  if (c->partialCap >= need) return;
  if (c->partial_d) cudaFree(c->partial_d);
  CODY_CUDA(cudaMalloc(&c->partial_d, need * sizeof(z_t)));
  c->partialCap = need;
}

}  // namespace

// Starts a Lanczos pass from the vector v (device, nS): basis[:,0] = v/|v|.
void launch_lanczos_start(cgpu_ctx* c, const z_t* v) {
  ensure_lz_partial(c);
  k_norm_partial<<<LZ_BLOCKS, LZ_THREADS, 0, c->stream>>>(c->partial_d, v, c->metric_d, c->nS);
  CODY_LAUNCHED(c);
  k_lz_start<<<LZ_BLOCKS, LZ_THREADS, 0, c->stream>>>(c->basis_d, v, c->partial_d, LZ_BLOCKS, c->nS, c->lz_d, 1.0e-14);
  CODY_LAUNCHED(c);
}

// After lw_d holds H v_j: CGS2 against v_1..v_j, beta_j, v_{j+1}.
void launch_lanczos_update(cgpu_ctx* c, int j, int maxDim) {
  ProfScope prof(c, CGPU_KERNEL_LANCZOS);
  ensure_lz_partial(c);
  size_t nS = c->nS;
  z_t* p1 = c->partial_d;
  z_t* p2 = c->partial_d + (size_t)LZ_BLOCKS * (CODY_MAX_KRYLOV + 1);
  auto passes = [&](auto tag) {
    constexpr int MV = decltype(tag)::value;
    k_mdot<MV><<<LZ_BLOCKS, LZ_THREADS, 0, c->stream>>>(p1, c->basis_d, nS, j, c->lw_d, c->metric_d, nS, c->lz_d);
    CODY_LAUNCHED(c);
    k_cgs_pass<MV><<<LZ_BLOCKS, LZ_THREADS, 0, c->stream>>>(c->lw_d, c->basis_d, nS, j, p1, LZ_BLOCKS, p2,
                                                             c->metric_d, nS, c->lz_d, 0, 1);
    CODY_LAUNCHED(c);
    k_cgs_pass<MV><<<LZ_BLOCKS, LZ_THREADS, 0, c->stream>>>(c->lw_d, c->basis_d, nS, j, p2, LZ_BLOCKS, p1,
                                                             c->metric_d, nS, c->lz_d, 1, 0);
    CODY_LAUNCHED(c);
  };
  if (j <= 8) passes(std::integral_constant<int, 8>());
  else if (j <= 16) passes(std::integral_constant<int, 16>());
  else passes(std::integral_constant<int, 32>());
  z_t* vNext = (j < maxDim) ? c->basis_d + nS * (size_t)j : nullptr;
  k_lz_finish<<<LZ_BLOCKS, LZ_THREADS, 0, c->stream>>>(vNext, c->lw_d, p1, LZ_BLOCKS, nS, c->lz_d, j, maxDim,
                                                        1.0e-14);
  CODY_LAUNCHED(c);
  k_lz_mark_done<<<1, 1, 0, c->stream>>>(c->lz_d, j);
  CODY_LAUNCHED(c);
}

void launch_lanczos_tail(cgpu_ctx* c, int j, double dt, int evalExp) {
  if (!evalExp) return;
  k_lz_expsub<<<1, 32, 0, c->stream>>>(c->lz_d, j, dt, 0.0);
  CODY_LAUNCHED(c);
}

void launch_lanczos_combine(cgpu_ctx* c, z_t* out) {
  k_lz_combine<<<LZ_BLOCKS, LZ_THREADS, 0, c->stream>>>(out, c->work_d, c->basis_d, c->nS, c->nS, c->lz_d);
  CODY_LAUNCHED(c);
}

__global__ void k_lz_set(double* lz, int idx, double v) { lz[idx] = v; }

void launch_lz_set(cgpu_ctx* c, int idx, double v) {
  k_lz_set<<<1, 1, 0, c->stream>>>(c->lz_d, idx, v);
  CODY_LAUNCHED(c);
}
