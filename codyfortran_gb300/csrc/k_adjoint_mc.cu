// k_adjoint_mc.cu -- gradient of a final-time MCTDHF objective with respect to
// every sample of the laser field, by the exact discrete adjoint of the Strang
// step (no counterpart in the reference; the forward map is the reference's
// step: src/Propagator/SplitStep/Order2/S_Propagator_SplitStep_Order2.f90:52-77
// with fixed-order SIL on OrbsLin, src/IntegratorList/Sil/S_IntegratorList_Sil.f90:207-310,
// and RK4 on CoeffsPlusOrbsNonLin, src/Method/Mb/OrbBased/Mctdhx/S_Method_Mb_OrbBased_Mctdhx.f90:180-226).
//
// Systems: restricted MCTDHF with two body types (spins) of one particle each,
// M <= 16 spatial orbitals: the two-electron problem of the 1D helium model.
// There the configuration space is the M x M matrix C (C[a, b]: orbital a of
// body type 1, b of body type 2; state index a + M b) and the reference's
// generic CI traversals reduce to dense algebra, checked against the
// configuration-table path to rounding:
//   H1 C = h1^T C + C h1,  H2 C = sum_ab g(a, b; c, d) C[a, b],
//   g(a, b; c, d) = <phi_a| W_bd |phi_c>_w,  W_bd(x) = sum_y V(x, y) conj(phi_b(y)) phi_d(y) w(y),
//   rho1 = conj(C) C^T + C^H C (spin-summed),
//   rho2[a, b, c, d] = C[c, d] conj(C[a, b]) + C[d, c] conj(C[b, a]),
//   Mreg = U n/(n^2 + eps) U^H (rho1 = U n U^H),  R[a, b, j, d] = sum_k rho2[a, b, k, d] Mreg[k, j],
//   dphi_j(x) += sum_{a, k, l} W_lk(x) phi_a(x) R[a, k, j, l],
// then the (1 - P) projector on the orbitals, P_C on the coefficients and -i.
//
// Field: piecewise constant, E(t) = field[floor(t / dt)] (zero outside), the
// convention of the sampled laser; the one-body operator is
// h = T + V0(x) + E(t) x.  Stage times are the reference's, so step n reads
// field[n] (both SIL halves, RK4 stages 1-3) and field[n + 1] (RK4 stage 4).
//
// Objective: J = 1 - |<Psi_ref | Psi_N>|^2 with the MCTDHF overlap
// <Psi_ref|Psi> = sum conj(C_ref[a, b]) (S C S^T)[a, b], S = phi_ref^H W phi.
//
// Adjoint: co-states in the convention dL = Re sum conj(xbar) dx.  The
// Lanczos step is differentiated as the three-term recurrence (its full
// re-orthogonalisation is the identity in exact arithmetic), exp(-i tau T) e1
// through the eigenvector form of its Frechet derivative, the NonLin
// derivative piece by piece (the regularised inverse by the Daleckii-Krein
// formula).  The forward sweep keeps the state every `checkpoint` steps; the
// backward sweep recomputes a segment at a time, and each step's
// intermediates (Krylov bases, RK4 stages, NonLin intermediates) again while
// it is differentiated.
#include <algorithm>
#include <cmath>
#include <vector>

#include "common.cuh"

namespace {

constexpr int MC_T = 256;
constexpr int MC_MAXM = 16;
constexpr int MC_MAXK = 32;
constexpr int MC_RED = 512;  // threads of the one-block reductions

unsigned nblk(size_t n) { return (unsigned)std::min<size_t>((n + MC_T - 1) / MC_T, 4096); }

#define MC_LOOP(e, n) for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < (size_t)(n); e += (size_t)gridDim.x * blockDim.x)

// ---------------------------------------------------------------------------
// Generic building blocks
// ---------------------------------------------------------------------------

// op: 0 = A, 1 = A^T, 2 = A^H, 3 = conj(A)
__device__ __forceinline__ z_t opget(const z_t* A, int lda, int op, int i, int k) {
  z_t v = (op == 0 || op == 3) ? A[i + (size_t)lda * k] : A[k + (size_t)lda * i];
  return op >= 2 ? zconj(v) : v;
}

// C = alpha op(A) diag(wk) op(B) + beta C (column-major; wk may be null)
__global__ void k_mc_zgemm(int M, int N, int K, z_t alpha, const z_t* __restrict__ A, int lda, int opA,
                           const z_t* __restrict__ B, int ldb, int opB, const double* __restrict__ wk, z_t beta,
                           z_t* __restrict__ C, int ldc) {
  MC_LOOP(e, (size_t)M * N) {
    const int i = (int)(e % M), j = (int)(e / M);
    z_t s = zmk(0.0, 0.0);
    for (int k = 0; k < K; k++) {
      z_t a = opget(A, lda, opA, i, k);
      if (wk) a = zscale(a, wk[k]);
      zfma(s, a, opget(B, ldb, opB, k, j));
    }
    z_t r = zmul(alpha, s);
    if (beta.x != 0.0 || beta.y != 0.0) r = zadd(r, zmul(beta, C[i + (size_t)ldc * j]));
    C[i + (size_t)ldc * j] = r;
  }
}

// k_mc_zgemm with one warp per output element (small outputs, long K): lanes
// stride K, a fixed-order shuffle tree sums them
__global__ void k_mc_zgemm_w(int M, int N, int K, z_t alpha, const z_t* __restrict__ A, int lda, int opA,
                             const z_t* __restrict__ B, int ldb, int opB, const double* __restrict__ wk, z_t beta,
                             z_t* __restrict__ C, int ldc) {
  const int lane = threadIdx.x & 31;
  const size_t nw = ((size_t)gridDim.x * blockDim.x) >> 5;
  for (size_t e = (blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5; e < (size_t)M * N; e += nw) {
    const int i = (int)(e % M), j = (int)(e / M);
    z_t s = zmk(0.0, 0.0);
    for (int k = lane; k < K; k += 32) {
      z_t a = opget(A, lda, opA, i, k);
      if (wk) a = zscale(a, wk[k]);
      zfma(s, a, opget(B, ldb, opB, k, j));
    }
    for (int o = 16; o > 0; o >>= 1) {
      s.x += __shfl_xor_sync(0xffffffffu, s.x, o);
      s.y += __shfl_xor_sync(0xffffffffu, s.y, o);
    }
    if (lane == 0) {
      z_t r = zmul(alpha, s);
      if (beta.x != 0.0 || beta.y != 0.0) r = zadd(r, zmul(beta, C[i + (size_t)ldc * j]));
      C[i + (size_t)ldc * j] = r;
    }
  }
}

// C = V B (+ C when acc): V the real symmetric nG x nG interaction matrix; one
// warp per output element (lanes over the row of V and the column of B)
__global__ void k_mc_vgemm(int nG, int N, const double* __restrict__ V, const z_t* __restrict__ B, z_t* __restrict__ C,
                           int acc) {
  const int lane = threadIdx.x & 31;
  const size_t nw = ((size_t)gridDim.x * blockDim.x) >> 5;
  for (size_t e = (blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5; e < (size_t)nG * N; e += nw) {
    const int x = (int)(e % nG), j = (int)(e / nG);
    const double* Vr = V + (size_t)x * nG;
    const z_t* b = B + (size_t)nG * j;
    z_t s = zmk(0.0, 0.0);
    for (int y = lane; y < nG; y += 32) {
      s.x = fma(Vr[y], b[y].x, s.x);
      s.y = fma(Vr[y], b[y].y, s.y);
    }
    for (int o = 16; o > 0; o >>= 1) {
      s.x += __shfl_xor_sync(0xffffffffu, s.x, o);
      s.y += __shfl_xor_sync(0xffffffffu, s.y, o);
    }
    if (lane == 0) C[e] = acc ? zadd(C[e], s) : s;
  }
}

// out[slot] = sum_i conj(a[i]) w[i] b[i] (w may be null): one block, fixed order
__global__ void __launch_bounds__(MC_RED) k_mc_dot(z_t* __restrict__ out, const z_t* __restrict__ a,
                                                   const z_t* __restrict__ b, const double* __restrict__ w, int n) {
  __shared__ double sx[MC_RED], sy[MC_RED];
  z_t s = zmk(0.0, 0.0);
  for (int i = threadIdx.x; i < n; i += MC_RED) {
    z_t v = zcmul(a[i], b[i]);
    if (w) v = zscale(v, w[i]);
    s = zadd(s, v);
  }
  sx[threadIdx.x] = s.x;
  sy[threadIdx.x] = s.y;
  __syncthreads();
  for (int o = MC_RED / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) {
      sx[threadIdx.x] += sx[threadIdx.x + o];
      sy[threadIdx.x] += sy[threadIdx.x + o];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = zmk(sx[0], sy[0]);
}

// One-body operator on the orbital part of state vectors: out_phi = s (T + V0 + E x) in_phi
// (trans: the transposed banded matrix), C part of out zero.  T: the banded
// rows of body type 1 ((2 band + 1) x nG).
__global__ void k_mc_apply_h(z_t* __restrict__ out, const z_t* __restrict__ in, const double* __restrict__ T,
                             const double* __restrict__ V0, const double* __restrict__ x, double E, int nG, int band,
                             int M, int offC, int trans) {
  const int nd = 2 * band + 1;
  MC_LOOP(e, (size_t)offC + (size_t)nG * M) {
    if ((int)e < offC) {
      out[e] = zmk(0.0, 0.0);
      continue;
    }
    const size_t f = e - offC;
    const int g = (int)(f % nG);
    const z_t* col = in + offC + (f - g);
    z_t acc = zscale(col[g], fma(E, x[g], V0[g]));
    for (int d = 0; d < nd; d++) {
      const int gg = g - band + d;
      if (gg < 0 || gg >= nG) continue;
      // row g of T at column gg is T[d][g]; row gg at column g is T[2 band - d][gg]
      const double c = trans ? T[(size_t)(nd - 1 - d) * nG + gg] : T[(size_t)d * nG + g];
      acc.x = fma(c, col[gg].x, acc.x);
      acc.y = fma(c, col[gg].y, acc.y);
    }
    out[e] = acc;
  }
}

// y = a x + b y with complex constants; n entries
__global__ void k_mc_axpby(z_t* __restrict__ y, const z_t* __restrict__ x, z_t a, z_t b, int n) {
  MC_LOOP(e, n) y[e] = zadd(zmul(a, x[e]), zmul(b, y[e]));
}

// y += s x with s = sgn * (*coef) (complex device scalar) * mul, n entries
__global__ void k_mc_axpy_dev(z_t* __restrict__ y, const z_t* __restrict__ x, const z_t* __restrict__ coef, double mul,
                              int conjc, int n) {
  z_t s = *coef;
  if (conjc) s = zconj(s);
  s = zscale(s, mul);
  MC_LOOP(e, n) zfma(y[e], s, x[e]);
}

// w_el = w[g] on orbital entries, 1 on the C part (the SIL metric), and w x
__global__ void k_mc_weights(double* __restrict__ m, double* __restrict__ wx, const double* __restrict__ w,
                             const double* __restrict__ x, int nG, int M, int offC) {
  MC_LOOP(e, (size_t)offC + (size_t)nG * M) {
    if ((int)e < offC) {
      m[e] = 1.0;
      continue;
    }
    const int g = (int)((e - offC) % nG);
    m[e] = w[g];
    if (e - offC < (size_t)nG) wx[g] = w[g] * x[g];
  }
}

// out_el = X v: x on the orbital entries, 0 on the C part
__global__ void k_mc_xmul(z_t* __restrict__ out, const z_t* __restrict__ v, const double* __restrict__ x, int nG, int M,
                          int offC) {
  MC_LOOP(e, (size_t)offC + (size_t)nG * M) {
    out[e] = (int)e < offC ? zmk(0.0, 0.0) : zscale(v[e], x[(e - offC) % nG]);
  }
}

// ---------------------------------------------------------------------------
// Small Hermitian eigenproblems (rho1: M x M; the Krylov tridiagonal: K x K)
// in one block: cyclic Jacobi in tournament order, A = V diag(ev) V^H.
// ---------------------------------------------------------------------------
constexpr int JM = 32;

__device__ void herm_jacobi(z_t (*A)[JM + 1], z_t (*V)[JM + 1], int n, double* ev) {
  __shared__ double rc[JM / 2], rs[JM / 2];
  __shared__ z_t rph[JM / 2];
  __shared__ int rp[JM / 2], rq[JM / 2];
  __shared__ double offs, diags;
  const int tid = threadIdx.x;
  for (int e = tid; e < n * n; e += blockDim.x) {
    const int i = e % n, j = e / n;
    V[i][j] = zmk(i == j ? 1.0 : 0.0, 0.0);
    if (i == j) A[i][i].y = 0.0;
  }
  __syncthreads();
  const int ne = (n + 1) & ~1, half = ne / 2;
  __shared__ double redOff[32], redDg[32];
  double prevOffs = -1.0;
  for (int sweep = 0; sweep < 40 && n > 1; sweep++) {
    {  // off-diagonal and diagonal mass: per-thread strided sums, warp trees, warps in order
      double off = 0.0, dg = 0.0;
      for (int e = tid; e < n * n; e += blockDim.x) {
        const int i = e % n, j = e / n;
        const double a2 = A[i][j].x * A[i][j].x + A[i][j].y * A[i][j].y;
        if (i == j) dg += a2;
        else off += a2;
      }
      for (int o = 16; o > 0; o >>= 1) {
        off += __shfl_xor_sync(0xffffffffu, off, o);
        dg += __shfl_xor_sync(0xffffffffu, dg, o);
      }
      if ((tid & 31) == 0) {
        redOff[tid >> 5] = off;
        redDg[tid >> 5] = dg;
      }
      __syncthreads();
      if (tid == 0) {
        double o2 = 0.0, d2 = 0.0;
        for (int w = 0; w < (int)(blockDim.x + 31) / 32; w++) {
          o2 += redOff[w];
          d2 += redDg[w];
        }
        offs = o2;
        diags = d2;
      }
      __syncthreads();
    }
    // converged, or at the rounding floor (below 1e-24 of the mass and no longer halving)
    if (offs <= 1e-30 * (diags + offs) || offs == 0.0) break;
    if (offs <= 1e-24 * (diags + offs) && prevOffs >= 0.0 && offs > 0.5 * prevOffs) break;
    prevOffs = offs;
    for (int r = 0; r < ne - 1; r++) {
      if (tid < half) {
        const int k = tid;
        auto pos = [&](int i) { return i == 0 ? 0 : ((i - 1 + r) % (ne - 1)) + 1; };
        int p = pos(k), q = pos(ne - 1 - k);
        if (p > q) {
          const int t = p;
          p = q;
          q = t;
        }
        rp[k] = p;
        rq[k] = q;
        double c = 1.0, s = 0.0;
        z_t ph = zmk(1.0, 0.0);
        if (q < n) {
          const z_t b = A[p][q];
          const double g = sqrt(b.x * b.x + b.y * b.y);
          if (g != 0.0) {
            ph = zmk(b.x / g, b.y / g);
            const double tau = (A[q][q].x - A[p][p].x) / (2.0 * g);
            const double t = (tau >= 0 ? 1.0 : -1.0) / (fabs(tau) + sqrt(1.0 + tau * tau));
            c = 1.0 / sqrt(1.0 + t * t);
            s = t * c;
          }
        } else {
          rq[k] = -1;
        }
        rc[k] = c;
        rs[k] = s;
        rph[k] = ph;
      }
      __syncthreads();
      for (int e = tid; e < n * half; e += blockDim.x) {
        const int i = e % n, k = e / n;
        const int p = rp[k], q = rq[k];
        if (q < 0 || rs[k] == 0.0) continue;
        const double c = rc[k], s = rs[k];
        const z_t phc = zconj(rph[k]);
        const z_t akp = A[i][p], akq = A[i][q];
        A[i][p] = zsub(zscale(akp, c), zscale(zmul(akq, phc), s));
        A[i][q] = zadd(zscale(akp, s), zscale(zmul(akq, phc), c));
        const z_t vkp = V[i][p], vkq = V[i][q];
        V[i][p] = zsub(zscale(vkp, c), zscale(zmul(vkq, phc), s));
        V[i][q] = zadd(zscale(vkp, s), zscale(zmul(vkq, phc), c));
      }
      __syncthreads();
      for (int e = tid; e < n * half; e += blockDim.x) {
        const int i = e % n, k = e / n;
        const int p = rp[k], q = rq[k];
        if (q < 0 || rs[k] == 0.0) continue;
        const double c = rc[k], s = rs[k];
        const z_t ph = rph[k];
        const z_t apk = A[p][i], aqk = A[q][i];
        A[p][i] = zsub(zscale(apk, c), zscale(zmul(ph, aqk), s));
        A[q][i] = zadd(zscale(apk, s), zscale(zmul(ph, aqk), c));
      }
      __syncthreads();
      if (tid < half) {
        const int p = rp[tid], q = rq[tid];
        if (q >= 0 && rs[tid] != 0.0) {
          A[p][q] = zmk(0.0, 0.0);
          A[q][p] = zmk(0.0, 0.0);
          A[p][p].y = 0.0;
          A[q][q].y = 0.0;
        }
      }
      __syncthreads();
    }
  }
  for (int e = tid; e < n; e += blockDim.x) ev[e] = A[e][e].x;
  __syncthreads();
}

// rho1 = U diag(occ) U^H, f = occ / (occ^2 + eps), Mreg = U diag(f) U^H
__global__ void k_mc_rdm_inverse(z_t* __restrict__ Mreg, z_t* __restrict__ Uo, double* __restrict__ occ,
                                 double* __restrict__ f, const z_t* __restrict__ r1, int M, double eps) {
  __shared__ z_t A[JM][JM + 1], V[JM][JM + 1];
  __shared__ double ev[JM];
  for (int e = threadIdx.x; e < M * M; e += blockDim.x) A[e % M][e / M] = r1[e];
  __syncthreads();
  herm_jacobi(A, V, M, ev);
  for (int e = threadIdx.x; e < M; e += blockDim.x) {
    occ[e] = ev[e];
    f[e] = ev[e] / (ev[e] * ev[e] + eps);
  }
  for (int e = threadIdx.x; e < M * M; e += blockDim.x) Uo[e] = V[e % M][e / M];
  __syncthreads();
  for (int e = threadIdx.x; e < M * M; e += blockDim.x) {
    const int k = e % M, j = e / M;
    z_t s = zmk(0.0, 0.0);
    for (int n = 0; n < M; n++) zfma(s, zscale(V[k][n], ev[n] / (ev[n] * ev[n] + eps)), zconj(V[j][n]));
    Mreg[e] = s;
  }
}

// Daleckii-Krein: r1bar = U (F o (U^H Mbar U)) U^H, F the divided differences of f
__global__ void k_mc_dk(z_t* __restrict__ r1bar, const z_t* __restrict__ Mbar, const z_t* __restrict__ U,
                        const double* __restrict__ occ, const double* __restrict__ f, int M, double eps) {
  __shared__ z_t B[JM][JM + 1], T[JM][JM + 1];
  for (int e = threadIdx.x; e < M * M; e += blockDim.x) {
    const int i = e % M, j = e / M;
    z_t s = zmk(0.0, 0.0);  // (Mbar U)[i, j]
    for (int k = 0; k < M; k++) zfma(s, Mbar[i + M * k], U[k + M * j]);
    T[i][j] = s;
  }
  __syncthreads();
  for (int e = threadIdx.x; e < M * M; e += blockDim.x) {
    const int i = e % M, j = e / M;
    z_t s = zmk(0.0, 0.0);  // (U^H Mbar U)[i, j]
    for (int k = 0; k < M; k++) zcfma(s, U[k + M * i], T[k][j]);
    const double dn = occ[i] - occ[j];
    double F;
    if (fabs(dn) > 1e-13 * fmax(1.0, fabs(occ[i]))) F = (f[i] - f[j]) / dn;
    else {
      const double fi = (eps - occ[i] * occ[i]) / ((occ[i] * occ[i] + eps) * (occ[i] * occ[i] + eps));
      const double fj = (eps - occ[j] * occ[j]) / ((occ[j] * occ[j] + eps) * (occ[j] * occ[j] + eps));
      F = 0.5 * (fi + fj);
    }
    B[i][j] = zscale(s, F);
  }
  __syncthreads();
  for (int e = threadIdx.x; e < M * M; e += blockDim.x) {
    const int i = e % M, j = e / M;
    z_t s = zmk(0.0, 0.0);  // (U B)[i, j]
    for (int k = 0; k < M; k++) zfma(s, U[i + M * k], B[k][j]);
    T[i][j] = s;
  }
  __syncthreads();
  for (int e = threadIdx.x; e < M * M; e += blockDim.x) {
    const int i = e % M, j = e / M;
    z_t s = zmk(0.0, 0.0);  // (U B U^H)[i, j]
    for (int k = 0; k < M; k++) zfma(s, T[i][k], zconj(U[j + M * k]));
    r1bar[e] = s;
  }
}

// y = exp(-i tau T) e1 for the K x K tridiagonal T (al, be); lam, Q kept for the adjoint
__global__ void k_mc_expsub(z_t* __restrict__ y, double* __restrict__ lam, double* __restrict__ Q,
                            const double* __restrict__ al, const double* __restrict__ be, int K, double tau) {
  __shared__ z_t A[JM][JM + 1], V[JM][JM + 1];
  __shared__ double ev[JM];
  for (int e = threadIdx.x; e < K * K; e += blockDim.x) {
    const int i = e % K, j = e / K;
    double v = i == j ? al[i] : (j == i + 1 ? be[i] : (i == j + 1 ? be[j] : 0.0));
    A[i][j] = zmk(v, 0.0);
  }
  __syncthreads();
  herm_jacobi(A, V, K, ev);
  for (int e = threadIdx.x; e < K * K; e += blockDim.x) Q[e] = V[e % K][e / K].x;
  for (int e = threadIdx.x; e < K; e += blockDim.x) lam[e] = ev[e];
  __syncthreads();
  for (int i = threadIdx.x; i < K; i += blockDim.x) {
    z_t s = zmk(0.0, 0.0);
    for (int j = 0; j < K; j++) {
      double sn, cs;
      sincos(-tau * ev[j], &sn, &cs);
      s = zadd(s, zscale(zmk(cs, sn), V[i][j].x * V[0][j].x));
    }
    y[i] = s;
  }
}

// Frechet adjoint of y = exp(-i tau T) e1: abar, bbar (+=) from ybar
__global__ void k_mc_expsub_vjp(double* __restrict__ abar, double* __restrict__ bbar, const z_t* __restrict__ ybar,
                                const double* __restrict__ lam, const double* __restrict__ Q, int K, double tau) {
  __shared__ z_t a[JM];
  __shared__ double Bb[JM][JM + 1], Tq[JM][JM + 1];
  for (int i = threadIdx.x; i < K; i += blockDim.x) {
    z_t s = zmk(0.0, 0.0);
    for (int k = 0; k < K; k++) s = zadd(s, zscale(ybar[k], Q[k + K * i]));
    a[i] = s;
  }
  __syncthreads();
  for (int e = threadIdx.x; e < K * K; e += blockDim.x) {
    const int i = e % K, j = e / K;
    double si, ci, sj, cj;
    sincos(-tau * lam[i], &si, &ci);
    sincos(-tau * lam[j], &sj, &cj);
    z_t F;
    const double dl = lam[i] - lam[j];
    if (fabs(dl) > 1e-12 * fmax(1.0, fabs(lam[i]))) F = zscale(zmk(ci - cj, si - sj), 1.0 / dl);
    else F = zmul(zmk(0.0, -tau), zmk(ci, si));
    const z_t t = zmul(zconj(a[i]), F);
    Bb[i][j] = t.x * Q[0 + K * j];
  }
  __syncthreads();
  for (int e = threadIdx.x; e < K * K; e += blockDim.x) {
    const int i = e % K, j = e / K;
    double s = 0.0;  // (Q Bb)[i, j]
    for (int k = 0; k < K; k++) s += Q[i + K * k] * Bb[k][j];
    Tq[i][j] = s;
  }
  __syncthreads();
  for (int j = threadIdx.x; j < K; j += blockDim.x) {
    auto Tbar = [&](int r, int c) {
      double s = 0.0;  // (Q Bb Q^T)[r, c]
      for (int k = 0; k < K; k++) s += Tq[r][k] * Q[c + K * k];
      return s;
    };
    abar[j] += Tbar(j, j);
    if (j < K - 1) bbar[j] += Tbar(j, j + 1) + Tbar(j + 1, j);
  }
}

// ---------------------------------------------------------------------------
// NonLin pieces (dense two-electron form)
// ---------------------------------------------------------------------------

// Sp[x, b + M d] = conj(phi_xb) phi_xd w_x
__global__ void k_mc_pairs(z_t* __restrict__ Sp, const z_t* __restrict__ phi, const double* __restrict__ w, int nG,
                           int M) {
  MC_LOOP(e, (size_t)nG * M * M) {
    const int x = (int)(e % nG), bd = (int)(e / nG), b = bd % M, d = bd / M;
    Sp[e] = zscale(zcmul(phi[x + (size_t)nG * b], phi[x + (size_t)nG * d]), w[x]);
  }
}

// dC0 = h1^T C + C h1 + sum_ab g(a, b; c, d) C[a, b],  g2[(a + M c) + Q (b + M d)]
__global__ void k_mc_dc0(z_t* __restrict__ dC0, const z_t* __restrict__ h1, const z_t* __restrict__ C,
                         const z_t* __restrict__ g2, int M) {
  const int Q = M * M;
  MC_LOOP(e, Q) {
    const int c = (int)(e % M), d = (int)(e / M);
    z_t s = zmk(0.0, 0.0);
    for (int a = 0; a < M; a++) zfma(s, h1[a + M * c], C[a + M * d]);
    for (int b = 0; b < M; b++) zfma(s, C[c + M * b], h1[b + M * d]);
    for (int b = 0; b < M; b++)
      for (int a = 0; a < M; a++) zfma(s, g2[(a + M * c) + (size_t)Q * (b + M * d)], C[a + M * b]);
    dC0[e] = s;
  }
}

// rho1 = conj(C) C^T + C^H C;  rho2[a + M b + Q c + Q M d] = C_cd conj(C_ab) + C_dc conj(C_ba)
__global__ void k_mc_rdms(z_t* __restrict__ r1, z_t* __restrict__ r2, const z_t* __restrict__ C, int M) {
  const int Q = M * M;
  MC_LOOP(e, (size_t)Q * Q) {
    const int a = (int)(e % M), b = (int)(e / M % M), c = (int)(e / Q % M), d = (int)(e / ((size_t)Q * M));
    r2[e] = zadd(zmul(C[c + M * d], zconj(C[a + M * b])), zmul(C[d + M * c], zconj(C[b + M * a])));
    if (e < (size_t)Q) {
      const int i = (int)(e % M), k = (int)(e / M);
      z_t s = zmk(0.0, 0.0);
      for (int j = 0; j < M; j++) {
        zfma(s, zconj(C[i + M * j]), C[k + M * j]);
        zcfma(s, C[j + M * i], C[j + M * k]);
      }
      r1[e] = s;
    }
  }
}

// R[a, b, j, d] = sum_k r2[a, b, k, d] Mreg[k, j]
__global__ void k_mc_build_R(z_t* __restrict__ R, const z_t* __restrict__ r2, const z_t* __restrict__ Mreg, int M) {
  const int Q = M * M;
  MC_LOOP(e, (size_t)Q * Q) {
    const int ab = (int)(e % Q), j = (int)(e / Q % M), d = (int)(e / ((size_t)Q * M));
    z_t s = zmk(0.0, 0.0);
    for (int k = 0; k < M; k++) zfma(s, r2[ab + (size_t)Q * (k + M * d)], Mreg[k + M * j]);
    R[e] = s;
  }
}

// dphi0[x, j] = sum_{a, k, l} Wp[x, l + M k] phi[x, a] R[a, k, j, l]
// the l-th term of k_mc_meanfield's sum, Y[x, j + M l], one thread each
// (nG M^2 threads; the sum over l follows in k_mc_meanfield_sum in order)
__global__ void k_mc_meanfield(z_t* __restrict__ Y, const z_t* __restrict__ Wp, const z_t* __restrict__ phi,
                               const z_t* __restrict__ R, int nG, int M) {
  const int Q = M * M;
  MC_LOOP(e, (size_t)nG * Q) {
    const int x = (int)(e % nG), jl = (int)(e / nG), j = jl % M, l = jl / M;
    z_t s = zmk(0.0, 0.0);
    for (int k = 0; k < M; k++) {
      z_t t = zmk(0.0, 0.0);
      for (int a = 0; a < M; a++) zfma(t, phi[x + (size_t)nG * a], R[a + M * k + (size_t)Q * (j + M * l)]);
      zfma(s, Wp[x + (size_t)nG * (l + M * k)], t);
    }
    Y[e] = s;
  }
}

// dphi[x, j] = sum_l Y[x, j + M l] (fixed order)
__global__ void k_mc_meanfield_sum(z_t* __restrict__ dphi, const z_t* __restrict__ Y, int nG, int M) {
  MC_LOOP(e, (size_t)nG * M) {
    const int x = (int)(e % nG), j = (int)(e / nG);
    z_t s = zmk(0.0, 0.0);
    for (int l = 0; l < M; l++) s = zadd(s, Y[x + (size_t)nG * (j + M * l)]);
    dphi[e] = s;
  }
}

// out = -i [dC0 - s c ; dphi] (dphi already projected), s = *sc
__global__ void k_mc_nonlin_out(z_t* __restrict__ out, const z_t* __restrict__ dC0, const z_t* __restrict__ c,
                                const z_t* __restrict__ sc, const z_t* __restrict__ dphi, int Q, int nGM) {
  const z_t s = *sc;
  MC_LOOP(e, (size_t)Q + nGM) {
    z_t v = (int)e < Q ? zsub(dC0[e], zmul(s, c[e])) : dphi[e - Q];
    out[e] = zmi(v);
  }
}

// ---- NonLin VJP pieces

// ubar = i obar; C part: dC0bar = ubar_C - c (c^H ubar_C), Cbar = -conj(s) ubar_C - conj(c^H ubar_C) dC0
__global__ void k_mc_proj_c_vjp(z_t* __restrict__ dC0bar, z_t* __restrict__ Cbar, const z_t* __restrict__ obar,
                                const z_t* __restrict__ c, const z_t* __restrict__ dC0, const z_t* __restrict__ sc,
                                const z_t* __restrict__ t1, int Q) {
  const z_t s = *sc, t = *t1;  // t1 = c^H (i obar_C)
  MC_LOOP(e, Q) {
    const z_t u = zpi(obar[e]);
    dC0bar[e] = zsub(u, zmul(c[e], t));
    Cbar[e] = zsub(zmul(zscale(zconj(s), -1.0), u), zmul(zconj(t), dC0[e]));
  }
}

// ubar_phi = i obar_phi (copy into u)
__global__ void k_mc_times_i(z_t* __restrict__ u, const z_t* __restrict__ obar, int n) {
  MC_LOOP(e, n) u[e] = zpi(obar[e]);
}

// out = w o a (row weights on nG x M)
__global__ void k_mc_wrows(z_t* __restrict__ out, const z_t* __restrict__ a, const double* __restrict__ w, int nG,
                           int M) {
  MC_LOOP(e, (size_t)nG * M) out[e] = zscale(a[e], w[e % nG]);
}

// Cbar += sum_cd conj(g(a, b; c, d)) dC0bar[c, d];  g2bar[(a + M c) + Q (b + M d)] = dC0bar[c, d] conj(C[a, b])
__global__ void k_mc_g_vjp(z_t* __restrict__ Cbar, z_t* __restrict__ g2bar, const z_t* __restrict__ g2,
                           const z_t* __restrict__ dC0bar, const z_t* __restrict__ C, int M) {
  const int Q = M * M;
  MC_LOOP(e, (size_t)Q * Q) {
    const int ac = (int)(e % Q), bd = (int)(e / Q);
    const int a = ac % M, c = ac / M, b = bd % M, d = bd / M;
    g2bar[e] = zmul(dC0bar[c + M * d], zconj(C[a + M * b]));
    if (e < (size_t)Q) {
      const int aa = (int)(e % M), bb = (int)(e / M);
      z_t s = zmk(0.0, 0.0);
      for (int dd = 0; dd < M; dd++)
        for (int cc = 0; cc < M; cc++) zcfma(s, g2[(aa + M * cc) + (size_t)Q * (bb + M * dd)], dC0bar[cc + M * dd]);
      Cbar[e] = zadd(Cbar[e], s);
    }
  }
}

// phibar[x, i] += w_x ( T1[x, i] + T2[x, i] )
__global__ void k_mc_add_w2(z_t* __restrict__ phibar, const z_t* __restrict__ T1, const z_t* __restrict__ T2,
                            const double* __restrict__ w, int nG, int M) {
  MC_LOOP(e, (size_t)nG * M) phibar[e] = zadd(phibar[e], zscale(zadd(T1[e], T2[e]), w[e % nG]));
}

// phibar[x, a] += w_x sum_c phi[x, c] Q1[x, a + M c]  (which = 0)
// phibar[x, c] += w_x sum_a phi[x, a] Q2[x, a + M c]  (which = 1)
__global__ void k_mc_phi_from_q(z_t* __restrict__ phibar, const z_t* __restrict__ Qm, const z_t* __restrict__ phi,
                                const double* __restrict__ w, int nG, int M, int which) {
  MC_LOOP(e, (size_t)nG * M) {
    const int x = (int)(e % nG), i = (int)(e / nG);
    z_t s = zmk(0.0, 0.0);
    for (int k = 0; k < M; k++) {
      const int col = which == 0 ? (i + M * k) : (k + M * i);
      zfma(s, phi[x + (size_t)nG * k], Qm[x + (size_t)nG * col]);
    }
    phibar[e] = zadd(phibar[e], zscale(s, w[x]));
  }
}

// Rbar[a, k, j, l] = sum_x conj(Wp[x, l + M k] phi[x, a]) dphi0bar[x, j]
__global__ void k_mc_Rbar(z_t* __restrict__ Rbar, const z_t* __restrict__ Wp, const z_t* __restrict__ phi,
                          const z_t* __restrict__ dphibar, int nG, int M) {
  const int Q = M * M;
  MC_LOOP(e, (size_t)Q * Q) {
    const int a = (int)(e % M), k = (int)(e / M % M), j = (int)(e / Q % M), l = (int)(e / ((size_t)Q * M));
    const z_t* wp = Wp + (size_t)nG * (l + M * k);
    const z_t* ph = phi + (size_t)nG * a;
    const z_t* db = dphibar + (size_t)nG * j;
    z_t s = zmk(0.0, 0.0);
    for (int x = 0; x < nG; x++) zcfma(s, zmul(wp[x], ph[x]), db[x]);
    Rbar[e] = s;
  }
}

// Wpbar[x, l + M k] += sum_{a, j} conj(phi[x, a] R[a, k, j, l]) dphi0bar[x, j]
// phibar[x, a] += sum_{l, k, j} conj(Wp[x, l + M k] R[a, k, j, l]) dphi0bar[x, j]
__global__ void k_mc_mf_vjp(z_t* __restrict__ Wpbar, z_t* __restrict__ phibar, const z_t* __restrict__ Wp,
                            const z_t* __restrict__ phi, const z_t* __restrict__ R, const z_t* __restrict__ dphibar,
                            int nG, int M) {
  const int Q = M * M;
  MC_LOOP(e, (size_t)nG * Q) {
    const int x = (int)(e % nG), lk = (int)(e / nG), l = lk % M, k = lk / M;
    z_t s = zmk(0.0, 0.0);
    for (int j = 0; j < M; j++) {
      const z_t db = dphibar[x + (size_t)nG * j];
      for (int a = 0; a < M; a++) zcfma(s, zmul(phi[x + (size_t)nG * a], R[a + M * k + (size_t)Q * (j + M * l)]), db);
    }
    Wpbar[e] = zadd(Wpbar[e], s);
    if (lk < M) {
      const int a = lk;
      z_t t = zmk(0.0, 0.0);
      for (int j = 0; j < M; j++) {
        const z_t db = dphibar[x + (size_t)nG * j];
        for (int kk = 0; kk < M; kk++)
          for (int ll = 0; ll < M; ll++)
            zcfma(t, zmul(Wp[x + (size_t)nG * (ll + M * kk)], R[a + M * kk + (size_t)Q * (j + M * ll)]), db);
      }
      phibar[x + (size_t)nG * a] = zadd(phibar[x + (size_t)nG * a], t);
    }
  }
}

// r2bar[a, b, k, d] = sum_j Rbar[a, b, j, d] conj(Mreg[k, j]);  Mbar[k, j] = sum_abd conj(r2[a, b, k, d]) Rbar[a, b, j, d]
__global__ void k_mc_R_vjp(z_t* __restrict__ r2bar, z_t* __restrict__ Mbar, const z_t* __restrict__ Rbar,
                           const z_t* __restrict__ Mreg, const z_t* __restrict__ r2, int M) {
  const int Q = M * M;
  MC_LOOP(e, (size_t)Q * Q) {
    const int ab = (int)(e % Q), k = (int)(e / Q % M), d = (int)(e / ((size_t)Q * M));
    z_t s = zmk(0.0, 0.0);
    for (int j = 0; j < M; j++) zfma(s, Rbar[ab + (size_t)Q * (j + M * d)], zconj(Mreg[k + M * j]));
    r2bar[e] = s;
    if (e < (size_t)Q) {
      const int kk = (int)(e % M), j = (int)(e / M);
      z_t t = zmk(0.0, 0.0);
      for (int dd = 0; dd < M; dd++)
        for (int q = 0; q < Q; q++) zcfma(t, r2[q + (size_t)Q * (kk + M * dd)], Rbar[q + (size_t)Q * (j + M * dd)]);
      Mbar[e] = t;
    }
  }
}

// Cbar += r1bar^T C + conj(r1bar) C + C r1bar + C r1bar^H  +  the rho2 terms
__global__ void k_mc_rdm_vjp(z_t* __restrict__ Cbar, const z_t* __restrict__ r1bar, const z_t* __restrict__ r2bar,
                             const z_t* __restrict__ C, int M) {
  const int Q = M * M;
  MC_LOOP(e, Q) {
    const int p = (int)(e % M), q = (int)(e / M);
    z_t s = zmk(0.0, 0.0);
    for (int k = 0; k < M; k++) {
      zfma(s, r1bar[k + M * p], C[k + M * q]);           // (r1bar^T C)[p, q]
      zfma(s, zconj(r1bar[p + M * k]), C[k + M * q]);    // (conj(r1bar) C)[p, q]
      zfma(s, C[p + M * k], r1bar[k + M * q]);           // (C r1bar)[p, q]
      zfma(s, C[p + M * k], zconj(r1bar[q + M * k]));    // (C r1bar^H)[p, q]
    }
    for (int b = 0; b < M; b++)
      for (int a = 0; a < M; a++) {
        zfma(s, r2bar[a + M * b + (size_t)Q * (p + M * q)], C[a + M * b]);
        zcfma(s, r2bar[p + M * q + (size_t)Q * (a + M * b)], C[a + M * b]);
        zfma(s, r2bar[a + M * b + (size_t)Q * (q + M * p)], C[b + M * a]);
        zcfma(s, r2bar[q + M * p + (size_t)Q * (a + M * b)], C[b + M * a]);
      }
    Cbar[e] = zadd(Cbar[e], s);
  }
}

// phibar[y, m] += w_y ( sum_b Spbar[y, b + M m] phi[y, b] + sum_d conj(Spbar[y, m + M d]) phi[y, d] )
__global__ void k_mc_pairs_vjp(z_t* __restrict__ phibar, const z_t* __restrict__ Spbar, const z_t* __restrict__ phi,
                               const double* __restrict__ w, int nG, int M) {
  MC_LOOP(e, (size_t)nG * M) {
    const int y = (int)(e % nG), m = (int)(e / nG);
    z_t s = zmk(0.0, 0.0);
    for (int b = 0; b < M; b++) {
      zfma(s, Spbar[y + (size_t)nG * (b + M * m)], phi[y + (size_t)nG * b]);
      zfma(s, zconj(Spbar[y + (size_t)nG * (m + M * b)]), phi[y + (size_t)nG * b]);
    }
    phibar[e] = zadd(phibar[e], zscale(s, w[y]));
  }
}

// dst += [Cbar ; phibar]
__global__ void k_mc_acc_state(z_t* __restrict__ dst, const z_t* __restrict__ Cbar, const z_t* __restrict__ phibar,
                               int Q, int nGM) {
  MC_LOOP(e, (size_t)Q + nGM) dst[e] = zadd(dst[e], (int)e < Q ? Cbar[e] : phibar[e - Q]);
}

// grad[n] += Re(*dot) * mul (one thread)
__global__ void k_mc_grad_add(double* __restrict__ grad, int n, const z_t* __restrict__ dot, double mul) {
  if (threadIdx.x == 0 && blockIdx.x == 0) grad[n] += dot->x * mul;
}

// ---- Lanczos scalar helpers (one thread)

// n0 = sqrt(Re <s,s>_m) into ls[0]; v1 = s / n0 done by k_mc_scale_inv
__global__ void k_mc_set_sqrt(double* __restrict__ dst, const z_t* __restrict__ dot) {
  if (threadIdx.x == 0 && blockIdx.x == 0) *dst = sqrt(dot->x);
}
__global__ void k_mc_set_re(double* __restrict__ dst, const z_t* __restrict__ dot) {
  if (threadIdx.x == 0 && blockIdx.x == 0) *dst = dot->x;
}
// y = x / *s
__global__ void k_mc_scale_inv(z_t* __restrict__ y, const z_t* __restrict__ x, const double* __restrict__ s, int n) {
  const double inv = 1.0 / *s;
  MC_LOOP(e, n) y[e] = zscale(x[e], inv);
}
// y -= (*s) x   (real device scalar)
__global__ void k_mc_sub_real(z_t* __restrict__ y, const z_t* __restrict__ x, const double* __restrict__ s, int n) {
  const double a = *s;
  MC_LOOP(e, n) {
    y[e].x -= a * x[e].x;
    y[e].y -= a * x[e].y;
  }
}
// w -= sum_k dots[k] V_k (classical Gram-Schmidt update against nv basis vectors)
__global__ void k_mc_cgs(z_t* __restrict__ w, const z_t* __restrict__ V, const z_t* __restrict__ dots, int nv, int nS) {
  MC_LOOP(e, nS) {
    z_t s = w[e];
    for (int k = 0; k < nv; k++) {
      const z_t d = dots[k], v = V[(size_t)nS * k + e];
      s.x -= d.x * v.x - d.y * v.y;
      s.y -= d.x * v.y + d.y * v.x;
    }
    w[e] = s;
  }
}
// dots[k] = <V_k, w>_m for k < nv: one block per k
__global__ void __launch_bounds__(MC_RED) k_mc_mdots(z_t* __restrict__ dots, const z_t* __restrict__ V,
                                                     const z_t* __restrict__ w, const double* __restrict__ m, int nS) {
  __shared__ double sx[MC_RED], sy[MC_RED];
  const z_t* v = V + (size_t)nS * blockIdx.x;
  z_t s = zmk(0.0, 0.0);
  for (int i = threadIdx.x; i < nS; i += MC_RED) s = zadd(s, zscale(zcmul(v[i], w[i]), m ? m[i] : 1.0));
  sx[threadIdx.x] = s.x;
  sy[threadIdx.x] = s.y;
  __syncthreads();
  for (int o = MC_RED / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) {
      sx[threadIdx.x] += sx[threadIdx.x + o];
      sy[threadIdx.x] += sy[threadIdx.x + o];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) dots[blockIdx.x] = zmk(sx[0], sy[0]);
}
// out = n0 sum_j y_j V_j
__global__ void k_mc_combine(z_t* __restrict__ out, const z_t* __restrict__ V, const z_t* __restrict__ y,
                             const double* __restrict__ n0, int K, int nS) {
  const double s0 = *n0;
  MC_LOOP(e, nS) {
    z_t s = zmk(0.0, 0.0);
    for (int j = 0; j < K; j++) zfma(s, y[j], V[(size_t)nS * j + e]);
    out[e] = zscale(s, s0);
  }
}
// vbar_j = n0 conj(y_j) obar for all j
__global__ void k_mc_vbar_init(z_t* __restrict__ vbar, const z_t* __restrict__ obar, const z_t* __restrict__ y,
                               const double* __restrict__ n0, int K, int nS) {
  const double s0 = *n0;
  MC_LOOP(e, (size_t)nS * K) {
    const int j = (int)(e / nS);
    vbar[e] = zscale(zmul(zconj(y[j]), obar[e % nS]), s0);
  }
}
// ybar_j = n0 dots_j (dots_j = V_j^H obar) ; n0bar = Re sum_j conj(y_j) dots_j  -> written to ybar[K] .x
__global__ void k_mc_ybar(z_t* __restrict__ ybar, double* __restrict__ n0bar, const z_t* __restrict__ dots,
                          const z_t* __restrict__ y, const double* __restrict__ n0, int K) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    double nb = 0.0;
    for (int j = 0; j < K; j++) {
      ybar[j] = zscale(dots[j], *n0);
      const z_t t = zcmul(dots[j], y[j]);  // conj(V_j^H obar) y_j = (V y)^H obar part
      nb += t.x;
    }
    *n0bar = nb;
  }
}

// Reverse step j of the three-term recurrence, part 1:
//   r = H v_j - beta_{j-1} v_{j-1} - alpha_j v_j  (u = H v_j computed before)
__global__ void k_mc_rj(z_t* __restrict__ r, const z_t* __restrict__ u, const z_t* __restrict__ vj,
                        const z_t* __restrict__ vjm, const double* __restrict__ al, const double* __restrict__ be,
                        int j, int nS) {
  const double a = al[j], b = j > 0 ? be[j - 1] : 0.0;
  MC_LOOP(e, nS) {
    z_t v = zsub(u[e], zscale(vj[e], a));
    if (j > 0) v = zsub(v, zscale(vjm[e], b));
    r[e] = v;
  }
}
// part 2 (j < K-1): bbar_j += -Re<vbar_{j+1}, r> / beta_j^2;  rbar = vbar_{j+1} / beta_j + bbar_j m r / beta_j
__global__ void k_mc_rbar(z_t* __restrict__ rbar, const z_t* __restrict__ vbn, const z_t* __restrict__ r,
                          const double* __restrict__ m, double* __restrict__ bbar, const double* __restrict__ be,
                          const z_t* __restrict__ dot, int j, int nS, int last) {
  if (last) {
    MC_LOOP(e, nS) rbar[e] = zmk(0.0, 0.0);
    return;
  }
  const double b = be[j];
  const double bb = bbar[j] - dot->x / (b * b);
  MC_LOOP(e, nS) rbar[e] = zadd(zscale(vbn[e], 1.0 / b), zscale(r[e], bb * m[e] / b));
}
__global__ void k_mc_store_bbar(double* __restrict__ bbar, const double* __restrict__ be, const z_t* __restrict__ dot,
                                int j) {
  if (threadIdx.x == 0 && blockIdx.x == 0) bbar[j] -= dot->x / (be[j] * be[j]);
}
// part 3: abar_j += -Re<rbar, v_j>;  wbar = rbar + abar_j m v_j;  vbar_j += -alpha_j rbar + abar_j m (r + alpha_j v_j)
__global__ void k_mc_wbar(z_t* __restrict__ wbar, z_t* __restrict__ vbj, const z_t* __restrict__ rbar,
                          const z_t* __restrict__ r, const z_t* __restrict__ vj, const double* __restrict__ m,
                          const double* __restrict__ al, const double* __restrict__ abar, const z_t* __restrict__ dot,
                          int j, int nS) {
  const double a = al[j], ab = abar[j] - dot->x;
  MC_LOOP(e, nS) {
    wbar[e] = zadd(rbar[e], zscale(vj[e], ab * m[e]));
    const z_t w = zadd(r[e], zscale(vj[e], a));
    vbj[e] = zadd(zsub(vbj[e], zscale(rbar[e], a)), zscale(w, ab * m[e]));
  }
}
__global__ void k_mc_store_abar(double* __restrict__ abar, const z_t* __restrict__ dot, int j) {
  if (threadIdx.x == 0 && blockIdx.x == 0) abar[j] -= dot->x;
}
// bbar_{j-1} += -Re<wbar, v_{j-1}>
__global__ void k_mc_bbar_prev(double* __restrict__ bbar, const z_t* __restrict__ dot, int j) {
  if (threadIdx.x == 0 && blockIdx.x == 0) bbar[j - 1] -= dot->x;
}
// sbar += vbar_1 / n0 + n0bar' m s / n0,  n0bar' = n0bar - Re<vbar_1, s> / n0^2
__global__ void k_mc_sbar(z_t* __restrict__ sbar, const z_t* __restrict__ vb1, const z_t* __restrict__ s,
                          const double* __restrict__ m, const double* __restrict__ n0, const double* __restrict__ n0bar,
                          const z_t* __restrict__ dot, int nS, int accumulate) {
  const double n = *n0, nb = *n0bar - dot->x / (n * n);
  MC_LOOP(e, nS) {
    const z_t v = zadd(zscale(vb1[e], 1.0 / n), zscale(s[e], nb * m[e] / n));
    sbar[e] = accumulate ? zadd(sbar[e], v) : v;
  }
}

// ---- objective: O = sum conj(Cr) (S C S^T), S = phi_ref^H W phi
__global__ void k_mc_overlap(z_t* __restrict__ O, const z_t* __restrict__ Cr, const z_t* __restrict__ S,
                             const z_t* __restrict__ C, int M) {
  __shared__ double sx[MC_RED], sy[MC_RED];
  z_t s = zmk(0.0, 0.0);
  for (int e = threadIdx.x; e < M * M; e += MC_RED) {
    const int a = e % M, b = e / M;
    z_t t = zmk(0.0, 0.0);
    for (int d = 0; d < M; d++)
      for (int c = 0; c < M; c++) zfma(t, zmul(S[a + M * c], C[c + M * d]), S[b + M * d]);
    s = zadd(s, zcmul(Cr[e], t));
  }
  sx[threadIdx.x] = s.x;
  sy[threadIdx.x] = s.y;
  __syncthreads();
  for (int o = MC_RED / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) {
      sx[threadIdx.x] += sx[threadIdx.x + o];
      sy[threadIdx.x] += sy[threadIdx.x + o];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) *O = zmk(sx[0], sy[0]);
}
// Cbar = Ob S^H Cr conj(S);  Sbar = Ob conj(P S C^T + P^T S C), P = conj(Cr), Ob = -2 O
__global__ void k_mc_overlap_vjp(z_t* __restrict__ Cbar, z_t* __restrict__ Sbar, const z_t* __restrict__ Cr,
                                 const z_t* __restrict__ S, const z_t* __restrict__ C, const z_t* __restrict__ O, int M) {
  const z_t Ob = zscale(*O, -2.0);
  for (int e = threadIdx.x; e < M * M; e += blockDim.x) {
    const int p = e % M, q = e / M;
    z_t cb = zmk(0.0, 0.0), g = zmk(0.0, 0.0);
    for (int b = 0; b < M; b++)
      for (int a = 0; a < M; a++) {
        // (S^H Cr conj(S))[p, q] = sum_ab conj(S[a, p]) Cr[a, b] conj(S[b, q])
        zfma(cb, zconj(S[a + M * p]), zmul(Cr[a + M * b], zconj(S[b + M * q])));
        // (P S C^T)[p, q] = sum_ab conj(Cr[p, a]) S[a, b] C[q, b];  (P^T S C)[p, q] = sum_ab conj(Cr[a, p]) S[a, b] C[b, q]
        zfma(g, zconj(Cr[p + M * a]), zmul(S[a + M * b], C[q + M * b]));
        zfma(g, zconj(Cr[a + M * p]), zmul(S[a + M * b], C[b + M * q]));
      }
    Cbar[e] = zmul(Ob, cb);
    Sbar[e] = zmul(Ob, zconj(g));
  }
}
__global__ void k_mc_objective(double* __restrict__ J, const z_t* __restrict__ O) {
  if (threadIdx.x == 0 && blockIdx.x == 0) *J = 1.0 - (O->x * O->x + O->y * O->y);
}

}  // namespace

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------
struct McAdjoint {
  int nG = 0, M = 0, Q = 0, nS = 0, band = 0, K = 0, nT = 0, chk = 0;
  double dt = 0.0, eps = 1e-10;
  std::vector<double> field;
  // constants
  double *m = nullptr, *wx = nullptr, *grad = nullptr, *J = nullptr;
  // state vectors
  z_t *ref = nullptr, *cur = nullptr, *chkStates = nullptr, *seg = nullptr, *co = nullptr;
  z_t *sA = nullptr, *sB = nullptr, *lam = nullptr, *lamB = nullptr;
  z_t *stage[4] = {}, *kv[4] = {};
  // Lanczos
  z_t *V = nullptr, *w = nullptr, *r = nullptr, *u = nullptr, *vbar = nullptr, *rbar = nullptr, *wbar = nullptr, *y = nullptr,
      *ybar = nullptr, *dots = nullptr, *tmpS = nullptr;
  double *al = nullptr, *be = nullptr, *abar = nullptr, *bbar = nullptr, *lz = nullptr, *lamK = nullptr, *Qk = nullptr;
  // NonLin
  z_t *Aphi = nullptr, *wphi = nullptr, *h1 = nullptr, *Sp = nullptr, *Wp = nullptr, *g2 = nullptr, *dC0 = nullptr,
      *r1 = nullptr, *U = nullptr, *Mreg = nullptr, *r2 = nullptr, *R = nullptr, *dphi0 = nullptr, *dphi = nullptr,
      *Gp = nullptr, *sc = nullptr;
  double *occ = nullptr, *fv = nullptr;
  // NonLin VJP
  z_t *dC0bar = nullptr, *Cbar = nullptr, *ubar = nullptr, *dphi0bar = nullptr, *phibar = nullptr, *G1 = nullptr,
      *h1bar = nullptr, *X1 = nullptr, *T1 = nullptr, *T2 = nullptr, *AT2 = nullptr, *g2bar = nullptr, *Q1 = nullptr,
      *Wpbar = nullptr, *Spbar = nullptr, *Rbar = nullptr, *r2bar = nullptr, *Mbar = nullptr, *r1bar = nullptr,
      *wd = nullptr, *sbarTmp = nullptr, *Sov = nullptr, *Sbar = nullptr, *Ov = nullptr;
  std::vector<void*> allocs;
  bool ready = false;

  template <class T>
  T* alloc(size_t n) {
    void* p = nullptr;
    CODY_CUDA(cudaMalloc(&p, sizeof(T) * std::max<size_t>(n, 1)));
    CODY_CUDA(cudaMemset(p, 0, sizeof(T) * std::max<size_t>(n, 1)));
    allocs.push_back(p);
    return (T*)p;
  }
  ~McAdjoint() {
    for (void* p : allocs) cudaFree(p);
  }
};

namespace {

double field_at(const McAdjoint& A, double t, int* idx) {
  const int n = (int)std::floor(t / A.dt + 1e-9);
  *idx = n;
  return (n >= 0 && n < A.nT) ? A.field[n] : 0.0;
}

void mc_zgemm(cgpu_ctx* c, int M, int N, int K, z_t alpha, const z_t* A, int lda, int opA, const z_t* B, int ldb,
              int opB, const double* wk, z_t beta, z_t* C, int ldc) {
  // small outputs over a long K (the M x M and Q x Q products over the grid,
  // whose operands are K-contiguous): a warp per output; otherwise a thread
  if ((size_t)M * N <= 8192 && K >= 128)
    k_mc_zgemm_w<<<nblk((size_t)M * N * 32), MC_T, 0, c->stream>>>(M, N, K, alpha, A, lda, opA, B, ldb, opB, wk, beta,
                                                                     C, ldc);
  else
    k_mc_zgemm<<<nblk((size_t)M * N), MC_T, 0, c->stream>>>(M, N, K, alpha, A, lda, opA, B, ldb, opB, wk, beta, C,
                                                             ldc);
  CODY_LAUNCHED(c);
}

void mc_dot(cgpu_ctx* c, z_t* out, const z_t* a, const z_t* b, const double* w, int n) {
  k_mc_dot<<<1, MC_RED, 0, c->stream>>>(out, a, b, w, n);
  CODY_LAUNCHED(c);
}

void mc_apply_h(cgpu_ctx* c, McAdjoint& A, z_t* out, const z_t* in, double E, int offC, int trans) {
  k_mc_apply_h<<<nblk((size_t)offC + (size_t)A.nG * A.M), MC_T, 0, c->stream>>>(out, in, c->T_d, c->V0_d, c->x_d, E,
                                                                                  A.nG, A.band, A.M, offC, trans);
  CODY_LAUNCHED(c);
}

const z_t ONE = {1.0, 0.0}, ZERO = {0.0, 0.0}, MONE = {-1.0, 0.0};

// NonLin derivative of state s into out, with field E; leaves the intermediates in A
void nonlin_forward(cgpu_ctx* c, McAdjoint& A, const z_t* s, z_t* out, double E) {
  const int nG = A.nG, M = A.M, Q = A.Q;
  const z_t* C = s;
  const z_t* phi = s + Q;
  mc_apply_h(c, A, A.Aphi, phi, E, 0, 0);
  mc_zgemm(c, M, M, nG, ONE, phi, nG, 2, A.Aphi, nG, 0, c->w_d, ZERO, A.h1, M);
  k_mc_pairs<<<nblk((size_t)nG * Q), MC_T, 0, c->stream>>>(A.Sp, phi, c->w_d, nG, M);
  CODY_LAUNCHED(c);
  k_mc_vgemm<<<nblk((size_t)nG * Q * 32), MC_T, 0, c->stream>>>(nG, Q, c->Vint_d, A.Sp, A.Wp, 0);
  CODY_LAUNCHED(c);
  mc_zgemm(c, Q, Q, nG, ONE, A.Sp, nG, 1, A.Wp, nG, 0, nullptr, ZERO, A.g2, Q);
  k_mc_dc0<<<nblk(Q), MC_T, 0, c->stream>>>(A.dC0, A.h1, C, A.g2, M);
  CODY_LAUNCHED(c);
  k_mc_rdms<<<nblk((size_t)Q * Q), MC_T, 0, c->stream>>>(A.r1, A.r2, C, M);
  CODY_LAUNCHED(c);
  k_mc_rdm_inverse<<<1, 256, 0, c->stream>>>(A.Mreg, A.U, A.occ, A.fv, A.r1, M, A.eps);
  CODY_LAUNCHED(c);
  k_mc_build_R<<<nblk((size_t)Q * Q), MC_T, 0, c->stream>>>(A.R, A.r2, A.Mreg, M);
  CODY_LAUNCHED(c);
  k_mc_meanfield<<<nblk((size_t)nG * Q), MC_T, 0, c->stream>>>(A.Q1, A.Wp, phi, A.R, nG, M);  // Q1: scratch here
  CODY_LAUNCHED(c);
  k_mc_meanfield_sum<<<nblk((size_t)nG * M), MC_T, 0, c->stream>>>(A.dphi0, A.Q1, nG, M);
  CODY_LAUNCHED(c);
  mc_dot(c, A.sc, C, A.dC0, nullptr, Q);
  mc_zgemm(c, M, M, nG, ONE, phi, nG, 2, A.dphi0, nG, 0, c->w_d, ZERO, A.Gp, M);
  CODY_CUDA(cudaMemcpyAsync(A.dphi, A.dphi0, sizeof(z_t) * (size_t)nG * M, cudaMemcpyDeviceToDevice, c->stream));
  mc_zgemm(c, nG, M, M, MONE, phi, nG, 0, A.Gp, M, 0, nullptr, ONE, A.dphi, nG);
  k_mc_nonlin_out<<<nblk(A.nS), MC_T, 0, c->stream>>>(out, A.dC0, C, A.sc, A.dphi, Q, nG * M);
  CODY_LAUNCHED(c);
}

// sbar += (dNonLin/ds)^H obar at the state of the last nonlin_forward; grad[n] += dNonLin/dE part
void nonlin_vjp(cgpu_ctx* c, McAdjoint& A, const z_t* s, const z_t* obar, z_t* sbar, double E, int nIdx) {
  (void)E;
  const int nG = A.nG, M = A.M, Q = A.Q;
  const z_t* C = s;
  const z_t* phi = s + Q;
  // C projection (t1 = c^H (i obar_C) into ubar[0] scratch)
  k_mc_times_i<<<nblk(Q), MC_T, 0, c->stream>>>(A.ubar, obar, Q);
  CODY_LAUNCHED(c);
  mc_dot(c, A.dots, C, A.ubar, nullptr, Q);
  k_mc_proj_c_vjp<<<nblk(Q), MC_T, 0, c->stream>>>(A.dC0bar, A.Cbar, obar, C, A.dC0, A.sc, A.dots, Q);
  CODY_LAUNCHED(c);
  // orbital projection: u = i obar_phi; dphi0bar = u - (w phi)(phi^H u); phibar = -u Gp^H - (w dphi0)(phi^H u)^H
  k_mc_times_i<<<nblk((size_t)nG * M), MC_T, 0, c->stream>>>(A.ubar, obar + Q, nG * M);
  CODY_LAUNCHED(c);
  mc_zgemm(c, M, M, nG, ONE, phi, nG, 2, A.ubar, nG, 0, nullptr, ZERO, A.G1, M);
  k_mc_wrows<<<nblk((size_t)nG * M), MC_T, 0, c->stream>>>(A.wphi, phi, c->w_d, nG, M);
  CODY_LAUNCHED(c);
  k_mc_wrows<<<nblk((size_t)nG * M), MC_T, 0, c->stream>>>(A.wd, A.dphi0, c->w_d, nG, M);
  CODY_LAUNCHED(c);
  CODY_CUDA(cudaMemcpyAsync(A.dphi0bar, A.ubar, sizeof(z_t) * (size_t)nG * M, cudaMemcpyDeviceToDevice, c->stream));
  mc_zgemm(c, nG, M, M, MONE, A.wphi, nG, 0, A.G1, M, 0, nullptr, ONE, A.dphi0bar, nG);
  mc_zgemm(c, nG, M, M, MONE, A.ubar, nG, 0, A.Gp, M, 2, nullptr, ZERO, A.phibar, nG);
  mc_zgemm(c, nG, M, M, MONE, A.wd, nG, 0, A.G1, M, 2, nullptr, ONE, A.phibar, nG);
  // dC0 = h1^T C + C h1 + G
  mc_zgemm(c, M, M, M, ONE, A.h1, M, 3, A.dC0bar, M, 0, nullptr, ONE, A.Cbar, M);
  mc_zgemm(c, M, M, M, ONE, A.dC0bar, M, 0, A.h1, M, 2, nullptr, ONE, A.Cbar, M);
  mc_zgemm(c, M, M, M, ONE, C, M, 3, A.dC0bar, M, 1, nullptr, ZERO, A.h1bar, M);
  mc_zgemm(c, M, M, M, ONE, C, M, 2, A.dC0bar, M, 0, nullptr, ONE, A.h1bar, M);
  k_mc_g_vjp<<<nblk((size_t)Q * Q), MC_T, 0, c->stream>>>(A.Cbar, A.g2bar, A.g2, A.dC0bar, C, M);
  CODY_LAUNCHED(c);
  // field: grad[n] += Re sum conj(h1bar) X1, X1 = phi^H (w x) phi
  if (nIdx >= 0 && nIdx < A.nT) {
    mc_zgemm(c, M, M, nG, ONE, phi, nG, 2, phi, nG, 0, A.wx, ZERO, A.X1, M);
    mc_dot(c, A.dots, A.h1bar, A.X1, nullptr, Q);
    k_mc_grad_add<<<1, 32, 0, c->stream>>>(A.grad, nIdx, A.dots, 1.0);
    CODY_LAUNCHED(c);
  }
  // h1 = phi^H W A phi: phibar += w (Aphi h1bar^H + A (phi h1bar))
  mc_zgemm(c, nG, M, M, ONE, A.Aphi, nG, 0, A.h1bar, M, 2, nullptr, ZERO, A.T1, nG);
  mc_zgemm(c, nG, M, M, ONE, phi, nG, 0, A.h1bar, M, 0, nullptr, ZERO, A.T2, nG);
  mc_apply_h(c, A, A.AT2, A.T2, E, 0, 0);
  k_mc_add_w2<<<nblk((size_t)nG * M), MC_T, 0, c->stream>>>(A.phibar, A.T1, A.AT2, c->w_d, nG, M);
  CODY_LAUNCHED(c);
  // g = Sp^T Wp: phibar (bra and ket), Wpbar
  mc_zgemm(c, nG, Q, Q, ONE, A.Wp, nG, 0, A.g2bar, Q, 2, nullptr, ZERO, A.Q1, nG);
  k_mc_phi_from_q<<<nblk((size_t)nG * M), MC_T, 0, c->stream>>>(A.phibar, A.Q1, phi, c->w_d, nG, M, 0);
  CODY_LAUNCHED(c);
  mc_zgemm(c, nG, Q, Q, ONE, A.Wp, nG, 3, A.g2bar, Q, 1, nullptr, ZERO, A.Q1, nG);
  k_mc_phi_from_q<<<nblk((size_t)nG * M), MC_T, 0, c->stream>>>(A.phibar, A.Q1, phi, c->w_d, nG, M, 1);
  CODY_LAUNCHED(c);
  mc_zgemm(c, nG, Q, Q, ONE, A.Sp, nG, 3, A.g2bar, Q, 0, nullptr, ZERO, A.Wpbar, nG);
  // mean field
  k_mc_Rbar<<<nblk((size_t)Q * Q), MC_T, 0, c->stream>>>(A.Rbar, A.Wp, phi, A.dphi0bar, nG, M);
  CODY_LAUNCHED(c);
  k_mc_mf_vjp<<<nblk((size_t)nG * Q), MC_T, 0, c->stream>>>(A.Wpbar, A.phibar, A.Wp, phi, A.R, A.dphi0bar, nG, M);
  CODY_LAUNCHED(c);
  k_mc_R_vjp<<<nblk((size_t)Q * Q), MC_T, 0, c->stream>>>(A.r2bar, A.Mbar, A.Rbar, A.Mreg, A.r2, M);
  CODY_LAUNCHED(c);
  k_mc_dk<<<1, 256, 0, c->stream>>>(A.r1bar, A.Mbar, A.U, A.occ, A.fv, M, A.eps);
  CODY_LAUNCHED(c);
  k_mc_rdm_vjp<<<nblk(Q), MC_T, 0, c->stream>>>(A.Cbar, A.r1bar, A.r2bar, C, M);
  CODY_LAUNCHED(c);
  // pair potentials
  k_mc_vgemm<<<nblk((size_t)nG * Q * 32), MC_T, 0, c->stream>>>(nG, Q, c->Vint_d, A.Wpbar, A.Spbar, 0);
  CODY_LAUNCHED(c);
  k_mc_pairs_vjp<<<nblk((size_t)nG * M), MC_T, 0, c->stream>>>(A.phibar, A.Spbar, phi, c->w_d, nG, M);
  CODY_LAUNCHED(c);
  k_mc_acc_state<<<nblk(A.nS), MC_T, 0, c->stream>>>(sbar, A.Cbar, A.phibar, Q, nG * M);
  CODY_LAUNCHED(c);
}

// Fixed-order Lanczos exp(-i tau H(E)) s into out (the basis, alpha, beta, y kept)
void lanczos_forward(cgpu_ctx* c, McAdjoint& A, const z_t* s, z_t* out, double E, double tau) {
  const int nS = A.nS, K = A.K;
  mc_dot(c, A.dots, s, s, A.m, nS);
  k_mc_set_sqrt<<<1, 32, 0, c->stream>>>(A.lz, A.dots);
  CODY_LAUNCHED(c);
  k_mc_scale_inv<<<nblk(nS), MC_T, 0, c->stream>>>(A.V, s, A.lz, nS);
  CODY_LAUNCHED(c);
  for (int j = 0; j < K; j++) {
    z_t* vj = A.V + (size_t)nS * j;
    mc_apply_h(c, A, A.w, vj, E, A.Q, 0);
    if (j > 0) {
      k_mc_sub_real<<<nblk(nS), MC_T, 0, c->stream>>>(A.w, vj - nS, A.be + (j - 1), nS);
      CODY_LAUNCHED(c);
    }
    mc_dot(c, A.dots, vj, A.w, A.m, nS);
    k_mc_set_re<<<1, 32, 0, c->stream>>>(A.al + j, A.dots);
    CODY_LAUNCHED(c);
    k_mc_sub_real<<<nblk(nS), MC_T, 0, c->stream>>>(A.w, vj, A.al + j, nS);
    CODY_LAUNCHED(c);
    // full re-orthogonalisation (two classical Gram-Schmidt passes)
    for (int pass = 0; pass < 2; pass++) {
      k_mc_mdots<<<j + 1, MC_RED, 0, c->stream>>>(A.dots, A.V, A.w, A.m, nS);
      CODY_LAUNCHED(c);
      k_mc_cgs<<<nblk(nS), MC_T, 0, c->stream>>>(A.w, A.V, A.dots, j + 1, nS);
      CODY_LAUNCHED(c);
    }
    mc_dot(c, A.dots, A.w, A.w, A.m, nS);
    k_mc_set_sqrt<<<1, 32, 0, c->stream>>>(A.be + j, A.dots);
    CODY_LAUNCHED(c);
    if (j < K - 1) {
      k_mc_scale_inv<<<nblk(nS), MC_T, 0, c->stream>>>(A.V + (size_t)nS * (j + 1), A.w, A.be + j, nS);
      CODY_LAUNCHED(c);
    }
  }
  k_mc_expsub<<<1, 256, 0, c->stream>>>(A.y, A.lamK, A.Qk, A.al, A.be, K, tau);
  CODY_LAUNCHED(c);
  k_mc_combine<<<nblk(nS), MC_T, 0, c->stream>>>(out, A.V, A.y, A.lz, K, nS);
  CODY_LAUNCHED(c);
}

// sbar (=, or += with accumulate) = (d out / d s)^H obar of the last lanczos_forward(s); grad[nIdx] += d/dE part
void lanczos_vjp(cgpu_ctx* c, McAdjoint& A, const z_t* s, const z_t* obar, z_t* sbar, double E, double tau, int nIdx,
                 int accumulate) {
  const int nS = A.nS, K = A.K;
  double* n0bar = A.lz + 1;
  CODY_CUDA(cudaMemsetAsync(A.abar, 0, sizeof(double) * K, c->stream));
  CODY_CUDA(cudaMemsetAsync(A.bbar, 0, sizeof(double) * K, c->stream));
  k_mc_mdots<<<K, MC_RED, 0, c->stream>>>(A.dots, A.V, obar, nullptr, nS);
  CODY_LAUNCHED(c);
  k_mc_ybar<<<1, 32, 0, c->stream>>>(A.ybar, n0bar, A.dots, A.y, A.lz, K);
  CODY_LAUNCHED(c);
  k_mc_vbar_init<<<nblk((size_t)nS * K), MC_T, 0, c->stream>>>(A.vbar, obar, A.y, A.lz, K, nS);
  CODY_LAUNCHED(c);
  k_mc_expsub_vjp<<<1, 256, 0, c->stream>>>(A.abar, A.bbar, A.ybar, A.lamK, A.Qk, K, tau);
  CODY_LAUNCHED(c);
  z_t* d1 = A.dots + MC_MAXK;
  for (int j = K - 1; j >= 0; j--) {
    z_t* vj = A.V + (size_t)nS * j;
    z_t* vbj = A.vbar + (size_t)nS * j;
    mc_apply_h(c, A, A.u, vj, E, A.Q, 0);
    k_mc_rj<<<nblk(nS), MC_T, 0, c->stream>>>(A.r, A.u, vj, j > 0 ? vj - nS : vj, A.al, A.be, j, nS);
    CODY_LAUNCHED(c);
    const int last = j == K - 1;
    if (!last) mc_dot(c, d1, vbj + nS, A.r, nullptr, nS);
    k_mc_rbar<<<nblk(nS), MC_T, 0, c->stream>>>(A.rbar, last ? vbj : vbj + nS, A.r, A.m, A.bbar, A.be, d1, j, nS,
                                                 last);
    CODY_LAUNCHED(c);
    if (!last) {
      k_mc_store_bbar<<<1, 32, 0, c->stream>>>(A.bbar, A.be, d1, j);
      CODY_LAUNCHED(c);
    }
    mc_dot(c, d1, A.rbar, vj, nullptr, nS);
    k_mc_wbar<<<nblk(nS), MC_T, 0, c->stream>>>(A.wbar, vbj, A.rbar, A.r, vj, A.m, A.al, A.abar, d1, j, nS);
    CODY_LAUNCHED(c);
    k_mc_store_abar<<<1, 32, 0, c->stream>>>(A.abar, d1, j);
    CODY_LAUNCHED(c);
    // vbar_j += H^T wbar; grad += Re<wbar, X v_j>; bbar_{j-1} -= Re<wbar, v_{j-1}>; vbar_{j-1} -= beta_{j-1} wbar
    mc_apply_h(c, A, A.u, A.wbar, E, A.Q, 1);
    k_mc_axpby<<<nblk(nS), MC_T, 0, c->stream>>>(vbj, A.u, ONE, ONE, nS);
    CODY_LAUNCHED(c);
    if (nIdx >= 0 && nIdx < A.nT) {
      k_mc_xmul<<<nblk(nS), MC_T, 0, c->stream>>>(A.u, vj, c->x_d, A.nG, A.M, A.Q);
      CODY_LAUNCHED(c);
      mc_dot(c, d1, A.wbar, A.u, nullptr, nS);
      k_mc_grad_add<<<1, 32, 0, c->stream>>>(A.grad, nIdx, d1, 1.0);
      CODY_LAUNCHED(c);
    }
    if (j > 0) {
      mc_dot(c, d1, A.wbar, vj - nS, nullptr, nS);
      k_mc_bbar_prev<<<1, 32, 0, c->stream>>>(A.bbar, d1, j);
      CODY_LAUNCHED(c);
      k_mc_sub_real<<<nblk(nS), MC_T, 0, c->stream>>>(vbj - nS, A.wbar, A.be + (j - 1), nS);
      CODY_LAUNCHED(c);
    }
  }
  mc_dot(c, d1, A.vbar, s, nullptr, nS);
  k_mc_sbar<<<nblk(nS), MC_T, 0, c->stream>>>(sbar, A.vbar, s, A.m, A.lz, n0bar, d1, nS, accumulate);
  CODY_LAUNCHED(c);
}

// RK4 of the NonLin derivative from s (t0, dt) into out (out == nullptr: the
// stage states and derivatives only); stage states kept in A.stage, derivatives in A.kv
void rk4_forward(cgpu_ctx* c, McAdjoint& A, const z_t* s, z_t* out, double t0) {
  const int nS = A.nS;
  const double dt = A.dt;
  int n1, n2, n4;
  const double E1 = field_at(A, t0, &n1), E2 = field_at(A, t0 + 0.5 * dt, &n2), E4 = field_at(A, t0 + dt, &n4);
  const double Es[4] = {E1, E2, E2, E4};
  const double cs[3] = {0.5 * dt, 0.5 * dt, dt};
  CODY_CUDA(cudaMemcpyAsync(A.stage[0], s, sizeof(z_t) * nS, cudaMemcpyDeviceToDevice, c->stream));
  for (int i = 0; i < 4; i++) {
    nonlin_forward(c, A, A.stage[i], A.kv[i], Es[i]);
    if (i < 3) {
      CODY_CUDA(cudaMemcpyAsync(A.stage[i + 1], s, sizeof(z_t) * nS, cudaMemcpyDeviceToDevice, c->stream));
      k_mc_axpby<<<nblk(nS), MC_T, 0, c->stream>>>(A.stage[i + 1], A.kv[i], zmk(cs[i], 0.0), ONE, nS);
      CODY_LAUNCHED(c);
    }
  }
  if (!out) return;
  // out = s + dt/6 k1 + dt/3 k2 + dt/3 k3 + dt/6 k4 (the reference's accumulation order)
  if (out != s) CODY_CUDA(cudaMemcpyAsync(out, s, sizeof(z_t) * nS, cudaMemcpyDeviceToDevice, c->stream));
  CODY_CUDA(cudaMemcpyAsync(A.tmpS, A.kv[0], sizeof(z_t) * nS, cudaMemcpyDeviceToDevice, c->stream));
  k_mc_axpby<<<nblk(nS), MC_T, 0, c->stream>>>(A.tmpS, A.kv[0], ZERO, zmk(dt / 6.0, 0.0), nS);
  CODY_LAUNCHED(c);
  k_mc_axpby<<<nblk(nS), MC_T, 0, c->stream>>>(A.tmpS, A.kv[1], zmk(dt / 3.0, 0.0), ONE, nS);
  CODY_LAUNCHED(c);
  k_mc_axpby<<<nblk(nS), MC_T, 0, c->stream>>>(A.tmpS, A.kv[2], zmk(dt / 3.0, 0.0), ONE, nS);
  CODY_LAUNCHED(c);
  k_mc_axpby<<<nblk(nS), MC_T, 0, c->stream>>>(A.tmpS, A.kv[3], zmk(dt / 6.0, 0.0), ONE, nS);
  CODY_LAUNCHED(c);
  k_mc_axpby<<<nblk(nS), MC_T, 0, c->stream>>>(out, A.tmpS, ONE, ONE, nS);
  CODY_LAUNCHED(c);
}

// sbar = (d RK4 / d s)^H obar (stages recomputed from s); grad += field parts
void rk4_vjp(cgpu_ctx* c, McAdjoint& A, const z_t* s, const z_t* obar, z_t* sbar, double t0) {
  const int nS = A.nS;
  const double dt = A.dt;
  int n1, n2, n4;
  const double E1 = field_at(A, t0, &n1), E2 = field_at(A, t0 + 0.5 * dt, &n2), E4 = field_at(A, t0 + dt, &n4);
  const double Es[4] = {E1, E2, E2, E4};
  const int ns[4] = {n1, n2, n2, n4};
  rk4_forward(c, A, s, nullptr, t0);  // stage states
  // kbar_i (kept in kv[i] once the stage values are no longer needed)
  const double wgt[4] = {dt / 6.0, dt / 3.0, dt / 3.0, dt / 6.0};
  const double cs[3] = {0.5 * dt, 0.5 * dt, dt};
  CODY_CUDA(cudaMemcpyAsync(sbar, obar, sizeof(z_t) * nS, cudaMemcpyDeviceToDevice, c->stream));
  for (int i = 0; i < 4; i++) {
    CODY_CUDA(cudaMemcpyAsync(A.kv[i], obar, sizeof(z_t) * nS, cudaMemcpyDeviceToDevice, c->stream));
    k_mc_axpby<<<nblk(nS), MC_T, 0, c->stream>>>(A.kv[i], obar, ZERO, zmk(wgt[i], 0.0), nS);
    CODY_LAUNCHED(c);
  }
  for (int i = 3; i >= 0; i--) {
    // intermediates of stage i, then its VJP into sbarTmp
    nonlin_forward(c, A, A.stage[i], A.u, Es[i]);
    CODY_CUDA(cudaMemsetAsync(A.sbarTmp, 0, sizeof(z_t) * nS, c->stream));
    nonlin_vjp(c, A, A.stage[i], A.kv[i], A.sbarTmp, Es[i], ns[i]);
    k_mc_axpby<<<nblk(nS), MC_T, 0, c->stream>>>(sbar, A.sbarTmp, ONE, ONE, nS);
    CODY_LAUNCHED(c);
    if (i > 0) {
      k_mc_axpby<<<nblk(nS), MC_T, 0, c->stream>>>(A.kv[i - 1], A.sbarTmp, zmk(cs[i - 1], 0.0), ONE, nS);
      CODY_LAUNCHED(c);
    }
  }
}

// One Strang step n: s -> out
void step_forward(cgpu_ctx* c, McAdjoint& A, const z_t* s, z_t* out, int n) {
  const double dt = A.dt, t0 = n * dt;
  int na, nc;
  const double Ea = field_at(A, t0 + 0.25 * dt, &na), Ec = field_at(A, t0 + 0.75 * dt, &nc);
  lanczos_forward(c, A, s, A.sA, Ea, 0.5 * dt);
  rk4_forward(c, A, A.sA, A.sB, t0);
  lanczos_forward(c, A, A.sB, out, Ec, 0.5 * dt);
}

// lam (co-state of the step's output) -> lam (co-state of its input s)
void step_vjp(cgpu_ctx* c, McAdjoint& A, const z_t* s, z_t* lam, int n) {
  const double dt = A.dt, t0 = n * dt;
  int na, nc;
  const double Ea = field_at(A, t0 + 0.25 * dt, &na), Ec = field_at(A, t0 + 0.75 * dt, &nc);
  // recompute the intermediate states
  lanczos_forward(c, A, s, A.sA, Ea, 0.5 * dt);
  rk4_forward(c, A, A.sA, A.sB, t0);
  lanczos_forward(c, A, A.sB, A.tmpS, Ec, 0.5 * dt);
  lanczos_vjp(c, A, A.sB, lam, A.lamB, Ec, 0.5 * dt, nc, 0);
  rk4_vjp(c, A, A.sA, A.lamB, A.lam, t0);
  lanczos_forward(c, A, s, A.sA, Ea, 0.5 * dt);
  lanczos_vjp(c, A, s, A.lam, lam, Ea, 0.5 * dt, na, 0);
}

}  // namespace

// ---------------------------------------------------------------------------
// Entry points (called from ctx.cu's C ABI)
// ---------------------------------------------------------------------------
void mc_adjoint_free(cgpu_ctx* c) {
  delete c->mcAdj;
  c->mcAdj = nullptr;
}

void mc_adjoint_forward(cgpu_ctx* c, const z_t* state0_h, const z_t* ref_h, const double* field_h, int nT, double dt,
                        int K, int checkpoint, double* J, double* overlap, z_t* final_h) {
  if (c->nb != 1) throw std::string("mc_adjoint: a single-system context");
  if (c->method != CGPU_METHOD_MCTDHX) throw std::string("mc_adjoint: an MCTDHX context");
  if (c->precision != CGPU_PREC_FP64) throw std::string("mc_adjoint: the FP64 form");
  const SysHost& s = c->sys[0];
  if (!c->restricted || c->nBt != 2 || s.nBodies[0] != 1 || s.nBodies[1] != 1)
    throw std::string("mc_adjoint: restricted systems of two body types with one particle each");
  if (s.nOS > MC_MAXM) throw std::string("mc_adjoint: at most 16 spatial orbitals");
  if (K < 1 || K > MC_MAXK) throw std::string("mc_adjoint: Krylov order in 1..32");
  if (nT < 1 || !(dt > 0.0)) throw std::string("mc_adjoint: need n_steps >= 1 and dt > 0");
  if (!c->hasInteraction) throw std::string("mc_adjoint: needs the interaction");
  if (checkpoint <= 0) checkpoint = 64;
  const int M = s.nOS, nG = s.nG, Q = M * M, nS = Q + nG * M;
  if (s.nC != Q) throw std::string("mc_adjoint: configuration count");
  McAdjoint* A = c->mcAdj;
  const int nChk = (nT + checkpoint - 1) / checkpoint;
  if (!A || A->K != K || A->nT != nT || A->chk != checkpoint) {
    delete A;
    A = new McAdjoint();
    c->mcAdj = A;
    A->nG = nG;
    A->M = M;
    A->Q = Q;
    A->nS = nS;
    A->band = s.band;
    A->K = K;
    A->nT = nT;
    A->chk = checkpoint;
    A->eps = s.regEps;
    A->m = A->alloc<double>(nS);
    A->wx = A->alloc<double>(nG);
    A->grad = A->alloc<double>(nT);
    A->J = A->alloc<double>(4);
    A->ref = A->alloc<z_t>(nS);
    A->cur = A->alloc<z_t>(nS);
    A->co = A->alloc<z_t>(nS);
    A->chkStates = A->alloc<z_t>((size_t)nS * nChk);
    A->seg = A->alloc<z_t>((size_t)nS * (checkpoint + 1));
    A->sA = A->alloc<z_t>(nS);
    A->sB = A->alloc<z_t>(nS);
    A->lam = A->alloc<z_t>(nS);
    A->lamB = A->alloc<z_t>(nS);
    for (int i = 0; i < 4; i++) {
      A->stage[i] = A->alloc<z_t>(nS);
      A->kv[i] = A->alloc<z_t>(nS);
    }
    A->V = A->alloc<z_t>((size_t)nS * K);
    A->vbar = A->alloc<z_t>((size_t)nS * K);
    A->w = A->alloc<z_t>(nS);
    A->r = A->alloc<z_t>(nS);
    A->u = A->alloc<z_t>(nS);
    A->rbar = A->alloc<z_t>(nS);
    A->wbar = A->alloc<z_t>(nS);
    A->tmpS = A->alloc<z_t>(nS);
    A->sbarTmp = A->alloc<z_t>(nS);
    A->y = A->alloc<z_t>(MC_MAXK);
    A->ybar = A->alloc<z_t>(MC_MAXK);
    A->dots = A->alloc<z_t>(2 * MC_MAXK + 8);
    A->al = A->alloc<double>(MC_MAXK);
    A->be = A->alloc<double>(MC_MAXK);
    A->abar = A->alloc<double>(MC_MAXK);
    A->bbar = A->alloc<double>(MC_MAXK);
    A->lz = A->alloc<double>(8);
    A->lamK = A->alloc<double>(MC_MAXK);
    A->Qk = A->alloc<double>(MC_MAXK * MC_MAXK);
    const size_t GM = (size_t)nG * M, GQ = (size_t)nG * Q, QQ = (size_t)Q * Q;
    A->Aphi = A->alloc<z_t>(GM);
    A->wphi = A->alloc<z_t>(GM);
    A->h1 = A->alloc<z_t>(Q);
    A->Sp = A->alloc<z_t>(GQ);
    A->Wp = A->alloc<z_t>(GQ);
    A->g2 = A->alloc<z_t>(QQ);
    A->dC0 = A->alloc<z_t>(Q);
    A->r1 = A->alloc<z_t>(Q);
    A->U = A->alloc<z_t>(Q);
    A->Mreg = A->alloc<z_t>(Q);
    A->r2 = A->alloc<z_t>(QQ);
    A->R = A->alloc<z_t>(QQ);
    A->dphi0 = A->alloc<z_t>(GM);
    A->dphi = A->alloc<z_t>(GM);
    A->Gp = A->alloc<z_t>(Q);
    A->sc = A->alloc<z_t>(2);
    A->occ = A->alloc<double>(M);
    A->fv = A->alloc<double>(M);
    A->dC0bar = A->alloc<z_t>(Q);
    A->Cbar = A->alloc<z_t>(Q);
    A->ubar = A->alloc<z_t>(std::max<size_t>(GM, Q));
    A->dphi0bar = A->alloc<z_t>(GM);
    A->phibar = A->alloc<z_t>(GM);
    A->G1 = A->alloc<z_t>(Q);
    A->h1bar = A->alloc<z_t>(Q);
    A->X1 = A->alloc<z_t>(Q);
    A->T1 = A->alloc<z_t>(GM);
    A->T2 = A->alloc<z_t>(GM);
    A->AT2 = A->alloc<z_t>(GM);
    A->g2bar = A->alloc<z_t>(QQ);
    A->Q1 = A->alloc<z_t>(GQ);
    A->Wpbar = A->alloc<z_t>(GQ);
    A->Spbar = A->alloc<z_t>(GQ);
    A->Rbar = A->alloc<z_t>(QQ);
    A->r2bar = A->alloc<z_t>(QQ);
    A->Mbar = A->alloc<z_t>(Q);
    A->r1bar = A->alloc<z_t>(Q);
    A->wd = A->alloc<z_t>(GM);
    A->Sov = A->alloc<z_t>(Q);
    A->Sbar = A->alloc<z_t>(Q);
    A->Ov = A->alloc<z_t>(2);
    k_mc_weights<<<nblk(nS), MC_T, 0, c->stream>>>(A->m, A->wx, c->w_d, c->x_d, nG, M, Q);
    CODY_LAUNCHED(c);
  }
  A->dt = dt;
  A->field.assign(field_h, field_h + nT);
  CODY_CUDA(cudaMemcpyAsync(A->cur, state0_h, sizeof(z_t) * nS, cudaMemcpyHostToDevice, c->stream));
  CODY_CUDA(cudaMemcpyAsync(A->ref, ref_h ? ref_h : state0_h, sizeof(z_t) * nS, cudaMemcpyHostToDevice, c->stream));
  for (int n = 0; n < nT; n++) {
    if (n % checkpoint == 0)
      CODY_CUDA(cudaMemcpyAsync(A->chkStates + (size_t)nS * (n / checkpoint), A->cur, sizeof(z_t) * nS,
                                cudaMemcpyDeviceToDevice, c->stream));
    step_forward(c, *A, A->cur, A->cur, n);
  }
  // objective
  mc_zgemm(c, M, M, nG, ONE, A->ref + Q, nG, 2, A->cur + Q, nG, 0, c->w_d, ZERO, A->Sov, M);
  k_mc_overlap<<<1, MC_RED, 0, c->stream>>>(A->Ov, A->ref, A->Sov, A->cur, M);
  CODY_LAUNCHED(c);
  k_mc_objective<<<1, 32, 0, c->stream>>>(A->J, A->Ov);
  CODY_LAUNCHED(c);
  double jo[1];
  z_t ov;
  CODY_CUDA(cudaMemcpyAsync(jo, A->J, sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  CODY_CUDA(cudaMemcpyAsync(&ov, A->Ov, sizeof(z_t), cudaMemcpyDeviceToHost, c->stream));
  if (final_h) CODY_CUDA(cudaMemcpyAsync(final_h, A->cur, sizeof(z_t) * nS, cudaMemcpyDeviceToHost, c->stream));
  CODY_CUDA(cudaStreamSynchronize(c->stream));
  if (J) *J = jo[0];
  if (overlap) {
    overlap[0] = ov.x;
    overlap[1] = ov.y;
  }
  A->ready = true;
}

void mc_adjoint_backward(cgpu_ctx* c, double* grad_h) {
  McAdjoint* A = c->mcAdj;
  if (!A || !A->ready) throw std::string("mc_adjoint_backward: call cgpu_mc_adjoint_forward first");
  const int nS = A->nS, M = A->M, Q = A->Q, nG = A->nG, nT = A->nT, chk = A->chk;
  CODY_CUDA(cudaMemsetAsync(A->grad, 0, sizeof(double) * nT, c->stream));
  // co-state of the final state: d J / d Psi_N
  k_mc_overlap_vjp<<<1, 256, 0, c->stream>>>(A->Cbar, A->Sbar, A->ref, A->Sov, A->cur, A->Ov, M);
  CODY_LAUNCHED(c);
  CODY_CUDA(cudaMemsetAsync(A->lam, 0, sizeof(z_t) * nS, c->stream));
  mc_zgemm(c, nG, M, M, ONE, A->ref + Q, nG, 0, A->Sbar, M, 0, nullptr, ZERO, A->phibar, nG);
  k_mc_wrows<<<nblk((size_t)nG * M), MC_T, 0, c->stream>>>(A->phibar, A->phibar, c->w_d, nG, M);
  CODY_LAUNCHED(c);
  z_t* lamN = A->lamB;
  CODY_CUDA(cudaMemsetAsync(lamN, 0, sizeof(z_t) * nS, c->stream));
  k_mc_acc_state<<<nblk(nS), MC_T, 0, c->stream>>>(lamN, A->Cbar, A->phibar, Q, nG * M);
  CODY_LAUNCHED(c);
  // the co-state between steps (step_vjp uses lam / lamB as scratch)
  CODY_CUDA(cudaMemcpyAsync(A->co, lamN, sizeof(z_t) * nS, cudaMemcpyDeviceToDevice, c->stream));
  const int nChk = (nT + chk - 1) / chk;
  for (int sgm = nChk - 1; sgm >= 0; sgm--) {
    const int n0 = sgm * chk, n1 = std::min(nT, n0 + chk);
    CODY_CUDA(cudaMemcpyAsync(A->seg, A->chkStates + (size_t)nS * sgm, sizeof(z_t) * nS, cudaMemcpyDeviceToDevice,
                              c->stream));
    for (int n = n0; n < n1 - 1; n++)
      step_forward(c, *A, A->seg + (size_t)nS * (n - n0), A->seg + (size_t)nS * (n - n0 + 1), n);
    for (int n = n1 - 1; n >= n0; n--) step_vjp(c, *A, A->seg + (size_t)nS * (n - n0), A->co, n);
  }
  CODY_CUDA(cudaMemcpyAsync(grad_h, A->grad, sizeof(double) * nT, cudaMemcpyDeviceToHost, c->stream));
  CODY_CUDA(cudaStreamSynchronize(c->stream));
}
