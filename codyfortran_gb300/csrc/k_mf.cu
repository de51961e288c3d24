// k_mf.cu -- interaction and mean-field kernels (FP64 form).
//
// The reference loops over unordered orbital pairs and, per pair, runs an
// O(nG^2) convolution, multiplies the potential onto every orbital and
// accumulates into dOrbs / h2 (ApplyCorrelationOp, AccumulateCorrelation,
// FillH2CorrelationBlock, FillH2: src/Method/Mb/OrbBased/S_Method_Mb_OrbBased.f90:227-329,
// 491-872).  Here the same sums are three dense contractions:
//
//   S[g,(l,k)] = conj(phi_l(g)) phi_k(g) w(g)                 (FillInteractionSrc)
//   W[g,(l,k)] = sum_g' V(g,g') S[g',(l,k)]    l <= k         (pair potentials, DGEMM)
//   W[g,(k,l)] = conj(W[g,(l,k)])                             (ConjugateInteractionPotential)
//   Z[g,(k1,j)] = sum_(l2,k2) W[g,(l2,k2)] R'[(l2,k2),(k1,j)]  (ZGEMM, R' = rho2 x_3 rho^-1)
//   dphi_j(g) += sum_k1 phi_k1(g) Z[g,(k1,j)]                 (AccumulateCorrelation)
//   h2[(i1,j1),(l2,k2)] = 1/2 sum_g S[g,(i1,j1)] W[g,(l2,k2)]  (ZGEMM^T, FillH2Block)
//
// plus the regularised inverse of the one-body RDM (RdmDiagonalize_Rdm1 +
// regInvMat, :722-754) by a parallel cyclic Jacobi eigensolver in one CTA.
// Every kernel covers all trajectories of the context (blockIdx.z).
#include <algorithm>

#include "common.cuh"

namespace {

// ---------------------------------------------------------------------------
// Pair sources and expansion
// ---------------------------------------------------------------------------
__global__ void k_pair_src(z_t* __restrict__ S, const z_t* __restrict__ orbs, const double* __restrict__ w,
                           const int* __restrict__ pl, const int* __restrict__ pk, TRAJ_ARGS) {
  const TrajShape& T = shp[blockIdx.z];
  const int nG = T.nG, nP = T.nPairs;
  S = bat(S, bs);
  orbs = bat(orbs, bs);
  w = bat(w, bs);
  pl = bat(pl, bs);
  pk = bat(pk, bs);
  GRID_STRIDE(e, (size_t)nG * nP) {
    int g = (int)(e / nP), p = (int)(e % nP);
    z_t a = orbs[(size_t)nG * pl[p] + g], b = orbs[(size_t)nG * pk[p] + g];
    S[e] = zscale(zcmul(a, b), w[g]);
  }
}

// Wfull[g][a*n+b] = W_(a,b)(g) for same-body-type pairs, Sfull[g][a*n+b] = conj(phi_a) phi_b w.
__global__ void k_expand(z_t* __restrict__ Wfull, z_t* __restrict__ Sfull, const z_t* __restrict__ W,
                         const z_t* __restrict__ orbs, const double* __restrict__ w, const int* __restrict__ pidx,
                         TRAJ_ARGS) {
  const TrajShape& T = shp[blockIdx.z];
  const int nG = T.nG, n = T.nOS, nP = T.nPairs;
  int Q = n * n;
  Wfull = bat(Wfull, bs);
  Sfull = bat(Sfull, bs);
  W = bat(W, bs);
  orbs = bat(orbs, bs);
  w = bat(w, bs);
  pidx = bat(pidx, bs);
  GRID_STRIDE(e, (size_t)nG * Q) {
    int g = (int)(e / Q), q = (int)(e % Q);
    int a = q / n, b = q % n;
    z_t v = zmk(0.0, 0.0);
    if (a <= b) {
      int p = pidx[a * n + b];
      if (p >= 0) v = W[(size_t)g * nP + p];
    } else {
      int p = pidx[b * n + a];
      if (p >= 0) v = zconj(W[(size_t)g * nP + p]);
    }
    Wfull[e] = v;
    if (Sfull) Sfull[e] = zscale(zcmul(orbs[(size_t)nG * a + g], orbs[(size_t)nG * b + g]), w[g]);
  }
}

// dOrbs[g + nG*j] += sum_k1 orbs[g + nG*k1] * Z[g][k1*n + j]
__global__ void k_corr_epilogue(z_t* __restrict__ dOrbs, const z_t* __restrict__ orbs, const z_t* __restrict__ Z,
                                TRAJ_ARGS) {
  const TrajShape& T = shp[blockIdx.z];
  const int nG = T.nG, n = T.nOS;
  int g = blockIdx.x * blockDim.x + threadIdx.x;
  int j = blockIdx.y;
  if (g >= nG || j >= n) return;
  dOrbs = bat(dOrbs, bs);
  orbs = bat(orbs, bs);
  Z = bat(Z, bs);
  z_t acc = zmk(0.0, 0.0);
  const z_t* zr = Z + (size_t)g * n * n;
  for (int k1 = 0; k1 < n; k1++) zfma(acc, orbs[(size_t)nG * k1 + g], zr[k1 * n + j]);
  size_t o = (size_t)nG * j + g;
  dOrbs[o] = zadd(dOrbs[o], acc);
}

// h2 (nO^4, Fortran order) from the spatial block H2s[(i1*n+j1)][(l2*n+k2)]:
// h2(i1,l2,j1,k2) = H2s, same body type within (i1,j1) and within (l2,k2);
// restricted runs duplicate the spatial block into the spin blocks.
__global__ void k_h2_layout(z_t* __restrict__ h2, const z_t* __restrict__ H2s, const int* __restrict__ btOf,
                            TRAJ_ARGS) {
  const TrajShape& T = shp[blockIdx.z];
  const int n = T.nOS;
  size_t N = T.nO;
  h2 = bat(h2, bs);
  H2s = bat(H2s, bs);
  btOf = bat(btOf, bs);
  GRID_STRIDE(e, N * N * N * N) {
    int i1 = (int)(e % N), l2 = (int)((e / N) % N), j1 = (int)((e / N / N) % N), k2 = (int)(e / N / N / N);
    h2[e] = h2_from_h2s(H2s, btOf, T.restricted, n, i1, l2, j1, k2);
  }
}

// ---------------------------------------------------------------------------
// Tiled GEMMs
// ---------------------------------------------------------------------------
// W[nG, 2P] = V[nG, nG] S[nG, 2P] (the complex pair sources viewed as interleaved
// doubles), all row-major, real FP64.  64x64 tile, 256 threads, 4x4 per thread.
constexpr int DG_BM = 64, DG_BN = 64, DG_BK = 16;

__global__ void __launch_bounds__(256) k_dgemm_pairs(const double* __restrict__ A, const double* __restrict__ B,
                                                     double* __restrict__ C, TRAJ_ARGS) {
  __shared__ double As[DG_BK][DG_BM + 1];
  __shared__ double Bs[DG_BK][DG_BN];
  const TrajShape& T = shp[blockIdx.z];
  const int M = T.nG, N = 2 * T.nPairs, K = T.nG, lda = T.nG, ldb = N, ldc = N;
  int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
  int m0 = blockIdx.y * DG_BM, n0 = blockIdx.x * DG_BN;
  if (m0 >= M || n0 >= N) return;
  A = bat(A, bs);
  B = bat(B, bs);
  C = bat(C, bs);
  double acc[4][4] = {};
  for (int k0 = 0; k0 < K; k0 += DG_BK) {
    for (int t = threadIdx.x; t < DG_BM * DG_BK; t += 256) {
      int r = t / DG_BK, kk = t % DG_BK;
      int m = m0 + r, k = k0 + kk;
      As[kk][r] = (m < M && k < K) ? A[(size_t)m * lda + k] : 0.0;
    }
    for (int t = threadIdx.x; t < DG_BK * DG_BN; t += 256) {
      int kk = t / DG_BN, cc = t % DG_BN;
      int k = k0 + kk, n = n0 + cc;
      Bs[kk][cc] = (k < K && n < N) ? B[(size_t)k * ldb + n] : 0.0;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < DG_BK; kk++) {
      double a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; i++) a[i] = As[kk][ty + 16 * i];
#pragma unroll
      for (int j = 0; j < 4; j++) b[j] = Bs[kk][tx + 16 * j];
#pragma unroll
      for (int i = 0; i < 4; i++)
#pragma unroll
        for (int j = 0; j < 4; j++) acc[i][j] = fma(a[i], b[j], acc[i][j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; i++)
#pragma unroll
    for (int j = 0; j < 4; j++) {
      int m = m0 + ty + 16 * i, n = n0 + tx + 16 * j;
      if (m < M && n < N) C[(size_t)m * ldc + n] = acc[i][j];
    }
}

// The two complex GEMMs of the mean field, row-major, per trajectory:
//   ZG_Z : Z[nG, Q]  = Wfull[nG, Q] R'[Q, Q]
//   ZG_H2: H2s[Q, Q] = Sfull[nG, Q]^T Wfull[nG, Q]   (scaled by 1/2 in the reduction)
// P[split][m][n] = sum_{k in split} opA(m,k) B[k][n].  32x32 tile, 256 threads,
// 2x2 per thread; blockIdx.z = trajectory * nSplit + split.
enum { ZG_Z = 0, ZG_H2 = 1 };
constexpr int ZG_BM = 32, ZG_BN = 32, ZG_BK = 8;

__device__ __forceinline__ void zgemm_dims(const TrajShape& T, int mode, int& M, int& N, int& K) {
  int Q = T.nOS * T.nOS;
  if (mode == ZG_Z) { M = T.nG; N = Q; K = Q; }
  else { M = Q; N = Q; K = T.nG; }
}

__global__ void __launch_bounds__(256) k_zgemm(int mode, int nSplit, int kPerSplit, const z_t* __restrict__ A,
                                               const z_t* __restrict__ B, z_t* __restrict__ P, TRAJ_ARGS) {
  __shared__ z_t As[ZG_BK][ZG_BM + 1];
  __shared__ z_t Bs[ZG_BK][ZG_BN];
  const int traj = blockIdx.z / nSplit, split = blockIdx.z % nSplit;
  const TrajShape& T = shp[traj];
  int M, N, K;
  zgemm_dims(T, mode, M, N, K);
  const int transA = mode == ZG_H2, lda = T.nOS * T.nOS, ldb = lda, ldp = N;
  int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
  int m0 = blockIdx.y * ZG_BM, n0 = blockIdx.x * ZG_BN;
  if (m0 >= M || n0 >= N) return;
  A = batn(A, bs, traj);
  B = batn(B, bs, traj);
  P = batn(P, bs, traj);
  int kBeg = split * kPerSplit, kEnd = min(K, kBeg + kPerSplit);
  z_t acc[2][2];
  for (int i = 0; i < 2; i++)
    for (int j = 0; j < 2; j++) acc[i][j] = zmk(0.0, 0.0);
  for (int k0 = kBeg; k0 < kEnd; k0 += ZG_BK) {
    {
      int t = threadIdx.x;  // 256 = 32 x 8
      int r, kk;
      if (transA) { r = t % ZG_BM; kk = t / ZG_BM; } else { kk = t % ZG_BK; r = t / ZG_BK; }
      int m = m0 + r, k = k0 + kk;
      z_t v = zmk(0.0, 0.0);
      if (m < M && k < kEnd) v = transA ? A[(size_t)k * lda + m] : A[(size_t)m * lda + k];
      As[kk][r] = v;
      int kb = t / ZG_BN, cc = t % ZG_BN;
      int kq = k0 + kb, n = n0 + cc;
      Bs[kb][cc] = (kq < kEnd && n < N) ? B[(size_t)kq * ldb + n] : zmk(0.0, 0.0);
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < ZG_BK; kk++) {
      z_t a0 = As[kk][ty], a1 = As[kk][ty + 16];
      z_t b0 = Bs[kk][tx], b1 = Bs[kk][tx + 16];
      zfma(acc[0][0], a0, b0);
      zfma(acc[0][1], a0, b1);
      zfma(acc[1][0], a1, b0);
      zfma(acc[1][1], a1, b1);
    }
    __syncthreads();
  }
  z_t* Pz = P + (size_t)split * M * ldp;
  for (int i = 0; i < 2; i++)
    for (int j = 0; j < 2; j++) {
      int m = m0 + ty + 16 * i, n = n0 + tx + 16 * j;
      if (m < M && n < N) Pz[(size_t)m * ldp + n] = acc[i][j];
    }
}

__global__ void k_split_reduce(z_t* __restrict__ C, const z_t* __restrict__ P, int nSplit, int mode, double scale,
                               TRAJ_ARGS) {
  const TrajShape& T = shp[blockIdx.z];
  int M, N, K;
  zgemm_dims(T, mode, M, N, K);
  size_t MN = (size_t)M * N;
  C = bat(C, bs);
  P = bat(P, bs);
  GRID_STRIDE(e, MN) {
    z_t s = zmk(0.0, 0.0);
    for (int z = 0; z < nSplit; z++) s = zadd(s, P[(size_t)z * MN + e]);
    C[e] = zscale(s, scale);
  }
}

// ---------------------------------------------------------------------------
// Regularised inverse of the spin-summed one-body RDM (one CTA per trajectory).
// Parallel cyclic Jacobi (round-robin pairing), complex Hermitian n <= 32.
// ---------------------------------------------------------------------------
constexpr int JB_MAX = 32;

// The eigenvectors of the previous call (Uprev, column-major n x n, identity
// at start) precondition the problem: Jacobi runs on Uprev^H rho Uprev, which
// is nearly diagonal between consecutive evaluations, so it converges in a few
// sweeps; Uprev V is stored for the next call.  Uprev is re-orthonormalised
// (one modified Gram-Schmidt pass) on load so rounding cannot accumulate.
// The result Mreg = U f(n) U^H depends only on rho (to rounding).
__global__ void __launch_bounds__(512) k_rdm_inverse(z_t* __restrict__ Mreg, z_t* __restrict__ r1s,
                                                     const z_t* __restrict__ rdm1, z_t* __restrict__ Uprev,
                                                     double* __restrict__ occ, TRAJ_ARGS) {
  extern __shared__ z_t jsm[];
  const TrajShape& T = shp[blockIdx.z];
  const int nO = T.nO, n = T.nOS, restricted = T.restricted;
  const double reg = T.regEps;
  Mreg = bat(Mreg, bs);
  r1s = bat(r1s, bs);
  rdm1 = bat(rdm1, bs);
  Uprev = bat(Uprev, bs);
  z_t(*A)[JB_MAX + 1] = reinterpret_cast<z_t(*)[JB_MAX + 1]>(jsm);
  z_t(*V)[JB_MAX + 1] = reinterpret_cast<z_t(*)[JB_MAX + 1]>(jsm + JB_MAX * (JB_MAX + 1));
  z_t(*U)[JB_MAX + 1] = reinterpret_cast<z_t(*)[JB_MAX + 1]>(jsm + 2 * JB_MAX * (JB_MAX + 1));
  __shared__ double rc[JB_MAX / 2], rs[JB_MAX / 2], ev[JB_MAX];
  __shared__ z_t rph[JB_MAX / 2];
  __shared__ int rp[JB_MAX / 2], rq[JB_MAX / 2];
  __shared__ double offs, diags;
  int tid = threadIdx.x;
  for (int e = tid; e < n * n; e += blockDim.x) {
    int i = e % n, j = e / n;
    z_t v = rdm1[i + (size_t)nO * j];
    if (restricted) v = zadd(v, rdm1[(n + i) + (size_t)nO * (n + j)]);
    A[i][j] = v;
    r1s[e] = v;
    U[i][j] = Uprev[i + (size_t)n * j];
  }
  __syncthreads();
  for (int e = tid; e < n; e += blockDim.x) A[e][e].y = 0.0;
  // re-orthonormalise U (unitary to rounding) by one Newton-Schulz polar
  // step, U <- U (3 I - U^H U) / 2: the deviation from orthonormality squares
  {
    for (int e = tid; e < n * n; e += blockDim.x) {
      int i = e % n, j = e / n;
      z_t g = zmk(0.0, 0.0);
      for (int k = 0; k < n; k++) zcfma(g, U[k][i], U[k][j]);
      V[i][j] = zmk((i == j ? 1.5 : 0.0) - 0.5 * g.x, -0.5 * g.y);
    }
    __syncthreads();
    z_t un[(JB_MAX * JB_MAX + 511) / 512];
    int q = 0;
    for (int e = tid; e < n * n; e += blockDim.x, q++) {
      int i = e % n, j = e / n;
      z_t s = zmk(0.0, 0.0);
      for (int k = 0; k < n; k++) zfma(s, U[i][k], V[k][j]);
      un[q] = s;
    }
    __syncthreads();
    q = 0;
    for (int e = tid; e < n * n; e += blockDim.x, q++) U[e % n][e / n] = un[q];
    __syncthreads();
  }
  // A <- U^H A U  (V as temporary), then V <- I
  for (int e = tid; e < n * n; e += blockDim.x) {
    int i = e % n, j = e / n;
    z_t s = zmk(0.0, 0.0);
    for (int k = 0; k < n; k++) zfma(s, A[i][k], U[k][j]);
    V[i][j] = s;
  }
  __syncthreads();
  for (int e = tid; e < n * n; e += blockDim.x) {
    int i = e % n, j = e / n;
    z_t s = zmk(0.0, 0.0);
    for (int k = 0; k < n; k++) s = zadd(s, zcmul(U[k][i], V[k][j]));
    A[i][j] = s;
  }
  __syncthreads();
  for (int e = tid; e < n * n; e += blockDim.x) {
    int i = e % n, j = e / n;
    V[i][j] = zmk(i == j ? 1.0 : 0.0, 0.0);
    if (i == j) A[i][i].y = 0.0;
  }
  __syncthreads();
  int ne = (n + 1) & ~1;
  int half = ne / 2;
  for (int sweep = 0; sweep < 30; sweep++) {
    if (tid == 0) {
      double off = 0.0, dg = 0.0;
      for (int j = 0; j < n; j++)
        for (int i = 0; i < n; i++) {
          double a2 = A[i][j].x * A[i][j].x + A[i][j].y * A[i][j].y;
          if (i == j) dg += a2; else off += a2;
        }
      offs = off;
      diags = dg;
    }
    __syncthreads();
    if (offs <= 1e-28 * (diags + offs) || offs == 0.0) break;  // rounding floor is ~1e-32
    for (int r = 0; r < ne - 1; r++) {
      if (tid < half) {
        int k = tid;
        auto pos = [&](int i) { return i == 0 ? 0 : ((i - 1 + r) % (ne - 1)) + 1; };
        int p = pos(k), q = pos(ne - 1 - k);
        if (p > q) { int t = p; p = q; q = t; }
        rp[k] = p;
        rq[k] = q;
        double c = 1.0, s = 0.0;
        z_t ph = zmk(1.0, 0.0);
        if (q < n) {
          z_t b = A[p][q];
          double g = sqrt(b.x * b.x + b.y * b.y);
          if (g != 0.0) {
            ph = zmk(b.x / g, b.y / g);
            double tau = (A[q][q].x - A[p][p].x) / (2.0 * g);
            double t = (tau >= 0 ? 1.0 : -1.0) / (fabs(tau) + sqrt(1.0 + tau * tau));
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
      // columns: A <- A U, V <- V U with U = [[c, s],[-s e^{-i th}, c e^{-i th}]]
      for (int e = tid; e < n * half; e += blockDim.x) {
        int i = e % n, k = e / n;
        int p = rp[k], q = rq[k];
        if (q < 0 || rs[k] == 0.0) continue;
        double c = rc[k], s = rs[k];
        z_t phc = zconj(rph[k]);
        z_t akp = A[i][p], akq = A[i][q];
        A[i][p] = zsub(zscale(akp, c), zscale(zmul(akq, phc), s));
        A[i][q] = zadd(zscale(akp, s), zscale(zmul(akq, phc), c));
        z_t vkp = V[i][p], vkq = V[i][q];
        V[i][p] = zsub(zscale(vkp, c), zscale(zmul(vkq, phc), s));
        V[i][q] = zadd(zscale(vkp, s), zscale(zmul(vkq, phc), c));
      }
      __syncthreads();
      // rows: A <- U^H A
      for (int e = tid; e < n * half; e += blockDim.x) {
        int i = e % n, k = e / n;
        int p = rp[k], q = rq[k];
        if (q < 0 || rs[k] == 0.0) continue;
        double c = rc[k], s = rs[k];
        z_t ph = rph[k];
        z_t apk = A[p][i], aqk = A[q][i];
        A[p][i] = zsub(zscale(apk, c), zscale(zmul(ph, aqk), s));
        A[q][i] = zadd(zscale(apk, s), zscale(zmul(ph, aqk), c));
      }
      __syncthreads();
      if (tid < half) {
        int p = rp[tid], q = rq[tid];
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
  // eigenvalues, eigenvectors U_new = U V (into A), stored for the next call
  occ = bat(occ, bs);
  for (int e = tid; e < n; e += blockDim.x) {
    ev[e] = A[e][e].x;
    occ[e] = ev[e];  // natural occupations (eigenvalues of the spin-summed rho1, unsorted)
  }
  __syncthreads();
  for (int e = tid; e < n * n; e += blockDim.x) {
    int i = e % n, j = e / n;
    z_t s = zmk(0.0, 0.0);
    for (int k = 0; k < n; k++) zfma(s, U[i][k], V[k][j]);
    A[i][j] = s;
    Uprev[i + (size_t)n * j] = s;
  }
  __syncthreads();
  // Mreg(k1,j1) = sum_j U(k1,j) n_j/(n_j^2+reg) conj(U(j1,j))
  for (int e = tid; e < n * n; e += blockDim.x) {
    int k1 = e % n, j1 = e / n;
    z_t acc = zmk(0.0, 0.0);
    for (int j = 0; j < n; j++) {
      double occ = ev[j];
      double f = occ / (occ * occ + reg);
      zfma(acc, zscale(A[k1][j], f), zconj(A[j1][j]));
    }
    Mreg[e] = acc;
  }
}

// r2s[(l2*n+k2)][(k1*n+k)] = rdm2(k1,k2,k,l2) summed over the spin blocks
// (restricted), or the spatial block masked by body types (unrestricted).
__global__ void k_build_r2s(z_t* __restrict__ r2s, const z_t* __restrict__ rdm2, const int* __restrict__ btOf,
                            TRAJ_ARGS) {
  const TrajShape& T = shp[blockIdx.z];
  const int n = T.nOS, restricted = T.restricted;
  size_t Q = (size_t)n * n;
  r2s = bat(r2s, bs);
  rdm2 = bat(rdm2, bs);
  btOf = bat(btOf, bs);
  const size_t N = T.nO;
  auto R2 = [&](int a, int b, int c, int d) { return rdm2[a + N * (b + N * (c + N * (size_t)d))]; };
  GRID_STRIDE(e, Q * Q) {
    int row = (int)(e / Q), col = (int)(e % Q);
    int l2 = row / n, k2 = row % n, k1 = col / n, k = col % n;
    z_t r = zmk(0.0, 0.0);
    if (restricted)
      r = zadd(zadd(zadd(R2(k1, k2, k, l2), R2(n + k1, k2, n + k, l2)), R2(k1, n + k2, k, n + l2)),
               R2(n + k1, n + k2, n + k, n + l2));
    else if (btOf[l2] == btOf[k2] && btOf[k1] == btOf[k])
      r = R2(k1, k2, k, l2);
    r2s[e] = r;
  }
}

// As k_build_r2s with the rdm2 entries formed from rdm2Lin (inside the NonLin
// derivative the nO^4 rdm2 is not formed); the same values.
__global__ void k_build_r2s_lin(z_t* __restrict__ r2s, const z_t* __restrict__ lin, const int* __restrict__ btOf,
                                TRAJ_ARGS) {
  const TrajShape& T = shp[blockIdx.z];
  const int n = T.nOS, restricted = T.restricted;
  size_t Q = (size_t)n * n;
  r2s = bat(r2s, bs);
  lin = bat(lin, bs);
  btOf = bat(btOf, bs);
  const size_t N = T.nO;
  auto R2 = [&](int a, int b, int c, int d) { return rdm2_from_lin(lin, btOf, N, a, b, c, d); };
  const int Qi = (int)Q;
  GRID_STRIDE(e, Q * Q) {  // Q^2 < 2^31: 32-bit index arithmetic
    const int ei = (int)e, row = ei / Qi, col = ei - row * Qi;
    const int l2 = row / n, k2 = row - l2 * n, k1 = col / n, k = col - k1 * n;
    z_t r = zmk(0.0, 0.0);
    if (restricted)
      r = zadd(zadd(zadd(R2(k1, k2, k, l2), R2(n + k1, k2, n + k, l2)), R2(k1, n + k2, k, n + l2)),
               R2(n + k1, n + k2, n + k, n + l2));
    else if (btOf[l2] == btOf[k2] && btOf[k1] == btOf[k])
      r = R2(k1, k2, k, l2);
    r2s[e] = r;
  }
}

// R'[(l2*n+k2)][(k1*n+j)] = sum_k r2s[(l2,k2)][(k1,k)] Mreg(k,j), masked by body types.
// One block per row (l2, k2) of R' (blockIdx.x), threads over its Q columns.
// DF: the products in double-float arithmetic (the fixed-point forms: 4 n FP64
// FMA per entry would hold the FP64 pipe), Mreg staged as double-floats.
template <bool DF>
__global__ void k_build_R(z_t* __restrict__ Rp, const z_t* __restrict__ r2s, const z_t* __restrict__ Mreg,
                          const int* __restrict__ btOf, TRAJ_ARGS) {
  const TrajShape& T = shp[blockIdx.z];
  const int n = T.nOS, restricted = T.restricted, Q = n * n, row = blockIdx.x;
  if (row >= Q) return;
  Rp = bat(Rp, bs);
  r2s = bat(r2s, bs);
  Mreg = bat(Mreg, bs);
  btOf = bat(btOf, bs);
  __shared__ float4 mdf[JB_MAX * JB_MAX];  // n <= JB_MAX (checked by the launcher)
  if (DF) {
    for (int i = threadIdx.x; i < Q; i += blockDim.x) mdf[i] = zdf_from(Mreg[i]);
    __syncthreads();
  }
  const int l2 = row / n, k2 = row - l2 * n;
  for (int col = threadIdx.x; col < Q; col += blockDim.x) {
    const int k1 = col / n, j = col - k1 * n;
    const bool ok = restricted || (btOf[l2] == btOf[k2] && btOf[k1] == btOf[j]);
    const z_t* rr = r2s + (size_t)row * Q + (size_t)k1 * n;
    z_t v = zmk(0.0, 0.0);
    if (ok && DF) {
      zdf_acc a = {0.0f, 0.0f, 0.0f, 0.0f};
      for (int k = 0; k < n; k++) zdf_fma(a, zdf_from(rr[k]), mdf[k + n * j], false);
      v = zdf_to_z(a);
    } else if (ok) {
      for (int k = 0; k < n; k++) zfma(v, rr[k], Mreg[k + (size_t)n * j]);
    }
    Rp[(size_t)row * Q + col] = v;
  }
}

// split count of a complex GEMM with M x N output and inner dimension K
int zgemm_splits(const cgpu_ctx* c, int M, int N, int K, int* kPer) {
  int tilesM = (M + ZG_BM - 1) / ZG_BM, tilesN = (N + ZG_BN - 1) / ZG_BN;
  long tiles = (long)tilesM * tilesN * c->nb;
  int nSplit = 1;
  if (tiles < 2 * 152 && K > 512) nSplit = (int)std::min<long>((2 * 152 + tiles - 1) / tiles, (K + 255) / 256);
  int per = ((K + nSplit - 1) / nSplit + ZG_BK - 1) / ZG_BK * ZG_BK;
  nSplit = (K + per - 1) / per;
  if (kPer) *kPer = per;
  return std::max(nSplit, 1);
}

void zgemm(cgpu_ctx* c, int mode, const z_t* A, const z_t* B, z_t* C, double scale) {
  int Q = c->nOS * c->nOS;
  int M = mode == ZG_Z ? c->nG : Q, N = Q, K = mode == ZG_Z ? Q : c->nG;
  int kPer = K;
  int nSplit = zgemm_splits(c, M, N, K, &kPer);
  int tilesM = (M + ZG_BM - 1) / ZG_BM, tilesN = (N + ZG_BN - 1) / ZG_BN;
  if (nSplit == 1 && scale == 1.0) {
    dim3 grid(tilesN, tilesM, c->nb);
    k_zgemm<<<grid, 256, 0, c->stream>>>(mode, 1, K, A, B, C, TRAJ_PASS(c));
    CODY_LAUNCHED(c);
    return;
  }
  if ((size_t)nSplit * M * N > c->partialCap) throw std::string("internal: zgemm scratch too small");
  dim3 grid(tilesN, tilesM, (unsigned)(c->nb * nSplit));
  k_zgemm<<<grid, 256, 0, c->stream>>>(mode, nSplit, kPer, A, B, c->partial_d, TRAJ_PASS(c));
  CODY_LAUNCHED(c);
  size_t MN = (size_t)M * N;
  k_split_reduce<<<bgrid(c, ew_blocks(c, MN)), 256, 0, c->stream>>>(C, c->partial_d, nSplit, mode, scale,
                                                                      TRAJ_PASS(c));
  CODY_LAUNCHED(c);
}

}  // namespace

size_t zgemm_partial_need(const cgpu_ctx* c) {
  int Q = c->nOS * c->nOS;
  size_t need = 0;
  // ZG_H2 always goes through the partial buffer (scale 1/2); ZG_Z only when split
  int s2 = zgemm_splits(c, Q, Q, c->nG, nullptr);
  need = std::max(need, (size_t)s2 * Q * Q);
  int s1 = zgemm_splits(c, c->nG, Q, Q, nullptr);
  if (s1 > 1) need = std::max(need, (size_t)s1 * c->nG * Q);
  return need;
}

// W = V S for the unordered same-body-type pairs (FP64).
void launch_pair_potentials(cgpu_ctx* c, const z_t* orbs) {
  ProfScope prof(c, CGPU_KERNEL_PAIR_POTENTIALS);
  size_t nGP = (size_t)c->nG * c->nPairs;
  k_pair_src<<<bgrid(c, ew_blocks(c, nGP)), 256, 0, c->stream>>>(c->S_d, orbs, c->w_d, c->pairL_d, c->pairK_d,
                                                                   TRAJ_PASS(c));
  CODY_LAUNCHED(c);
  int N = 2 * c->nPairs;  // complex columns viewed as interleaved doubles
  dim3 grid(ceil_div(N, DG_BN), ceil_div(c->nG, DG_BM), c->nb);
  k_dgemm_pairs<<<grid, 256, 0, c->stream>>>(c->Vint_d, (const double*)c->S_d, (double*)c->W_d, TRAJ_PASS(c));
  CODY_LAUNCHED(c);
}

static void expand_pairs(cgpu_ctx* c, const z_t* orbs, int wantS) {
  int n = c->nOS;
  size_t tot = (size_t)c->nG * n * n;
  k_expand<<<bgrid(c, ew_blocks(c, tot)), 256, 0, c->stream>>>(c->Wfull_d, wantS ? c->Sfull_d : nullptr, c->W_d,
                                                                 orbs, c->w_d, c->pidx_d, TRAJ_PASS(c));
  CODY_LAUNCHED(c);
}

static void h2_from_pairs(cgpu_ctx* c) {
  ProfScope prof(c, CGPU_KERNEL_H2);
  // H2s = 1/2 Sfull^T Wfull  (Q x nG)(nG x Q)
  zgemm(c, ZG_H2, c->Sfull_d, c->Wfull_d, c->h2s_d, 0.5);
  launch_h2_layout(c);
}

void launch_rdm_inverse(cgpu_ctx* c) {
  ProfScope prof(c, CGPU_KERNEL_RDM_INVERSE);
  int n = c->nOS;
  if (n > JB_MAX) throw std::string("ApplyCorrelationOp: more than 32 stored orbitals is not supported");
  constexpr size_t jsmem = 3 * sizeof(z_t) * JB_MAX * (JB_MAX + 1);
  static bool attr = false;
  if (!attr) {
    CODY_CUDA(cudaFuncSetAttribute(k_rdm_inverse, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)jsmem));
    attr = true;
  }
  k_rdm_inverse<<<bgrid(c, 1), 512, jsmem, c->stream>>>(c->Mreg_d, c->r1s_d, c->rdm1_d, c->Uprev_d,
                                                        c->scal_d + CODY_SCAL_OCC, TRAJ_PASS(c));
  CODY_LAUNCHED(c);
  size_t Q = (size_t)n * n;
  if (c->fuseLayouts)
    k_build_r2s_lin<<<bgrid(c, ew_blocks(c, Q * Q)), 256, 0, c->stream>>>(c->r2s_d, c->rdm2Lin_d, c->btOfOrb_d,
                                                                         TRAJ_PASS(c));
  else
    k_build_r2s<<<bgrid(c, ew_blocks(c, Q * Q)), 256, 0, c->stream>>>(c->r2s_d, c->rdm2_d, c->btOfOrb_d,
                                                                     TRAJ_PASS(c));
  CODY_LAUNCHED(c);
  auto buildR = c->ciDf ? k_build_R<true> : k_build_R<false>;
  buildR<<<dim3((unsigned)Q, 1, c->nb), 128, 0, c->stream>>>(c->Rp_d, c->r2s_d, c->Mreg_d, c->btOfOrb_d,
                                                             TRAJ_PASS(c));
  CODY_LAUNCHED(c);
}

// ApplyCorrelationOp: dOrbs += contraction; h2 (nO^4) filled when wantH2.
// Requires rdm1_d / rdm2_d to hold the current RDMs.
void launch_correlation(cgpu_ctx* c, z_t* dOrbs, const z_t* orbs, int wantH2) {
  launch_rdm_inverse(c);
  if (!c->hasInteraction) {
    if (wantH2) {
      batch_zero(c, c->h2_d, sizeof(z_t) * (size_t)c->nO * c->nO * c->nO * c->nO);
      batch_zero(c, c->h2s_d, sizeof(z_t) * (size_t)c->nOS * c->nOS * c->nOS * c->nOS);
    }
    return;
  }
  launch_pair_potentials(c, orbs);
  expand_pairs(c, orbs, wantH2);
  int n = c->nOS, Q = n * n;
  // Z = Wfull R'  (nG x Q)(Q x Q), stored in the second half of the Wfull allocation
  z_t* Z = c->Wfull_d + (size_t)c->nG * Q;
  {
    ProfScope prof(c, CGPU_KERNEL_CORRELATION);
    zgemm(c, ZG_Z, c->Wfull_d, c->Rp_d, Z, 1.0);
    launch_corr_epilogue(c, dOrbs, orbs, Z);
  }
  if (wantH2) h2_from_pairs(c);
}

// FillH2: h2 of the given orbitals.
void launch_fill_h2(cgpu_ctx* c, const z_t* orbs) {
  if (!c->hasInteraction) {
    batch_zero(c, c->h2_d, sizeof(z_t) * (size_t)c->nO * c->nO * c->nO * c->nO);
    return;
  }
  launch_pair_potentials(c, orbs);
  expand_pairs(c, orbs, 1);
  h2_from_pairs(c);
}

void launch_corr_epilogue(cgpu_ctx* c, z_t* dOrbs, const z_t* orbs, const z_t* Z) {
  // FP64 in every form: a double-float variant (a thread per grid point and
  // batch of orbitals) measured 0.1 ms per step slower at the 512-trajectory batch
  dim3 grid(ceil_div(c->nG, 256), c->nOS, c->nb);
  k_corr_epilogue<<<grid, 256, 0, c->stream>>>(dOrbs, orbs, Z, TRAJ_PASS(c));
  CODY_LAUNCHED(c);
}

void launch_h2_layout(cgpu_ctx* c) {
  if (c->fuseLayouts) return;  // launch_fold_h2 reads H2s directly
  size_t n4 = (size_t)c->nO * c->nO * c->nO * c->nO;
  k_h2_layout<<<bgrid(c, ew_blocks(c, n4)), 256, 0, c->stream>>>(c->h2_d, c->h2s_d, c->btOfOrb_d, TRAJ_PASS(c));
  CODY_LAUNCHED(c);
}
