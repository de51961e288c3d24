// k_adjoint.cu -- gradient of a pulse objective with respect to the sampled
// field, by the exact discrete adjoint of the fixed-orbital (TDCI) propagation
// (src/Method/Mb/OrbBased/Tdci/S_Method_Mb_OrbBased_Tdci.f90:75-107 with the
// RK4 integrator, src/IntegratorList/Rk/O4Expl/S_IntegratorList_Rk_O4Expl.f90:90-141).
//
// With fixed orbitals the CI equation is linear, dC/dt = -i (A + E(t) X) C:
// A = H1 + H2 at zero field, X = the CI matrix of the one-body dipole x
// (length gauge, +E x).  The field is constant over step n (E_n), so one RK4
// step is the degree-4 Taylor polynomial C_{n+1} = R(z_n) C_n, z_n = -i dt H_n.
// For J = 1 - |a|^2, a = C_0^H C_N:
//   mu_N = C_0,  mu_n = R(z_n)^H mu_{n+1},
//   da/dE_n = mu_{n+1}^H (dR/dE_n) C_n
//           = -i dt sum_{m+q<=3} w_m^H X u_q / (m+q+1)!,
//   u_q = z^q C_n,  w_m = (z^H)^m mu_{n+1} = (i dt H_n^H)^m mu_{n+1},
//   dJ/dE_n = -2 Re(conj(a) da/dE_n).
// States are checkpointed every K steps in the forward sweep and recomputed a
// segment at a time in the backward sweep.  A and X are dense (nC <= 64,
// held in shared memory); one CTA runs both sweeps.
#include <algorithm>
#include <cmath>

#include "common.cuh"

namespace {

constexpr int ADJ_MAXC = 64;     // configurations held in shared memory
constexpr int ADJ_THREADS = 256;

// out[:, i] = x * orbs[:, i]
__global__ void k_x_orbs(z_t* __restrict__ out, const z_t* __restrict__ orbs, const double* __restrict__ x, int nG,
                         int nOS) {
  GRID_STRIDE(e, (size_t)nG * nOS) {
    int g = (int)(e % nG);
    out[e] = zscale(orbs[e], x[g]);
  }
}

// Dense CI matrix M[I][J] (row-major, nC x nC) of the operator whose folded
// integrals are h1Lin / h2Lin: the matrix k_ci_apply applies.  One thread per row.
__global__ void k_ci_dense(z_t* __restrict__ M, const z_t* __restrict__ h1Lin, const z_t* __restrict__ h2Lin,
                           TRAJ_ARGS, int useH1, int useH2) {
  const CiView& v = shp[0].view;
  const int nC = v.nC, nO2 = v.nO * v.nO;
  for (int I0 = blockIdx.x * blockDim.x + threadIdx.x; I0 < nC; I0 += gridDim.x * blockDim.x) {
    z_t* row = M + (size_t)I0 * nC;
    for (int J = 0; J < nC; J++) row[J] = zmk(0.0, 0.0);
    int conf[CODY_MAX_BT], t = I0;
    for (int b = 0; b < v.nBt; b++) {
      conf[b] = t % v.nConf[b] + 1;
      t /= v.nConf[b];
    }
    for (int b = 0; b < v.nBt; b++) {
      int c = conf[b], st = v.stride[b];
      size_t col = (size_t)v.maxS[b] * (c - 1);
      if (useH1)
        for (int k = 0; k < v.sN[b][c - 1]; k++) {
          int J = I0 + (v.sExc[b][col + k] - c) * st;
          z_t h = h1Lin[v.sCode[b][col + k]];
          row[J] = zadd(row[J], v.sFac[b][col + k] < 0 ? zmk(-h.x, -h.y) : h);
        }
      if (useH2) {
        size_t cd = (size_t)v.maxD[b] * (c - 1);
        for (int k = 0; k < v.dN[b][c - 1]; k++) {
          int J = I0 + (v.dExc[b][cd + k] - c) * st;
          z_t h = h2Lin[v.dCode[b][cd + k]];
          row[J] = zadd(row[J], v.dFac[b][cd + k] < 0 ? zmk(-h.x, -h.y) : h);
        }
        for (int b2 = b + 1; b2 < v.nBt; b2++) {
          int c2 = conf[b2], st2 = v.stride[b2];
          size_t col2 = (size_t)v.maxS[b2] * (c2 - 1);
          for (int k1 = 0; k1 < v.sN[b][c - 1]; k1++)
            for (int k2 = 0; k2 < v.sN[b2][c2 - 1]; k2++) {
              int J = I0 + (v.sExc[b][col + k1] - c) * st + (v.sExc[b2][col2 + k2] - c2) * st2;
              z_t h = h2Lin[(v.sCode[b][col + k1] - 1) * nO2 + v.sCode[b2][col2 + k2]];
              bool neg = (v.sFac[b][col + k1] * v.sFac[b2][col2 + k2]) < 0;
              row[J] = zadd(row[J], neg ? zmk(-h.x, -h.y) : h);
            }
        }
      }
    }
  }
}

// y = s * (H x) for the nC x nC matrix H in shared memory; 4 threads per row.
__device__ void mat_vec(z_t* __restrict__ y, const z_t* __restrict__ H, const z_t* __restrict__ x, int nC, z_t s) {
  const int r = threadIdx.x >> 2, q = threadIdx.x & 3;
  z_t acc = zmk(0.0, 0.0);
  if (r < nC)
    for (int j = q; j < nC; j += 4) zfma(acc, H[r * nC + j], x[j]);
  for (int o = 1; o < 4; o <<= 1) {
    acc.x += __shfl_xor_sync(0xffffffffu, acc.x, o);
    acc.y += __shfl_xor_sync(0xffffffffu, acc.y, o);
  }
  __syncthreads();  // x may alias a vector being written by another call
  if (r < nC && q == 0) y[r] = zmul(s, acc);
  __syncthreads();
}

// y = s * (H^H x) (conjugate transpose of the shared-memory matrix H)
__device__ void mat_vec_h(z_t* __restrict__ y, const z_t* __restrict__ H, const z_t* __restrict__ x, int nC, z_t s) {
  const int r = threadIdx.x >> 2, q = threadIdx.x & 3;
  z_t acc = zmk(0.0, 0.0);
  if (r < nC)
    for (int j = q; j < nC; j += 4) zcfma(acc, H[j * nC + r], x[j]);
  for (int o = 1; o < 4; o <<= 1) {
    acc.x += __shfl_xor_sync(0xffffffffu, acc.x, o);
    acc.y += __shfl_xor_sync(0xffffffffu, acc.y, o);
  }
  __syncthreads();
  if (r < nC && q == 0) y[r] = zmul(s, acc);
  __syncthreads();
}

// conj(a) . b over nC entries, result in all threads
__device__ z_t dotc(const z_t* a, const z_t* b, int nC, z_t* red) {
  z_t s = zmk(0.0, 0.0);
  for (int i = threadIdx.x; i < nC; i += blockDim.x) s = zadd(s, zcmul(a[i], b[i]));
  for (int o = 16; o > 0; o >>= 1) {
    s.x += __shfl_xor_sync(0xffffffffu, s.x, o);
    s.y += __shfl_xor_sync(0xffffffffu, s.y, o);
  }
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  z_t t = zmk(0.0, 0.0);
  for (int w = 0; w < (int)(blockDim.x >> 5); w++) t = zadd(t, red[w]);
  __syncthreads();
  return t;
}

// H = A + E X into shared memory
__device__ void form_h(z_t* H, const z_t* A, const z_t* X, double E, int nC) {
  for (int e = threadIdx.x; e < nC * nC; e += blockDim.x) H[e] = zadd(A[e], zscale(X[e], E));
  __syncthreads();
}

// One RK4 step C <- R(-i dt H) C (u scratch 5 x nC)
__device__ void rk4_poly(z_t* C, const z_t* H, double dt, int nC, z_t* u) {
  const z_t z = zmk(0.0, -dt);
  for (int i = threadIdx.x; i < nC; i += blockDim.x) u[i] = C[i];
  __syncthreads();
  for (int p = 1; p <= 4; p++) mat_vec(u + p * nC, H, u + (p - 1) * nC, nC, z);
  const double f[5] = {1.0, 1.0, 0.5, 1.0 / 6.0, 1.0 / 24.0};
  for (int i = threadIdx.x; i < nC; i += blockDim.x) {
    z_t s = zmk(0.0, 0.0);
    for (int p = 0; p <= 4; p++) s = zadd(s, zscale(u[p * nC + i], f[p]));
    C[i] = s;
  }
  __syncthreads();
}

// Forward sweep (checkpoints every K steps, final state, a) and, with grad,
// the backward sweep producing dJ/dE_n.  One CTA; A and X in global memory,
// copied to shared memory.
__global__ void __launch_bounds__(ADJ_THREADS, 1)
    k_adj_run(const z_t* __restrict__ Ag, const z_t* __restrict__ Xg, const z_t* __restrict__ C0,
              const double* __restrict__ E, int nT, double dt, int K, int nC, z_t* __restrict__ ckpt,
              z_t* __restrict__ seg, z_t* __restrict__ CN, double* __restrict__ out, double* __restrict__ grad) {
  extern __shared__ z_t smA[];
  z_t* A = smA;                   // nC^2
  z_t* X = A + nC * nC;           // nC^2
  z_t* H = X + nC * nC;           // nC^2
  z_t* C = H + nC * nC;           // nC
  z_t* u = C + nC;                // 5 nC (u_0..u_4)
  z_t* w = u + 5 * nC;            // 5 nC (w_0..w_4)
  z_t* Bu = w + 5 * nC;           // 4 nC
  z_t* mu = Bu + 4 * nC;          // nC
  __shared__ z_t red[ADJ_THREADS / 32];
  for (int e = threadIdx.x; e < nC * nC; e += blockDim.x) {
    A[e] = Ag[e];
    X[e] = Xg[e];
  }
  for (int i = threadIdx.x; i < nC; i += blockDim.x) C[i] = C0[i];
  __syncthreads();
  // forward
  for (int n = 0; n < nT; n++) {
    if (n % K == 0)
      for (int i = threadIdx.x; i < nC; i += blockDim.x) ckpt[(size_t)(n / K) * nC + i] = C[i];
    form_h(H, A, X, E[n], nC);
    rk4_poly(C, H, dt, nC, u);
  }
  for (int i = threadIdx.x; i < nC; i += blockDim.x) CN[i] = C[i];
  z_t a = dotc(C0, C, nC, red);
  if (threadIdx.x == 0) {
    out[0] = 1.0 - (a.x * a.x + a.y * a.y);
    out[1] = a.x;
    out[2] = a.y;
  }
  if (!grad) return;
  // backward: mu_N = C0
  for (int i = threadIdx.x; i < nC; i += blockDim.x) mu[i] = C0[i];
  __syncthreads();
  const double fact[5] = {1.0, 1.0, 2.0, 6.0, 24.0};
  const int nSeg = (nT + K - 1) / K;
  for (int s = nSeg - 1; s >= 0; s--) {
    const int n0 = s * K, n1 = min(nT, n0 + K);
    // recompute the segment's states from its checkpoint: seg[j] = C_{n0+j}
    for (int i = threadIdx.x; i < nC; i += blockDim.x) C[i] = ckpt[(size_t)s * nC + i];
    __syncthreads();
    for (int n = n0; n < n1; n++) {
      for (int i = threadIdx.x; i < nC; i += blockDim.x) seg[(size_t)(n - n0) * nC + i] = C[i];
      __syncthreads();
      if (n + 1 < n1) {
        form_h(H, A, X, E[n], nC);
        rk4_poly(C, H, dt, nC, u);
      }
    }
    for (int n = n1 - 1; n >= n0; n--) {
      form_h(H, A, X, E[n], nC);
      // u_q = z^q C_n (q <= 3), X u_q
      for (int i = threadIdx.x; i < nC; i += blockDim.x) u[i] = seg[(size_t)(n - n0) * nC + i];
      __syncthreads();
      for (int q = 1; q <= 3; q++) mat_vec(u + q * nC, H, u + (q - 1) * nC, nC, zmk(0.0, -dt));
      for (int q = 0; q <= 3; q++) mat_vec(Bu + q * nC, X, u + q * nC, nC, zmk(1.0, 0.0));
      // w_m = (z^H)^m mu_{n+1} = (i dt H^H)^m mu_{n+1} (m <= 4)
      for (int i = threadIdx.x; i < nC; i += blockDim.x) w[i] = mu[i];
      __syncthreads();
      for (int m = 1; m <= 4; m++) mat_vec_h(w + m * nC, H, w + (m - 1) * nC, nC, zmk(0.0, dt));
      // da/dE_n
      z_t da = zmk(0.0, 0.0);
      for (int m = 0; m <= 3; m++)
        for (int q = 0; m + q <= 3; q++) da = zadd(da, zscale(dotc(w + m * nC, Bu + q * nC, nC, red), 1.0 / fact[m + q + 1]));
      da = zmul(zmk(0.0, -dt), da);
      if (threadIdx.x == 0) grad[n] = -2.0 * (a.x * da.x + a.y * da.y);  // -2 Re(conj(a) da)
      // mu_n = R^H mu_{n+1} = sum_m w_m / m!
      for (int i = threadIdx.x; i < nC; i += blockDim.x) {
        z_t sum = zmk(0.0, 0.0);
        for (int m = 0; m <= 4; m++) sum = zadd(sum, zscale(w[m * nC + i], 1.0 / fact[m]));
        mu[i] = sum;
      }
      __syncthreads();
    }
  }
}

}  // namespace

// Dense A (zero field) and X (dipole) for the TDCI context's orbitals; returns them on the device.
void adjoint_matrices(cgpu_ctx* c, z_t* A, z_t* X) {
  const int nG = c->nG, nOS = c->nOS;
  // X: h1 = <phi_i| x |phi_j>_w, no two-body part
  k_x_orbs<<<ew_blocks(c, (size_t)nG * nOS), 256, 0, c->stream>>>(c->orbTmp_d, c->tdciOrbs_d, c->x_d, nG, nOS);
  CODY_LAUNCHED(c);
  launch_fill_h1_from(c, c->tdciOrbs_d, c->orbTmp_d, c->h1_d);
  launch_fold_h1(c);
  k_ci_dense<<<1, 128, 0, c->stream>>>(X, c->h1Lin_d, c->h2Lin_d, TRAJ_PASS(c), 1, 0);
  CODY_LAUNCHED(c);
  // A: one-body part at zero field (a time before the pulse or the samples start) plus h2
  const SysHost& s = c->sys[0];
  const double tz = -1.0 - std::fabs(s.sampleT0) - std::fabs(s.tStart);
  c->useStepTime = 0;
  launch_onebody(c, c->orbTmp_d, c->tdciOrbs_d, tz, zmk(1.0, 0.0), 0);
  launch_fill_h1_from(c, c->tdciOrbs_d, c->orbTmp_d, c->h1_d);
  launch_fill_h2(c, c->tdciOrbs_d);
  launch_fold_h1(c);
  launch_fold_h2(c);
  k_ci_dense<<<1, 128, 0, c->stream>>>(A, c->h1Lin_d, c->h2Lin_d, TRAJ_PASS(c), 1, 1);
  CODY_LAUNCHED(c);
}

// J, a = C0^H C_N, C_N and (grad != nullptr) dJ/dE_n for the sampled field E (nT steps of dt).
void adjoint_tdci(cgpu_ctx* c, const z_t* C0_h, const double* E_h, int nT, double dt, int K, double* J,
                  double* aOut, z_t* CN_h, double* grad_h) {
  if (c->method != CGPU_METHOD_TDCI || c->nb != 1) throw std::string("adjoint: needs a single TDCI context");
  const int nC = c->nC;
  if (nC > ADJ_MAXC) throw std::string("adjoint: at most 64 configurations");
  if (nT <= 0 || K <= 0 || !(dt > 0.0)) throw std::string("adjoint: bad step arguments");
  const int nSeg = (nT + K - 1) / K;
  size_t bytes = sizeof(z_t) * ((size_t)2 * nC * nC + (size_t)nC * (2 + nSeg + K)) +
                 sizeof(double) * ((size_t)(grad_h ? 2 : 1) * nT + 3);
  char* buf = nullptr;
  const size_t slack = 16 * 256;  // rounding of the sub-buffers to 256 bytes
  CODY_CUDA(cudaMalloc(&buf, bytes + slack));
  auto at = [&](size_t& off, size_t n) { char* p = buf + off; off += (n + 255) & ~(size_t)255; return p; };
  size_t off = 0;
  z_t* A = (z_t*)at(off, sizeof(z_t) * nC * nC);
  z_t* X = (z_t*)at(off, sizeof(z_t) * nC * nC);
  z_t* C0 = (z_t*)at(off, sizeof(z_t) * nC);
  z_t* CN = (z_t*)at(off, sizeof(z_t) * nC);
  z_t* ckpt = (z_t*)at(off, sizeof(z_t) * nC * nSeg);
  z_t* seg = (z_t*)at(off, sizeof(z_t) * nC * K);
  double* E = (double*)at(off, sizeof(double) * nT);
  double* out = (double*)at(off, sizeof(double) * 3);
  double* grad = grad_h ? (double*)at(off, sizeof(double) * nT) : nullptr;
  try {
    if (off > bytes + slack) throw std::string("internal: adjoint scratch");
    adjoint_matrices(c, A, X);
    CODY_CUDA(cudaMemcpyAsync(C0, C0_h, sizeof(z_t) * nC, cudaMemcpyHostToDevice, c->stream));
    CODY_CUDA(cudaMemcpyAsync(E, E_h, sizeof(double) * nT, cudaMemcpyHostToDevice, c->stream));
    size_t smem = sizeof(z_t) * ((size_t)3 * nC * nC + (size_t)16 * nC);
    static bool attr = false;
    if (!attr) {
      CODY_CUDA(cudaFuncSetAttribute(k_adj_run, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)(sizeof(z_t) * (3 * ADJ_MAXC * ADJ_MAXC + 16 * ADJ_MAXC))));
      attr = true;
    }
    k_adj_run<<<1, ADJ_THREADS, smem, c->stream>>>(A, X, C0, E, nT, dt, K, nC, ckpt, seg, CN, out, grad);
    CODY_LAUNCHED(c);
    double o[3];
    CODY_CUDA(cudaMemcpyAsync(o, out, sizeof(o), cudaMemcpyDeviceToHost, c->stream));
    if (CN_h) CODY_CUDA(cudaMemcpyAsync(CN_h, CN, sizeof(z_t) * nC, cudaMemcpyDeviceToHost, c->stream));
    if (grad_h) CODY_CUDA(cudaMemcpyAsync(grad_h, grad, sizeof(double) * nT, cudaMemcpyDeviceToHost, c->stream));
    CODY_CUDA(cudaStreamSynchronize(c->stream));
    *J = o[0];
    if (aOut) {
      aOut[0] = o[1];
      aOut[1] = o[2];
    }
    // restore the context's TDCI integrals at t = 0
    launch_onebody(c, c->orbTmp_d, c->tdciOrbs_d, 0.0, zmk(1.0, 0.0), 0);
    launch_fill_h1_from(c, c->tdciOrbs_d, c->orbTmp_d, c->h1_d);
    launch_fill_h2(c, c->tdciOrbs_d);
    launch_fold_h1(c);
    launch_fold_h2(c);
    CODY_CUDA(cudaStreamSynchronize(c->stream));
  } catch (...) {
    cudaFree(buf);
    throw;
  }
  cudaFree(buf);
}
