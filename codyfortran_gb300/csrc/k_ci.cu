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

#include "common.cuh"

namespace {

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

__global__ void k_ci_apply(CiView v, const z_t* __restrict__ C, z_t* __restrict__ dC, const z_t* __restrict__ h1Lin,
                           const z_t* __restrict__ h2Lin, int useH1, int useH2) {
  int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  int lane = threadIdx.x & 31;
  if (warp >= v.nC) return;
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
        z_t hc = zmul(h1Lin[oc], C[jG - 1]);
        if (v.sFac[b][col + k] < 0) hc = zmk(-hc.x, -hc.y);
        acc = zadd(acc, hc);
      }
    }
    if (useH2) {
      int n = v.dN[b][c - 1];
      size_t col = (size_t)v.maxD[b] * (c - 1);
      for (int k = lane; k < n; k += 32) {
        int oc = v.dCode[b][col + k];
        int jG = I + (v.dExc[b][col + k] - c) * st;
        z_t hc = zmul(h2Lin[oc], C[jG - 1]);
        if (v.dFac[b][col + k] < 0) hc = zmk(-hc.x, -hc.y);
        acc = zadd(acc, hc);
      }
      // inter-body-type terms: products of singles on b and b2 > b (Generic :266-300)
      int n1 = v.sN[b][c - 1];
      size_t col1 = (size_t)v.maxS[b] * (c - 1);
      for (int b2 = b + 1; b2 < v.nBt; b2++) {
        int c2 = conf[b2];
        int n2 = v.sN[b2][c2 - 1];
        size_t col2 = (size_t)v.maxS[b2] * (c2 - 1);
        int st2 = v.stride[b2];
        for (int t = lane; t < n1 * n2; t += 32) {
          int k1 = t / n2, k2 = t % n2;
          int oc = (v.sCode[b][col1 + k1] - 1) * nO2 + v.sCode[b2][col2 + k2];
          int jG = I + (v.sExc[b][col1 + k1] - c) * st + (v.sExc[b2][col2 + k2] - c2) * st2;
          z_t hc = zmul(h2Lin[oc], C[jG - 1]);
          if ((v.sFac[b][col1 + k1] * v.sFac[b2][col2 + k2]) < 0) hc = zmk(-hc.x, -hc.y);
          acc = zadd(acc, hc);
        }
      }
    }
  }
  acc = warp_sum(acc);
  if (lane == 0) dC[warp] = zadd(dC[warp], acc);
}

__device__ __forceinline__ void atomic_zadd(z_t* p, z_t v) {
  atomicAdd(&p->x, v.x);
  atomicAdd(&p->y, v.y);
}

__global__ void k_ci_rdm(CiView v, const z_t* __restrict__ C, z_t* __restrict__ r1Lin, z_t* __restrict__ r2Lin,
                         int want1, int want2) {
  int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  int lane = threadIdx.x & 31;
  if (warp >= v.nC) return;
  int I = warp + 1;
  int conf[CODY_MAX_BT];
  conf_from_index(v, I, conf);
  z_t cI = C[warp];
  if (cI.x == 0.0 && cI.y == 0.0) return;  // every contribution carries the factor C_I
  int nO2 = v.nO * v.nO;
  for (int b = 0; b < v.nBt; b++) {
    int c = conf[b];
    int st = v.stride[b];
    if (want1) {
      int n = v.sN[b][c - 1];
      size_t col = (size_t)v.maxS[b] * (c - 1);
      for (int k = lane; k < n; k += 32) {
        int oc = v.sCode[b][col + k];
        int jG = I + (v.sExc[b][col + k] - c) * st;
        z_t r = zcmul(C[jG - 1], cI);
        if (v.sFac[b][col + k] < 0) r = zmk(-r.x, -r.y);
        atomic_zadd(&r1Lin[oc], r);
      }
    }
    if (want2) {
      int n = v.dN[b][c - 1];
      size_t col = (size_t)v.maxD[b] * (c - 1);
      for (int k = lane; k < n; k += 32) {
        int oc = v.dCode[b][col + k];
        int jG = I + (v.dExc[b][col + k] - c) * st;
        z_t r = zcmul(C[jG - 1], cI);
        if (v.dFac[b][col + k] < 0) r = zmk(-r.x, -r.y);
        atomic_zadd(&r2Lin[oc], r);
      }
      int n1 = v.sN[b][c - 1];
      size_t col1 = (size_t)v.maxS[b] * (c - 1);
      for (int b2 = b + 1; b2 < v.nBt; b2++) {
        int c2 = conf[b2];
        int n2 = v.sN[b2][c2 - 1];
        size_t col2 = (size_t)v.maxS[b2] * (c2 - 1);
        int st2 = v.stride[b2];
        for (int t = lane; t < n1 * n2; t += 32) {
          int k1 = t / n2, k2 = t % n2;
          int oc = (v.sCode[b][col1 + k1] - 1) * nO2 + v.sCode[b2][col2 + k2];
          int jG = I + (v.sExc[b][col1 + k1] - c) * st + (v.sExc[b2][col2 + k2] - c2) * st2;
          z_t r = zcmul(C[jG - 1], cI);
          if ((v.sFac[b][col1 + k1] * v.sFac[b2][col2 + k2]) < 0) r = zmk(-r.x, -r.y);
          atomic_zadd(&r2Lin[oc], r);
        }
      }
    }
  }
}

// FillH1Lin: h1Lin((i1-1)*nO + j1) = h1(i1, j1)
__global__ void k_fold_h1(z_t* __restrict__ h1Lin, const z_t* __restrict__ h1, int nO) {
  int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= nO * nO) return;
  int i1 = e % nO, j1 = e / nO;  // 0-based
  h1Lin[i1 * nO + j1 + 1] = h1[e];
}

__device__ __forceinline__ bool bt_rule_ok(const int* btOf, int i1, int i2, int j1, int j2) {
  int bi1 = btOf[i1], bi2 = btOf[i2], bj1 = btOf[j1], bj2 = btOf[j2];
  if (bi1 == bi2 && bj1 != bj2) return false;
  if (bi1 != bi2 && bj1 == bj2) return false;
  return true;
}

// FillH2Lin (fermions; inter-body-type pairs use the same antisymmetric form)
__global__ void k_fold_h2(z_t* __restrict__ h2Lin, const z_t* __restrict__ h2, const int* __restrict__ btOf, int nO) {
  size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  size_t n4 = (size_t)nO * nO * nO * nO;
  if (e >= n4) return;
  // e = orbCode - 1 with orbCode = (((i1-1) nO + j1 - 1) nO + i2 - 1) nO + j2
  int j2 = (int)(e % nO), i2 = (int)((e / nO) % nO), j1 = (int)((e / nO / nO) % nO), i1 = (int)(e / nO / nO / nO);
  z_t v = zmk(0.0, 0.0);
  if (i1 <= i2 && j1 <= j2 && bt_rule_ok(btOf, i1, i2, j1, j2) && i1 != i2 && j1 != j2) {
    size_t n = nO;
    auto H = [&](int a, int b, int c, int d) { return h2[a + n * (b + n * (c + n * d))]; };
    v = zadd(zsub(zsub(H(i1, i2, j1, j2), H(i1, i2, j2, j1)), H(i2, i1, j1, j2)), H(i2, i1, j2, j1));
  }
  h2Lin[e + 1] = v;
}

__global__ void k_unfold_rdm1(z_t* __restrict__ rdm1, const z_t* __restrict__ lin, int nO) {
  int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= nO * nO) return;
  int i1 = e % nO, j1 = e / nO;
  rdm1[e] = lin[i1 * nO + j1 + 1];
}

// FillRdm2FromRdm2Lin written per output element: rdm2(a,b,c,d) gathers the
// (up to four) signed lin entries the reference scatters into it.
__global__ void k_unfold_rdm2(z_t* __restrict__ rdm2, const z_t* __restrict__ lin, const int* __restrict__ btOf,
                              int nO) {
  size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  size_t n = nO;
  if (e >= n * n * n * n) return;
  int a = (int)(e % n), b = (int)((e / n) % n), c = (int)((e / n / n) % n), d = (int)(e / n / n / n);
  auto L = [&](int i1, int j1, int i2, int j2) { return lin[(((size_t)i1 * n + j1) * n + i2) * n + j2 + 1]; };
  z_t s = zmk(0.0, 0.0);
  if (a <= b && c <= d && bt_rule_ok(btOf, a, b, c, d)) s = zadd(s, L(a, c, b, d));
  if (b <= a && c <= d && bt_rule_ok(btOf, b, a, c, d)) s = zsub(s, L(b, c, a, d));
  if (a <= b && d <= c && bt_rule_ok(btOf, a, b, d, c)) s = zsub(s, L(a, d, b, c));
  if (b <= a && d <= c && bt_rule_ok(btOf, b, a, d, c)) s = zadd(s, L(b, d, a, c));
  rdm2[e] = s;
}

long long binom_h(int n, int k) {
  if (k < 0 || n < 0 || k > n) return (n == k) ? 1 : 0;
  long double r = 1.0;
  for (int i = 1; i <= k; i++) r = r * (n - k + i) / i;
  return (long long)llroundl(r);
}

}  // namespace

// ConfigList_Setup: codes in GSL lexicographic order on the host, tables on the device.
void ci_build_tables(cgpu_ctx* c) {
  c->view.nBt = c->nBt;
  c->view.nO = c->nO;
  int stride = 1;
  for (int b = 0; b < c->nBt; b++) {
    CiTables& t = c->tab[b];
    int M = c->nOrbs[b], N = c->nBodies[b];
    t.nOrbs = M;
    t.nBodies = N;
    t.shift = c->orbStart[b];
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
      k_build_tables<<<blocks, threads, 0, c->stream>>>(kind, 0, t.codes, t.nConf, M, c->nO, t.shift, t.rankTab,
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
      k_build_tables<<<blocks, threads, 0, c->stream>>>(kind, 1, t.codes, t.nConf, M, c->nO, t.shift, t.rankTab,
                                                         rankBase, nConn, mxa, *exc, *oc, *fac);
      CODY_LAUNCHED(c);
      if (kind == 0) t.maxS = mx; else t.maxD = mx;
    }
    CiView& v = c->view;
    v.stride[b] = stride;
    v.nConf[b] = t.nConf;
    v.maxS[b] = std::max(t.maxS, 1);
    v.maxD[b] = std::max(t.maxD, 1);
    v.sN[b] = t.sN; v.sExc[b] = t.sExc; v.sCode[b] = t.sCode; v.sFac[b] = t.sFac;
    v.dN[b] = t.dN; v.dExc[b] = t.dExc; v.dCode[b] = t.dCode; v.dFac[b] = t.dFac;
    stride *= t.nConf;
  }
  c->view.nC = stride;
  CODY_CUDA(cudaStreamSynchronize(c->stream));
}

void launch_ci_apply(cgpu_ctx* c, const z_t* C, z_t* dC, int useH1, int useH2) {
  ProfScope prof(c, CGPU_KERNEL_CI_APPLY);
  int threads = 256;
  int blocks = (int)(((size_t)c->nC * 32 + threads - 1) / threads);
  k_ci_apply<<<blocks, threads, 0, c->stream>>>(c->view, C, dC, c->h1Lin_d, c->h2Lin_d, useH1, useH2);
  CODY_LAUNCHED(c);
}

void launch_ci_rdm(cgpu_ctx* c, const z_t* C, int want1, int want2) {
  ProfScope prof(c, CGPU_KERNEL_CI_RDM);
  size_t n2 = (size_t)c->nO * c->nO, n4 = n2 * n2;
  if (want1) CODY_CUDA(cudaMemsetAsync(c->rdm1Lin_d, 0, sizeof(z_t) * (n2 + 1), c->stream));
  if (want2) CODY_CUDA(cudaMemsetAsync(c->rdm2Lin_d, 0, sizeof(z_t) * (n4 + 1), c->stream));
  int threads = 256;
  int blocks = (int)(((size_t)c->nC * 32 + threads - 1) / threads);
  k_ci_rdm<<<blocks, threads, 0, c->stream>>>(c->view, C, c->rdm1Lin_d, c->rdm2Lin_d, want1, want2);
  CODY_LAUNCHED(c);
  if (want1) {
    k_unfold_rdm1<<<(int)((n2 + 255) / 256), 256, 0, c->stream>>>(c->rdm1_d, c->rdm1Lin_d, c->nO);
    CODY_LAUNCHED(c);
  }
  if (want2) {
    k_unfold_rdm2<<<(int)((n4 + 255) / 256), 256, 0, c->stream>>>(c->rdm2_d, c->rdm2Lin_d, c->btOfOrb_d, c->nO);
    CODY_LAUNCHED(c);
  }
}

void launch_fold_h1(cgpu_ctx* c) {
  int n2 = c->nO * c->nO;
  k_fold_h1<<<(n2 + 255) / 256, 256, 0, c->stream>>>(c->h1Lin_d, c->h1_d, c->nO);
  CODY_LAUNCHED(c);
}

void launch_fold_h2(cgpu_ctx* c) {
  size_t n4 = (size_t)c->nO * c->nO * c->nO * c->nO;
  k_fold_h2<<<(int)((n4 + 255) / 256), 256, 0, c->stream>>>(c->h2Lin_d, c->h2_d, c->btOfOrb_d, c->nO);
  CODY_LAUNCHED(c);
}
