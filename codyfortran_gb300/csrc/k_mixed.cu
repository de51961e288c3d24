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
#include <cuda_bf16.h>

#include <algorithm>

#include "common.cuh"
#include "tc.cuh"

struct MixedBufs {
  int terms = 3;            // 3: bf16x3, 6: bf16x6
  int Kg = 0, Kp = 0;       // padded K of the grid contraction and of the pair contraction
  __nv_bfloat16 *VxB = nullptr, *SxA = nullptr, *WxA = nullptr, *WTxB = nullptr, *RxB = nullptr;
  float *P1 = nullptr, *P2 = nullptr, *P3 = nullptr;
  size_t cap1 = 0, cap2 = 0, cap3 = 0;
  int* err = nullptr;
  double* Zd = nullptr;     // (nG, Q) complex
  double* Gd = nullptr;     // (2P, 2P)
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

// out[row][seg*Kpad + k] = part(value(row,k)), zero for k >= K.
__device__ __forceinline__ void write_split(__nv_bfloat16* out, int row, int k, int K, int Kpad, int terms, int isB,
                                            double v) {
  size_t base = (size_t)row * terms * Kpad;
  for (int seg = 0; seg < terms; seg++) {
    __nv_bfloat16 h = (k < K) ? split_part(v, terms, seg_part(terms, isB, seg)) : __double2bfloat16(0.0);
    out[base + (size_t)seg * Kpad + k] = h;
  }
}

__global__ void k_split_V(__nv_bfloat16* __restrict__ out, const double* __restrict__ V, int nG, int Kpad, int terms) {
  size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (e >= (size_t)nG * Kpad) return;
  int row = (int)(e / Kpad), k = (int)(e % Kpad);
  double v = (k < nG) ? V[(size_t)row * nG + k] : 0.0;
  write_split(out, row, k, nG, Kpad, terms, 1, v);
}

// S_s(p, g) = (re, im)[conj(phi_l) phi_k w] for pair p = (l, k), A pattern.
__global__ void k_split_S(__nv_bfloat16* __restrict__ outA, const z_t* __restrict__ orbs, const double* __restrict__ w, const int* __restrict__ pl,
                          const int* __restrict__ pk, int nG, int nP, int Kpad, int terms) {
  size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (e >= (size_t)2 * nP * Kpad) return;
  int row = (int)(e / Kpad), g = (int)(e % Kpad);
  int p = row >> 1, s = row & 1;
  double v = 0.0;
  if (g < nG) {
    z_t a = orbs[(size_t)nG * pl[p] + g], b = orbs[(size_t)nG * pk[p] + g];
    z_t sv = zscale(zcmul(a, b), w[g]);
    v = s ? sv.y : sv.x;
  }
  write_split(outA, row, g, nG, Kpad, terms, 0, v);
}

// W[g][n] = sum_z P1[z][g][n] (FP64), split to WxA (g-major, K = 2P) and WTxB (pair-major, K = nG).
__global__ void k_split_W(__nv_bfloat16* __restrict__ WxA, __nv_bfloat16* __restrict__ WTxB,
                          const float* __restrict__ P1, int nSplit, int nG, int N2P, int KpP, int KpG, int terms) {
  size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (e >= (size_t)nG * KpP) return;
  int g = (int)(e / KpP), n = (int)(e % KpP);
  double v = 0.0;
  if (n < N2P)
    for (int z = 0; z < nSplit; z++) v += (double)P1[((size_t)z * nG + g) * N2P + n];
  write_split(WxA, g, n, N2P, KpP, terms, 0, v);
  if (n < N2P) write_split(WTxB, n, g, nG, KpG, terms, 1, v);
}

// zero the K padding columns of WTxB (g in [nG, KpG)) for every pair row
__global__ void k_pad_WT(__nv_bfloat16* __restrict__ WTxB, int nG, int N2P, int KpG, int terms) {
  int pad = KpG - nG;
  size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (e >= (size_t)N2P * pad) return;
  int n = (int)(e / pad), g = nG + (int)(e % pad);
  write_split(WTxB, n, g, nG, KpG, terms, 1, 0.0);
}

// R'' rows n = 2q + s (s: re/im of the output), K = 2p + t (t: a or b of W_p).
__global__ void k_split_R(__nv_bfloat16* __restrict__ RxB, const z_t* __restrict__ Rp, const int* __restrict__ pl,
                          const int* __restrict__ pk, int n, int nP, int KpP, int terms) {
  int Q = n * n;
  size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (e >= (size_t)2 * Q * KpP) return;
  int row = (int)(e / KpP), k = (int)(e % KpP);
  int q = row >> 1, s = row & 1;
  double v = 0.0;
  if (k < 2 * nP) {
    int p = k >> 1, t = k & 1;
    int l = pl[p], kk = pk[p];
    z_t R1 = Rp[(size_t)(l * n + kk) * Q + q];
    z_t R2 = (l < kk) ? Rp[(size_t)(kk * n + l) * Q + q] : zmk(0.0, 0.0);
    z_t X = zadd(R1, R2);
    z_t D = zsub(R1, R2);
    z_t Y = zmk(-D.y, D.x);
    z_t val = t ? Y : X;
    v = s ? val.y : val.x;
  }
  write_split(RxB, row, k, 2 * nP, KpP, terms, 1, v);
}

// Z[g][q] (complex) = sum_z P2[z][g][2q+s]
__global__ void k_reduce_Z(z_t* __restrict__ Z, const float* __restrict__ P2, int nSplit, int nG, int Q) {
  size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (e >= (size_t)nG * Q) return;
  int g = (int)(e / Q), q = (int)(e % Q);
  double re = 0.0, im = 0.0;
  for (int z = 0; z < nSplit; z++) {
    const float* r = P2 + ((size_t)z * nG + g) * 2 * Q + 2 * q;
    re += (double)r[0];
    im += (double)r[1];
  }
  Z[e] = zmk(re, im);
}

// H2s[(i1*n+j1)][(l2*n+k2)] = 1/2 sum_g S_(i1j1) W_(l2k2) from the unordered-pair products.
__global__ void k_reduce_H2(z_t* __restrict__ H2s, const float* __restrict__ P3, int nSplit, const int* __restrict__ pidx,
                            int n, int nP) {
  int Q = n * n;
  size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (e >= (size_t)Q * Q) return;
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
      const float* G = P3 + (size_t)z * N2 * N2;
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

template <typename T>
T* dalloc_t(size_t n) {
  T* p = nullptr;
  CODY_CUDA(cudaMalloc(&p, std::max<size_t>(n, 1) * sizeof(T)));
  return p;
}

int blocks(size_t n) { return (int)((n + 255) / 256); }

}  // namespace

void mixed_free(cgpu_ctx* c) {
  MixedBufs* m = c->mixed;
  if (!m) return;
  void* ptrs[] = {m->VxB, m->SxA, m->WxA, m->WTxB, m->RxB, m->P1, m->P2, m->P3, m->err, m->Zd, m->Gd};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  delete m;
  c->mixed = nullptr;
}

void mixed_setup(cgpu_ctx* c) {
  if (c->mixed || !c->hasInteraction) return;
  MixedBufs* m = new MixedBufs();
  c->mixed = m;
  m->terms = c->precision == CGPU_PREC_MIXED_X6 ? 6 : 3;
  int nG = c->nG, nP = c->nPairs, n = c->nOS, Q = n * n, T = m->terms;
  m->Kg = (nG + 63) / 64 * 64;
  m->Kp = (2 * nP + 63) / 64 * 64;
  m->VxB = dalloc_t<__nv_bfloat16>((size_t)nG * T * m->Kg);
  m->SxA = dalloc_t<__nv_bfloat16>((size_t)2 * nP * T * m->Kg);
  m->WxA = dalloc_t<__nv_bfloat16>((size_t)nG * T * m->Kp);
  m->WTxB = dalloc_t<__nv_bfloat16>((size_t)2 * nP * T * m->Kg);
  m->RxB = dalloc_t<__nv_bfloat16>((size_t)2 * Q * T * m->Kp);
  m->err = dalloc_t<int>(1);
  CODY_CUDA(cudaMemset(m->err, 0, sizeof(int)));
  m->Zd = dalloc_t<double>((size_t)2 * nG * Q);
  // split-K partial buffers sized for the splits the GEMMs will use
  int kt1 = T * m->Kg / 64, kt2 = T * m->Kp / 64;
  int s1 = tc_split_count(nG, 2 * nP, tc_tile_n(2 * nP), kt1);
  int s2 = tc_split_count(nG, 2 * Q, tc_tile_n(2 * Q), kt2);
  int s3 = tc_split_count(2 * nP, 2 * nP, tc_tile_n(2 * nP), kt1);
  m->cap1 = (size_t)s1 * nG * 2 * nP;
  m->cap2 = (size_t)s2 * nG * 2 * Q;
  m->cap3 = (size_t)s3 * 2 * nP * 2 * nP;
  m->P1 = dalloc_t<float>(m->cap1);
  m->P2 = dalloc_t<float>(m->cap2);
  m->P3 = dalloc_t<float>(m->cap3);
  k_split_V<<<blocks((size_t)nG * m->Kg), 256, 0, c->stream>>>(m->VxB, c->Vint_d, nG, m->Kg, T);
  CODY_LAUNCHED(c);
  CODY_CUDA(cudaStreamSynchronize(c->stream));
}

int mixed_error(cgpu_ctx* c) {
  if (!c->mixed) return 0;
  int e = 0;
  CODY_CUDA(cudaMemcpy(&e, c->mixed->err, sizeof(int), cudaMemcpyDeviceToHost));
  return e;
}

// ApplyCorrelationOp in the mixed form: dOrbs += rho^-1 rho2 W phi; h2 (FP64 nO^4) when wantH2.
void launch_correlation_mixed(cgpu_ctx* c, z_t* dOrbs, const z_t* orbs, int wantH2) {
  launch_rdm_inverse(c);
  if (!c->hasInteraction) {
    if (wantH2) CODY_CUDA(cudaMemsetAsync(c->h2_d, 0, sizeof(z_t) * (size_t)c->nO * c->nO * c->nO * c->nO, c->stream));
    return;
  }
  mixed_setup(c);
  MixedBufs* m = c->mixed;
  int nG = c->nG, nP = c->nPairs, n = c->nOS, Q = n * n, T = m->terms;
  int K1 = T * m->Kg, K2 = T * m->Kp;
  {
    ProfScope prof(c, CGPU_KERNEL_PAIR_POTENTIALS);
    k_split_S<<<blocks((size_t)2 * nP * m->Kg), 256, 0, c->stream>>>(m->SxA, orbs, c->w_d, c->pairL_d, c->pairK_d,
                                                                      nG, nP, m->Kg, T);
    CODY_LAUNCHED(c);
    int s1 = tc_split_count(nG, 2 * nP, tc_tile_n(2 * nP), K1 / 64);
    // V carries the B split pattern, S the A pattern: hi*hi + lo*hi + hi*lo (x3)
    s1 = tc_gemm(c, m->VxB, nG, m->SxA, 2 * nP, K1, m->P1, s1, m->err);
    k_split_W<<<blocks((size_t)nG * m->Kp), 256, 0, c->stream>>>(m->WxA, m->WTxB, m->P1, s1, nG, 2 * nP, m->Kp,
                                                                  m->Kg, T);
    CODY_LAUNCHED(c);
    if (m->Kg > nG) {
      k_pad_WT<<<blocks((size_t)2 * nP * (m->Kg - nG)), 256, 0, c->stream>>>(m->WTxB, nG, 2 * nP, m->Kg, T);
      CODY_LAUNCHED(c);
    }
  }
  {
    ProfScope prof(c, CGPU_KERNEL_CORRELATION);
    k_split_R<<<blocks((size_t)2 * Q * m->Kp), 256, 0, c->stream>>>(m->RxB, c->Rp_d, c->pairL_d, c->pairK_d, n, nP,
                                                                     m->Kp, T);
    CODY_LAUNCHED(c);
    int s2 = tc_split_count(nG, 2 * Q, tc_tile_n(2 * Q), K2 / 64);
    s2 = tc_gemm(c, m->WxA, nG, m->RxB, 2 * Q, K2, m->P2, s2, m->err);
    z_t* Z = (z_t*)m->Zd;
    k_reduce_Z<<<blocks((size_t)nG * Q), 256, 0, c->stream>>>(Z, m->P2, s2, nG, Q);
    CODY_LAUNCHED(c);
    launch_corr_epilogue(c, dOrbs, orbs, Z);
  }
  if (wantH2) {
    ProfScope prof(c, CGPU_KERNEL_H2);
    int s3 = tc_split_count(2 * nP, 2 * nP, tc_tile_n(2 * nP), K1 / 64);
    s3 = tc_gemm(c, m->SxA, 2 * nP, m->WTxB, 2 * nP, K1, m->P3, s3, m->err);
    k_reduce_H2<<<blocks((size_t)Q * Q), 256, 0, c->stream>>>(c->h2s_d, m->P3, s3, c->pidx_d, n, nP);
    CODY_LAUNCHED(c);
    launch_h2_layout(c);
  }
}
