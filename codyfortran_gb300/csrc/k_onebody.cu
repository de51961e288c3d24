// k_onebody.cu -- streaming one-body kernels of the MCTDHX hot path.
//
//   * banded kinetic + soft-Yukawa + length-gauge apply (ApplySingleBodyOp,
//     src/Method/Mb/OrbBased/S_Method_Mb_OrbBased.f90:976-1034)
//   * weighted Gram matrices (Grid_InnerProduct, src/Grid/Linear/S_Grid_Linear.f90:53-61)
//     used by FillH1 (:164-224) and the (1-P) projector (src/Grid/S_Grid.f90:170-203)
//   * coefficient projection / normalisation (src/Coeffs/S_Coeffs.f90:84-111)
//   * MGS x2 orthonormalisation (src/Grid/S_Grid.f90:120-151)
//   * RK4 stage updates and the RDM energy contraction
//     (src/Utils/M_Utils_RdmObservables.f90:17-52)
//
// All reductions are deterministic: fixed grids, per-block partials in a
// fixed order, no floating-point atomics.
#include "common.cuh"

namespace {

constexpr int OB_THREADS = 256;
constexpr int RED_BLOCKS = 148;  // partial-sum blocks for grid reductions

// ---------------------------------------------------------------------------
// out[:, i] = alpha * ((T_bt + V0 + E x) orbs[:, i]) (+ out[:, i] if accumulate)
// T is stored as (2b+1) diagonals per body type: T[(bt*(2b+1) + d+b)*nG + g]
// multiplies orbs[g+d].  One CTA covers OB_THREADS grid points of one orbital;
// the tile and its halo are staged in shared memory.
// ---------------------------------------------------------------------------
// Laser field E(t): sin^2 pulse (pattern of src/SysPotential/Ylm/CoulombLaser/
// S_SysPotential_Ylm_CoulombLaser.f90:60-83) or piecewise-constant samples.
__device__ double field_amplitude_dev(const LaserDev& L, double t) {
  if (L.kind == CGPU_LASER_SIN2) {
    if (L.omega <= 0.0) return 0.0;
    const double PI = 3.14159265358979323846264338327950288;
    double duration = 2.0 * PI * L.nCycles / L.omega;
    double tRel = t - L.tStart;
    if (tRel < 0.0 || tRel > duration) return 0.0;
    double env = sin(PI * tRel / duration);
    env = env * env;
    return L.E0 * env * cos(L.omega * (tRel - 0.5 * duration) + L.cep);
  }
  if (L.kind == CGPU_LASER_SAMPLED) {
    double u = (t - L.sampleT0) / L.sampleDt;
    long n = (long)floor(u + 1e-9);
    if (n < 0 || n >= L.nSamples) return 0.0;
    return L.samples[n];
  }
  return 0.0;
}

__global__ void k_onebody(z_t* __restrict__ out, const z_t* __restrict__ orbs, const double* __restrict__ T,
                          const double* __restrict__ V0, const double* __restrict__ x, const int* __restrict__ btOf,
                          int nG, int band, int restricted, LaserDev laser, const double* __restrict__ tBase,
                          double tOff, int hasPot, z_t alpha, int accumulate) {
  extern __shared__ z_t sh[];
  __shared__ double Eshared;
  if (threadIdx.x == 0) Eshared = field_amplitude_dev(laser, *tBase + tOff);
  int i = blockIdx.y;
  int g0 = blockIdx.x * OB_THREADS;
  const z_t* f = orbs + (size_t)nG * i;
  int nTile = OB_THREADS + 2 * band;
  for (int t = threadIdx.x; t < nTile; t += OB_THREADS) {
    int g = g0 - band + t;
    sh[t] = (g >= 0 && g < nG) ? f[g] : zmk(0.0, 0.0);
  }
  __syncthreads();
  int g = g0 + threadIdx.x;
  if (g >= nG) return;
  int bt = restricted ? 0 : btOf[i];
  int nd = 2 * band + 1;
  const double* Tb = T + (size_t)bt * nd * nG;
  z_t acc = zmk(0.0, 0.0);
  for (int d = 0; d < nd; d++) {
    double c = Tb[(size_t)d * nG + g];
    z_t v = sh[threadIdx.x + d];
    acc.x = fma(c, v.x, acc.x);
    acc.y = fma(c, v.y, acc.y);
  }
  if (hasPot) {
    double pot = V0[g] + Eshared * x[g];
    z_t v = sh[threadIdx.x + band];
    acc.x = fma(pot, v.x, acc.x);
    acc.y = fma(pot, v.y, acc.y);
  }
  z_t r = zmul(alpha, acc);
  size_t o = (size_t)nG * i + g;
  if (accumulate) r = zadd(out[o], r);
  out[o] = r;
}

// ---------------------------------------------------------------------------
// Weighted Gram partials: part[blk][i + n*j] = sum_{g in chunks of blk}
//   conj(A[g, colA0+i]) * B[g, colB0+j] * w[g]
// ---------------------------------------------------------------------------
constexpr int GR_CHUNK = 32;
constexpr int GR_PER_THREAD = 16;  // 256 threads x 16 = 4096 = 64^2 Gram entries

__global__ void k_gram_partial(z_t* __restrict__ part, const z_t* __restrict__ A, const z_t* __restrict__ B,
                               const double* __restrict__ w, int nG, int n, int colA0, int colB0, int chunk) {
  extern __shared__ z_t sh[];
  z_t* sa = sh;                 // chunk x n
  z_t* sb = sh + chunk * n;     // chunk x n
  int nn = n * n;
  z_t acc[GR_PER_THREAD];
  for (int q = 0; q < GR_PER_THREAD; q++) acc[q] = zmk(0.0, 0.0);
  for (int c0 = blockIdx.x * chunk; c0 < nG; c0 += gridDim.x * chunk) {
    __syncthreads();
    for (int t = threadIdx.x; t < chunk * n; t += blockDim.x) {
      int col = t / chunk, r = t % chunk;
      int g = c0 + r;
      z_t a = zmk(0.0, 0.0), b = zmk(0.0, 0.0);
      if (g < nG) {
        a = A[(size_t)nG * (colA0 + col) + g];
        b = B[(size_t)nG * (colB0 + col) + g];
        b = zscale(b, w[g]);
      }
      sa[r * n + col] = a;
      sb[r * n + col] = b;
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < GR_PER_THREAD; q++) {
      int e = threadIdx.x + q * blockDim.x;
      if (e >= nn) break;
      int ii = e % n, jj = e / n;
      z_t s = acc[q];
      for (int r = 0; r < chunk; r++) {
        z_t a = sa[r * n + ii], b = sb[r * n + jj];
        s.x += a.x * b.x + a.y * b.y;
        s.y += a.x * b.y - a.y * b.x;
      }
      acc[q] = s;
    }
  }
#pragma unroll
  for (int q = 0; q < GR_PER_THREAD; q++) {
    int e = threadIdx.x + q * blockDim.x;
    if (e >= nn) break;
    part[(size_t)blockIdx.x * nn + e] = acc[q];
  }
}

// one warp per Gram entry, lanes over the block partials (fixed order)
__global__ void k_gram_final(z_t* __restrict__ G, const z_t* __restrict__ part, int nBlk, int n, int ldG,
                             double scale) {
  int e = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  int lane = threadIdx.x & 31;
  int nn = n * n;
  if (e >= nn) return;
  z_t s = zmk(0.0, 0.0);
  for (int b = lane; b < nBlk; b += 32) s = zadd(s, part[(size_t)b * nn + e]);
  for (int o = 16; o > 0; o >>= 1) {
    s.x += __shfl_xor_sync(0xffffffffu, s.x, o);
    s.y += __shfl_xor_sync(0xffffffffu, s.y, o);
  }
  if (lane == 0) {
    int i = e % n, j = e / n;
    G[i + (size_t)ldG * j] = zscale(s, scale);
  }
}

// dOrbs[:, c0+j] -= sum_i orbs[:, c0+i] * G[i + n*j]
__global__ void k_project_apply(z_t* __restrict__ dOrbs, const z_t* __restrict__ orbs, const z_t* __restrict__ G,
                                int nG, int n, int c0) {
  int g = blockIdx.x * blockDim.x + threadIdx.x;
  int j = blockIdx.y;
  if (g >= nG) return;
  z_t acc = zmk(0.0, 0.0);
  for (int i = 0; i < n; i++) zfma(acc, orbs[(size_t)nG * (c0 + i) + g], G[i + (size_t)n * j]);
  size_t o = (size_t)nG * (c0 + j) + g;
  dOrbs[o] = zsub(dOrbs[o], acc);
}

// h1 (nO x nO) from the stored-orbital Gram G (nOS x nOS): same body type only,
// restricted runs duplicate the block for the second spin (FillH1 :203-222).
__global__ void k_h1_layout(z_t* __restrict__ h1, const z_t* __restrict__ G, const int* __restrict__ btOf, int nO,
                            int nOS, int restricted) {
  int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= nO * nO) return;
  int i = e % nO, j = e / nO;
  z_t v = zmk(0.0, 0.0);
  if (restricted) {
    if ((i < nOS) == (j < nOS)) v = G[(i % nOS) + (size_t)nOS * (j % nOS)];
  } else {
    if (btOf[i] == btOf[j]) v = G[i + (size_t)nOS * j];
  }
  h1[e] = v;
}

// ---------------------------------------------------------------------------
// Vector kernels
// ---------------------------------------------------------------------------
__global__ void k_axpby(z_t* __restrict__ y, const z_t* __restrict__ x, z_t a, z_t b, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    z_t r = zmul(b, y[i]);
    zfma(r, a, x[i]);
    y[i] = r;
  }
}

__global__ void k_scale(z_t* __restrict__ y, z_t a, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    y[i] = zmul(a, y[i]);
}

// RK4 stage bookkeeping (S_IntegratorList_Rk_O4Expl.f90:109-135):
// inc = (first ? 0 : inc) + d*wInc; tmp = state + d*wTmp
__global__ void k_rk_stage(z_t* __restrict__ inc, z_t* __restrict__ tmp, const z_t* __restrict__ state,
                           const z_t* __restrict__ d, double wInc, double wTmp, int first, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    z_t di = d[i];
    z_t v = zscale(di, wInc);
    inc[i] = first ? v : zadd(inc[i], v);
    if (tmp) tmp[i] = zadd(state[i], zscale(di, wTmp));
  }
}

// block reduction helper (sum of complex)
__device__ z_t block_sum(z_t v) {
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
  return v;  // valid in thread 0
}

// part[blk] = sum conj(a) b over the block's stride
__global__ void k_dot_partial(z_t* __restrict__ part, const z_t* __restrict__ a, const z_t* __restrict__ b, size_t n) {
  z_t s = zmk(0.0, 0.0);
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    z_t u = a[i], v = b[i];
    s.x += u.x * v.x + u.y * v.y;
    s.y += u.x * v.y - u.y * v.x;
  }
  s = block_sum(s);
  if (threadIdx.x == 0) part[blockIdx.x] = s;
}

// dC -= (sum of partials) * C   (dot_product(coeffs, dCoeffs) = sum conj(C) dC)
__global__ void k_project_coeffs_apply(z_t* __restrict__ dC, const z_t* __restrict__ C, const z_t* __restrict__ part,
                                       int nBlk, size_t n) {
  __shared__ z_t ov[1];
  sum_partials(part, nBlk, 1, 1, ov);
  z_t o = ov[0];
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    z_t r = dC[i];
    z_t c = C[i];
    r.x -= o.x * c.x - o.y * c.y;
    r.y -= o.x * c.y + o.y * c.x;
    dC[i] = r;
  }
}

__global__ void k_normalize_apply(z_t* __restrict__ C, const z_t* __restrict__ part, int nBlk, size_t n) {
  __shared__ z_t tot[1];
  sum_partials(part, nBlk, 1, 1, tot);
  double nr = sqrt(tot[0].x);
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    z_t c = C[i];
    C[i] = zmk(c.x / nr, c.y / nr);
  }
}

// Modified Gram-Schmidt, two sweeps, one CTA (src/Grid/S_Grid.f90:120-151).
// Used only for relaxation / set-up, not in the real-time step.
__global__ void k_mgs2(z_t* __restrict__ f, const double* __restrict__ w, int nG, int c0, int n, int* status) {
  for (int i1 = c0; i1 < c0 + n; i1++) {
    for (int pass = 0; pass < 2; pass++)
      for (int j1 = c0; j1 < i1; j1++) {
        z_t s = zmk(0.0, 0.0);
        for (int g = threadIdx.x; g < nG; g += blockDim.x) {
          z_t a = f[(size_t)nG * j1 + g], b = f[(size_t)nG * i1 + g];
          double wg = w[g];
          s.x += (a.x * b.x + a.y * b.y) * wg;
          s.y += (a.x * b.y - a.y * b.x) * wg;
        }
        s = block_sum(s);
        __shared__ z_t ov;
        if (threadIdx.x == 0) ov = s;
        __syncthreads();
        z_t o = ov;
        for (int g = threadIdx.x; g < nG; g += blockDim.x) {
          z_t a = f[(size_t)nG * j1 + g];
          z_t& b = f[(size_t)nG * i1 + g];
          b.x -= a.x * o.x - a.y * o.y;
          b.y -= a.x * o.y + a.y * o.x;
        }
        __syncthreads();
      }
    z_t s = zmk(0.0, 0.0);
    for (int g = threadIdx.x; g < nG; g += blockDim.x) {
      z_t b = f[(size_t)nG * i1 + g];
      s.x += (b.x * b.x + b.y * b.y) * w[g];
    }
    s = block_sum(s);
    __shared__ double nrm;
    if (threadIdx.x == 0) {
      nrm = s.x;
      if (!(s.x > 0.0)) *status = 1;
    }
    __syncthreads();
    double sq = sqrt(nrm);
    for (int g = threadIdx.x; g < nG; g += blockDim.x) {
      z_t& b = f[(size_t)nG * i1 + g];
      b.x /= sq;
      b.y /= sq;
    }
    __syncthreads();
  }
}

// E = Re[ sum h1(k,l) rho1(l,k) + sum h2(k1,k2,l1,l2) rho2(l1,l2,k1,k2) ]
__global__ void k_energy(double* out, const z_t* __restrict__ h1, const z_t* __restrict__ r1,
                         const z_t* __restrict__ h2, const z_t* __restrict__ r2, int nO) {
  z_t s = zmk(0.0, 0.0);
  size_t n2 = (size_t)nO * nO;
  for (size_t e = threadIdx.x; e < n2; e += blockDim.x) {
    size_t k = e % nO, l = e / nO;
    zfma(s, h1[k + nO * l], r1[l + nO * k]);
  }
  for (size_t e = threadIdx.x; e < n2 * n2; e += blockDim.x) {
    size_t kk = e % n2, ll = e / n2;  // kk = (k1,k2), ll = (l1,l2)
    zfma(s, h2[kk + n2 * ll], r2[ll + n2 * kk]);
  }
  s = block_sum(s);
  if (threadIdx.x == 0) *out = s.x;
}

int grid_for(size_t n, int threads) {
  size_t b = (n + threads - 1) / threads;
  if (b > 152 * 8) b = 152 * 8;
  if (b < 1) b = 1;
  return (int)b;
}

void ensure_partial(cgpu_ctx* c, size_t n) {
  if (c->partialCap >= n) return;
  if (c->partial_d) cudaFree(c->partial_d);
  CODY_CUDA(cudaMalloc(&c->partial_d, n * sizeof(z_t)));
  c->partialCap = n;
}

}  // namespace

double cody_field_amplitude(const cgpu_ctx* c, double t) {
  if (c->laserKind == CGPU_LASER_SIN2) {
    if (c->omega <= 0.0) return 0.0;
    const double PI = 3.14159265358979323846264338327950288;
    double duration = 2.0 * PI * c->nCycles / c->omega;
    double tRel = t - c->tStart;
    if (tRel < 0.0 || tRel > duration) return 0.0;
    double env = sin(PI * tRel / duration);
    env = env * env;
    return c->E0 * env * cos(c->omega * (tRel - 0.5 * duration) + c->cep);
  }
  if (c->laserKind == CGPU_LASER_SAMPLED) {
    double u = (t - c->sampleT0) / c->sampleDt;
    long n = (long)floor(u + 1e-9);
    if (n < 0 || n >= (long)c->samples.size()) return 0.0;
    return c->samples[n];
  }
  return 0.0;
}

void launch_onebody(cgpu_ctx* c, z_t* out, const z_t* orbs, double t, z_t alpha, int accumulate) {
  ProfScope prof(c, CGPU_KERNEL_ONEBODY);
  int hasPot = c->hasPotential || c->laserKind != CGPU_LASER_NONE;
  dim3 grid((c->nG + OB_THREADS - 1) / OB_THREADS, c->nOS);
  size_t sh = sizeof(z_t) * (OB_THREADS + 2 * c->band);
  const double* base = c->inCapture ? c->stepT_d : c->zero_d;
  double off = c->inCapture ? t - c->captureT0 : t;
  k_onebody<<<grid, OB_THREADS, sh, c->stream>>>(out, orbs, c->T_d, c->V0_d, c->x_d, c->btOfOrb_d, c->nG, c->band,
                                                 c->restricted, c->laserDev, base, off, hasPot, alpha, accumulate);
  CODY_LAUNCHED(c);
}

void launch_gram(cgpu_ctx* c, z_t* G, const z_t* A, const z_t* B, int n, int colA0, int colB0, int ldG, double scale) {
  int chunk = std::max(1, std::min(GR_CHUNK, 1024 / std::max(n, 1)));  // <= 32 KB of shared memory
  int nBlk = std::min(RED_BLOCKS, (c->nG + chunk - 1) / chunk);
  ensure_partial(c, (size_t)nBlk * n * n);
  size_t sh = 2 * sizeof(z_t) * chunk * n;
  int threads = 256;
  if (n * n > GR_PER_THREAD * threads) throw std::string("launch_gram: more than 64 orbitals");
  k_gram_partial<<<nBlk, threads, sh, c->stream>>>(c->partial_d, A, B, c->w_d, c->nG, n, colA0, colB0, chunk);
  CODY_LAUNCHED(c);
  k_gram_final<<<(n * n * 32 + 255) / 256, 256, 0, c->stream>>>(G, c->partial_d, nBlk, n, ldG, scale);
  CODY_LAUNCHED(c);
}

// Orbs_ProjectOnSubspace: one block when restricted, otherwise per body type.
void launch_project_orbs(cgpu_ctx* c, z_t* dOrbs, const z_t* orbs) {
  int nGroups = c->restricted ? 1 : c->nBt;
  for (int b = 0; b < nGroups; b++) {
    int c0 = c->restricted ? 0 : c->orbStart[b];
    int n = c->restricted ? c->nOS : c->nOrbs[b];
    launch_gram(c, c->gram_d, orbs, dOrbs, n, c0, c0, n, 1.0);
    dim3 grid((c->nG + 255) / 256, n);
    k_project_apply<<<grid, 256, 0, c->stream>>>(dOrbs, orbs, c->gram_d, c->nG, n, c0);
    CODY_LAUNCHED(c);
  }
}

void launch_project_coeffs(cgpu_ctx* c, z_t* dC, const z_t* C) {
  int nBlk = std::min(RED_BLOCKS, grid_for(c->nC, 256));
  ensure_partial(c, nBlk);
  k_dot_partial<<<nBlk, 256, 0, c->stream>>>(c->partial_d, C, dC, c->nC);
  CODY_LAUNCHED(c);
  k_project_coeffs_apply<<<grid_for(c->nC, 256), 256, 0, c->stream>>>(dC, C, c->partial_d, nBlk, c->nC);
  CODY_LAUNCHED(c);
}

void launch_normalize_coeffs(cgpu_ctx* c, z_t* C) {
  int nBlk = std::min(RED_BLOCKS, grid_for(c->nC, 256));
  ensure_partial(c, nBlk);
  k_dot_partial<<<nBlk, 256, 0, c->stream>>>(c->partial_d, C, C, c->nC);
  CODY_LAUNCHED(c);
  k_normalize_apply<<<grid_for(c->nC, 256), 256, 0, c->stream>>>(C, c->partial_d, nBlk, c->nC);
  CODY_LAUNCHED(c);
}

void launch_fill_h1_from(cgpu_ctx* c, const z_t* orbs, const z_t* hOrbs, z_t* h1) {
  launch_gram(c, c->gram_d, orbs, hOrbs, c->nOS, 0, 0, c->nOS, 1.0);
  int nn = c->nO * c->nO;
  k_h1_layout<<<(nn + 127) / 128, 128, 0, c->stream>>>(h1, c->gram_d, c->btOfOrb_d, c->nO, c->nOS, c->restricted);
  CODY_LAUNCHED(c);
}

void launch_axpby(cgpu_ctx* c, z_t* y, const z_t* x, z_t a, z_t b, size_t n) {
  k_axpby<<<grid_for(n, 256), 256, 0, c->stream>>>(y, x, a, b, n);
  CODY_LAUNCHED(c);
}

void launch_scale(cgpu_ctx* c, z_t* y, z_t a, size_t n) {
  k_scale<<<grid_for(n, 256), 256, 0, c->stream>>>(y, a, n);
  CODY_LAUNCHED(c);
}

void launch_rk_stage(cgpu_ctx* c, z_t* inc, z_t* tmp, const z_t* state, const z_t* d, double wInc, double wTmp,
                     int first, size_t n) {
  k_rk_stage<<<grid_for(n, 256), 256, 0, c->stream>>>(inc, tmp, state, d, wInc, wTmp, first, n);
  CODY_LAUNCHED(c);
}

void launch_orthonormalize(cgpu_ctx* c, z_t* orbs, int col0, int nCols) {
  CODY_CUDA(cudaMemsetAsync(c->scal_d, 0, sizeof(int), c->stream));
  k_mgs2<<<1, 1024, 0, c->stream>>>(orbs, c->w_d, c->nG, col0, nCols, (int*)c->scal_d);
  CODY_LAUNCHED(c);
}

void launch_energy(cgpu_ctx* c, double* out_d) {
  k_energy<<<1, 1024, 0, c->stream>>>(out_d, c->h1_d, c->rdm1_d, c->h2_d, c->rdm2_d, c->nO);
  CODY_LAUNCHED(c);
}
