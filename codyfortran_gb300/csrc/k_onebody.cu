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
// fixed order, no floating-point atomics.  Every kernel covers all
// trajectories of the context (blockIdx.z).
#include <algorithm>

#include "common.cuh"

namespace {

constexpr int OB_THREADS = 256;
constexpr int RED_BLOCKS = 148;  // partial-sum blocks for grid reductions (one trajectory)

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

// Eout (one slot per trajectory) = E(*tBase + tOff) for every trajectory.
__global__ void k_field(double* __restrict__ Eout, TRAJ_ARGS, const double* __restrict__ tBase, double tOff) {
  Eout = bat(Eout, bs);
  *Eout = field_amplitude_dev(shp[blockIdx.z].laser, *bat(tBase, bs) + tOff);
}

__global__ void k_onebody(z_t* __restrict__ out, const z_t* __restrict__ orbs, const double* __restrict__ T,
                          const double* __restrict__ V0, const double* __restrict__ x, const int* __restrict__ btOf,
                          TRAJ_ARGS, const double* __restrict__ Efield, z_t alpha, int accumulate) {
  extern __shared__ z_t sh[];
  const TrajShape& S = shp[blockIdx.z];
  const int nG = S.nG, band = S.band;
  const int g0 = blockIdx.x * OB_THREADS;
  if (g0 >= nG) return;
  out = bat(out, bs);
  orbs = bat(orbs, bs);
  T = bat(T, bs);
  V0 = bat(V0, bs);
  x = bat(x, bs);
  btOf = bat(btOf, bs);
  const double E = *bat(Efield, bs);
  const int nTile = OB_THREADS + 2 * band, nd = 2 * band + 1;
  const int g = g0 + threadIdx.x;
  const bool live = g < nG;
  const double pot = (S.hasPot && live) ? V0[g] + E * x[g] : 0.0;
  // orbitals blockIdx.y, blockIdx.y + gridDim.y, ... of the grid tile (a batch
  // launches one orbital group: one block per tile instead of per orbital and tile)
  for (int i = blockIdx.y; i < S.nOS; i += gridDim.y) {
    const z_t* f = orbs + (size_t)nG * i;
    if (i != (int)blockIdx.y) __syncthreads();  // the previous orbital's tile has been read
    for (int t = threadIdx.x; t < nTile; t += OB_THREADS) {
      const int gg = g0 - band + t;
      sh[t] = (gg >= 0 && gg < nG) ? f[gg] : zmk(0.0, 0.0);
    }
    __syncthreads();
    if (!live) continue;
    const int bt = S.restricted ? 0 : btOf[i];
    const double* Tb = T + (size_t)bt * nd * nG;
    z_t acc = zmk(0.0, 0.0);
    for (int d = 0; d < nd; d++) {
      double c = Tb[(size_t)d * nG + g];
      z_t v = sh[threadIdx.x + d];
      acc.x = fma(c, v.x, acc.x);
      acc.y = fma(c, v.y, acc.y);
    }
    if (S.hasPot) {
      z_t v = sh[threadIdx.x + band];
      acc.x = fma(pot, v.x, acc.x);
      acc.y = fma(pot, v.y, acc.y);
    }
    // alpha is 1 or -i on the propagation paths: no FP64 multiply for those
    z_t r = (alpha.x == 1.0 && alpha.y == 0.0) ? acc : (alpha.x == 0.0 && alpha.y == -1.0) ? zmi(acc)
                                                                                             : zmul(alpha, acc);
    size_t o = (size_t)nG * i + g;
    if (accumulate) r = zadd(out[o], r);
    out[o] = r;
  }
}

// The one-body apply in double-float arithmetic (the fixed-point forms): the
// orbital tile staged as double-floats, the static double-float band, every
// product error-free in FP32 with two-sum accumulation; the potential V0 + E x
// formed in FP64 (one FMA) and split.
__global__ void k_onebody_df(z_t* __restrict__ out, const z_t* __restrict__ orbs, const float2* __restrict__ Tdf,
                             const double* __restrict__ V0, const double* __restrict__ x,
                             const int* __restrict__ btOf, TRAJ_ARGS, const double* __restrict__ Efield, z_t alpha,
                             int accumulate) {
  extern __shared__ float4 shf[];
  const TrajShape& S = shp[blockIdx.z];
  const int nG = S.nG, band = S.band;
  const int g0 = blockIdx.x * OB_THREADS;
  if (g0 >= nG) return;
  out = bat(out, bs);
  orbs = bat(orbs, bs);
  Tdf = bat(Tdf, bs);
  V0 = bat(V0, bs);
  x = bat(x, bs);
  btOf = bat(btOf, bs);
  const double E = *bat(Efield, bs);
  const int nTile = OB_THREADS + 2 * band, nd = 2 * band + 1;
  const int g = g0 + threadIdx.x;
  const bool live = g < nG;
  const float2 pd = (S.hasPot && live) ? df_split(fma(E, x[g], V0[g])) : make_float2(0.0f, 0.0f);
  for (int i = blockIdx.y; i < S.nOS; i += gridDim.y) {  // the block's orbitals of the grid tile
    const z_t* f = orbs + (size_t)nG * i;
    if (i != (int)blockIdx.y) __syncthreads();
    for (int t = threadIdx.x; t < nTile; t += OB_THREADS) {
      const int gg = g0 - band + t;
      shf[t] = (gg >= 0 && gg < nG) ? zdf_from(f[gg]) : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    }
    __syncthreads();
    if (!live) continue;
    const int bt = S.restricted ? 0 : btOf[i];
    const float2* Tb = Tdf + (size_t)bt * nd * nG;
    zdf_acc acc = {0.0f, 0.0f, 0.0f, 0.0f};
    for (int d = 0; d < nd; d++) {
      const float2 cf = Tb[(size_t)d * nG + g];
      const float4 v = shf[threadIdx.x + d];
      df_mul_acc(acc.rs, acc.rc, cf.x, cf.y, v.x, v.y);
      df_mul_acc(acc.is, acc.ic, cf.x, cf.y, v.z, v.w);
    }
    if (S.hasPot) {
      const float4 v = shf[threadIdx.x + band];
      df_mul_acc(acc.rs, acc.rc, pd.x, pd.y, v.x, v.y);
      df_mul_acc(acc.is, acc.ic, pd.x, pd.y, v.z, v.w);
    }
    const z_t a = zdf_to_z(acc);
    z_t r = (alpha.x == 1.0 && alpha.y == 0.0) ? a : (alpha.x == 0.0 && alpha.y == -1.0) ? zmi(a) : zmul(alpha, a);
    size_t o = (size_t)nG * i + g;
    if (accumulate) r = zadd(out[o], r);
    out[o] = r;
  }
}

// Sum of v over the block (the block total in thread 0).
__device__ z_t ob_block_sum(z_t v) {
  __shared__ z_t red[OB_THREADS / 32];
  for (int o = 16; o > 0; o >>= 1) {
    v.x += __shfl_down_sync(0xffffffffu, v.x, o);
    v.y += __shfl_down_sync(0xffffffffu, v.y, o);
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) red[wid] = v;
  __syncthreads();
  v = (threadIdx.x < OB_THREADS / 32) ? red[threadIdx.x] : zmk(0.0, 0.0);
  if (wid == 0)
    for (int o = 16; o > 0; o >>= 1) {
      v.x += __shfl_down_sync(0xffffffffu, v.x, o);
      v.y += __shfl_down_sync(0xffffffffu, v.y, o);
    }
  return v;
}

// The OrbsLin apply of Lanczos iteration j (three-term recurrence on
// unnormalised basis vectors u_k, scales s_k in lz) in double-float arithmetic,
// fused with the recurrence's first pass: h = (T + V0 + E x) u_j on the
// orbitals into out (0 on the coefficients, which OrbsLin does not move) and,
// with x = s_j h - beta_{j-1} s_{j-1} u_{j-1}, per block b the partials
//   part[2 b] = s_j sum m Re(conj(u_j) x),   part[2 b + 1] = sum m |x|^2
// (b = blockIdx.x + gridDim.x blockIdx.y), the layout the pass-2 kernel reads.
// The one-body apply has just read u_j; the pass reads u_{j-1} and m besides,
// instead of a separate pass over h, u_j, u_{j-1} and m.
__global__ void __launch_bounds__(OB_THREADS, 4) k_onebody_lz_df(z_t* __restrict__ out, const z_t* __restrict__ vCur, const z_t* __restrict__ vPrev,
                                const double* __restrict__ m, z_t* __restrict__ part, const float2* __restrict__ Tdf,
                                const double* __restrict__ V0, const double* __restrict__ x,
                                const int* __restrict__ btOf, TRAJ_ARGS, const double* __restrict__ Efield,
                                const double* __restrict__ lz, int j) {
  extern __shared__ float4 shf[];
  const TrajShape& S = shp[blockIdx.z];
  lz = bat(lz, bs);
  if (lz[CODY_LZ_DONE] != 0.0) return;  // the recurrence stopped: the pass-2 kernel returns too
  const int nG = S.nG, band = S.band;
  const int g0 = blockIdx.x * OB_THREADS;
  const int bid = blockIdx.x + gridDim.x * blockIdx.y;
  const double sj = lz[CODY_LZ_S + j - 1];
  const double bp = (j > 1) ? lz[CODY_LZ_BETA + j - 2] * lz[CODY_LZ_S + j - 2] : 0.0;
  out = bat(out, bs);
  vCur = bat(vCur, bs);
  vPrev = (j > 1) ? bat(vPrev, bs) : nullptr;
  m = bat(m, bs);
  part = bat(part, bs);
  // the pass is summed in double-float arithmetic (the FP64 pipe is the scarce one)
  const float2 sj2 = df_split(sj), nbp2 = df_split(-bp), zero2 = make_float2(0.0f, 0.0f);
  float as = 0.0f, ac = 0.0f, qs = 0.0f, qc = 0.0f;
  // a += m Re(conj(v) x), q += m |x|^2 for the double-floats x, v, m
  auto pass_df = [&](float2 xr, float2 xi, float2 vr, float2 vi, double mi) {
    const float2 m2 = df_split(mi);
    const float2 t = df_dot2(vr, xr, vi, xi), u = df_dot2(xr, xr, xi, xi);
    df_mul_acc(as, ac, m2.x, m2.y, t.x, t.y);
    df_mul_acc(qs, qc, m2.x, m2.y, u.x, u.y);
  };
  auto pass = [&](float2 xr, float2 xi, const z_t v, double mi) {
    pass_df(xr, xi, df_split(v.x), df_split(v.y), mi);
  };
  if (bid == 0)  // the coefficient part: h = 0, x = -bp u_{j-1}
    for (int l = threadIdx.x; l < S.nC; l += OB_THREADS) {
      out[l] = zmk(0.0, 0.0);
      if (vPrev) {
        const z_t p = vPrev[l];
        const float2 pr = df_split(p.x), pi = df_split(p.y);
        pass(df_dot2(nbp2, pr, zero2, zero2), df_dot2(nbp2, pi, zero2, zero2), vCur[l], m[l]);
      }
    }
  if (g0 < nG) {
    Tdf = bat(Tdf, bs);
    V0 = bat(V0, bs);
    x = bat(x, bs);
    btOf = bat(btOf, bs);
    const double E = *bat(Efield, bs);
    const z_t* orbCur = vCur + S.nCpad;
    const z_t* orbPrev = vPrev ? vPrev + S.nCpad : nullptr;
    const double* mo = m + S.nCpad;
    z_t* oo = out + S.nCpad;
    const int nTile = OB_THREADS + 2 * band, nd = 2 * band + 1;
    const int g = g0 + threadIdx.x;
    const bool live = g < nG;
    const float2 pd = (S.hasPot && live) ? df_split(fma(E, x[g], V0[g])) : make_float2(0.0f, 0.0f);
    // restricted orbitals share one band: its coefficients for this grid tile
    // are staged in shared memory once (after the orbital tile, nd rows of
    // OB_THREADS double-floats)
    float2* shT = reinterpret_cast<float2*>(shf + nTile);
    if (S.restricted) {
      for (int d = 0; d < nd; d++) shT[d * OB_THREADS + threadIdx.x] = live ? Tdf[(size_t)d * nG + g] : zero2;
    }
    // the orbital tile (entries threadIdx.x and threadIdx.x + OB_THREADS) and
    // this thread's v_{j-1} and metric entries are fetched one orbital ahead
    auto tile_at = [&](int i, int t) {
      const int gg = g0 - band + t;
      return (t < nTile && gg >= 0 && gg < nG) ? orbCur[(size_t)nG * i + gg] : zmk(0.0, 0.0);
    };
    const int i0 = blockIdx.y;
    z_t nx0 = zmk(0.0, 0.0), nx1 = zmk(0.0, 0.0), np = zmk(0.0, 0.0);
    double nm = 0.0;
    if (i0 < S.nOS) {
      nx0 = tile_at(i0, threadIdx.x);
      nx1 = tile_at(i0, threadIdx.x + OB_THREADS);
      if (live) {
        if (orbPrev) np = orbPrev[(size_t)nG * i0 + g];
        nm = mo[(size_t)nG * i0 + g];
      }
    }
    for (int i = i0; i < S.nOS; i += gridDim.y) {
      if (i != i0) __syncthreads();
      shf[threadIdx.x] = zdf_from(nx0);
      if (threadIdx.x + OB_THREADS < nTile) shf[threadIdx.x + OB_THREADS] = zdf_from(nx1);
      const z_t p = np;
      const double mi = nm;
      const int in = i + gridDim.y;
      if (in < S.nOS) {
        nx0 = tile_at(in, threadIdx.x);
        nx1 = tile_at(in, threadIdx.x + OB_THREADS);
        if (live) {
          if (orbPrev) np = orbPrev[(size_t)nG * in + g];
          nm = mo[(size_t)nG * in + g];
        }
      }
      __syncthreads();
      if (!live) continue;
      zdf_acc acc = {0.0f, 0.0f, 0.0f, 0.0f};
      if (S.restricted) {
        for (int d = 0; d < nd; d++) {
          const float2 cf = shT[d * OB_THREADS + threadIdx.x];
          const float4 v = shf[threadIdx.x + d];
          df_mul_acc(acc.rs, acc.rc, cf.x, cf.y, v.x, v.y);
          df_mul_acc(acc.is, acc.ic, cf.x, cf.y, v.z, v.w);
        }
      } else {
        const float2* Tb = Tdf + (size_t)btOf[i] * nd * nG;
        for (int d = 0; d < nd; d++) {
          const float2 cf = Tb[(size_t)d * nG + g];
          const float4 v = shf[threadIdx.x + d];
          df_mul_acc(acc.rs, acc.rc, cf.x, cf.y, v.x, v.y);
          df_mul_acc(acc.is, acc.ic, cf.x, cf.y, v.z, v.w);
        }
      }
      if (S.hasPot) {
        const float4 v = shf[threadIdx.x + band];
        df_mul_acc(acc.rs, acc.rc, pd.x, pd.y, v.x, v.y);
        df_mul_acc(acc.is, acc.ic, pd.x, pd.y, v.z, v.w);
      }
      const size_t o = (size_t)nG * i + g;
      oo[o] = zdf_to_z(acc);
      const float2 hr = df_norm(acc.rs, acc.rc), hi = df_norm(acc.is, acc.ic);
      float2 pr = zero2, pi = zero2;
      if (orbPrev) {
        pr = df_split(p.x);
        pi = df_split(p.y);
      }
      const float4 vc = shf[threadIdx.x + band];  // u_j at g, already split
      pass_df(df_dot2(sj2, hr, nbp2, pr), df_dot2(sj2, hi, nbp2, pi), make_float2(vc.x, vc.y),
              make_float2(vc.z, vc.w), mi);
    }
  }
  const double a = f2d_exact(as) + f2d_exact(ac), q = f2d_exact(qs) + f2d_exact(qc);
  const z_t t = ob_block_sum(zmk(a * sj, q));
  if (threadIdx.x == 0) {
    part[(size_t)bid * 2] = zmk(t.x, 0.0);
    part[(size_t)bid * 2 + 1] = zmk(t.y, 0.0);
  }
}

// Column range of a Gram / projector call: group < 0 = all stored orbitals,
// otherwise projector group `group` (false when the trajectory has none).
__device__ __forceinline__ bool gram_cols(const TrajShape& S, int group, int& c0, int& n) {
  if (group < 0) {
    c0 = 0;
    n = S.nOS;
    return true;
  }
  if (group >= S.nGroups) return false;
  c0 = S.grpStart[group];
  n = S.grpSize[group];
  return n > 0;
}

// ---------------------------------------------------------------------------
// Weighted Gram partials: part[blk][i + n*j] = sum_{g in chunks of blk}
//   conj(A[g, c0+i]) * B[g, c0+j] * w[g]
// ---------------------------------------------------------------------------
constexpr int GR_CHUNK = 32;
constexpr int GR_PER_THREAD = 16;  // 256 threads x 16 = 4096 = 64^2 Gram entries

__global__ void k_gram_partial(z_t* __restrict__ part, const z_t* __restrict__ A, const z_t* __restrict__ B,
                               const double* __restrict__ w, TRAJ_ARGS, int group, int chunk) {
  extern __shared__ z_t sh[];
  const TrajShape& S = shp[blockIdx.z];
  int c0, n;
  if (!gram_cols(S, group, c0, n)) return;
  const int nG = S.nG;
  part = bat(part, bs);
  A = bat(A, bs);
  B = bat(B, bs);
  w = bat(w, bs);
  z_t* sa = sh;                 // chunk x n
  z_t* sb = sh + chunk * n;     // chunk x n
  int nn = n * n;
  z_t acc[GR_PER_THREAD];
  for (int q = 0; q < GR_PER_THREAD; q++) acc[q] = zmk(0.0, 0.0);
  for (int r0 = blockIdx.x * chunk; r0 < nG; r0 += gridDim.x * chunk) {
    __syncthreads();
    for (int t = threadIdx.x; t < chunk * n; t += blockDim.x) {
      int col = t / chunk, r = t % chunk;
      int g = r0 + r;
      z_t a = zmk(0.0, 0.0), b = zmk(0.0, 0.0);
      if (g < nG) {
        a = A[(size_t)nG * (c0 + col) + g];
        b = B[(size_t)nG * (c0 + col) + g];
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

// one warp per Gram entry, lanes over the block partials (fixed order); G is n x n
__global__ void k_gram_final(z_t* __restrict__ G, const z_t* __restrict__ part, int nBlk, TRAJ_ARGS, int group,
                             double scale) {
  const TrajShape& S = shp[blockIdx.z];
  int c0, n;
  if (!gram_cols(S, group, c0, n)) return;
  int e = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  int lane = threadIdx.x & 31;
  int nn = n * n;
  if (e >= nn) return;
  G = bat(G, bs);
  part = bat(part, bs);
  z_t s = zmk(0.0, 0.0);
  for (int b = lane; b < nBlk; b += 32) s = zadd(s, part[(size_t)b * nn + e]);
  for (int o = 16; o > 0; o >>= 1) {
    s.x += __shfl_xor_sync(0xffffffffu, s.x, o);
    s.y += __shfl_xor_sync(0xffffffffu, s.y, o);
  }
  if (lane == 0) {
    int i = e % n, j = e / n;
    G[i + (size_t)n * j] = zscale(s, scale);
  }
}

// dOrbs[:, c0+j] -= sum_i orbs[:, c0+i] * G[i + n*j]
__global__ void k_project_apply(z_t* __restrict__ dOrbs, const z_t* __restrict__ orbs, const z_t* __restrict__ G,
                                TRAJ_ARGS, int group) {
  const TrajShape& S = shp[blockIdx.z];
  int c0, n;
  if (!gram_cols(S, group, c0, n)) return;
  int g = blockIdx.x * blockDim.x + threadIdx.x;
  int j = blockIdx.y;
  const int nG = S.nG;
  if (g >= nG || j >= n) return;
  dOrbs = bat(dOrbs, bs);
  orbs = bat(orbs, bs);
  G = bat(G, bs);
  z_t acc = zmk(0.0, 0.0);
  for (int i = 0; i < n; i++) zfma(acc, orbs[(size_t)nG * (c0 + i) + g], G[i + (size_t)n * j]);
  size_t o = (size_t)nG * (c0 + j) + g;
  dOrbs[o] = zsub(dOrbs[o], acc);
}

// k_project_apply in double-float arithmetic (the fixed-point forms): one
// thread per grid point and batch of PA_J orbitals j (blockIdx.y), G staged as
// double-floats (n <= PA_MAXN), phi_i(g) split once per batch.
constexpr int PA_J = 8, PA_MAXN = 32;
__global__ void __launch_bounds__(128) k_project_apply_df(z_t* __restrict__ dOrbs, const z_t* __restrict__ orbs,
                                                           const z_t* __restrict__ G, TRAJ_ARGS, int group) {
  const TrajShape& S = shp[blockIdx.z];
  int c0, n;
  if (!gram_cols(S, group, c0, n)) return;
  const int nG = S.nG;
  dOrbs = bat(dOrbs, bs);
  orbs = bat(orbs, bs);
  G = bat(G, bs);
  __shared__ float4 gdf[PA_MAXN * PA_MAXN];
  for (int e = threadIdx.x; e < n * n; e += blockDim.x) {  // -G, so that the sums subtract
    const z_t v = G[e];
    gdf[e] = zdf_from(zmk(-v.x, -v.y));
  }
  __syncthreads();
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  const int j0 = blockIdx.y * PA_J;
  if (g >= nG || j0 >= n) return;
  {
    zdf_acc acc[PA_J];
#pragma unroll
    for (int q = 0; q < PA_J; q++) {
      const float4 d =
          (j0 + q < n) ? zdf_from(dOrbs[(size_t)nG * (c0 + j0 + q) + g]) : make_float4(0.f, 0.f, 0.f, 0.f);
      acc[q] = {d.x, d.y, d.z, d.w};
    }
    for (int i = 0; i < n; i++) {
      const float4 o = zdf_from(orbs[(size_t)nG * (c0 + i) + g]);
#pragma unroll
      for (int q = 0; q < PA_J; q++)
        if (j0 + q < n) zdf_fma(acc[q], gdf[i + n * (j0 + q)], o, false);
    }
#pragma unroll
    for (int q = 0; q < PA_J; q++)
      if (j0 + q < n) dOrbs[(size_t)nG * (c0 + j0 + q) + g] = zdf_to_z(acc[q]);
  }
}

// h1 (nO x nO) from the stored-orbital Gram G (nOS x nOS): same body type only,
// restricted runs duplicate the block for the second spin (FillH1 :203-222).
__global__ void k_h1_layout(z_t* __restrict__ h1, const z_t* __restrict__ G, const int* __restrict__ btOf,
                            TRAJ_ARGS) {
  const TrajShape& S = shp[blockIdx.z];
  const int nO = S.nO, nOS = S.nOS;
  int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= nO * nO) return;
  h1 = bat(h1, bs);
  G = bat(G, bs);
  btOf = bat(btOf, bs);
  int i = e % nO, j = e / nO;
  z_t v = zmk(0.0, 0.0);
  if (S.restricted) {
    if ((i < nOS) == (j < nOS)) v = G[(i % nOS) + (size_t)nOS * (j % nOS)];
  } else {
    if (btOf[i] == btOf[j]) v = G[i + (size_t)nOS * j];
  }
  h1[e] = v;
}

// ---------------------------------------------------------------------------
// Vector kernels over a state vector (sel VSEL_STATE) or its coefficients
// ---------------------------------------------------------------------------
__global__ void k_axpby(z_t* __restrict__ y, const z_t* __restrict__ x, z_t a, z_t b, TRAJ_ARGS, int sel) {
  const TrajShape& S = shp[blockIdx.z];
  y = bat(y, bs);
  x = bat(x, bs);
  size_t n = vlen(S, sel);
  for (size_t l = blockIdx.x * (size_t)blockDim.x + threadIdx.x; l < n; l += (size_t)gridDim.x * blockDim.x) {
    size_t i = vidx(S, l);
    z_t r = zmul(b, y[i]);
    zfma(r, a, x[i]);
    y[i] = r;
  }
}

__global__ void k_scale(z_t* __restrict__ y, z_t a, TRAJ_ARGS, int sel) {
  const TrajShape& S = shp[blockIdx.z];
  y = bat(y, bs);
  size_t n = vlen(S, sel);
  for (size_t l = blockIdx.x * (size_t)blockDim.x + threadIdx.x; l < n; l += (size_t)gridDim.x * blockDim.x) {
    size_t i = vidx(S, l);
    y[i] = zmul(a, y[i]);
  }
}

// RK4 stage bookkeeping (S_IntegratorList_Rk_O4Expl.f90:109-135):
// inc = (first ? 0 : inc) + d*wInc; tmp = state + d*wTmp
__global__ void k_rk_stage(z_t* __restrict__ inc, z_t* __restrict__ tmp, const z_t* __restrict__ state,
                           const z_t* __restrict__ d, double wInc, double wTmp, int first, TRAJ_ARGS) {
  const TrajShape& S = shp[blockIdx.z];
  inc = bat(inc, bs);
  tmp = bat(tmp, bs);
  state = bat(state, bs);
  d = bat(d, bs);
  size_t n = S.nS;
  for (size_t l = blockIdx.x * (size_t)blockDim.x + threadIdx.x; l < n; l += (size_t)gridDim.x * blockDim.x) {
    size_t i = vidx(S, l);
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

// part[blk] = sum conj(a) b over the block's stride of the coefficients
__global__ void k_dot_partial(z_t* __restrict__ part, const z_t* __restrict__ a, const z_t* __restrict__ b,
                              TRAJ_ARGS) {
  const TrajShape& S = shp[blockIdx.z];
  part = bat(part, bs);
  a = bat(a, bs);
  b = bat(b, bs);
  size_t n = S.nC;
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
                                       int nBlk, TRAJ_ARGS) {
  const TrajShape& S = shp[blockIdx.z];
  dC = bat(dC, bs);
  C = bat(C, bs);
  part = bat(part, bs);
  __shared__ z_t ov[1];
  sum_partials(part, nBlk, 1, 1, ov);
  z_t o = ov[0];
  size_t n = S.nC;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    z_t r = dC[i];
    z_t c = C[i];
    r.x -= o.x * c.x - o.y * c.y;
    r.y -= o.x * c.y + o.y * c.x;
    dC[i] = r;
  }
}

__global__ void k_normalize_apply(z_t* __restrict__ C, const z_t* __restrict__ part, int nBlk, TRAJ_ARGS) {
  const TrajShape& S = shp[blockIdx.z];
  C = bat(C, bs);
  part = bat(part, bs);
  __shared__ z_t tot[1];
  sum_partials(part, nBlk, 1, 1, tot);
  double nr = sqrt(tot[0].x);
  size_t n = S.nC;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    z_t c = C[i];
    C[i] = zmk(c.x / nr, c.y / nr);
  }
}

// Modified Gram-Schmidt, two sweeps, one CTA per trajectory (src/Grid/S_Grid.f90:120-151).
// Used only for relaxation / set-up, not in the real-time step.
__global__ void k_mgs2(z_t* __restrict__ f, const double* __restrict__ w, TRAJ_ARGS, int c0, int n, int* status) {
  const TrajShape& S = shp[blockIdx.z];
  const int nG = S.nG;
  f = bat(f, bs);
  w = bat(w, bs);
  status = bat(status, bs);
  if (c0 + n > S.nOS) n = S.nOS - c0;
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
                         const z_t* __restrict__ h2, const z_t* __restrict__ r2, TRAJ_ARGS) {
  const TrajShape& S = shp[blockIdx.z];
  const size_t nO = S.nO;
  out = bat(out, bs);
  h1 = bat(h1, bs);
  r1 = bat(r1, bs);
  h2 = bat(h2, bs);
  r2 = bat(r2, bs);
  z_t s = zmk(0.0, 0.0);
  size_t n2 = nO * nO;
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

// out[:, i] = x * orbs[:, i] (dipole operator on the orbitals)
__global__ void k_x_apply(z_t* __restrict__ out, const z_t* __restrict__ orbs, const double* __restrict__ x,
                          TRAJ_ARGS) {
  const TrajShape& S = shp[blockIdx.z];
  out = bat(out, bs);
  orbs = bat(orbs, bs);
  x = bat(x, bs);
  GRID_STRIDE(e, (size_t)S.nG * S.nOS) out[e] = zscale(orbs[e], x[e % S.nG]);
}

// scal[NORM] = ||C||, scal[DIPOLE] = Re sum_kl xm(k,l) rho1(l,k) (xm: the dipole
// matrix in the spin-orbital layout of h1)
__global__ void k_norm_dipole(double* __restrict__ scal, const z_t* __restrict__ C, const z_t* __restrict__ xm,
                              const z_t* __restrict__ r1, TRAJ_ARGS) {
  const TrajShape& S = shp[blockIdx.z];
  scal = bat(scal, bs);
  C = bat(C, bs);
  xm = bat(xm, bs);
  r1 = bat(r1, bs);
  z_t s = zmk(0.0, 0.0);
  for (int i = threadIdx.x; i < S.nC; i += blockDim.x) s.x += C[i].x * C[i].x + C[i].y * C[i].y;
  const size_t nO = S.nO;
  for (size_t e = threadIdx.x; e < nO * nO; e += blockDim.x) {
    size_t k = e % nO, l = e / nO;
    z_t p = zmul(xm[k + nO * l], r1[l + nO * k]);
    s.y += p.x;
  }
  s = block_sum(s);
  if (threadIdx.x == 0) {
    scal[CODY_SCAL_NORM] = sqrt(s.x);
    scal[CODY_SCAL_DIPOLE] = s.y;
  }
}

// Absorber mask (src/Absorber/Linear/Cosinus/S_Absorber_Linear_Cosinus.f90:75-104):
// 1 inside |x| < onset, cos(pi/2 xi)^(1/order) outside, xi = (|x| - onset) / (x_last - onset).
__global__ void k_absorber_mask(double* __restrict__ mask, const double* __restrict__ x, double onset, double order,
                                TRAJ_ARGS) {
  const TrajShape& S = shp[blockIdx.z];
  mask = bat(mask, bs);
  x = bat(x, bs);
  const double xMax = x[S.nG - 1];
  const double PI = 3.14159265358979323846264338327950288;
  GRID_STRIDE(g, S.nG) {
    double xi = fabs(x[g]);
    double t = (xi - onset) / (xMax - onset);
    mask[g] = xi < onset ? 1.0 : pow(cos(0.5 * PI * t), 1.0 / order);
  }
}

// ApplyAbsorber (:115-128): every stored orbital times the mask
__global__ void k_absorber_apply(z_t* __restrict__ orbs, const double* __restrict__ mask, TRAJ_ARGS) {
  const TrajShape& S = shp[blockIdx.z];
  orbs = bat(orbs, bs);
  mask = bat(mask, bs);
  GRID_STRIDE(e, (size_t)S.nG * S.nOS) orbs[e] = zscale(orbs[e], mask[e % S.nG]);
}

__global__ void k_set_scalar(double* p, double v, size_t bs) { *bat(p, bs) = v; }
__global__ void k_add_scalar(double* p, double v, size_t bs) { *bat(p, bs) += v; }

// Blocks per trajectory for a grid-stride kernel over n items.
unsigned vec_blocks(const cgpu_ctx* c, size_t n) {
  size_t b = (n + 255) / 256;
  size_t cap = std::max<size_t>(4, 4864 / (size_t)c->nb);
  return (unsigned)std::max<size_t>(1, std::min(b, cap));
}

int gram_chunk(int n) { return std::max(1, std::min(GR_CHUNK, 1024 / std::max(n, 1))); }  // <= 32 KB shared

int gram_blocks(const cgpu_ctx* c, int chunk) {
  int nBlk = std::min(RED_BLOCKS, (c->nG + chunk - 1) / chunk);
  if (c->nb > 1) nBlk = std::max(1, std::min(nBlk, (c->nG + 4 * chunk - 1) / (4 * chunk)));
  return nBlk;
}

int coeff_blocks(const cgpu_ctx* c) {
  return (int)std::min<unsigned>(RED_BLOCKS, vec_blocks(c, c->nC));
}

void check_partial(const cgpu_ctx* c, size_t need) {
  if (need > c->partialCap) throw std::string("internal: reduction scratch too small");
}

// grid/launch of the two-kernel Gram: G (n x n) = scale * A^H W B over the group's columns
// The weighted Gram partials in double-float arithmetic (the fixed-point forms):
// the chunk of A and w B staged as double-floats, every term conj(a) b an
// error-free FP32 product with two-sum accumulation, FP64 partials out.
__global__ void k_gram_partial_df(z_t* __restrict__ part, const z_t* __restrict__ A, const z_t* __restrict__ B,
                                  const double* __restrict__ w, TRAJ_ARGS, int group, int chunk) {
  extern __shared__ float4 shg[];
  const TrajShape& S = shp[blockIdx.z];
  int c0, n;
  if (!gram_cols(S, group, c0, n)) return;
  const int nG = S.nG;
  part = bat(part, bs);
  A = bat(A, bs);
  B = bat(B, bs);
  w = bat(w, bs);
  float4* sa = shg;              // chunk x n
  float4* sb = shg + chunk * n;  // chunk x n
  int nn = n * n;
  // small blocks (n^2 <= blockDim / 2): the rows of a chunk spread over R phases;
  // their R x n^2 partials reuse the tiles' 2 chunk n >= 2 chunk n (batch maximum)
  // double-floats, hence R <= 2 chunk / n
  const int R = nn * 2 <= (int)blockDim.x ? min(min(chunk, (int)blockDim.x / nn), 2 * chunk / n) : 1;
  const int e0 = threadIdx.x % nn, ph = threadIdx.x / nn, ii0 = e0 % n, jj0 = e0 / n;
  zdf_acc acc[GR_PER_THREAD];
  for (int q = 0; q < GR_PER_THREAD; q++) acc[q] = {0.0f, 0.0f, 0.0f, 0.0f};
  for (int r0 = blockIdx.x * chunk; r0 < nG; r0 += gridDim.x * chunk) {
    __syncthreads();
    for (int t = threadIdx.x; t < chunk * n; t += blockDim.x) {
      int col = t / chunk, r = t % chunk;
      int g = r0 + r;
      float4 a = make_float4(0.0f, 0.0f, 0.0f, 0.0f), b = a;
      if (g < nG) {
        a = zdf_from(A[(size_t)nG * (c0 + col) + g]);
        const float4 bb = zdf_from(B[(size_t)nG * (c0 + col) + g]);
        const float2 wg = df_split(w[g]);
        zdf_acc t2 = {0.0f, 0.0f, 0.0f, 0.0f};
        df_mul_acc(t2.rs, t2.rc, wg.x, wg.y, bb.x, bb.y);
        df_mul_acc(t2.is, t2.ic, wg.x, wg.y, bb.z, bb.w);
        b = make_float4(t2.rs, t2.rc, t2.is, t2.ic);
      }
      sa[r * n + col] = a;
      sb[r * n + col] = b;
    }
    __syncthreads();
    if (R > 1) {  // entry threadIdx.x % nn, rows of phase threadIdx.x / nn
      if (ph < R) {
        zdf_acc s = acc[0];
        for (int r = ph; r < chunk; r += R) zdf_cfma(s, sa[r * n + ii0], sb[r * n + jj0], false);
        acc[0] = s;
      }
    } else {
#pragma unroll
      for (int q = 0; q < GR_PER_THREAD; q++) {
        int e = threadIdx.x + q * blockDim.x;
        if (e >= nn) break;
        int ii = e % n, jj = e / n;
        zdf_acc s = acc[q];
        for (int r = 0; r < chunk; r++) zdf_cfma(s, sa[r * n + ii], sb[r * n + jj], false);
        acc[q] = s;
      }
    }
  }
  if (R > 1) {  // the R phase partials of each entry, summed in a fixed order
    __syncthreads();
    float4* red = shg;  // R x nn <= blockDim entries (the tiles are no longer read)
    if (ph < R) red[ph * nn + e0] = make_float4(acc[0].rs, acc[0].rc, acc[0].is, acc[0].ic);
    __syncthreads();
    if (threadIdx.x < nn) {
      zdf_acc t = {0.0f, 0.0f, 0.0f, 0.0f};
      for (int k = 0; k < R; k++) {
        const float4 v = red[k * nn + threadIdx.x];
        df_acc(t.rs, t.rc, v.x, v.y);
        df_acc(t.is, t.ic, v.z, v.w);
      }
      part[(size_t)blockIdx.x * nn + threadIdx.x] = zdf_to_z(t);
    }
    return;
  }
#pragma unroll
  for (int q = 0; q < GR_PER_THREAD; q++) {
    int e = threadIdx.x + q * blockDim.x;
    if (e >= nn) break;
    part[(size_t)blockIdx.x * nn + e] = zdf_to_z(acc[q]);
  }
}

void launch_gram(cgpu_ctx* c, z_t* G, const z_t* A, const z_t* B, int group, int nMax, double scale) {
  int chunk = gram_chunk(nMax);
  int nBlk = gram_blocks(c, chunk);
  check_partial(c, (size_t)nBlk * nMax * nMax);
  size_t sh = 2 * sizeof(z_t) * chunk * nMax;
  int threads = 256;
  if (nMax * nMax > GR_PER_THREAD * threads) throw std::string("launch_gram: more than 64 orbitals");
  if (c->ciDf)
    k_gram_partial_df<<<bgrid(c, nBlk), threads, sh, c->stream>>>(c->partial_d, A, B, c->w_d, TRAJ_PASS(c), group,
                                                                  chunk);
  else
    k_gram_partial<<<bgrid(c, nBlk), threads, sh, c->stream>>>(c->partial_d, A, B, c->w_d, TRAJ_PASS(c), group,
                                                               chunk);
  CODY_LAUNCHED(c);
  k_gram_final<<<bgrid(c, ceil_div((size_t)nMax * nMax * 32, 256)), 256, 0, c->stream>>>(G, c->partial_d, nBlk,
                                                                                         TRAJ_PASS(c), group, scale);
  CODY_LAUNCHED(c);
}

int max_group_size(const cgpu_ctx* c, int g) {
  int m = 0;
  for (const TrajShape& s : c->shape_h)
    if (g < s.nGroups) m = std::max(m, s.grpSize[g]);
  return m;
}

}  // namespace

size_t gram_partial_need(const cgpu_ctx* c, int n) {
  int chunk = gram_chunk(n);
  return (size_t)gram_blocks(c, chunk) * n * n;
}

void launch_field(cgpu_ctx* c, double* E, double t) {
  const double* base = (c->inCapture || c->useStepTime) ? c->stepT_d : c->zero_d;
  const double off = c->inCapture ? t - c->captureT0 : t;
  k_field<<<bgrid(c, 1), 1, 0, c->stream>>>(E, TRAJ_PASS(c), base, off);
  CODY_LAUNCHED(c);
}

int launch_onebody_lz(cgpu_ctx* c, int j, double t) {
  if (!c->Tdf_d || c->krylovWindow != 1 || c->method == CGPU_METHOD_TDCI) return 0;
  const unsigned tiles = ceil_div(c->nG, OB_THREADS);
  const unsigned groups = (size_t)tiles * c->nb >= 4 * (size_t)c->numSms ? 1 : (unsigned)c->nOS;
  const int nPart = (int)(tiles * groups);
  // the pass-1 partials share the region the separate pass writes
  if ((size_t)2 * nPart > (size_t)c->lzBlocks * (c->maxKrylov + 1)) return 0;
  ProfScope prof(c, CGPU_KERNEL_ONEBODY);
  double* E = c->scal_d + CODY_SCAL_FIELD;
  launch_field(c, E, t);
  const z_t* vCur = c->basis_d + (size_t)c->nS * (j - 1);
  const z_t* vPrev = j > 1 ? c->basis_d + (size_t)c->nS * (j - 2) : nullptr;
  dim3 grid(tiles, groups, c->nb);
  // the orbital tile (double-floats) and the band coefficients of the tile
  size_t sh = sizeof(float4) * (OB_THREADS + 2 * c->band) + sizeof(float2) * (2 * c->band + 1) * OB_THREADS;
  k_onebody_lz_df<<<grid, OB_THREADS, sh, c->stream>>>(c->lw_d, vCur, vPrev, c->metric_d, c->partial_d, c->Tdf_d,
                                                        c->V0_d, c->x_d, c->btOfOrb_d, TRAJ_PASS(c), E, c->lz_d, j);
  CODY_LAUNCHED(c);
  return nPart;
}

void launch_onebody(cgpu_ctx* c, z_t* out, const z_t* orbs, double t, z_t alpha, int accumulate) {
  ProfScope prof(c, CGPU_KERNEL_ONEBODY);
  // one block per grid tile walking every orbital when the tiles alone fill
  // the SMs several times over (batches), else one block per tile and orbital
  const unsigned tiles = ceil_div(c->nG, OB_THREADS);
  const unsigned groups = (size_t)tiles * c->nb >= 4 * (size_t)c->numSms ? 1 : (unsigned)c->nOS;
  dim3 grid(tiles, groups, c->nb);
  size_t sh = sizeof(z_t) * (OB_THREADS + 2 * c->band);
  const double* base = (c->inCapture || c->useStepTime) ? c->stepT_d : c->zero_d;
  double off = c->inCapture ? t - c->captureT0 : t;
  double* E = c->scal_d + CODY_SCAL_FIELD;
  k_field<<<bgrid(c, 1), 1, 0, c->stream>>>(E, TRAJ_PASS(c), base, off);
  CODY_LAUNCHED(c);
  if (c->Tdf_d)
    k_onebody_df<<<grid, OB_THREADS, sh, c->stream>>>(out, orbs, c->Tdf_d, c->V0_d, c->x_d, c->btOfOrb_d,
                                                      TRAJ_PASS(c), E, alpha, accumulate);
  else
    k_onebody<<<grid, OB_THREADS, sh, c->stream>>>(out, orbs, c->T_d, c->V0_d, c->x_d, c->btOfOrb_d, TRAJ_PASS(c), E,
                                                   alpha, accumulate);
  CODY_LAUNCHED(c);
}

// Orbs_ProjectOnSubspace: one group when restricted, otherwise per body type.
void launch_project_orbs(cgpu_ctx* c, z_t* dOrbs, const z_t* orbs) {
  ProfScope prof(c, CGPU_KERNEL_PROJECTORS);
  int nGroups = c->restricted ? 1 : c->nBt;
  for (int g = 0; g < nGroups; g++) {
    int n = max_group_size(c, g);
    if (n <= 0) continue;
    launch_gram(c, c->gram_d, orbs, dOrbs, g, n, 1.0);
    if (c->ciDf && n <= PA_MAXN) {
      k_project_apply_df<<<dim3(ceil_div(c->nG, 128), ceil_div(n, PA_J), c->nb), 128, 0, c->stream>>>(
          dOrbs, orbs, c->gram_d, TRAJ_PASS(c), g);
    } else {
      dim3 grid(ceil_div(c->nG, 256), n, c->nb);
      k_project_apply<<<grid, 256, 0, c->stream>>>(dOrbs, orbs, c->gram_d, TRAJ_PASS(c), g);
    }
    CODY_LAUNCHED(c);
  }
}

void launch_project_coeffs(cgpu_ctx* c, z_t* dC, const z_t* C) {
  ProfScope prof(c, CGPU_KERNEL_PROJECTORS);
  int nBlk = coeff_blocks(c);
  check_partial(c, nBlk);
  k_dot_partial<<<bgrid(c, nBlk), 256, 0, c->stream>>>(c->partial_d, C, dC, TRAJ_PASS(c));
  CODY_LAUNCHED(c);
  k_project_coeffs_apply<<<bgrid(c, vec_blocks(c, c->nC)), 256, 0, c->stream>>>(dC, C, c->partial_d, nBlk,
                                                                                  TRAJ_PASS(c));
  CODY_LAUNCHED(c);
}

void launch_normalize_coeffs(cgpu_ctx* c, z_t* C) {
  int nBlk = coeff_blocks(c);
  check_partial(c, nBlk);
  k_dot_partial<<<bgrid(c, nBlk), 256, 0, c->stream>>>(c->partial_d, C, C, TRAJ_PASS(c));
  CODY_LAUNCHED(c);
  k_normalize_apply<<<bgrid(c, vec_blocks(c, c->nC)), 256, 0, c->stream>>>(C, c->partial_d, nBlk, TRAJ_PASS(c));
  CODY_LAUNCHED(c);
}

void launch_fill_h1_from(cgpu_ctx* c, const z_t* orbs, const z_t* hOrbs, z_t* h1) {
  ProfScope prof(c, CGPU_KERNEL_PROJECTORS);
  launch_gram(c, c->gram_d, orbs, hOrbs, -1, c->nOS, 1.0);
  int nn = c->nO * c->nO;
  k_h1_layout<<<bgrid(c, ceil_div(nn, 128)), 128, 0, c->stream>>>(h1, c->gram_d, c->btOfOrb_d, TRAJ_PASS(c));
  CODY_LAUNCHED(c);
}

void launch_axpby(cgpu_ctx* c, z_t* y, const z_t* x, z_t a, z_t b, int sel) {
  ProfScope prof(c, CGPU_KERNEL_VECTOR);
  size_t n = sel == VSEL_STATE ? c->nS : c->nC;
  k_axpby<<<bgrid(c, vec_blocks(c, n)), 256, 0, c->stream>>>(y, x, a, b, TRAJ_PASS(c), sel);
  CODY_LAUNCHED(c);
}

void launch_scale(cgpu_ctx* c, z_t* y, z_t a, int sel) {
  ProfScope prof(c, CGPU_KERNEL_VECTOR);
  size_t n = sel == VSEL_STATE ? c->nS : c->nC;
  k_scale<<<bgrid(c, vec_blocks(c, n)), 256, 0, c->stream>>>(y, a, TRAJ_PASS(c), sel);
  CODY_LAUNCHED(c);
}

void launch_rk_stage(cgpu_ctx* c, z_t* inc, z_t* tmp, const z_t* state, const z_t* d, double wInc, double wTmp,
                     int first) {
  ProfScope prof(c, CGPU_KERNEL_VECTOR);
  k_rk_stage<<<bgrid(c, vec_blocks(c, c->nS)), 256, 0, c->stream>>>(inc, tmp, state, d, wInc, wTmp, first,
                                                                      TRAJ_PASS(c));
  CODY_LAUNCHED(c);
}

void launch_orthonormalize(cgpu_ctx* c, z_t* orbs, int col0, int nCols, int resetStatus) {
  if (resetStatus) batch_zero(c, c->scal_d, sizeof(int));
  k_mgs2<<<bgrid(c, 1), 1024, 0, c->stream>>>(orbs, c->w_d, TRAJ_PASS(c), col0, nCols, (int*)c->scal_d);
  CODY_LAUNCHED(c);
}

void launch_norm_dipole(cgpu_ctx* c, const z_t* state) {
  const z_t* orbs = (c->method == CGPU_METHOD_TDCI) ? c->tdciOrbs_d : state + c->nC;
  k_x_apply<<<bgrid(c, ew_blocks(c, (size_t)c->nG * c->nOS)), 256, 0, c->stream>>>(c->orbTmp_d, orbs, c->x_d,
                                                                                    TRAJ_PASS(c));
  CODY_LAUNCHED(c);
  launch_fill_h1_from(c, orbs, c->orbTmp_d, c->h1_d);  // h1 <- dipole matrix
  k_norm_dipole<<<bgrid(c, 1), 256, 0, c->stream>>>(c->scal_d, state, c->h1_d, c->rdm1_d, TRAJ_PASS(c));
  CODY_LAUNCHED(c);
}

void launch_energy(cgpu_ctx* c, double* out_d) {
  k_energy<<<bgrid(c, 1), 1024, 0, c->stream>>>(out_d, c->h1_d, c->rdm1_d, c->h2_d, c->rdm2_d, TRAJ_PASS(c));
  CODY_LAUNCHED(c);
}

void launch_set_scalar(cgpu_ctx* c, double* p, double v) {
  k_set_scalar<<<bgrid(c, 1), 1, 0, c->stream>>>(p, v, c->bs);
  CODY_LAUNCHED(c);
}

void launch_add_scalar(cgpu_ctx* c, double* p, double v) {
  k_add_scalar<<<bgrid(c, 1), 1, 0, c->stream>>>(p, v, c->bs);
  CODY_LAUNCHED(c);
}

void launch_absorber_setup(cgpu_ctx* c, double onset, double order) {
  k_absorber_mask<<<bgrid(c, ew_blocks(c, c->nG)), 256, 0, c->stream>>>(c->mask_d, c->x_d, onset, order,
                                                                          TRAJ_PASS(c));
  CODY_LAUNCHED(c);
}

void launch_absorber_apply(cgpu_ctx* c, z_t* orbs) {
  ProfScope prof(c, CGPU_KERNEL_VECTOR);
  k_absorber_apply<<<bgrid(c, ew_blocks(c, (size_t)c->nG * c->nOS)), 256, 0, c->stream>>>(orbs, c->mask_d,
                                                                                            TRAJ_PASS(c));
  CODY_LAUNCHED(c);
}
