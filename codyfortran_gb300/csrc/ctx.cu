// ctx.cu -- context set-up (the hot path's Fabricate/Setup chain), the
// equation-of-motion orchestration, the integrators and the C ABI.
//
// A context holds nb >= 1 systems.  Set-up builds each system on the host
// (grid, kinetic band, potential, pairs, configuration tables), then places
// the device data of all systems in one arena: trajectory b's buffers sit at
// byte offset b * bs from trajectory 0's, every buffer sized for the largest
// system.  The orchestration below is written once for all trajectories.
#include <sys/stat.h>

#include <algorithm>
#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>

#include "common.cuh"

namespace {

std::string g_lastGlobalError;
std::mutex g_errMutex;

constexpr double PI = 3.14159265358979323846264338327950288;

// ---------------------------------------------------------------------------
// Host-side set-up of one system
// ---------------------------------------------------------------------------
// Gauss-Legendre-Lobatto points/weights on [a,b]: interior nodes are the roots
// of P'_{n-1}, found by Newton's method from Chebyshev-Lobatto guesses;
// weights 2 / (n (n-1) P_{n-1}(x)^2).
void gll_points(int npts, double a, double b, std::vector<double>& x, std::vector<double>& w) {
  int deg = npts - 1;
  x.assign(npts, 0.0);
  w.assign(npts, 0.0);
  auto legendre = [&](double t, double& p, double& dp) {
    double pm = 1.0, pc = t;
    if (deg == 0) { p = 1.0; dp = 0.0; return; }
    for (int k = 2; k <= deg; k++) {
      double pn = ((2.0 * k - 1.0) * t * pc - (k - 1.0) * pm) / k;
      pm = pc;
      pc = pn;
    }
    p = pc;
    dp = (1.0 - t * t) != 0.0 ? deg * (pm - t * pc) / (1.0 - t * t) : 0.0;
  };
  for (int i = 0; i < npts; i++) {
    double t;
    if (i == 0) t = -1.0;
    else if (i == deg) t = 1.0;
    else {
      t = -std::cos(PI * i / deg);
      for (int it = 0; it < 100; it++) {
        double p, dp;
        legendre(t, p, dp);
        double d2p = (2.0 * t * dp - deg * (deg + 1.0) * p) / (1.0 - t * t);
        double step = dp / d2p;
        t -= step;
        if (std::fabs(step) < 1e-16) break;
      }
    }
    double p, dp;
    legendre(t, p, dp);
    x[i] = 0.5 * (b - a) * t + 0.5 * (a + b);
    w[i] = 0.5 * (b - a) * 2.0 / (deg * (deg + 1.0) * p * p);
  }
}

double lagrange_dprime(const std::vector<double>& xr, int basis, int node) {
  int n = (int)xr.size();
  if (basis == node) {
    double r = 0.0;
    for (int k = 0; k < n; k++)
      if (k != basis) r += 1.0 / (xr[node] - xr[k]);
    return r;
  }
  double r = 1.0 / (xr[basis] - xr[node]);
  for (int k = 0; k < n; k++)
    if (k != basis && k != node) r *= (xr[node] - xr[k]) / (xr[basis] - xr[k]);
  return r;
}

void setup_grid_and_kinetic(SysHost* c, int restricted, int nBt, const cgpu_desc* d) {
  std::vector<double>& x = c->x;
  std::vector<double>& w = c->w;
  std::vector<double> lap;  // (2b+1) x nG second-derivative band (mass independent)
  if (d->grid_kind == CGPU_GRID_CONST) {
    // grid.linear.const (src/Grid/Linear/Const/S_Grid_Linear_Const.f90:34-52) and the
    // 8th-order zero-ends stencil (src/Utils/M_Utils_DerivativeFinDiff.f90:66-71,179-198)
    int n = d->n_points;
    if (n < 2) throw std::string("grid.linear.const: nPoints must be >= 2");
    double dx = (d->xmax - d->xmin) / (n - 1);
    x.resize(n);
    w.assign(n, dx);
    for (int i = 0; i < n; i++) x[i] = d->xmin + w[i] * i;
    c->nG = n;
    c->band = 4;
    const double cst[5] = {-205.0 / 72.0, 8.0 / 5.0, -1.0 / 5.0, 8.0 / 315.0, -1.0 / 560.0};
    lap.assign((size_t)9 * n, 0.0);
    for (int dd = -4; dd <= 4; dd++)
      for (int g = 0; g < n; g++)
        if (g + dd >= 0 && g + dd < n) lap[(size_t)(dd + 4) * n + g] = cst[std::abs(dd)] / (dx * dx);
  } else if (d->grid_kind == CGPU_GRID_FEDVR) {
    // FEDVR grid (src/Utils/M_Utils_Fedvr.f90:76-149) with nLocals points per element and the
    // weak-form second derivative (src/Utils/M_Utils_DerivativeFedvr.f90:29-76,115-152):
    // (D2 f)_i = (sum_e K_ref f_e / dx_e)_i / w_i, K_ref(i,j) = -sum_k w_k D_ki D_kj on [-1/2,1/2].
    int nE = d->n_elements, nL = d->n_locals;
    if (nE < 1 || nL < 2) throw std::string("grid.linear.fedvr: need nElements >= 1 and nLocals >= 2");
    double es = (d->xmax - d->xmin) / nE;
    int np = nE * (nL - 1) + 1 - (d->xmin_excluded ? 1 : 0) - (d->xmax_excluded ? 1 : 0);
    x.assign(np, 0.0);
    w.assign(np, 0.0);
    std::vector<int> elStart(nE);
    std::vector<double> ep, ew;
    int iGrid = -1;
    for (int e = 0; e < nE; e++) {
      gll_points(nL, d->xmin + e * es, d->xmin + (e + 1) * es, ep, ew);
      int st = -1;
      for (int l = 0; l < nL; l++) {
        if (e == 0 && l == 0 && d->xmin_excluded) continue;
        if (e == nE - 1 && l == nL - 1 && d->xmax_excluded) continue;
        if (e == 0 || l != 0) iGrid++;
        if (st < 0) st = iGrid;
        x[iGrid] = ep[l];
        w[iGrid] += ew[l];
      }
      elStart[e] = st;
    }
    std::vector<double> xr, wr;
    gll_points(nL, -0.5, 0.5, xr, wr);
    std::vector<double> D((size_t)nL * nL), K((size_t)nL * nL, 0.0);
    for (int i = 0; i < nL; i++)
      for (int j = 0; j < nL; j++) D[i + (size_t)nL * j] = lagrange_dprime(xr, j, i);
    for (int i = 0; i < nL; i++)
      for (int j = 0; j < nL; j++) {
        double s = 0.0;
        for (int k = 0; k < nL; k++) s -= wr[k] * D[k + (size_t)nL * i] * D[k + (size_t)nL * j];
        K[i + (size_t)nL * j] = s;
      }
    c->nG = np;
    c->band = nL - 1;
    int b = c->band, nd = 2 * b + 1;
    lap.assign((size_t)nd * np, 0.0);
    for (int e = 0; e < nE; e++) {
      int l0 = (d->xmin_excluded && e == 0) ? 1 : 0;
      int l1 = (d->xmax_excluded && e == nE - 1) ? nL - 2 : nL - 1;
      for (int a = l0; a <= l1; a++)
        for (int bb = l0; bb <= l1; bb++) {
          int gi = elStart[e] + (a - l0), gj = elStart[e] + (bb - l0);
          lap[(size_t)(gj - gi + b) * np + gi] += K[a + (size_t)nL * bb] / es;
        }
    }
    for (int dd = 0; dd < nd; dd++)
      for (int g = 0; g < np; g++) lap[(size_t)dd * np + g] /= w[g];
  } else {
    throw std::string("unknown grid kind");
  }
  int nd = 2 * c->band + 1;
  c->nBtK = restricted ? 1 : nBt;
  c->band_h.assign((size_t)c->nBtK * nd * c->nG, 0.0);
  for (int bt = 0; bt < c->nBtK; bt++) {
    double m = c->mass[bt];
    if (!(m > 0.0)) throw std::string("sysKinetic: body masses must be positive");
    for (size_t k = 0; k < (size_t)nd * c->nG; k++) c->band_h[(size_t)bt * nd * c->nG + k] = -0.5 * lap[k] / m;
  }
}


template <typename T>
T* dalloc(size_t n) {
  T* p = nullptr;
  if (n == 0) n = 1;
  CODY_CUDA(cudaMalloc(&p, n * sizeof(T)));
  return p;
}

template <typename T>
T* dupload(const std::vector<T>& v) {
  T* p = dalloc<T>(v.size());
  CODY_CUDA(cudaMemcpy(p, v.data(), sizeof(T) * v.size(), cudaMemcpyHostToDevice));
  return p;
}

double soft_kernel(double s, double s1, double s2, double damp, double dist) {
  return s * std::exp(-dist * damp) / (std::sqrt(dist * dist + s1 * s1) + s2);
}

__global__ void k_build_vint(double* __restrict__ V, const double* __restrict__ x, int nG, int toeplitz, double dx,
                             double s, double s1, double s2, double damp) {
  size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (e >= (size_t)nG * nG) return;
  int i = (int)(e / nG), j = (int)(e % nG);
  double dist = toeplitz ? (double)abs(i - j) * dx : fabs(x[i] - x[j]);
  V[e] = s * exp(-dist * damp) / (sqrt(dist * dist + s1 * s1) + s2);
}

__global__ void k_set_step_times(double* __restrict__ stepT, const double* __restrict__ t0s, int nb, size_t bs) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b < nb) *(double*)((char*)stepT + (size_t)b * bs) = t0s[b];
}

__global__ void k_scatter_states(z_t* __restrict__ dst, const z_t* __restrict__ src, const long* __restrict__ off,
                                 TRAJ_ARGS) {
  const TrajShape& S = shp[blockIdx.z];
  dst = bat(dst, bs);
  src += off[blockIdx.z];
  for (size_t l = blockIdx.x * (size_t)blockDim.x + threadIdx.x; l < (size_t)S.nS; l += (size_t)gridDim.x * blockDim.x)
    dst[vidx(S, l)] = src[l];
}

__global__ void k_gather_states(z_t* __restrict__ dst, const z_t* __restrict__ src, const long* __restrict__ off,
                                TRAJ_ARGS) {
  const TrajShape& S = shp[blockIdx.z];
  src = bat(src, bs);
  dst += off[blockIdx.z];
  for (size_t l = blockIdx.x * (size_t)blockDim.x + threadIdx.x; l < (size_t)S.nS; l += (size_t)gridDim.x * blockDim.x)
    dst[l] = src[vidx(S, l)];
}

// One system from its descriptor (host data; CI tables on the device).
void build_system(cgpu_ctx* c, SysHost& s, const cgpu_desc* d) {
  if (d->n_body_types != c->nBt) throw std::string("batch: every system needs the same number of body types");
  if ((d->restricted ? 1 : 0) != c->restricted) throw std::string("batch: mixed restricted / unrestricted systems");
  if (d->method != c->method || d->precision != c->precision)
    throw std::string("batch: every system needs the same method and precision");
  if ((d->has_interaction ? 1 : 0) != c->hasInteraction) throw std::string("batch: mixed interaction settings");
  s.regEps = d->regularization > 0 ? d->regularization : 1e-10;
  s.nO = 0;
  for (int b = 0; b < c->nBt; b++) {
    s.nBodies[b] = d->n_bodies[b];
    s.nOrbs[b] = d->n_orbs[b];
    s.mass[b] = d->body_mass[b];
    s.orbStart[b] = s.nO;
    if (s.nOrbs[b] < 1 || s.nBodies[b] < 0 || s.nBodies[b] > s.nOrbs[b])
      throw std::string("method.mb: invalid nOrbs / nBodies");
    for (int i = 0; i < s.nOrbs[b]; i++) s.btOfOrb.push_back(b);
    s.nO += s.nOrbs[b];
  }
  if (c->restricted) {
    for (int b = 1; b < c->nBt; b++)
      if (s.nOrbs[b] != s.nOrbs[0]) throw std::string("orbs.restrictedQ needs equal nOrbs per body type");
    if (c->nBt != 2) throw std::string("orbs.restrictedQ needs two body types (spins)");
  }
  s.nOS = c->restricted ? s.nOrbs[0] : s.nO;
  if (s.nOS > 64) throw std::string("more than 64 stored orbitals is not supported");
  if (c->method != CGPU_METHOD_TDCI && s.nOS > 32)
    throw std::string("MCTDHX: more than 32 stored orbitals is not supported");
  setup_grid_and_kinetic(&s, c->restricted, c->nBt, d);
  for (int bt = 0; bt < s.nBtK; bt++)
    if (!(s.mass[bt] > 0.0)) throw std::string("sysKinetic: body masses must be positive");
  int nG = s.nG;
  // potential (src/SysPotential/Linear/SoftYukawa/StdImpl/*.f90:82-113)
  s.V0.assign(nG, 0.0);
  s.hasPotential = d->n_nuclei > 0;
  if (d->n_nuclei < 0 || d->n_nuclei > 8) throw std::string("sysPotential: 0..8 nuclei supported");
  for (int k = 0; k < d->n_nuclei; k++)
    for (int g = 0; g < nG; g++)
      s.V0[g] -= soft_kernel(d->nuc_charge[k], d->nuc_softening1[k], d->nuc_softening2[k], d->nuc_dampening[k],
                             std::fabs(s.x[g] - d->nuc_position[k]));
  // laser
  s.laserKind = d->laser_kind;
  s.E0 = d->laser_E0;
  s.omega = d->laser_omega;
  s.nCycles = d->laser_n_cycles;
  s.cep = d->laser_cep;
  s.tStart = d->laser_t_start;
  if (d->laser_kind == CGPU_LASER_SAMPLED) {
    if (!d->field_samples || d->n_field_samples <= 0) throw std::string("sampled field needs samples");
    s.samples.assign(d->field_samples, d->field_samples + d->n_field_samples);
    s.sampleDt = d->field_dt;
    s.sampleT0 = d->field_t0;
    s.samples_d = dupload(s.samples);
  }
  // interaction parameters (S_SysInteraction_Linear_SoftYukawa.f90:67-73)
  s.intToeplitz = d->int_kind == CGPU_INT_TOEPLITZ;
  s.intS = d->int_strength;
  s.intS1 = d->int_softening1;
  s.intS2 = d->int_softening2;
  s.intDamp = d->int_dampening;
  // pairs (l <= k, same body type) in the order of the reference's loops
  int n = s.nOS;
  s.pidx.assign((size_t)n * n, -1);
  for (int l = 0; l < n; l++)
    for (int k = l; k < n; k++) {
      if (!c->restricted && s.btOfOrb[l] != s.btOfOrb[k]) continue;
      s.pidx[(size_t)l * n + k] = (int)s.pl.size();
      s.pl.push_back(l);
      s.pk.push_back(k);
    }
  s.nPairs = (int)s.pl.size();
  // CI tables
  ci_build_tables(c, s);
  s.nC = s.view.nC;
  s.nS = (c->method == CGPU_METHOD_TDCI) ? s.nC : s.nC + nG * n;
}

size_t take(size_t& off, size_t bytes) {
  size_t o = (off + 255) & ~(size_t)255;
  off = o + std::max<size_t>(bytes, 1);
  return o;
}

// Sizes (base == nullptr) or places (base = the arena) the buffers of one
// trajectory block; returns the block size.
size_t layout(cgpu_ctx* c, char* base) {
  size_t off = 0;
  size_t nG = c->nG, nO2 = (size_t)c->nO * c->nO, nO4 = nO2 * nO2, n = c->nOS, Q = n * n, P = std::max(c->nPairs, 1);
  size_t nS = c->nS;
  int nd = 2 * c->band + 1;
  auto D = [&](double*& p, size_t cnt) { size_t o = take(off, sizeof(double) * cnt); if (base) p = (double*)(base + o); };
  auto I = [&](int*& p, size_t cnt) { size_t o = take(off, sizeof(int) * cnt); if (base) p = (int*)(base + o); };
  auto Z = [&](z_t*& p, size_t cnt) { size_t o = take(off, sizeof(z_t) * cnt); if (base) p = (z_t*)(base + o); };
  D(c->x_d, nG);
  D(c->mask_d, nG);
  D(c->w_d, nG);
  D(c->V0_d, nG);
  D(c->T_d, (size_t)c->nBtK * nd * nG);
  if (c->ciDf) {
    size_t o = take(off, sizeof(float2) * (size_t)c->nBtK * nd * nG);
    if (base) c->Tdf_d = (float2*)(base + o);
  }
  if (c->hasInteraction) D(c->Vint_d, nG * nG);
  D(c->metricW_d, nS);
  D(c->metricOne_d, nS);
  D(c->scal_d, 64);
  D(c->lz_d, 512);
  D(c->zero_d, 1);
  D(c->stepT_d, 1);
  I(c->btOfOrb_d, c->nO);
  I(c->pairL_d, P);
  I(c->pairK_d, P);
  I(c->pidx_d, Q);
  Z(c->h1Lin_d, nO2 + 1);
  Z(c->rdm1Lin_d, nO2 + 1);
  Z(c->h2Lin_d, nO4 + 1);
  if (c->ciDf) {
    size_t o1 = take(off, sizeof(float4) * (nO2 + 1));
    size_t o2 = take(off, sizeof(float4) * (nO4 + 1));
    if (base) {
      c->h1Df_d = (float4*)(base + o1);
      c->h2Df_d = (float4*)(base + o2);
    }
  }
  Z(c->rdm2Lin_d, nO4 + 1);
  Z(c->rdm1_d, nO2);
  Z(c->h1_d, nO2);
  Z(c->rdm2_d, nO4);
  Z(c->h2_d, nO4);
  Z(c->S_d, nG * P);
  Z(c->W_d, nG * P);
  Z(c->Sfull_d, nG * Q);
  Z(c->Wfull_d, 2 * nG * Q);
  Z(c->Rp_d, Q * Q);
  Z(c->h2s_d, Q * Q);
  Z(c->Mreg_d, Q);
  Z(c->Uprev_d, Q);
  Z(c->r1s_d, Q);
  Z(c->r2s_d, Q * Q);
  Z(c->gram_d, Q);
  Z(c->orbTmp_d, nG * n);
  Z(c->state_d, nS);
  Z(c->dstate_d, nS);
  Z(c->rkInc_d, nS);
  Z(c->rkTmp_d, nS);
  Z(c->rkStage_d, nS);
  Z(c->trial_d, nS);
  Z(c->work_d, nS);
  Z(c->lw_d, nS);
  Z(c->warm_d, nS);
  Z(c->basis_d, nS * (size_t)c->maxKrylov);
  if (c->method == CGPU_METHOD_TDCI) Z(c->tdciOrbs_d, nG * n);
  Z(c->partial_d, c->partialCap);
  off = mixed_layout(c, base, off);
  return (off + 1023) & ~(size_t)1023;
}

template <typename T>
void put(cgpu_ctx* c, int b, T* dst0, const std::vector<T>& v) {
  if (v.empty()) return;
  CODY_CUDA(cudaMemcpy((char*)dst0 + (size_t)b * c->bs, v.data(), sizeof(T) * v.size(), cudaMemcpyHostToDevice));
}


// Fixed-point form of a batch: when every trajectory has the same dense
// interaction and its grid is a contiguous, bitwise-equal piece of one of a
// few root grids (FEDVR boxes of different length with the same elements: the
// grids with an even and with an odd element count on [-n, n] form two
// families), every interaction matrix is a principal block of its root's; the
// contraction W = V S then reads one shared set of V slices per root
// (resident in L2) at the trajectory's row offset.
constexpr int FX_MAX_ROOTS = 8;
void detect_shared_interaction(cgpu_ctx* c) {
  const size_t n = c->sys.size();
  c->fxShared = 0;
  c->fxVRow.assign(n, 0);
  c->fxVRoot.assign(n, 0);
  c->fxRoots.clear();
  c->fxKgMax = (c->nG + 63) / 64 * 64;
  const bool fx = c->precision == CGPU_PREC_MIXED_FX || c->precision == CGPU_PREC_MIXED_FX6;
  if (!fx || !c->hasInteraction || n < 2) return;
  std::vector<int> order(n);
  for (size_t b = 0; b < n; b++) order[b] = (int)b;
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return c->sys[a].nG > c->sys[b].nG; });
  const SysHost& S0 = c->sys[order[0]];
  std::vector<int> roots, rows(n, 0), rootOf(n, 0);
  int kgMax = 0;
  for (int b : order) {
    const SysHost& s = c->sys[b];
    if (s.intToeplitz || s.intS != S0.intS || s.intS1 != S0.intS1 || s.intS2 != S0.intS2 ||
        s.intDamp != S0.intDamp || s.nG < 1)
      return;
    int found = -1;
    for (size_t r = 0; r < roots.size() && found < 0; r++) {
      const SysHost& B = c->sys[roots[r]];
      auto it = std::lower_bound(B.x.begin(), B.x.end(), s.x[0]);
      size_t off = (size_t)(it - B.x.begin());
      if (off + (size_t)s.nG <= B.x.size() && std::memcmp(&B.x[off], s.x.data(), sizeof(double) * s.nG) == 0) {
        found = (int)r;
        rows[b] = (int)off;
      }
    }
    if (found < 0) {  // a new root: the largest grid of its family
      if ((int)roots.size() == FX_MAX_ROOTS) return;
      found = (int)roots.size();
      roots.push_back(b);
      rows[b] = 0;
    }
    rootOf[b] = found;
    kgMax = std::max(kgMax, (rows[b] % 64 + s.nG + 63) / 64 * 64);
  }
  c->fxShared = 1;
  c->fxRoots = roots;
  c->fxVRow = rows;
  c->fxVRoot = rootOf;
  c->fxKgMax = kgMax;
}

void build_ctx(cgpu_ctx* c, const cgpu_desc* descs, int nSys) {
  const cgpu_desc* d0 = &descs[0];
  if (d0->n_body_types < 1 || d0->n_body_types > CODY_MAX_BT) throw std::string("method.mb.nBodyTypes out of range");
  if (d0->precision < CGPU_PREC_FP64 || d0->precision > CGPU_PREC_MIXED_FX6) throw std::string("unknown precision");
  c->nb = nSys;
  c->nBt = d0->n_body_types;
  c->restricted = d0->restricted ? 1 : 0;
  c->method = d0->method;
  c->precision = d0->precision;
  c->ciDf = (c->precision == CGPU_PREC_MIXED_FX || c->precision == CGPU_PREC_MIXED_FX6) ? 1 : 0;
  c->hasInteraction = d0->has_interaction ? 1 : 0;
  CODY_CUDA(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
  {
    int dev = 0;
    CODY_CUDA(cudaGetDevice(&dev));
    CODY_CUDA(cudaDeviceGetAttribute(&c->numSms, cudaDevAttrMultiProcessorCount, dev));
  }
  c->sys.resize(nSys);
  for (int b = 0; b < nSys; b++) build_system(c, c->sys[b], &descs[b]);
  // maxima over the systems
  int nGO = 0, minS = 1 << 30, maxK = 0;
  for (const SysHost& s : c->sys) {
    c->nG = std::max(c->nG, s.nG);
    c->nO = std::max(c->nO, s.nO);
    c->nOS = std::max(c->nOS, s.nOS);
    c->nC = std::max(c->nC, s.nC);
    c->nPairs = std::max(c->nPairs, s.nPairs);
    c->band = std::max(c->band, s.band);
    c->nBtK = std::max(c->nBtK, s.nBtK);
    c->anyLaser |= s.laserKind != CGPU_LASER_NONE;
    nGO = std::max(nGO, s.nG * s.nOS);
    minS = std::min(minS, s.nS);
  }
  for (int b = 0; b < nSys; b++) maxK = std::max(maxK, descs[b].max_krylov);
  c->krylovWindow = descs[0].krylov_window;
  for (int b = 0; b < nSys; b++)
    if (descs[b].krylov_window != c->krylovWindow || descs[b].krylov_window < 0)
      throw std::string("krylov_window must be >= 0 and the same for every trajectory of a batch");
  c->nGO = nGO;
  detect_shared_interaction(c);
  ci_build_work(c);
  c->nS = (c->method == CGPU_METHOD_TDCI) ? c->nC : c->nC + nGO;
  c->minS = minS;
  c->maxKrylov = std::max(1, std::min(maxK > 0 ? maxK : 32, 32));
  // Lanczos reductions: one system spreads 256-entry chunks over up to 4 blocks
  // per SM; a batch gives each trajectory a few blocks of 1024-entry chunks
  // (about 4k blocks in total: few partials, little per-block overhead).
  c->lzElems = nSys == 1 ? 1 : 4;
  {
    size_t chunk = (size_t)256 * c->lzElems;
    size_t need = ((size_t)c->nS + chunk - 1) / chunk;
    size_t cap = nSys == 1 ? 4 * 148 : std::max<size_t>(2, 4096 / (size_t)nSys);
    c->lzBlocks = (int)std::max<size_t>(1, std::min(cap, need));
    // the partials hold twice as many blocks (room for the tile tuner)
    c->lzBlocksHeur = c->lzBlocks;
    c->lzBlocksCap = (int)std::max<size_t>(1, std::min(need, (size_t)2 * c->lzBlocks));
  }
  c->lzBlocks = c->lzBlocksCap;
  c->partialCap = std::max({lanczos_partial_need(c), gram_partial_need(c, c->nOS), zgemm_partial_need(c),
                            (size_t)148});
  c->lzBlocks = c->lzBlocksHeur;
  // arena
  c->bs = layout(c, nullptr);
  size_t total = c->bs * (size_t)nSys;
  CODY_CUDA(cudaMalloc(&c->arena, total));
  CODY_CUDA(cudaMemset(c->arena, 0, total));
  CODY_CUDA(cudaDeviceSynchronize());
  layout(c, c->arena);
  // per-system static data
  c->shape_h.resize(nSys);
  for (int b = 0; b < nSys; b++) {
    SysHost& s = c->sys[b];
    put(c, b, c->x_d, s.x);
    put(c, b, c->mask_d, std::vector<double>(s.nG, 1.0));
    put(c, b, c->w_d, s.w);
    put(c, b, c->V0_d, s.V0);
    put(c, b, c->T_d, s.band_h);
    if (c->Tdf_d) {
      std::vector<float2> tdf(s.band_h.size());
      for (size_t k = 0; k < s.band_h.size(); k++) tdf[k] = df_split(s.band_h[k]);
      put(c, b, c->Tdf_d, tdf);
    }
    put(c, b, c->btOfOrb_d, s.btOfOrb);
    put(c, b, c->pairL_d, s.pl);
    put(c, b, c->pairK_d, s.pk);
    put(c, b, c->pidx_d, s.pidx);
    std::vector<double> mw(c->nS, 1.0), m1(c->nS, 1.0);
    if (c->method != CGPU_METHOD_TDCI)
      for (int o = 0; o < s.nOS; o++)
        for (int g = 0; g < s.nG; g++) mw[(size_t)c->nC + (size_t)o * s.nG + g] = s.w[g];
    put(c, b, c->metricW_d, mw);
    put(c, b, c->metricOne_d, m1);
    std::vector<z_t> eye((size_t)s.nOS * s.nOS, zmk(0.0, 0.0));
    for (int i = 0; i < s.nOS; i++) eye[(size_t)i * s.nOS + i] = zmk(1.0, 0.0);
    put(c, b, c->Uprev_d, eye);
    if (c->hasInteraction) {
      double dx = s.nG > 1 ? s.x[1] - s.x[0] : 0.0;
      size_t tot = (size_t)s.nG * s.nG;
      double* V = (double*)((char*)c->Vint_d + (size_t)b * c->bs);
      const double* xb = (const double*)((const char*)c->x_d + (size_t)b * c->bs);
      k_build_vint<<<(unsigned)((tot + 255) / 256), 256, 0, c->stream>>>(V, xb, s.nG, s.intToeplitz, dx, s.intS,
                                                                         s.intS1, s.intS2, s.intDamp);
      CODY_LAUNCHED(c);
    }
    TrajShape& t = c->shape_h[b];
    std::memset(&t, 0, sizeof(t));
    t.nG = s.nG;
    t.nOS = s.nOS;
    t.nO = s.nO;
    t.nC = s.nC;
    t.nS = s.nS;
    t.nGO = s.nG * s.nOS;
    t.nPairs = s.nPairs;
    t.band = s.band;
    t.restricted = c->restricted;
    t.hasPot = s.hasPotential || s.laserKind != CGPU_LASER_NONE;
    t.nBt = c->nBt;
    t.nCpad = c->nC;
    t.nGroups = c->restricted ? 1 : c->nBt;
    for (int g = 0; g < t.nGroups; g++) {
      t.grpStart[g] = c->restricted ? 0 : s.orbStart[g];
      t.grpSize[g] = c->restricted ? s.nOS : s.nOrbs[g];
    }
    t.vRow = c->fxShared ? c->fxVRow[b] : 0;
    t.gShift = t.vRow % 64;
    t.vRoot = c->fxShared ? c->fxVRoot[b] : 0;
    t.vExp = t.vRoot * c->nG + t.vRow;  // shared row exponents: [root][c->nG]
    t.Kg = (t.gShift + s.nG + 63) / 64 * 64;
    t.Kp = (2 * s.nPairs + 63) / 64 * 64;
    t.regEps = s.regEps;
    t.laser = LaserDev{s.laserKind, s.E0, s.omega, s.nCycles, s.cep, s.tStart, s.sampleDt, s.sampleT0,
                       (int)s.samples.size(), s.samples_d};
    t.view = s.view;
  }
  CODY_CUDA(cudaMalloc(&c->shape_d, sizeof(TrajShape) * nSys));
  CODY_CUDA(cudaMemcpy(c->shape_d, c->shape_h.data(), sizeof(TrajShape) * nSys, cudaMemcpyHostToDevice));
  CODY_CUDA(cudaMalloc(&c->stageOff_d, sizeof(long) * (nSys + 1)));
  std::vector<long> so(nSys + 1, 0);
  for (int b = 0; b < nSys; b++) so[b + 1] = so[b] + c->sys[b].nS;
  c->stageOff = so;
  CODY_CUDA(cudaMemcpy(c->stageOff_d, so.data(), sizeof(long) * (nSys + 1), cudaMemcpyHostToDevice));
  mixed_init(c);
  CODY_CUDA(cudaMallocHost(&c->lz_h, sizeof(double) * 512));
  CODY_CUDA(cudaDeviceSynchronize());
}

void free_ctx(cgpu_ctx* c) {
  mixed_free(c);
  mc_adjoint_free(c);
  if (c->stepGraph) cudaGraphExecDestroy(c->stepGraph);
  for (cudaEvent_t e : c->profEvents) cudaEventDestroy(e);
  for (SysHost& s : c->sys) {
    for (int b = 0; b < CODY_MAX_BT; b++) {
      CiTables& t = s.tab[b];
      void* tp[] = {t.codes, t.sN,     t.sExc,   t.sCode,  t.sFac,  t.dN,      t.dExc,   t.dCode,
                    t.dFac,  t.rankTab, t.sxCode, t.sxStart, t.sxSrc, t.sxDst,  t.sxFac,  t.dxCode,
                    t.dxStart, t.dxSrc, t.dxDst,  t.dxFac};
      for (void* p : tp)
        if (p) cudaFree(p);
    }
    if (s.samples_d) cudaFree(s.samples_d);
  }
  void* ptrs[] = {c->arena,      c->shape_d,     c->metricUser_d, c->stageOff_d, c->stage_d,
                  c->tStage_d,    c->applyWork_d, c->rdmWork_d,    c->pairWork_d,  c->sysTmp_d};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  if (c->lz_h) cudaFreeHost(c->lz_h);
  if (c->stream) cudaStreamDestroy(c->stream);
}

// ---------------------------------------------------------------------------
// Equation of motion on device buffers (all trajectories).  out = post * dState,
// where dState is the reference's time derivative (carrying its -i).
// ---------------------------------------------------------------------------
void td_device(cgpu_ctx* c, int which, z_t* out, const z_t* in, double t, z_t post) {
  z_t f = zmul(post, zmk(0.0, -1.0));
  bool unit = (f.x == 1.0 && f.y == 0.0);
  if (which == CGPU_TD_TDCI || c->method == CGPU_METHOD_TDCI) {
    if (c->method != CGPU_METHOD_TDCI) throw std::string("TDCI derivative needs a TDCI context");
    if (c->anyLaser) {  // time-dependent one-body part (Tdci :90-92)
      launch_onebody(c, c->orbTmp_d, c->tdciOrbs_d, t, zmk(1.0, 0.0), 0);
      launch_fill_h1_from(c, c->tdciOrbs_d, c->orbTmp_d, c->h1_d);
      launch_fold_h1(c);
    }
    batch_zero(c, out, sizeof(z_t) * c->nC);
    launch_ci_apply(c, in, out, 1, 1);
    if (!unit) launch_scale(c, out, f, VSEL_COEFFS);
    return;
  }
  const z_t* C = in;
  const z_t* orbs = in + c->nC;
  z_t* dC = out;
  z_t* dOrbs = out + c->nC;
  size_t nGO = c->nGO;
  if (which == CGPU_TD_ORBS_LIN) {
    batch_zero(c, dC, sizeof(z_t) * c->nC);
    launch_onebody(c, dOrbs, orbs, t, f, 0);
    return;
  }
  if (which != CGPU_TD_FULL && which != CGPU_TD_NONLIN) throw std::string("unknown time-derivative selector");
  // the nO^4 rdm2 / h2 tensors are not needed inside the derivative
  struct FuseScope {
    cgpu_ctx* c;
    int prev;
    explicit FuseScope(cgpu_ctx* cc) : c(cc), prev(cc->fuseLayouts) { c->fuseLayouts = 1; }
    ~FuseScope() { c->fuseLayouts = prev; }
  } fuse(c);
  launch_ci_rdm(c, C, 1, 1);
  if (which == CGPU_TD_FULL) {
    launch_onebody(c, dOrbs, orbs, t, zmk(1.0, 0.0), 0);
    launch_fill_h1_from(c, orbs, dOrbs, c->h1_d);
  } else {
    launch_onebody(c, c->orbTmp_d, orbs, t, zmk(1.0, 0.0), 0);
    launch_fill_h1_from(c, orbs, c->orbTmp_d, c->h1_d);
    batch_zero(c, dOrbs, sizeof(z_t) * nGO);
  }
  if (c->precision == CGPU_PREC_FP64) launch_correlation(c, dOrbs, orbs, 1);
  else launch_correlation_mixed(c, dOrbs, orbs, 1);
  launch_fold_h1(c);
  launch_fold_h2(c);
  batch_zero(c, dC, sizeof(z_t) * c->nC);
  launch_ci_apply(c, C, dC, 1, 1);
  launch_project_coeffs(c, dC, C);
  launch_project_orbs(c, dOrbs, orbs);
  if (!unit) launch_scale(c, out, f, VSEL_STATE);
}

// RK4 (src/IntegratorList/Rk/O4Expl/S_IntegratorList_Rk_O4Expl.f90:90-141) on state_d-like buffers.
void rk4_device(cgpu_ctx* c, int which, z_t* state, double t0, double t1) {
  double dt = t1 - t0, dt2 = dt / 2.0, dt3 = dt / 3.0, dt6 = dt / 6.0;
  z_t one = zmk(1.0, 0.0);
  td_device(c, which, c->dstate_d, state, t0, one);
  launch_rk_stage(c, c->rkInc_d, c->rkTmp_d, state, c->dstate_d, dt6, dt2, 1);
  double tp = t0 + dt2;
  td_device(c, which, c->dstate_d, c->rkTmp_d, tp, one);
  launch_rk_stage(c, c->rkInc_d, c->rkTmp_d, state, c->dstate_d, dt3, dt2, 0);
  td_device(c, which, c->dstate_d, c->rkTmp_d, tp, one);
  launch_rk_stage(c, c->rkInc_d, c->rkTmp_d, state, c->dstate_d, dt3, dt, 0);
  tp = t0 + dt;
  td_device(c, which, c->dstate_d, c->rkTmp_d, tp, one);
  launch_rk_stage(c, c->rkInc_d, nullptr, state, c->dstate_d, dt6, 0.0, 0);
  launch_axpby(c, state, c->rkInc_d, one, one, VSEL_STATE);
}

void euler_device(cgpu_ctx* c, int which, int imag, z_t* state, double t0, double t1) {
  z_t post = imag ? zmk(0.0, -1.0) : zmk(1.0, 0.0);
  td_device(c, which, c->dstate_d, state, t0, post);
  launch_axpby(c, state, c->dstate_d, zmk(t1 - t0, 0.0), zmk(1.0, 0.0), VSEL_STATE);
}

// One PerformLanczosStep from start (device) into out (may be start itself).
// Returns converged (adaptive) or -1 (not checked).
int lanczos_pass(cgpu_ctx* c, int which, double tBase, double dt, int maxDim, double tol, double* errOut,
                 const z_t* start, z_t* out) {
  launch_lanczos_start(c, start);
  double tEval = tBase + 0.5 * dt;
  int adaptive = tol > 0.0;
  if (adaptive && c->nb > 1) throw std::string("SIL: adaptive (tolerance > 0) steps need a single system");
  int converged = -1;
  int mUsed = maxDim;
  for (int j = 1; j <= maxDim; j++) {
    z_t* v = c->basis_d + (size_t)c->nS * (j - 1);
    // w = i * TimeDerivative(v); on OrbsLin with the three-term recurrence the
    // one-body apply also emits the recurrence's first-pass partials
    const int nPass1 = (which == CGPU_TD_ORBS_LIN && c->fuseOrbsLinLz) ? launch_onebody_lz(c, j, tEval) : 0;
    if (nPass1 == 0) td_device(c, which, c->lw_d, v, tEval, zmk(0.0, 1.0));
    launch_lanczos_update(c, j, maxDim, nPass1);
    if (adaptive) {
      launch_lanczos_tail(c, j, dt, 1);
      CODY_CUDA(cudaMemcpyAsync(c->lz_h, c->lz_d, sizeof(double) * 400, cudaMemcpyDeviceToHost, c->stream));
      CODY_CUDA(cudaStreamSynchronize(c->stream));
      double err = c->lz_h[CODY_LZ_ERR];
      bool breakdown = c->lz_h[CODY_LZ_BREAKJ] == (double)j;
      bool conv = err <= tol;
      if (errOut) *errOut = err;
      if (conv || breakdown || j == maxDim) {
        mUsed = j;
        converged = conv ? 1 : 0;
        break;
      }
    }
  }
  if (adaptive) {
    launch_lz_set(c, CODY_LZ_MDIM, (double)mUsed);
  } else {
    launch_lanczos_tail(c, 0, dt, 1);
  }
  launch_lanczos_combine(c, out, start);
  return converged;
}

// SIL Integrate (src/IntegratorList/Sil/S_IntegratorList_Sil.f90:114-177) on a device state.
int sil_device(cgpu_ctx* c, int which, z_t* state, double t0, double t1, int krylovDim, double tol, int maxRestarts,
               const double* metric_d) {
  const double zeroThreshold = 1.0e-14;
  if (std::fabs(t1 - t0) <= zeroThreshold) return 0;
  int maxDim = std::max(1, std::min(krylovDim, c->minS));
  if (maxDim > c->maxKrylov) throw std::string("SIL: krylovDim exceeds the context's max_krylov");
  c->metric_d = const_cast<double*>(metric_d);
  int warnings = 0;
  if (!(tol > 0.0)) {
    // fixed order: one pass, no acceptance test; the basis holds the start
    // vector, so the pass reads and overwrites the state in place (the
    // reference counts the unconverged pass as a warning)
    lanczos_pass(c, which, t0, t1 - t0, maxDim, tol, nullptr, state, state);
    return 1;
  }
  batch_copy(c, c->work_d, state, sizeof(z_t) * c->nS);
  double tCur = t0, rem = t1 - t0;
  while (std::fabs(rem) > zeroThreshold) {
    double dtS = rem;
    int restarts = 0;
    int conv = 0;
    for (;;) {
      double err = 0.0;
      conv = lanczos_pass(c, which, tCur, dtS, maxDim, tol, &err, c->work_d, c->trial_d);
      if (conv == 1) break;
      if (conv < 0) break;  // fixed-order pass: no convergence test (tolerance 0)
      if (std::fabs(dtS) <= zeroThreshold || restarts >= maxRestarts) break;
      dtS = 0.5 * dtS;
      restarts++;
    }
    if (conv != 1) warnings++;
    batch_copy(c, c->work_d, c->trial_d, sizeof(z_t) * c->nS);
    tCur = tCur + dtS;
    rem = rem - dtS;
  }
  batch_copy(c, state, c->work_d, sizeof(z_t) * c->nS);
  return warnings;
}

void split2_device(cgpu_ctx* c, z_t* state, double t0, double t1, int krylov, double tol, int maxRestarts,
                   int useMetric) {
  double dt = t1 - t0, time1 = t0, time2 = time1 + 0.5 * dt;
  const double* m = useMetric ? c->metricW_d : c->metricOne_d;
  if (krylov > 0) sil_device(c, CGPU_TD_ORBS_LIN, state, time1, time1 + 0.5 * dt, krylov, tol, maxRestarts, m);
  else rk4_device(c, CGPU_TD_ORBS_LIN, state, time1, time1 + 0.5 * dt);
  rk4_device(c, CGPU_TD_NONLIN, state, time1, time1 + 1.0 * dt);
  if (krylov > 0) sil_device(c, CGPU_TD_ORBS_LIN, state, time2, time2 + 0.5 * dt, krylov, tol, maxRestarts, m);
  else rk4_device(c, CGPU_TD_ORBS_LIN, state, time2, time2 + 0.5 * dt);
}

// Captures one fixed-order Strang step on state_d (every trajectory) as a CUDA
// graph.  The step reads its start times from stepT_d (the laser is evaluated
// on the device) and advances them by dt, so the graph can be replayed for
// consecutive steps.  A first step on a scratch copy of the state makes every
// launch of the capture valid outside it.
void capture_step_graph(cgpu_ctx* c, double t0, double dt, int krylov, int useMetric) {
  if (c->stepGraph) {
    cudaGraphExecDestroy(c->stepGraph);
    c->stepGraph = nullptr;
  }
  batch_copy(c, c->warm_d, c->state_d, sizeof(z_t) * c->nS);
  split2_device(c, c->warm_d, t0, t0 + dt, krylov, 0.0, 0, useMetric);
  CODY_CUDA(cudaStreamSynchronize(c->stream));
  // profiling events of the selected kernel family become event-record nodes of the graph
  c->profUsed = 0;
  long before = c->launches;
  cudaGraph_t g = nullptr;
  CODY_CUDA(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
  c->inCapture = 1;
  c->captureT0 = t0;
  try {
    split2_device(c, c->state_d, t0, t0 + dt, krylov, 0.0, 0, useMetric);
    if (c->absorbEachStep && c->method != CGPU_METHOD_TDCI) launch_absorber_apply(c, c->state_d + c->nC);
    launch_add_scalar(c, c->stepT_d, dt);
  } catch (...) {
    c->inCapture = 0;
    cudaStreamEndCapture(c->stream, &g);
    if (g) cudaGraphDestroy(g);
    throw;
  }
  c->inCapture = 0;
  c->graphProf = c->profTarget;
  c->graphProfUsed = c->profUsed;
  CODY_CUDA(cudaStreamEndCapture(c->stream, &g));
  c->graphKernels = (int)(c->launches - before);
  c->launches = before;
  cudaError_t e = cudaGraphInstantiate(&c->stepGraph, g, 0);
  cudaGraphDestroy(g);
  CODY_CUDA(e);
  c->graphDt = dt;
  c->graphKrylov = krylov;
  c->graphMetric = useMetric;
  c->graphAbsorb = c->absorbEachStep;
}

}  // namespace

void td_device_public(cgpu_ctx* c, int which, z_t* out, const z_t* in, double t) {
  td_device(c, which, out, in, t, zmk(0.0, 1.0));
}

void drop_step_graph(cgpu_ctx* c) {
  if (c->stepGraph) {
    cudaGraphExecDestroy(c->stepGraph);
    c->stepGraph = nullptr;
  }
  c->graphDt = 0.0;
}

double time_sil_lanczos(cgpu_ctx* c, int krylov) {
  drop_step_graph(c);
  batch_copy(c, c->warm_d, c->state_d, sizeof(z_t) * c->nS);
  c->profTarget = CGPU_KERNEL_LANCZOS;
  c->profUsed = 0;
  sil_device(c, CGPU_TD_ORBS_LIN, c->warm_d, 0.0, 0.005, krylov, 0.0, 0, c->metricW_d);
  CODY_CUDA(cudaStreamSynchronize(c->stream));
  double tot = 0.0;
  for (size_t i = 0; i + 1 < c->profUsed; i += 2) {
    float ms = 0.f;
    CODY_CUDA(cudaEventElapsedTime(&ms, c->profEvents[i], c->profEvents[i + 1]));
    tot += ms;
  }
  c->profTarget = 0;
  c->profUsed = 0;
  return tot;
}

namespace {

// Step start time of every trajectory (t0s has nb entries): one contiguous
// copy and a kernel that writes each trajectory's slot (a strided copy of nb
// single doubles costs the CUDA driver one transfer per trajectory).
void set_step_times(cgpu_ctx* c, const double* t0s) {
  if (!c->tStage_d) CODY_CUDA(cudaMalloc(&c->tStage_d, sizeof(double) * c->nb));
  CODY_CUDA(cudaMemcpyAsync(c->tStage_d, t0s, sizeof(double) * c->nb, cudaMemcpyHostToDevice, c->stream));
  k_set_step_times<<<ceil_div(c->nb, 256), 256, 0, c->stream>>>(c->stepT_d, c->tStage_d, c->nb, c->bs);
  CODY_LAUNCHED(c);
}

// n_steps replays of the step graph (captured when dt, order or metric changed).
void propagate_graph(cgpu_ctx* c, const double* t0s, double dt, int nSteps, int krylov, int useMetric) {
  if (!c->stepGraph || c->graphDt != dt || c->graphKrylov != krylov || c->graphMetric != useMetric ||
      c->graphProf != c->profTarget || c->graphAbsorb != c->absorbEachStep)
    capture_step_graph(c, t0s[0], dt, krylov, useMetric);
  if (c->profTarget) c->profUsed = c->graphProfUsed;
  set_step_times(c, t0s);
  for (int s = 0; s < nSteps; s++) CODY_CUDA(cudaGraphLaunch(c->stepGraph, c->stream));
  c->launches += (long)nSteps * c->graphKernels;
}

// energies of every trajectory (device), E of trajectory b at out_d + b*bs
void energy_launch(cgpu_ctx* c, const z_t* state, double t) {
  const z_t* C = state;
  const z_t* orbs = (c->method == CGPU_METHOD_TDCI) ? c->tdciOrbs_d : state + c->nC;
  launch_ci_rdm(c, C, 1, 1);
  launch_onebody(c, c->orbTmp_d, orbs, t, zmk(1.0, 0.0), 0);
  launch_fill_h1_from(c, orbs, c->orbTmp_d, c->h1_d);
  launch_fill_h2(c, orbs);
  launch_energy(c, c->scal_d + CODY_SCAL_ENERGY);
}

double energy_device(cgpu_ctx* c, const z_t* state, double t) {
  energy_launch(c, state, t);
  double e = 0.0;
  CODY_CUDA(cudaMemcpyAsync(&e, c->scal_d + CODY_SCAL_ENERGY, sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  CODY_CUDA(cudaStreamSynchronize(c->stream));
  return e;
}

// helpers for host <-> device staging (trajectory 0, contiguous)
void up(cgpu_ctx* c, z_t* dst, const cgpu_complex* src, size_t n) {
  CODY_CUDA(cudaMemcpyAsync(dst, src, sizeof(z_t) * n, cudaMemcpyHostToDevice, c->stream));
}
void down(cgpu_ctx* c, cgpu_complex* dst, const z_t* src, size_t n) {
  CODY_CUDA(cudaMemcpyAsync(dst, src, sizeof(z_t) * n, cudaMemcpyDeviceToHost, c->stream));
}
// state vector of trajectory b ([C | orbitals], nS_b entries) <-> its device layout
void up_state(cgpu_ctx* c, int b, z_t* dst0, const cgpu_complex* src) {
  const SysHost& s = c->sys[b];
  char* base = (char*)dst0 + (size_t)b * c->bs;
  CODY_CUDA(cudaMemcpyAsync(base, src, sizeof(z_t) * s.nC, cudaMemcpyHostToDevice, c->stream));
  if (s.nS > s.nC)
    CODY_CUDA(cudaMemcpyAsync(base + sizeof(z_t) * c->nC, src + s.nC, sizeof(z_t) * (s.nS - s.nC),
                              cudaMemcpyHostToDevice, c->stream));
}
void down_state(cgpu_ctx* c, int b, cgpu_complex* dst, const z_t* src0) {
  const SysHost& s = c->sys[b];
  const char* base = (const char*)src0 + (size_t)b * c->bs;
  CODY_CUDA(cudaMemcpyAsync(dst, base, sizeof(z_t) * s.nC, cudaMemcpyDeviceToHost, c->stream));
  if (s.nS > s.nC)
    CODY_CUDA(cudaMemcpyAsync(dst + s.nC, base + sizeof(z_t) * c->nC, sizeof(z_t) * (s.nS - s.nC),
                              cudaMemcpyDeviceToHost, c->stream));
}
// ---- restart files (M_Utils_DataStorage raw format) of one trajectory --------
// coeffs.in (nC complex), orbBB_KK.in per stored orbital (nG complex each), and
// with rdm2 the blocks rdm2BtXX_YY.in (n1 x n2 x n1 x n2, Fortran order).
std::string dir_prefix(const char* dir) {
  std::string pre = dir ? std::string(dir) : std::string();
  if (!pre.empty() && pre.back() != '/') pre += '/';
  return pre;
}

void write_file(const std::string& path, const void* p, size_t bytes) {
  FILE* f = std::fopen(path.c_str(), "wb");
  if (!f) throw std::string("save_restart: cannot open ") + path;
  const size_t w = std::fwrite(p, 1, bytes, f);
  std::fclose(f);
  if (w != bytes) throw std::string("save_restart: short write to ") + path;
}

void read_file(const std::string& path, void* p, size_t bytes) {
  FILE* f = std::fopen(path.c_str(), "rb");
  if (!f) throw std::string("load_restart: cannot open ") + path;
  const size_t r = std::fread(p, 1, bytes, f);
  std::fclose(f);
  if (r != bytes) throw std::string("load_restart: more data requested than stored in ") + path;
}

void down_state(cgpu_ctx* c, int b, cgpu_complex* dst, const z_t* src0);
void up_state(cgpu_ctx* c, int b, z_t* dst0, const cgpu_complex* src);
void sync(cgpu_ctx* c);

// Trajectory b's resident state (and, when withRdm2, its rdm2 as left by
// launch_ci_rdm) into the files under pre.
void save_traj(cgpu_ctx* c, int b, const std::string& pre, bool withRdm2) {
  const SysHost& s = c->sys[b];
  std::vector<cgpu_complex> st(s.nS);
  down_state(c, b, st.data(), c->state_d);
  std::vector<cgpu_complex> r2;
  const size_t nO = s.nO;
  if (withRdm2) {
    r2.resize(nO * nO * nO * nO);
    CODY_CUDA(cudaMemcpyAsync(r2.data(), (const char*)c->rdm2_d + (size_t)b * c->bs, sizeof(z_t) * r2.size(),
                              cudaMemcpyDeviceToHost, c->stream));
  }
  sync(c);
  write_file(pre + "coeffs.in", st.data(), sizeof(cgpu_complex) * s.nC);
  if (c->method != CGPU_METHOD_TDCI) {
    const int nBt = c->restricted ? 1 : c->nBt;
    int i1 = 0;
    for (int bt = 0; bt < nBt; bt++)
      for (int k = 0; k < s.nOrbs[bt]; k++, i1++) {
        char name[32];
        std::snprintf(name, sizeof(name), "orb%02d_%02d.in", bt + 1, k + 1);
        write_file(pre + name, st.data() + s.nC + (size_t)i1 * s.nG, sizeof(cgpu_complex) * s.nG);
      }
  }
  if (!withRdm2) return;
  for (int b1 = 0; b1 < c->nBt; b1++)
    for (int b2 = 0; b2 < c->nBt; b2++) {
      const int s1 = s.orbStart[b1], n1 = s.nOrbs[b1], s2 = s.orbStart[b2], n2 = s.nOrbs[b2];
      std::vector<cgpu_complex> blk((size_t)n1 * n2 * n1 * n2);
      size_t q = 0;
      for (int l = 0; l < n2; l++)
        for (int k = 0; k < n1; k++)
          for (int j = 0; j < n2; j++)
            for (int i = 0; i < n1; i++, q++)
              blk[q] = r2[(s1 + i) + nO * ((s2 + j) + nO * ((s1 + k) + nO * (size_t)(s2 + l)))];
      char name[32];
      std::snprintf(name, sizeof(name), "rdm2Bt%02d_%02d.in", b1 + 1, b2 + 1);
      write_file(pre + name, blk.data(), sizeof(cgpu_complex) * blk.size());
    }
}

// The files under pre into trajectory b's resident state.
void load_traj(cgpu_ctx* c, int b, const std::string& pre) {
  const SysHost& s = c->sys[b];
  std::vector<cgpu_complex> st(s.nS);
  read_file(pre + "coeffs.in", st.data(), sizeof(cgpu_complex) * s.nC);
  if (c->method != CGPU_METHOD_TDCI) {
    const int nBt = c->restricted ? 1 : c->nBt;
    int i1 = 0;
    for (int bt = 0; bt < nBt; bt++)
      for (int k = 0; k < s.nOrbs[bt]; k++, i1++) {
        char name[32];
        std::snprintf(name, sizeof(name), "orb%02d_%02d.in", bt + 1, k + 1);
        read_file(pre + name, st.data() + s.nC + (size_t)i1 * s.nG, sizeof(cgpu_complex) * s.nG);
      }
  }
  up_state(c, b, c->state_d, st.data());
  sync(c);  // st is freed on return
}

// Subdirectory of trajectory b of a batch: <dir>/trajNNNNN/ (created on save).
std::string traj_prefix(const char* dir, int b, bool create) {
  std::string base = dir_prefix(dir);
  char name[32];
  std::snprintf(name, sizeof(name), "traj%05d", b);
  std::string path = base + name;
  if (create && mkdir(path.c_str(), 0755) != 0 && errno != EEXIST)
    throw std::string("batch_save_restart: cannot create ") + path;
  return path + "/";
}

void sync(cgpu_ctx* c) {
  CODY_CUDA(cudaStreamSynchronize(c->stream));
  if (c->mixed && mixed_error(c)) throw std::string("tensor-core GEMM: a bounded mbarrier wait expired");
}

int fail(cgpu_ctx* c, const std::string& msg, int code) {
  if (c) c->lastError = msg;
  std::lock_guard<std::mutex> g(g_errMutex);
  g_lastGlobalError = msg;
  return code;
}

#define CODY_API_BEGIN(ctx)                                    \
  if (!(ctx)) return fail(nullptr, "null context", CGPU_ERR_ARG); \
  try {
#define CODY_API_END(ctx)                                                       \
  }                                                                             \
  catch (const std::string& e) {                                                \
    int code = (e.find("cuda") != std::string::npos || e.find("Cuda") != std::string::npos) ? CGPU_ERR_CUDA : CGPU_ERR_ARG; \
    return fail(ctx, e, code);                                                  \
  }                                                                             \
  catch (const std::exception& e) {                                             \
    return fail(ctx, e.what(), CGPU_ERR_ARG);                                    \
  }                                                                             \
  return CGPU_OK;

cgpu_ctx* create_ctx(const cgpu_desc* descs, int n, int* rc) {
  cgpu_ctx* c = new cgpu_ctx();
  try {
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
      cudaGetLastError();
      throw std::string("cuda: no CUDA device available");
    }
    build_ctx(c, descs, n);
  } catch (const std::string& e) {
    free_ctx(c);
    delete c;
    *rc = fail(nullptr, e, e.find("cuda") != std::string::npos ? CGPU_ERR_CUDA : CGPU_ERR_ARG);
    return nullptr;
  } catch (const std::exception& e) {
    free_ctx(c);
    delete c;
    *rc = fail(nullptr, e.what(), CGPU_ERR_ARG);
    return nullptr;
  }
  *rc = CGPU_OK;
  return c;
}

// Observables of every trajectory (RDM observables, src/Utils/M_Utils_RdmObservables.f90:17-52,
// and the printers' quantities, src/Utils/M_Utils_PrinterObservableLinear.f90:25-103):
// out[b*stride + 0..2] = energy, ||C||, <x>; then the natural occupations in
// descending order (zeros past the trajectory's orbital count).  stride = 3 + nOS(max).
void observables(cgpu_ctx* c, const double* tHost, double* out) {
  const int stride = 3 + c->nOS;
  set_step_times(c, tHost);
  c->useStepTime = 1;
  try {
    energy_launch(c, c->state_d, 0.0);
  } catch (...) {
    c->useStepTime = 0;
    throw;
  }
  c->useStepTime = 0;
  const bool occ = c->method != CGPU_METHOD_TDCI && c->nOS <= 32;
  if (occ) launch_rdm_inverse(c);
  launch_norm_dipole(c, c->state_d);
  std::vector<double> rows((size_t)c->nb * 64);
  CODY_CUDA(cudaMemcpy2DAsync(rows.data(), 64 * sizeof(double), c->scal_d, c->bs, 64 * sizeof(double), c->nb,
                              cudaMemcpyDeviceToHost, c->stream));
  sync(c);
  for (int b = 0; b < c->nb; b++) {
    const double* r = rows.data() + (size_t)b * 64;
    double* o = out + (size_t)b * stride;
    o[0] = r[CODY_SCAL_ENERGY];
    o[1] = r[CODY_SCAL_NORM];
    o[2] = r[CODY_SCAL_DIPOLE];
    int n = c->sys[b].nOS;
    std::vector<double> ev(occ ? r + CODY_SCAL_OCC : r, occ ? r + CODY_SCAL_OCC + n : r);
    std::sort(ev.begin(), ev.end(), [](double a, double bb) { return a > bb; });
    for (int k = 0; k < c->nOS; k++) o[3 + k] = k < (int)ev.size() ? ev[k] : 0.0;
  }
}

}  // namespace

void batch_zero(cgpu_ctx* c, void* p, size_t bytes) {
  ProfScope prof(c, CGPU_KERNEL_VECTOR);
  CODY_CUDA(cudaMemset2DAsync(p, c->bs, 0, bytes, c->nb, c->stream));
}

void batch_copy(cgpu_ctx* c, void* dst, const void* src, size_t bytes) {
  ProfScope prof(c, CGPU_KERNEL_VECTOR);
  CODY_CUDA(cudaMemcpy2DAsync(dst, c->bs, src, c->bs, bytes, c->nb, cudaMemcpyDeviceToDevice, c->stream));
}

// Records the message returned by cgpu_last_global_error (for entry points without a context).
void cody_record_global_error(const std::string& msg) {
  std::lock_guard<std::mutex> g(g_errMutex);
  g_lastGlobalError = msg;
}

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
extern "C" {

int cgpu_ctx_create(const cgpu_desc* desc, cgpu_ctx** out) {
  if (!desc || !out) return fail(nullptr, "cgpu_ctx_create: null argument", CGPU_ERR_ARG);
  int rc = CGPU_OK;
  *out = create_ctx(desc, 1, &rc);
  return rc;
}

int cgpu_ctx_destroy(cgpu_ctx* ctx) {
  if (!ctx) return CGPU_OK;
  free_ctx(ctx);
  delete ctx;
  return CGPU_OK;
}

const char* cgpu_last_error(const cgpu_ctx* ctx) { return ctx ? ctx->lastError.c_str() : g_lastGlobalError.c_str(); }
const char* cgpu_last_global_error(void) { return g_lastGlobalError.c_str(); }

int cgpu_host_alloc(size_t bytes, void** out) {
  if (!out) {
    cody_record_global_error("cgpu_host_alloc: null argument");
    return CGPU_ERR_ARG;
  }
  *out = nullptr;
  if (bytes == 0) return CGPU_OK;
  const cudaError_t e = cudaHostAlloc(out, bytes, cudaHostAllocDefault);
  if (e != cudaSuccess) {
    *out = nullptr;
    cody_record_global_error(std::string("cgpu_host_alloc: ") + cudaGetErrorString(e));
    return CGPU_ERR_CUDA;
  }
  return CGPU_OK;
}

int cgpu_select_device(int device) {
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e == cudaSuccess && (device < 0 || device >= n)) {
    cody_record_global_error("cgpu_select_device: no device " + std::to_string(device));
    return CGPU_ERR_ARG;
  }
  if (e == cudaSuccess) e = cudaSetDevice(device);
  if (e != cudaSuccess) {
    cody_record_global_error(std::string("cgpu_select_device: ") + cudaGetErrorString(e));
    return CGPU_ERR_CUDA;
  }
  return CGPU_OK;
}

int cgpu_host_free(void* ptr) {
  if (!ptr) return CGPU_OK;
  const cudaError_t e = cudaFreeHost(ptr);
  if (e != cudaSuccess) {
    cody_record_global_error(std::string("cgpu_host_free: ") + cudaGetErrorString(e));
    return CGPU_ERR_CUDA;
  }
  return CGPU_OK;
}

int cgpu_sizes(const cgpu_ctx* c, int* out) {
  if (!c || !out) return CGPU_ERR_ARG;
  out[0] = c->nG; out[1] = c->nO; out[2] = c->nOS; out[3] = c->nC; out[4] = c->nBt; out[5] = c->nS;
  return CGPU_OK;
}

int cgpu_grid(const cgpu_ctx* c, double* x, double* w) {
  if (!c) return CGPU_ERR_ARG;
  const SysHost& s = c->sys[0];
  if (x) std::memcpy(x, s.x.data(), sizeof(double) * s.nG);
  if (w) std::memcpy(w, s.w.data(), sizeof(double) * s.nG);
  return CGPU_OK;
}

int cgpu_configlist_tables(cgpu_ctx* c, int bt, int kind, int* n_conf, int* max_conn, int64_t* codes,
                           int* n_connected, int* excited_c, int* orb_code, double* factor) {
  CODY_API_BEGIN(c)
  if (bt < 0 || bt >= c->nBt) throw std::string("configlist: body type out of range");
  CiTables& t = c->sys[0].tab[bt];
  int mc = kind == 0 ? t.maxS : t.maxD;
  if (n_conf) *n_conf = t.nConf;
  if (max_conn) *max_conn = mc;
  size_t tot = (size_t)mc * t.nConf;
  if (codes) CODY_CUDA(cudaMemcpy(codes, t.codes, sizeof(int64_t) * t.nConf, cudaMemcpyDeviceToHost));
  if (n_connected)
    CODY_CUDA(cudaMemcpy(n_connected, kind == 0 ? t.sN : t.dN, sizeof(int) * t.nConf, cudaMemcpyDeviceToHost));
  if (excited_c && tot)
    CODY_CUDA(cudaMemcpy(excited_c, kind == 0 ? t.sExc : t.dExc, sizeof(int) * tot, cudaMemcpyDeviceToHost));
  if (orb_code && tot)
    CODY_CUDA(cudaMemcpy(orb_code, kind == 0 ? t.sCode : t.dCode, sizeof(int) * tot, cudaMemcpyDeviceToHost));
  if (factor && tot) {
    std::vector<int8_t> f(tot);
    CODY_CUDA(cudaMemcpy(f.data(), kind == 0 ? t.sFac : t.dFac, tot, cudaMemcpyDeviceToHost));
    for (size_t i = 0; i < tot; i++) factor[i] = (double)f[i];
  }
  CODY_API_END(c)
}

int cgpu_synchronize(cgpu_ctx* c) {
  CODY_API_BEGIN(c)
  sync(c);
  CODY_API_END(c)
}

long cgpu_launch_count(cgpu_ctx* c, int reset) {
  if (!c) return -1;
  long n = c->launches;
  if (reset) c->launches = 0;
  return n;
}

int cgpu_time_derivative(cgpu_ctx* c, int which, cgpu_complex* d_state, const cgpu_complex* state, double time) {
  CODY_API_BEGIN(c)
  if (!d_state || !state) throw std::string("time_derivative: null array");
  up(c, c->rkStage_d, state, c->nS);
  td_device(c, which, c->dstate_d, c->rkStage_d, time, zmk(1.0, 0.0));
  down(c, d_state, c->dstate_d, c->nS);
  sync(c);
  CODY_API_END(c)
}

int cgpu_apply_single_body_op(cgpu_ctx* c, cgpu_complex* d_orbs, const cgpu_complex* orbs, double time,
                              cgpu_complex* h1) {
  CODY_API_BEGIN(c)
  size_t n = (size_t)c->nG * c->nOS;
  up(c, c->rkStage_d, orbs, n);
  up(c, c->orbTmp_d, d_orbs, n);
  launch_onebody(c, c->orbTmp_d, c->rkStage_d, time, zmk(1.0, 0.0), 1);
  if (h1) {
    launch_fill_h1_from(c, c->rkStage_d, c->orbTmp_d, c->h1_d);
    down(c, h1, c->h1_d, (size_t)c->nO * c->nO);
  }
  down(c, d_orbs, c->orbTmp_d, n);
  sync(c);
  CODY_API_END(c)
}

int cgpu_fill_h1(cgpu_ctx* c, cgpu_complex* h1, const cgpu_complex* orbs, double time) {
  CODY_API_BEGIN(c)
  size_t n = (size_t)c->nG * c->nOS;
  up(c, c->rkStage_d, orbs, n);
  launch_onebody(c, c->orbTmp_d, c->rkStage_d, time, zmk(1.0, 0.0), 0);
  launch_fill_h1_from(c, c->rkStage_d, c->orbTmp_d, c->h1_d);
  down(c, h1, c->h1_d, (size_t)c->nO * c->nO);
  sync(c);
  CODY_API_END(c)
}

int cgpu_fill_h2(cgpu_ctx* c, cgpu_complex* h2, const cgpu_complex* orbs, double time) {
  CODY_API_BEGIN(c)
  (void)time;
  size_t n = (size_t)c->nG * c->nOS;
  up(c, c->rkStage_d, orbs, n);
  launch_fill_h2(c, c->rkStage_d);
  down(c, h2, c->h2_d, (size_t)c->nO * c->nO * c->nO * c->nO);
  sync(c);
  CODY_API_END(c)
}

int cgpu_apply_correlation_op(cgpu_ctx* c, cgpu_complex* d_orbs, const cgpu_complex* orbs, const cgpu_complex* rdm1,
                              const cgpu_complex* rdm2, double time, cgpu_complex* h2) {
  CODY_API_BEGIN(c)
  (void)time;
  size_t n = (size_t)c->nG * c->nOS, nO2 = (size_t)c->nO * c->nO;
  up(c, c->rkStage_d, orbs, n);
  up(c, c->orbTmp_d, d_orbs, n);
  up(c, c->rdm1_d, rdm1, nO2);
  up(c, c->rdm2_d, rdm2, nO2 * nO2);
  if (c->precision == CGPU_PREC_FP64) launch_correlation(c, c->orbTmp_d, c->rkStage_d, h2 != nullptr);
  else launch_correlation_mixed(c, c->orbTmp_d, c->rkStage_d, h2 != nullptr);
  down(c, d_orbs, c->orbTmp_d, n);
  if (h2) down(c, h2, c->h2_d, nO2 * nO2);
  sync(c);
  CODY_API_END(c)
}

int cgpu_energy(cgpu_ctx* c, const cgpu_complex* state, double time, double* energy) {
  CODY_API_BEGIN(c)
  up(c, c->rkStage_d, state, c->nS);
  *energy = energy_device(c, c->rkStage_d, time);
  CODY_API_END(c)
}

int cgpu_ci_apply_h1_fill_rdm1(cgpu_ctx* c, const cgpu_complex* coeffs, cgpu_complex* rdm1, cgpu_complex* d_coeffs,
                               const cgpu_complex* h1) {
  CODY_API_BEGIN(c)
  size_t nO2 = (size_t)c->nO * c->nO;
  up(c, c->rkStage_d, coeffs, c->nC);
  if (rdm1) {
    launch_ci_rdm(c, c->rkStage_d, 1, 0);
    down(c, rdm1, c->rdm1_d, nO2);
  }
  if (d_coeffs && h1) {
    up(c, c->h1_d, h1, nO2);
    launch_fold_h1(c);
    up(c, c->dstate_d, d_coeffs, c->nC);
    launch_ci_apply(c, c->rkStage_d, c->dstate_d, 1, 0);
    down(c, d_coeffs, c->dstate_d, c->nC);
  }
  sync(c);
  CODY_API_END(c)
}

int cgpu_ci_apply_h2_fill_rdm2(cgpu_ctx* c, const cgpu_complex* coeffs, cgpu_complex* rdm2, cgpu_complex* d_coeffs,
                               const cgpu_complex* h2) {
  CODY_API_BEGIN(c)
  size_t nO2 = (size_t)c->nO * c->nO;
  up(c, c->rkStage_d, coeffs, c->nC);
  if (rdm2) {
    launch_ci_rdm(c, c->rkStage_d, 0, 1);
    down(c, rdm2, c->rdm2_d, nO2 * nO2);
  }
  if (d_coeffs && h2) {
    up(c, c->h2_d, h2, nO2 * nO2);
    launch_fold_h2(c);
    up(c, c->dstate_d, d_coeffs, c->nC);
    launch_ci_apply(c, c->rkStage_d, c->dstate_d, 0, 1);
    down(c, d_coeffs, c->dstate_d, c->nC);
  }
  sync(c);
  CODY_API_END(c)
}

int cgpu_project_coeffs(cgpu_ctx* c, cgpu_complex* d_coeffs, const cgpu_complex* coeffs) {
  CODY_API_BEGIN(c)
  up(c, c->rkStage_d, coeffs, c->nC);
  up(c, c->dstate_d, d_coeffs, c->nC);
  launch_project_coeffs(c, c->dstate_d, c->rkStage_d);
  down(c, d_coeffs, c->dstate_d, c->nC);
  sync(c);
  CODY_API_END(c)
}

int cgpu_normalize_coeffs(cgpu_ctx* c, cgpu_complex* coeffs) {
  CODY_API_BEGIN(c)
  up(c, c->rkStage_d, coeffs, c->nC);
  launch_normalize_coeffs(c, c->rkStage_d);
  down(c, coeffs, c->rkStage_d, c->nC);
  sync(c);
  CODY_API_END(c)
}

int cgpu_project_orbs(cgpu_ctx* c, cgpu_complex* d_orbs, const cgpu_complex* orbs) {
  CODY_API_BEGIN(c)
  size_t n = (size_t)c->nG * c->nOS;
  up(c, c->rkStage_d, orbs, n);
  up(c, c->orbTmp_d, d_orbs, n);
  launch_project_orbs(c, c->orbTmp_d, c->rkStage_d);
  down(c, d_orbs, c->orbTmp_d, n);
  sync(c);
  CODY_API_END(c)
}

int cgpu_orthonormalize_orbs(cgpu_ctx* c, cgpu_complex* orbs) {
  CODY_API_BEGIN(c)
  const SysHost& s = c->sys[0];
  size_t n = (size_t)c->nG * c->nOS;
  up(c, c->orbTmp_d, orbs, n);
  if (c->restricted) launch_orthonormalize(c, c->orbTmp_d, 0, c->nOS);
  else
    for (int b = 0; b < c->nBt; b++) launch_orthonormalize(c, c->orbTmp_d, s.orbStart[b], s.nOrbs[b]);
  down(c, orbs, c->orbTmp_d, n);
  int status = 0;
  CODY_CUDA(cudaMemcpyAsync(&status, c->scal_d, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  sync(c);
  if (status) throw std::string("Grid Orthonormalize: vector with non-positive norm (linearly dependent input set?)");
  CODY_API_END(c)
}

int cgpu_integrate_rk4(cgpu_ctx* c, int which, cgpu_complex* state, double t0, double t1) {
  CODY_API_BEGIN(c)
  up(c, c->state_d, state, c->nS);
  rk4_device(c, which, c->state_d, t0, t1);
  down(c, state, c->state_d, c->nS);
  sync(c);
  CODY_API_END(c)
}

int cgpu_integrate_euler(cgpu_ctx* c, int which, int imag, cgpu_complex* state, double t0, double t1) {
  CODY_API_BEGIN(c)
  up(c, c->state_d, state, c->nS);
  euler_device(c, which, imag, c->state_d, t0, t1);
  down(c, state, c->state_d, c->nS);
  sync(c);
  CODY_API_END(c)
}

int cgpu_integrate_sil(cgpu_ctx* c, int which, cgpu_complex* state, double t0, double t1, int krylov_dim,
                       double tolerance, int max_restarts, const double* metric, int* warnings) {
  CODY_API_BEGIN(c)
  up(c, c->state_d, state, c->nS);
  const double* m = c->metricOne_d;
  if (metric) {
    if (!c->metricUser_d) c->metricUser_d = dalloc<double>(c->nS);
    CODY_CUDA(cudaMemcpyAsync(c->metricUser_d, metric, sizeof(double) * c->nS, cudaMemcpyHostToDevice, c->stream));
    m = c->metricUser_d;
  }
  int w = sil_device(c, which, c->state_d, t0, t1, krylov_dim, tolerance, max_restarts, m);
  if (warnings) *warnings = w;
  down(c, state, c->state_d, c->nS);
  sync(c);
  CODY_API_END(c)
}

int cgpu_propagate_split2(cgpu_ctx* c, cgpu_complex* state, double t0, double t1, int krylov_dim, double tolerance,
                          int max_restarts, int use_metric) {
  CODY_API_BEGIN(c)
  up(c, c->state_d, state, c->nS);
  if (krylov_dim > 0 && tolerance == 0.0 && max_restarts == 0) {
    // fixed-order SIL: the step has no host-side decisions, replay it as one graph
    propagate_graph(c, &t0, t1 - t0, 1, krylov_dim, use_metric);
  } else {
    split2_device(c, c->state_d, t0, t1, krylov_dim, tolerance, max_restarts, use_metric);
  }
  down(c, state, c->state_d, c->nS);
  sync(c);
  CODY_API_END(c)
}

int cgpu_state_upload(cgpu_ctx* c, const cgpu_complex* state) {
  CODY_API_BEGIN(c)
  up_state(c, 0, c->state_d, state);
  sync(c);
  CODY_API_END(c)
}

int cgpu_state_download(cgpu_ctx* c, cgpu_complex* state) {
  CODY_API_BEGIN(c)
  down_state(c, 0, state, c->state_d);
  sync(c);
  CODY_API_END(c)
}

int cgpu_propagate_resident(cgpu_ctx* c, double t0, double dt, int n_steps, int krylov_dim, int use_metric,
                            int use_graph) {
  CODY_API_BEGIN(c)
  if (!use_graph) {
    double t = t0;
    for (int s = 0; s < n_steps; s++) {
      split2_device(c, c->state_d, t, t + dt, krylov_dim, 0.0, 0, use_metric);
      if (c->absorbEachStep && c->method != CGPU_METHOD_TDCI) launch_absorber_apply(c, c->state_d + c->nC);
      t = t + dt;
    }
    CODY_CUDA(cudaGetLastError());
  } else {
    std::vector<double> t0s(c->nb, t0);
    propagate_graph(c, t0s.data(), dt, n_steps, krylov_dim, use_metric);
  }
  CODY_API_END(c)
}

int cgpu_propagate_resident_timed(cgpu_ctx* c, double t0, double dt, int n_steps, int krylov_dim, int use_metric,
                                  int use_graph, double* elapsed_ms) {
  CODY_API_BEGIN(c)
  cudaEvent_t e0, e1;
  CODY_CUDA(cudaEventCreate(&e0));
  CODY_CUDA(cudaEventCreate(&e1));
  CODY_CUDA(cudaEventRecord(e0, c->stream));
  int rc = cgpu_propagate_resident(c, t0, dt, n_steps, krylov_dim, use_metric, use_graph);
  CODY_CUDA(cudaEventRecord(e1, c->stream));
  CODY_CUDA(cudaEventSynchronize(e1));
  float ms = 0.f;
  CODY_CUDA(cudaEventElapsedTime(&ms, e0, e1));
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (rc != CGPU_OK) return rc;
  if (elapsed_ms) *elapsed_ms = ms;
  CODY_API_END(c)
}

int cgpu_profile_begin(cgpu_ctx* c, int kernel) {
  CODY_API_BEGIN(c)
  c->profTarget = kernel;
  c->profUsed = 0;
  CODY_API_END(c)
}

int cgpu_profile_end(cgpu_ctx* c, long* launches, double* total_ms) {
  CODY_API_BEGIN(c)
  sync(c);
  double tot = 0.0;
  for (size_t i = 0; i + 1 < c->profUsed; i += 2) {
    float ms = 0.f;
    CODY_CUDA(cudaEventElapsedTime(&ms, c->profEvents[i], c->profEvents[i + 1]));
    tot += ms;
  }
  if (launches) *launches = (long)(c->profUsed / 2);
  if (total_ms) *total_ms = tot;
  c->profTarget = 0;
  c->profUsed = 0;
  CODY_API_END(c)
}

int cgpu_energy_resident(cgpu_ctx* c, double time, double* energy) {
  CODY_API_BEGIN(c)
  *energy = energy_device(c, c->state_d, time);
  CODY_API_END(c)
}

int cgpu_tdci_set_orbitals(cgpu_ctx* c, const cgpu_complex* orbs) {
  CODY_API_BEGIN(c)
  if (c->method != CGPU_METHOD_TDCI) throw std::string("tdci_set_orbitals: not a TDCI context");
  size_t n = (size_t)c->nG * c->nOS;
  up(c, c->tdciOrbs_d, orbs, n);
  launch_onebody(c, c->orbTmp_d, c->tdciOrbs_d, 0.0, zmk(1.0, 0.0), 0);
  launch_fill_h1_from(c, c->tdciOrbs_d, c->orbTmp_d, c->h1_d);
  launch_fill_h2(c, c->tdciOrbs_d);
  launch_fold_h1(c);
  launch_fold_h2(c);
  sync(c);
  CODY_API_END(c)
}

int cgpu_observables(cgpu_ctx* c, double time, double* out) {
  CODY_API_BEGIN(c)
  if (!out) throw std::string("observables: null output");
  std::vector<double> t(c->nb, time);
  observables(c, t.data(), out);
  CODY_API_END(c)
}

// Imaginary-time relaxation (T_He1d_04_ImagTimePropagationMctdhx.f90:82-99 with
// M_Utils_Actions.f90:66-78): n_inner Euler steps on the imaginary-time
// derivative, each followed by Coeffs_Normalize and Orbs_Orthonormalize (MGS
// twice), then GetEnergy; stop when |dE| <= conv_thresh or after max_outer rounds.
int cgpu_relax(cgpu_ctx* c, cgpu_complex* state, double dt, int n_inner, double conv_thresh, int max_outer,
               double* energy, int* n_outer) {
  CODY_API_BEGIN(c)
  if (c->nb != 1) throw std::string("relax: a single system (use the context of one trajectory)");
  if (c->method == CGPU_METHOD_TDCI) throw std::string("relax: MCTDHX contexts only");
  if (!state || n_inner <= 0) throw std::string("relax: bad argument");
  const SysHost& s = c->sys[0];
  up_state(c, 0, c->state_d, state);
  z_t* orbs = c->state_d + c->nC;
  double eNew = 0.0, eOld = 0.0, conv = 1.0, time = 0.0;
  int outer = 0;
  while (std::fabs(conv) > conv_thresh && outer < max_outer) {
    outer++;
    batch_zero(c, c->scal_d, sizeof(int));
    for (int k = 0; k < n_inner; k++) {
      euler_device(c, CGPU_TD_FULL, 1, c->state_d, time, time + dt);
      time = time + dt;
      launch_normalize_coeffs(c, c->state_d);
      if (c->restricted) launch_orthonormalize(c, orbs, 0, c->nOS, 0);
      else
        for (int b = 0; b < c->nBt; b++) launch_orthonormalize(c, orbs, s.orbStart[b], s.nOrbs[b], 0);
    }
    int status = 0;
    CODY_CUDA(cudaMemcpyAsync(&status, c->scal_d, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    eOld = eNew;
    eNew = energy_device(c, c->state_d, time);
    if (status) throw std::string("relax: Orthonormalize met a vector with non-positive norm");
    conv = eNew - eOld;
  }
  down_state(c, 0, state, c->state_d);
  sync(c);
  if (energy) *energy = eNew;
  if (n_outer) *n_outer = outer;
  CODY_API_END(c)
}

// Restart files in the reference's raw format (src/Utils/M_Utils_DataStorage.f90:20-106:
// unformatted stream of the complex(R64) array): coeffs.in (S_Coeffs.f90:167-175),
// orbBB_II.in per stored orbital (S_Orbs.f90:251-276; restricted runs store
// body type 1 only) and, when asked, rdm2BtXX_YY.in body-type blocks of rho2
// (S_Coeffs.f90:177-214).  `dir` is a directory prefix ("" = current).
int cgpu_save_restart(cgpu_ctx* c, const char* dir, int with_rdm2) {
  CODY_API_BEGIN(c)
  if (c->nb != 1) throw std::string("save_restart: a single system");
  if (with_rdm2) launch_ci_rdm(c, c->state_d, 0, 1);
  save_traj(c, 0, dir_prefix(dir), with_rdm2 != 0);
  CODY_API_END(c)
}

// Loads coeffs.in and the orbital files written by cgpu_save_restart (or by the
// reference) into the resident state (CoeffsInit / OrbsInit with "load").
int cgpu_load_restart(cgpu_ctx* c, const char* dir) {
  CODY_API_BEGIN(c)
  if (c->nb != 1) throw std::string("load_restart: a single system");
  load_traj(c, 0, dir_prefix(dir));
  sync(c);
  CODY_API_END(c)
}

int cgpu_absorber_setup(cgpu_ctx* c, double onset, double order, int apply_each_step) {
  CODY_API_BEGIN(c)
  if (!(order > 0.0)) throw std::string("absorber: order must be positive");
  launch_absorber_setup(c, onset, order);
  c->absorbEachStep = apply_each_step ? 1 : 0;
  sync(c);
  CODY_API_END(c)
}

int cgpu_absorber_apply(cgpu_ctx* c) {
  CODY_API_BEGIN(c)
  if (c->method == CGPU_METHOD_TDCI) throw std::string("absorber: no orbitals in a TDCI state");
  launch_absorber_apply(c, c->state_d + c->nC);
  sync(c);
  CODY_API_END(c)
}

int cgpu_tdci_adjoint(cgpu_ctx* c, const cgpu_complex* c0, const double* field, int n_steps, double dt,
                      int checkpoint, double* objective, double* overlap, cgpu_complex* c_final, double* d_objective) {
  CODY_API_BEGIN(c)
  if (!c0 || !field || !objective) throw std::string("tdci_adjoint: null argument");
  adjoint_tdci(c, (const z_t*)c0, field, n_steps, dt, checkpoint > 0 ? checkpoint : 64, objective, overlap,
               (z_t*)c_final, d_objective);
  CODY_API_END(c)
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Batched trajectories: one context with nb systems; every launch of the step
// covers all of them, and the step is replayed as one CUDA graph.
// ---------------------------------------------------------------------------
struct cgpu_batch {
  cgpu_ctx* c = nullptr;
};

namespace {
cgpu_ctx* bctx(const cgpu_batch* b) {
  if (!b || !b->c) throw std::string("null batch");
  return b->c;
}

// device staging area for packed host states (all trajectories, nS_b each)
void ensure_stage(cgpu_ctx* c) {
  size_t need = (size_t)c->stageOff.back();
  if (c->stage_d && c->stageCap >= need) return;
  if (c->stage_d) cudaFree(c->stage_d);
  c->stage_d = nullptr;
  CODY_CUDA(cudaMalloc(&c->stage_d, sizeof(z_t) * std::max<size_t>(need, 1)));
  c->stageCap = need;
}
}  // namespace

#define CODY_BATCH_BEGIN(b) \
  cgpu_ctx* c_ = nullptr;   \
  try {                     \
    c_ = bctx(b);
#define CODY_BATCH_END CODY_API_END(c_)

extern "C" {

int cgpu_batch_create(const cgpu_desc* descs, int n, cgpu_batch** out) {
  if (!descs || !out || n <= 0) return fail(nullptr, "cgpu_batch_create: bad argument", CGPU_ERR_ARG);
  if (n > 65535) return fail(nullptr, "cgpu_batch_create: at most 65535 systems", CGPU_ERR_ARG);
  *out = nullptr;
  int rc = CGPU_OK;
  cgpu_ctx* c = create_ctx(descs, n, &rc);
  if (!c) return rc;
  cgpu_batch* b = new cgpu_batch();
  b->c = c;
  *out = b;
  return CGPU_OK;
}

int cgpu_batch_destroy(cgpu_batch* b) {
  if (!b) return CGPU_OK;
  if (b->c) cgpu_ctx_destroy(b->c);
  delete b;
  return CGPU_OK;
}

int cgpu_batch_size(const cgpu_batch* b) { return (b && b->c) ? b->c->nb : 0; }

int cgpu_batch_sizes(const cgpu_batch* b, int i, int* out) {
  if (!b || !b->c || !out || i < 0 || i >= b->c->nb) return CGPU_ERR_ARG;
  const SysHost& s = b->c->sys[i];
  out[0] = s.nG; out[1] = s.nO; out[2] = s.nOS; out[3] = s.nC; out[4] = b->c->nBt; out[5] = s.nS;
  return CGPU_OK;
}

int cgpu_batch_grid(const cgpu_batch* b, int i, double* x, double* w) {
  if (!b || !b->c || i < 0 || i >= b->c->nb) return CGPU_ERR_ARG;
  const SysHost& s = b->c->sys[i];
  if (x) std::memcpy(x, s.x.data(), sizeof(double) * s.nG);
  if (w) std::memcpy(w, s.w.data(), sizeof(double) * s.nG);
  return CGPU_OK;
}

int cgpu_batch_upload(cgpu_batch* b, const cgpu_complex* states) {
  CODY_BATCH_BEGIN(b)
  cgpu_ctx* c = c_;
  ensure_stage(c);
  CODY_CUDA(cudaMemcpyAsync(c->stage_d, states, sizeof(z_t) * c->stageOff.back(), cudaMemcpyHostToDevice, c->stream));
  k_scatter_states<<<bgrid(c, 64), 256, 0, c->stream>>>(c->state_d, c->stage_d, c->stageOff_d, TRAJ_PASS(c));
  CODY_LAUNCHED(c);
  sync(c);
  CODY_BATCH_END
}

int cgpu_batch_download(cgpu_batch* b, cgpu_complex* states) {
  CODY_BATCH_BEGIN(b)
  cgpu_ctx* c = c_;
  ensure_stage(c);
  k_gather_states<<<bgrid(c, 64), 256, 0, c->stream>>>(c->stage_d, c->state_d, c->stageOff_d, TRAJ_PASS(c));
  CODY_LAUNCHED(c);
  CODY_CUDA(cudaMemcpyAsync(states, c->stage_d, sizeof(z_t) * c->stageOff.back(), cudaMemcpyDeviceToHost, c->stream));
  sync(c);
  CODY_BATCH_END
}

int cgpu_batch_save_restart(cgpu_batch* b, const char* dir, int with_rdm2) {
  CODY_BATCH_BEGIN(b)
  cgpu_ctx* c = c_;
  if (!dir) throw std::string("batch_save_restart: null directory");
  if (with_rdm2) launch_ci_rdm(c, c->state_d, 0, 1);
  for (int i = 0; i < c->nb; i++) save_traj(c, i, traj_prefix(dir, i, true), with_rdm2 != 0);
  CODY_BATCH_END
}

int cgpu_batch_load_restart(cgpu_batch* b, const char* dir) {
  CODY_BATCH_BEGIN(b)
  cgpu_ctx* c = c_;
  if (!dir) throw std::string("batch_load_restart: null directory");
  for (int i = 0; i < c->nb; i++) load_traj(c, i, traj_prefix(dir, i, false));
  CODY_BATCH_END
}

int cgpu_batch_propagate(cgpu_batch* b, const double* t0, double dt, int n_steps, int krylov_dim, int use_metric,
                         double* elapsed_ms) {
  CODY_BATCH_BEGIN(b)
  cgpu_ctx* c = c_;
  if (!t0 || n_steps < 0 || krylov_dim <= 0) throw std::string("batch_propagate: bad argument");
  if (!c->stepGraph || c->graphDt != dt || c->graphKrylov != krylov_dim || c->graphMetric != use_metric ||
      c->graphProf != c->profTarget || c->graphAbsorb != c->absorbEachStep) {
    set_step_times(c, t0);
    capture_step_graph(c, t0[0], dt, krylov_dim, use_metric);
  }
  if (c->profTarget) c->profUsed = c->graphProfUsed;
  cudaEvent_t e0, e1;
  CODY_CUDA(cudaEventCreate(&e0));
  CODY_CUDA(cudaEventCreate(&e1));
  set_step_times(c, t0);
  CODY_CUDA(cudaEventRecord(e0, c->stream));
  for (int s = 0; s < n_steps; s++) CODY_CUDA(cudaGraphLaunch(c->stepGraph, c->stream));
  c->launches += (long)n_steps * c->graphKernels;
  CODY_CUDA(cudaEventRecord(e1, c->stream));
  CODY_CUDA(cudaEventSynchronize(e1));
  float ms = 0.f;
  CODY_CUDA(cudaEventElapsedTime(&ms, e0, e1));
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (elapsed_ms) *elapsed_ms = ms;
  sync(c);
  CODY_BATCH_END
}

int cgpu_batch_energies(cgpu_batch* b, const double* t, double* energies) {
  CODY_BATCH_BEGIN(b)
  cgpu_ctx* c = c_;
  if (!t || !energies) throw std::string("batch_energies: null array");
  // E(t_b) per trajectory: the field reads the per-trajectory time slots
  set_step_times(c, t);
  c->useStepTime = 1;
  try {
    energy_launch(c, c->state_d, 0.0);
  } catch (...) {
    c->useStepTime = 0;
    throw;
  }
  c->useStepTime = 0;
  CODY_CUDA(cudaMemcpy2DAsync(energies, sizeof(double), c->scal_d + CODY_SCAL_ENERGY, c->bs, sizeof(double), c->nb,
                              cudaMemcpyDeviceToHost, c->stream));
  sync(c);
  CODY_BATCH_END
}

int cgpu_batch_absorber_setup(cgpu_batch* b, double onset, double order, int apply_each_step) {
  if (!b || !b->c) return fail(nullptr, "null batch", CGPU_ERR_ARG);
  return cgpu_absorber_setup(b->c, onset, order, apply_each_step);
}

int cgpu_batch_observables(cgpu_batch* b, const double* t, double* out) {
  CODY_BATCH_BEGIN(b)
  if (!t || !out) throw std::string("batch_observables: null array");
  observables(c_, t, out);
  CODY_BATCH_END
}

long cgpu_batch_kernels_per_step(const cgpu_batch* b) { return (b && b->c) ? b->c->graphKernels : 0; }

long cgpu_batch_launch_count(cgpu_batch* b, int reset) { return (b && b->c) ? cgpu_launch_count(b->c, reset) : -1; }

int cgpu_batch_shared_interactions(const cgpu_batch* b) {
  return (b && b->c && b->c->fxShared) ? (int)b->c->fxRoots.size() : 0;
}

int cgpu_batch_profile_begin(cgpu_batch* b, int kernel) {
  if (!b || !b->c) return fail(nullptr, "null batch", CGPU_ERR_ARG);
  return cgpu_profile_begin(b->c, kernel);
}

int cgpu_batch_profile_end(cgpu_batch* b, long* launches, double* total_ms) {
  if (!b || !b->c) return fail(nullptr, "null batch", CGPU_ERR_ARG);
  return cgpu_profile_end(b->c, launches, total_ms);
}

// ---- Sys* operators on one orbital ------------------------------------------
}  // extern "C"

namespace {
// Three nG-point device vectors for the Sys* entry points (allocated on first use).
z_t* sys_scratch(cgpu_ctx* c) {
  if (c->nb != 1) throw std::string("Sys* operators: a single-system context");
  if (!c->sysTmp_d) CODY_CUDA(cudaMalloc(&c->sysTmp_d, sizeof(z_t) * 3 * (size_t)c->nG));
  return c->sysTmp_d;
}
}  // namespace

extern "C" {

int cgpu_sys_kinetic_multiply(cgpu_ctx* c, cgpu_complex* d_orb, const cgpu_complex* orb, double time, int bt) {
  CODY_API_BEGIN(c)
  (void)time;  // the kinetic operators are time independent (src/SysKinetic/M_SysKinetic.f90:139)
  if (!d_orb || !orb) throw std::string("sys_kinetic_multiply: null array");
  const int b = bt <= 0 ? 0 : bt - 1;
  if (b >= c->nBt) throw std::string("sys_kinetic_multiply: body type out of range");
  z_t* v = sys_scratch(c);
  up(c, v, orb, c->nG);
  sys_kinetic(c, v + c->nG, v, c->restricted ? 0 : b);
  down(c, d_orb, v + c->nG, c->nG);
  sync(c);
  CODY_API_END(c)
}

int cgpu_sys_potential_fill(cgpu_ctx* c, cgpu_complex* potential, double time, int bt) {
  CODY_API_BEGIN(c)
  if (!potential) throw std::string("sys_potential_fill: null array");
  if (bt > c->nBt) throw std::string("sys_potential_fill: body type out of range");
  z_t* v = sys_scratch(c);
  sys_potential(c, v, time);
  down(c, potential, v, c->nG);
  sync(c);
  CODY_API_END(c)
}

int cgpu_sys_potential_multiply(cgpu_ctx* c, cgpu_complex* d_orb, const cgpu_complex* potential,
                                const cgpu_complex* orb) {
  CODY_API_BEGIN(c)
  if (!d_orb || !potential || !orb) throw std::string("sys_potential_multiply: null array");
  z_t* v = sys_scratch(c);
  up(c, v, potential, c->nG);
  up(c, v + c->nG, orb, c->nG);
  sys_multiply(c, v + 2 * c->nG, v, v + c->nG);
  down(c, d_orb, v + 2 * c->nG, c->nG);
  sync(c);
  CODY_API_END(c)
}

int cgpu_sys_interaction_src(cgpu_ctx* c, cgpu_complex* src, const cgpu_complex* orb_conjg, const cgpu_complex* orb) {
  CODY_API_BEGIN(c)
  if (!src || !orb_conjg || !orb) throw std::string("sys_interaction_src: null array");
  z_t* v = sys_scratch(c);
  up(c, v, orb_conjg, c->nG);
  up(c, v + c->nG, orb, c->nG);
  sys_interaction_src(c, v + 2 * c->nG, v, v + c->nG);
  down(c, src, v + 2 * c->nG, c->nG);
  sync(c);
  CODY_API_END(c)
}

int cgpu_sys_interaction_potential(cgpu_ctx* c, cgpu_complex* potential, const cgpu_complex* src, double time,
                                   int bt1, int bt2) {
  CODY_API_BEGIN(c)
  (void)time;  // the soft-Yukawa interaction is time independent
  if (!potential || !src) throw std::string("sys_interaction_potential: null array");
  if (!c->hasInteraction) throw std::string("sys_interaction_potential: the context has no interaction");
  if (bt1 > c->nBt || bt2 > c->nBt) throw std::string("sys_interaction_potential: body type out of range");
  z_t* v = sys_scratch(c);
  up(c, v, src, c->nG);
  sys_interaction_potential(c, v + c->nG, v);
  down(c, potential, v + c->nG, c->nG);
  sync(c);
  CODY_API_END(c)
}

int cgpu_sys_interaction_multiply(cgpu_ctx* c, cgpu_complex* res, const cgpu_complex* potential,
                                  const cgpu_complex* orb) {
  return cgpu_sys_potential_multiply(c, res, potential, orb);
}

// ---- MCTDHF pulse gradient -------------------------------------------------
int cgpu_mc_adjoint_forward(cgpu_ctx* c, const cgpu_complex* state0, const cgpu_complex* ref_state,
                            const double* field, int n_steps, double dt, int krylov_dim, int checkpoint,
                            double* objective, double* overlap, cgpu_complex* state_final) {
  CODY_API_BEGIN(c)
  if (!state0 || !field) throw std::string("mc_adjoint_forward: null array");
  mc_adjoint_forward(c, (const z_t*)state0, (const z_t*)ref_state, field, n_steps, dt, krylov_dim, checkpoint,
                     objective, overlap, (z_t*)state_final);
  CODY_API_END(c)
}

int cgpu_mc_adjoint_backward(cgpu_ctx* c, double* d_objective) {
  CODY_API_BEGIN(c)
  if (!d_objective) throw std::string("mc_adjoint_backward: null array");
  mc_adjoint_backward(c, d_objective);
  CODY_API_END(c)
}

// ---- tile autotuner -------------------------------------------------------
int cgpu_autotune(cgpu_ctx* c, const char* cache_path, int mode, char* report, int report_len) {
  CODY_API_BEGIN(c)
  if (mode != CGPU_TUNE_CACHED && mode != CGPU_TUNE_FORCE) throw std::string("autotune: unknown mode");
  std::string rep;
  autotune_run(c, cache_path, mode == CGPU_TUNE_FORCE, rep);
  sync(c);
  if (report && report_len > 0) {
    std::strncpy(report, rep.c_str(), (size_t)report_len - 1);
    report[report_len - 1] = '\0';
  }
  CODY_API_END(c)
}

int cgpu_get_tiles(const cgpu_ctx* c, int* tiles) {
  if (!c || !tiles) return fail(nullptr, "get_tiles: null argument", CGPU_ERR_ARG);
  tiles_get(c, tiles);
  return CGPU_OK;
}

int cgpu_set_tiles(cgpu_ctx* c, const int* tiles) {
  CODY_API_BEGIN(c)
  if (!tiles) throw std::string("set_tiles: null table");
  tiles_set(c, tiles);
  sync(c);
  CODY_API_END(c)
}

int cgpu_batch_autotune(cgpu_batch* b, const char* cache_path, int mode, char* report, int report_len) {
  if (!b || !b->c) return fail(nullptr, "null batch", CGPU_ERR_ARG);
  return cgpu_autotune(b->c, cache_path, mode, report, report_len);
}

int cgpu_batch_get_tiles(const cgpu_batch* b, int* tiles) {
  if (!b || !b->c) return fail(nullptr, "null batch", CGPU_ERR_ARG);
  return cgpu_get_tiles(b->c, tiles);
}

int cgpu_batch_set_tiles(cgpu_batch* b, const int* tiles) {
  if (!b || !b->c) return fail(nullptr, "null batch", CGPU_ERR_ARG);
  return cgpu_set_tiles(b->c, tiles);
}

}  // extern "C"
