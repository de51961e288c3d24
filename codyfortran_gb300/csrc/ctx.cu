// ctx.cu -- context set-up (the hot path's Fabricate/Setup chain), the
// equation-of-motion orchestration, the integrators and the C ABI.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>

#include "common.cuh"

namespace {

std::string g_lastGlobalError;
std::mutex g_errMutex;

constexpr double PI = 3.14159265358979323846264338327950288;

// ---------------------------------------------------------------------------
// Host-side set-up
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

// Grid + banded kinetic operator.  T[(bt*(2b+1) + d+b)*nG + g] multiplies
// orbs[g+d] in (T orbs)[g] = -1/(2 m_bt) (d^2/dx^2 orbs)[g].
void setup_grid_and_kinetic(cgpu_ctx* c, const cgpu_desc* d) {
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
  c->nBtK = c->restricted ? 1 : c->nBt;
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

void build_ctx(cgpu_ctx* c, const cgpu_desc* d) {
  if (d->n_body_types < 1 || d->n_body_types > CODY_MAX_BT) throw std::string("method.mb.nBodyTypes out of range");
  c->nBt = d->n_body_types;
  c->restricted = d->restricted ? 1 : 0;
  c->method = d->method;
  c->precision = d->precision;
  c->regEps = d->regularization > 0 ? d->regularization : 1e-10;
  c->nO = 0;
  for (int b = 0; b < c->nBt; b++) {
    c->nBodies[b] = d->n_bodies[b];
    c->nOrbs[b] = d->n_orbs[b];
    c->mass[b] = d->body_mass[b];
    c->orbStart[b] = c->nO;
    if (c->nOrbs[b] < 1 || c->nBodies[b] < 0 || c->nBodies[b] > c->nOrbs[b])
      throw std::string("method.mb: invalid nOrbs / nBodies");
    for (int i = 0; i < c->nOrbs[b]; i++) c->btOfOrb.push_back(b);
    c->nO += c->nOrbs[b];
  }
  if (c->restricted) {
    for (int b = 1; b < c->nBt; b++)
      if (c->nOrbs[b] != c->nOrbs[0]) throw std::string("orbs.restrictedQ needs equal nOrbs per body type");
    if (c->nBt != 2) throw std::string("orbs.restrictedQ needs two body types (spins)");
  }
  c->nOS = c->restricted ? c->nOrbs[0] : c->nO;
  if (c->nOS > 64) throw std::string("more than 64 stored orbitals is not supported");
  if (c->method != CGPU_METHOD_TDCI && c->nOS > 32)
    throw std::string("MCTDHX: more than 32 stored orbitals is not supported");
  if (d->precision != CGPU_PREC_FP64 && d->precision != CGPU_PREC_MIXED && d->precision != CGPU_PREC_MIXED_X6)
    throw std::string("unknown precision");
  setup_grid_and_kinetic(c, d);
  int nG = c->nG;
  // potential (src/SysPotential/Linear/SoftYukawa/StdImpl/*.f90:82-113)
  c->V0.assign(nG, 0.0);
  c->hasPotential = d->n_nuclei > 0;
  if (d->n_nuclei < 0 || d->n_nuclei > 8) throw std::string("sysPotential: 0..8 nuclei supported");
  for (int k = 0; k < d->n_nuclei; k++)
    for (int g = 0; g < nG; g++)
      c->V0[g] -= soft_kernel(d->nuc_charge[k], d->nuc_softening1[k], d->nuc_softening2[k], d->nuc_dampening[k],
                              std::fabs(c->x[g] - d->nuc_position[k]));
  // laser
  c->laserKind = d->laser_kind;
  c->E0 = d->laser_E0;
  c->omega = d->laser_omega;
  c->nCycles = d->laser_n_cycles;
  c->cep = d->laser_cep;
  c->tStart = d->laser_t_start;
  if (d->laser_kind == CGPU_LASER_SAMPLED) {
    if (!d->field_samples || d->n_field_samples <= 0) throw std::string("sampled field needs samples");
    c->samples.assign(d->field_samples, d->field_samples + d->n_field_samples);
    c->sampleDt = d->field_dt;
    c->sampleT0 = d->field_t0;
  }
  // device operators
  CODY_CUDA(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
  c->zero_d = dalloc<double>(1);
  c->stepT_d = dalloc<double>(1);
  CODY_CUDA(cudaMemset(c->zero_d, 0, sizeof(double)));
  CODY_CUDA(cudaMemset(c->stepT_d, 0, sizeof(double)));
  if (!c->samples.empty()) c->samples_d = dupload(c->samples);
  c->laserDev = LaserDev{c->laserKind, c->E0, c->omega, c->nCycles, c->cep, c->tStart, c->sampleDt, c->sampleT0,
                         (int)c->samples.size(), c->samples_d};
  c->x_d = dupload(c->x);
  c->w_d = dupload(c->w);
  c->V0_d = dupload(c->V0);
  c->T_d = dupload(c->band_h);
  c->btOfOrb_d = dupload(c->btOfOrb);
  c->hasInteraction = d->has_interaction ? 1 : 0;
  if (c->hasInteraction) {
    // interaction matrix V(x_i, x_j) (S_SysInteraction_Linear_SoftYukawa.f90:67-73), built on the device
    double dx = nG > 1 ? c->x[1] - c->x[0] : 0.0;
    c->Vint_d = dalloc<double>((size_t)nG * nG);
    size_t tot = (size_t)nG * nG;
    k_build_vint<<<(int)((tot + 255) / 256), 256, 0, c->stream>>>(
        c->Vint_d, c->x_d, nG, d->int_kind == CGPU_INT_TOEPLITZ, dx, d->int_strength, d->int_softening1,
        d->int_softening2, d->int_dampening);
    CODY_LAUNCHED(c);
  }
  // pairs (l <= k, same body type) in the order of the reference's loops
  int n = c->nOS;
  std::vector<int> pl, pk, pidx((size_t)n * n, -1);
  for (int l = 0; l < n; l++)
    for (int k = l; k < n; k++) {
      if (!c->restricted && c->btOfOrb[l] != c->btOfOrb[k]) continue;
      pidx[(size_t)l * n + k] = (int)pl.size();
      pl.push_back(l);
      pk.push_back(k);
    }
  c->nPairs = (int)pl.size();
  c->pairL_d = dupload(pl);
  c->pairK_d = dupload(pk);
  c->pidx_d = dupload(pidx);
  // CI tables
  ci_build_tables(c);
  c->nC = c->view.nC;
  c->nS = (c->method == CGPU_METHOD_TDCI) ? c->nC : c->nC + nG * n;
  size_t nS = c->nS;
  std::vector<double> mw(nS, 1.0), m1(nS, 1.0);
  if (c->method != CGPU_METHOD_TDCI)
    for (int o = 0; o < n; o++)
      for (int g = 0; g < nG; g++) mw[(size_t)c->nC + (size_t)o * nG + g] = c->w[g];
  c->metricW_d = dupload(mw);
  c->metricOne_d = dupload(m1);
  c->metric_d = c->metricOne_d;
  // work buffers
  size_t nO2 = (size_t)c->nO * c->nO, nO4 = nO2 * nO2, Q = (size_t)n * n;
  c->h1Lin_d = dalloc<z_t>(nO2 + 1);
  c->rdm1Lin_d = dalloc<z_t>(nO2 + 1);
  c->h2Lin_d = dalloc<z_t>(nO4 + 1);
  c->rdm2Lin_d = dalloc<z_t>(nO4 + 1);
  CODY_CUDA(cudaMemset(c->h1Lin_d, 0, sizeof(z_t) * (nO2 + 1)));
  CODY_CUDA(cudaMemset(c->h2Lin_d, 0, sizeof(z_t) * (nO4 + 1)));
  c->rdm1_d = dalloc<z_t>(nO2);
  c->h1_d = dalloc<z_t>(nO2);
  c->rdm2_d = dalloc<z_t>(nO4);
  c->h2_d = dalloc<z_t>(nO4);
  CODY_CUDA(cudaMemset(c->h1_d, 0, sizeof(z_t) * nO2));
  CODY_CUDA(cudaMemset(c->h2_d, 0, sizeof(z_t) * nO4));
  c->S_d = dalloc<z_t>((size_t)nG * std::max(c->nPairs, 1));
  c->W_d = dalloc<z_t>((size_t)nG * std::max(c->nPairs, 1));
  c->Sfull_d = dalloc<z_t>((size_t)nG * Q);
  c->Wfull_d = dalloc<z_t>(2 * (size_t)nG * Q);
  c->Rp_d = dalloc<z_t>(Q * Q);
  c->h2s_d = dalloc<z_t>(Q * Q);
  c->Mreg_d = dalloc<z_t>(Q);
  {
    std::vector<z_t> eye(Q, zmk(0.0, 0.0));
    for (int i = 0; i < n; i++) eye[(size_t)i * n + i] = zmk(1.0, 0.0);
    c->Uprev_d = dupload(eye);
  }
  c->r1s_d = dalloc<z_t>(Q);
  c->gram_d = dalloc<z_t>(Q);
  c->orbTmp_d = dalloc<z_t>((size_t)nG * n);
  c->scal_d = dalloc<double>(64);
  c->state_d = dalloc<z_t>(nS);
  c->dstate_d = dalloc<z_t>(nS);
  c->rkInc_d = dalloc<z_t>(nS);
  c->rkTmp_d = dalloc<z_t>(nS);
  c->rkStage_d = dalloc<z_t>(nS);
  c->trial_d = dalloc<z_t>(nS);
  c->work_d = dalloc<z_t>(nS);
  c->lw_d = dalloc<z_t>(nS);
  c->maxKrylov = std::max(1, std::min(d->max_krylov > 0 ? d->max_krylov : 32, 32));
  c->basis_d = dalloc<z_t>(nS * (size_t)c->maxKrylov);
  c->lz_d = dalloc<double>(512);
  CODY_CUDA(cudaMemset(c->lz_d, 0, sizeof(double) * 512));
  CODY_CUDA(cudaMallocHost(&c->lz_h, sizeof(double) * 512));
  if (c->method == CGPU_METHOD_TDCI) c->tdciOrbs_d = dalloc<z_t>((size_t)nG * n);
  CODY_CUDA(cudaDeviceSynchronize());
}

void free_ctx(cgpu_ctx* c) {
  mixed_free(c);
  if (c->stepGraph) cudaGraphExecDestroy(c->stepGraph);
  if (c->stepGraphRaw) cudaGraphDestroy(c->stepGraphRaw);
  for (cudaEvent_t e : c->profEvents) cudaEventDestroy(e);
  void* ptrs[] = {c->x_d, c->w_d, c->V0_d, c->T_d, c->Vint_d, c->metricW_d, c->metricOne_d, c->metricUser_d, c->Vint_f,
                  c->btOfOrb_d, c->h1Lin_d, c->h2Lin_d, c->rdm1Lin_d, c->rdm2Lin_d, c->rdm1_d, c->rdm2_d, c->h1_d,
                  c->h2_d, c->pairL_d, c->pairK_d, c->pidx_d, c->S_d, c->W_d, c->Sfull_d, c->Wfull_d, c->Rp_d,
                  c->h2s_d, c->Mreg_d, c->r1s_d, c->r2s_d, c->partial_d, c->gram_d, c->orbTmp_d, c->scal_d,
                  c->state_d, c->dstate_d, c->rkInc_d, c->rkTmp_d, c->rkStage_d, c->basis_d, c->lw_d, c->trial_d,
                  c->work_d, c->lz_d, c->tdciOrbs_d, c->zero_d, c->stepT_d, c->samples_d, c->warm_d,
                  c->Uprev_d};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  for (int b = 0; b < CODY_MAX_BT; b++) {
    CiTables& t = c->tab[b];
    void* tp[] = {t.codes, t.sN, t.sExc, t.sCode, t.sFac, t.dN, t.dExc, t.dCode, t.dFac, t.rankTab};
    for (void* p : tp)
      if (p) cudaFree(p);
  }
  if (c->lz_h) cudaFreeHost(c->lz_h);
  if (c->stream) cudaStreamDestroy(c->stream);
}

// ---------------------------------------------------------------------------
// Equation of motion on device buffers.  out = post * dState, where dState is
// the reference's time derivative (carrying its -i).
// ---------------------------------------------------------------------------
void td_device(cgpu_ctx* c, int which, z_t* out, const z_t* in, double t, z_t post) {
  z_t f = zmul(post, zmk(0.0, -1.0));
  bool unit = (f.x == 1.0 && f.y == 0.0);
  if (which == CGPU_TD_TDCI || c->method == CGPU_METHOD_TDCI) {
    if (c->method != CGPU_METHOD_TDCI) throw std::string("TDCI derivative needs a TDCI context");
    if (c->laserKind != CGPU_LASER_NONE) {  // time-dependent one-body part (Tdci :90-92)
      launch_onebody(c, c->orbTmp_d, c->tdciOrbs_d, t, zmk(1.0, 0.0), 0);
      launch_fill_h1_from(c, c->tdciOrbs_d, c->orbTmp_d, c->h1_d);
      launch_fold_h1(c);
    }
    CODY_CUDA(cudaMemsetAsync(out, 0, sizeof(z_t) * c->nC, c->stream));
    launch_ci_apply(c, in, out, 1, 1);
    if (!unit) launch_scale(c, out, f, c->nC);
    return;
  }
  const z_t* C = in;
  const z_t* orbs = in + c->nC;
  z_t* dC = out;
  z_t* dOrbs = out + c->nC;
  size_t nGO = (size_t)c->nG * c->nOS;
  if (which == CGPU_TD_ORBS_LIN) {
    CODY_CUDA(cudaMemsetAsync(dC, 0, sizeof(z_t) * c->nC, c->stream));
    launch_onebody(c, dOrbs, orbs, t, f, 0);
    return;
  }
  if (which != CGPU_TD_FULL && which != CGPU_TD_NONLIN) throw std::string("unknown time-derivative selector");
  launch_ci_rdm(c, C, 1, 1);
  if (which == CGPU_TD_FULL) {
    launch_onebody(c, dOrbs, orbs, t, zmk(1.0, 0.0), 0);
    launch_fill_h1_from(c, orbs, dOrbs, c->h1_d);
  } else {
    launch_onebody(c, c->orbTmp_d, orbs, t, zmk(1.0, 0.0), 0);
    launch_fill_h1_from(c, orbs, c->orbTmp_d, c->h1_d);
    CODY_CUDA(cudaMemsetAsync(dOrbs, 0, sizeof(z_t) * nGO, c->stream));
  }
  if (c->precision == CGPU_PREC_FP64) launch_correlation(c, dOrbs, orbs, 1);
  else launch_correlation_mixed(c, dOrbs, orbs, 1);
  launch_fold_h1(c);
  launch_fold_h2(c);
  CODY_CUDA(cudaMemsetAsync(dC, 0, sizeof(z_t) * c->nC, c->stream));
  launch_ci_apply(c, C, dC, 1, 1);
  launch_project_coeffs(c, dC, C);
  launch_project_orbs(c, dOrbs, orbs);
  if (!unit) launch_scale(c, out, f, c->nS);
}

// RK4 (src/IntegratorList/Rk/O4Expl/S_IntegratorList_Rk_O4Expl.f90:90-141) on state_d-like buffers.
void rk4_device(cgpu_ctx* c, int which, z_t* state, double t0, double t1) {
  double dt = t1 - t0, dt2 = dt / 2.0, dt3 = dt / 3.0, dt6 = dt / 6.0;
  size_t n = c->nS;
  z_t one = zmk(1.0, 0.0);
  td_device(c, which, c->dstate_d, state, t0, one);
  launch_rk_stage(c, c->rkInc_d, c->rkTmp_d, state, c->dstate_d, dt6, dt2, 1, n);
  double tp = t0 + dt2;
  td_device(c, which, c->dstate_d, c->rkTmp_d, tp, one);
  launch_rk_stage(c, c->rkInc_d, c->rkTmp_d, state, c->dstate_d, dt3, dt2, 0, n);
  td_device(c, which, c->dstate_d, c->rkTmp_d, tp, one);
  launch_rk_stage(c, c->rkInc_d, c->rkTmp_d, state, c->dstate_d, dt3, dt, 0, n);
  tp = t0 + dt;
  td_device(c, which, c->dstate_d, c->rkTmp_d, tp, one);
  launch_rk_stage(c, c->rkInc_d, nullptr, state, c->dstate_d, dt6, 0.0, 0, n);
  launch_axpby(c, state, c->rkInc_d, one, one, n);
}

void euler_device(cgpu_ctx* c, int which, int imag, z_t* state, double t0, double t1) {
  z_t post = imag ? zmk(0.0, -1.0) : zmk(1.0, 0.0);
  td_device(c, which, c->dstate_d, state, t0, post);
  launch_axpby(c, state, c->dstate_d, zmk(t1 - t0, 0.0), zmk(1.0, 0.0), c->nS);
}

// One PerformLanczosStep on work_d -> trial_d.  Returns converged (adaptive) or -1 (not checked).
int lanczos_pass(cgpu_ctx* c, int which, double tBase, double dt, int maxDim, double tol, double* errOut) {
  launch_lanczos_start(c, c->work_d);
  double tEval = tBase + 0.5 * dt;
  int adaptive = tol > 0.0;
  int converged = -1;
  int mUsed = maxDim;
  for (int j = 1; j <= maxDim; j++) {
    z_t* v = c->basis_d + (size_t)c->nS * (j - 1);
    // w = i * TimeDerivative(v)
    td_device(c, which, c->lw_d, v, tEval, zmk(0.0, 1.0));
    launch_lanczos_update(c, j, maxDim);
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
  launch_lanczos_combine(c, c->trial_d);
  return converged;
}

// SIL Integrate (src/IntegratorList/Sil/S_IntegratorList_Sil.f90:114-177) on a device state.
int sil_device(cgpu_ctx* c, int which, z_t* state, double t0, double t1, int krylovDim, double tol, int maxRestarts,
               const double* metric_d) {
  const double zeroThreshold = 1.0e-14;
  if (std::fabs(t1 - t0) <= zeroThreshold) return 0;
  int maxDim = std::max(1, std::min(krylovDim, c->nS));
  if (maxDim > c->maxKrylov) throw std::string("SIL: krylovDim exceeds the context's max_krylov");
  c->metric_d = const_cast<double*>(metric_d);
  int warnings = 0;
  CODY_CUDA(cudaMemcpyAsync(c->work_d, state, sizeof(z_t) * c->nS, cudaMemcpyDeviceToDevice, c->stream));
  double tCur = t0, rem = t1 - t0;
  while (std::fabs(rem) > zeroThreshold) {
    double dtS = rem;
    int restarts = 0;
    int conv = 0;
    for (;;) {
      double err = 0.0;
      conv = lanczos_pass(c, which, tCur, dtS, maxDim, tol, &err);
      if (conv == 1) break;
      if (conv < 0) break;  // fixed-order pass: no convergence test (tolerance 0)
      if (std::fabs(dtS) <= zeroThreshold || restarts >= maxRestarts) break;
      dtS = 0.5 * dtS;
      restarts++;
    }
    if (conv != 1) warnings++;
    CODY_CUDA(cudaMemcpyAsync(c->work_d, c->trial_d, sizeof(z_t) * c->nS, cudaMemcpyDeviceToDevice, c->stream));
    tCur = tCur + dtS;
    rem = rem - dtS;
  }
  CODY_CUDA(cudaMemcpyAsync(state, c->work_d, sizeof(z_t) * c->nS, cudaMemcpyDeviceToDevice, c->stream));
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

__global__ void k_advance_time(double* t, double dt) { *t = *t + dt; }

// Captures one fixed-order Strang step on state_d as a CUDA graph.  The step
// reads its start time from stepT_d (the laser is evaluated on the device) and
// advances it by dt, so the graph can be replayed for consecutive steps.  A
// first step on a scratch copy of the state allocates every lazily sized
// buffer outside the capture.
void capture_step_graph(cgpu_ctx* c, double t0, double dt, int krylov, int useMetric) {
  if (c->stepGraph) {
    cudaGraphExecDestroy(c->stepGraph);
    c->stepGraph = nullptr;
  }
  if (!c->warm_d) c->warm_d = dalloc<z_t>(c->nS);
  CODY_CUDA(cudaMemcpyAsync(c->warm_d, c->state_d, sizeof(z_t) * c->nS, cudaMemcpyDeviceToDevice, c->stream));
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
    k_advance_time<<<1, 1, 0, c->stream>>>(c->stepT_d, dt);
    CODY_LAUNCHED(c);
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
  if (c->stepGraphRaw) cudaGraphDestroy(c->stepGraphRaw);
  c->stepGraphRaw = g;  // kept: a batch embeds it as a child graph
  CODY_CUDA(e);
  c->graphDt = dt;
  c->graphKrylov = krylov;
  c->graphMetric = useMetric;
}

double energy_device(cgpu_ctx* c, const z_t* state, double t) {
  const z_t* C = state;
  const z_t* orbs = (c->method == CGPU_METHOD_TDCI) ? c->tdciOrbs_d : state + c->nC;
  launch_ci_rdm(c, C, 1, 1);
  launch_onebody(c, c->orbTmp_d, orbs, t, zmk(1.0, 0.0), 0);
  launch_fill_h1_from(c, orbs, c->orbTmp_d, c->h1_d);
  launch_fill_h2(c, orbs);
  launch_energy(c, c->scal_d + 8);
  double e = 0.0;
  CODY_CUDA(cudaMemcpyAsync(&e, c->scal_d + 8, sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  CODY_CUDA(cudaStreamSynchronize(c->stream));
  return e;
}

// helpers for host <-> device staging
void up(cgpu_ctx* c, z_t* dst, const cgpu_complex* src, size_t n) {
  CODY_CUDA(cudaMemcpyAsync(dst, src, sizeof(z_t) * n, cudaMemcpyHostToDevice, c->stream));
}
void down(cgpu_ctx* c, cgpu_complex* dst, const z_t* src, size_t n) {
  CODY_CUDA(cudaMemcpyAsync(dst, src, sizeof(z_t) * n, cudaMemcpyDeviceToHost, c->stream));
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

}  // namespace

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
  *out = nullptr;
  cgpu_ctx* c = new cgpu_ctx();
  try {
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
      cudaGetLastError();
      throw std::string("cuda: no CUDA device available");
    }
    build_ctx(c, desc);
  } catch (const std::string& e) {
    free_ctx(c);
    delete c;
    return fail(nullptr, e, e.find("cuda") != std::string::npos ? CGPU_ERR_CUDA : CGPU_ERR_ARG);
  } catch (const std::exception& e) {
    free_ctx(c);
    delete c;
    return fail(nullptr, e.what(), CGPU_ERR_ARG);
  }
  *out = c;
  return CGPU_OK;
}

int cgpu_ctx_destroy(cgpu_ctx* ctx) {
  if (!ctx) return CGPU_OK;
  free_ctx(ctx);
  delete ctx;
  return CGPU_OK;
}

const char* cgpu_last_error(const cgpu_ctx* ctx) { return ctx ? ctx->lastError.c_str() : g_lastGlobalError.c_str(); }
const char* cgpu_last_global_error(void) { return g_lastGlobalError.c_str(); }

int cgpu_sizes(const cgpu_ctx* c, int* out) {
  if (!c || !out) return CGPU_ERR_ARG;
  out[0] = c->nG; out[1] = c->nO; out[2] = c->nOS; out[3] = c->nC; out[4] = c->nBt; out[5] = c->nS;
  return CGPU_OK;
}

int cgpu_grid(const cgpu_ctx* c, double* x, double* w) {
  if (!c) return CGPU_ERR_ARG;
  if (x) std::memcpy(x, c->x.data(), sizeof(double) * c->nG);
  if (w) std::memcpy(w, c->w.data(), sizeof(double) * c->nG);
  return CGPU_OK;
}

int cgpu_configlist_tables(cgpu_ctx* c, int bt, int kind, int* n_conf, int* max_conn, int64_t* codes,
                           int* n_connected, int* excited_c, int* orb_code, double* factor) {
  CODY_API_BEGIN(c)
  if (bt < 0 || bt >= c->nBt) throw std::string("configlist: body type out of range");
  CiTables& t = c->tab[bt];
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
  size_t n = (size_t)c->nG * c->nOS;
  up(c, c->orbTmp_d, orbs, n);
  if (c->restricted) launch_orthonormalize(c, c->orbTmp_d, 0, c->nOS);
  else
    for (int b = 0; b < c->nBt; b++) launch_orthonormalize(c, c->orbTmp_d, c->orbStart[b], c->nOrbs[b]);
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
    double dt = t1 - t0;
    if (!c->stepGraph || c->graphDt != dt || c->graphKrylov != krylov_dim || c->graphMetric != use_metric ||
        c->graphProf != c->profTarget)
      capture_step_graph(c, t0, dt, krylov_dim, use_metric);
    if (c->profTarget) c->profUsed = c->graphProfUsed;
    CODY_CUDA(cudaMemcpyAsync(c->stepT_d, &t0, sizeof(double), cudaMemcpyHostToDevice, c->stream));
    CODY_CUDA(cudaGraphLaunch(c->stepGraph, c->stream));
    c->launches += c->graphKernels;
  } else {
    split2_device(c, c->state_d, t0, t1, krylov_dim, tolerance, max_restarts, use_metric);
  }
  down(c, state, c->state_d, c->nS);
  sync(c);
  CODY_API_END(c)
}

int cgpu_state_upload(cgpu_ctx* c, const cgpu_complex* state) {
  CODY_API_BEGIN(c)
  up(c, c->state_d, state, c->nS);
  sync(c);
  CODY_API_END(c)
}

int cgpu_state_download(cgpu_ctx* c, cgpu_complex* state) {
  CODY_API_BEGIN(c)
  down(c, state, c->state_d, c->nS);
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
      t = t + dt;
    }
    CODY_CUDA(cudaGetLastError());
  } else {
    if (!c->stepGraph || c->graphDt != dt || c->graphKrylov != krylov_dim || c->graphMetric != use_metric ||
        c->graphProf != c->profTarget) {
      capture_step_graph(c, t0, dt, krylov_dim, use_metric);
    }
    if (c->profTarget) c->profUsed = c->graphProfUsed;
    CODY_CUDA(cudaMemcpyAsync(c->stepT_d, &t0, sizeof(double), cudaMemcpyHostToDevice, c->stream));
    for (int s = 0; s < n_steps; s++) CODY_CUDA(cudaGraphLaunch(c->stepGraph, c->stream));
    c->launches += n_steps * c->graphKernels;
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

}  // extern "C"

// ---------------------------------------------------------------------------
// Batched trajectories: one context per trajectory; the step graph of every
// context is a child node (no dependencies between them) of one batch graph.
// ---------------------------------------------------------------------------
struct cgpu_batch {
  std::vector<cgpu_ctx*> ctx;
  cudaStream_t stream = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  double dt = 0.0;
  int krylov = -1, metric = -1;
  long kernelsPerStep = 0;
  std::vector<double> t0;  // start times the graph was last launched from
};

namespace {
void batch_free_graph(cgpu_batch* b) {
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  b->exec = nullptr;
  b->graph = nullptr;
  b->kernelsPerStep = 0;
}

void batch_build_graph(cgpu_batch* b, const double* t0, double dt, int krylov, int useMetric) {
  batch_free_graph(b);
  CODY_CUDA(cudaGraphCreate(&b->graph, 0));
  for (size_t i = 0; i < b->ctx.size(); i++) {
    cgpu_ctx* c = b->ctx[i];
    c->profTarget = 0;
    capture_step_graph(c, t0[i], dt, krylov, useMetric);
    cudaGraphNode_t node;
    CODY_CUDA(cudaGraphAddChildGraphNode(&node, b->graph, nullptr, 0, c->stepGraphRaw));
    b->kernelsPerStep += c->graphKernels;
  }
  CODY_CUDA(cudaGraphInstantiate(&b->exec, b->graph, 0));
  b->dt = dt;
  b->krylov = krylov;
  b->metric = useMetric;
}
}  // namespace

#define CODY_BATCH_BEGIN(b)                                          \
  if (!(b)) return fail(nullptr, "null batch", CGPU_ERR_ARG);        \
  try {

extern "C" {

int cgpu_batch_create(const cgpu_desc* descs, int n, cgpu_batch** out) {
  if (!descs || !out || n <= 0) return fail(nullptr, "cgpu_batch_create: bad argument", CGPU_ERR_ARG);
  *out = nullptr;
  cgpu_batch* b = new cgpu_batch();
  for (int i = 0; i < n; i++) {
    cgpu_ctx* c = nullptr;
    int rc = cgpu_ctx_create(&descs[i], &c);
    if (rc != CGPU_OK) {
      std::string msg = "batch trajectory " + std::to_string(i) + ": " + g_lastGlobalError;
      cgpu_batch_destroy(b);
      return fail(nullptr, msg, rc);
    }
    b->ctx.push_back(c);
  }
  if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess) {
    cgpu_batch_destroy(b);
    return fail(nullptr, "cuda: batch stream creation failed", CGPU_ERR_CUDA);
  }
  *out = b;
  return CGPU_OK;
}

int cgpu_batch_destroy(cgpu_batch* b) {
  if (!b) return CGPU_OK;
  if (b->stream) cudaStreamSynchronize(b->stream);
  batch_free_graph(b);
  if (b->stream) cudaStreamDestroy(b->stream);
  for (cgpu_ctx* c : b->ctx) cgpu_ctx_destroy(c);
  delete b;
  return CGPU_OK;
}

int cgpu_batch_size(const cgpu_batch* b) { return b ? (int)b->ctx.size() : 0; }

cgpu_ctx* cgpu_batch_context(cgpu_batch* b, int i) {
  if (!b || i < 0 || i >= (int)b->ctx.size()) return nullptr;
  return b->ctx[i];
}

long cgpu_batch_kernels_per_step(const cgpu_batch* b) { return b ? b->kernelsPerStep : 0; }

int cgpu_batch_propagate(cgpu_batch* b, const double* t0, double dt, int n_steps, int krylov_dim, int use_metric,
                         double* elapsed_ms) {
  CODY_BATCH_BEGIN(b)
  if (!t0 || n_steps < 0 || krylov_dim <= 0) throw std::string("batch_propagate: bad argument");
  // uploads and other work queued on the contexts' own streams come first
  for (cgpu_ctx* c : b->ctx) CODY_CUDA(cudaStreamSynchronize(c->stream));
  if (!b->exec || b->dt != dt || b->krylov != krylov_dim || b->metric != use_metric)
    batch_build_graph(b, t0, dt, krylov_dim, use_metric);
  for (size_t i = 0; i < b->ctx.size(); i++)
    CODY_CUDA(cudaMemcpyAsync(b->ctx[i]->stepT_d, &t0[i], sizeof(double), cudaMemcpyHostToDevice, b->stream));
  cudaEvent_t e0, e1;
  CODY_CUDA(cudaEventCreate(&e0));
  CODY_CUDA(cudaEventCreate(&e1));
  CODY_CUDA(cudaEventRecord(e0, b->stream));
  for (int s = 0; s < n_steps; s++) CODY_CUDA(cudaGraphLaunch(b->exec, b->stream));
  CODY_CUDA(cudaEventRecord(e1, b->stream));
  CODY_CUDA(cudaEventSynchronize(e1));
  float ms = 0.f;
  CODY_CUDA(cudaEventElapsedTime(&ms, e0, e1));
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (elapsed_ms) *elapsed_ms = ms;
  for (cgpu_ctx* c : b->ctx) {
    c->launches += n_steps * c->graphKernels;
    if (c->mixed && mixed_error(c)) throw std::string("tensor-core GEMM: a bounded mbarrier wait expired");
  }
  CODY_API_END(nullptr)
}

}  // extern "C"
