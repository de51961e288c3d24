// cody_oracle.cpp -- CPU restatement of CodyFortran's MCTDHX/TDCI hot path.
//
// TEST INFRASTRUCTURE ONLY.  This file is the parity oracle for the GB300
// engine in codyfortran_gb300/.  Only tests/, __graft_entry__.smoke() and the
// cpu_baseline leg of bench.py may load it; the product never does.
//
// Every routine restates the reference algorithm it names (paths are relative
// to the CodyFortran source tree).  Loop orders, index encodings and sign
// conventions follow the reference so that the configuration tables are
// bit-exact and the floating point results agree to ~1e-15.
//
// Third-party arithmetic the reference delegates to libraries is restated from
// the published methods:
//   * LAPACK ZHEEV / DSYEV  -> cyclic Jacobi eigenvalue method (Jacobi 1846,
//     Rutishauser 1966) for Hermitian / real symmetric matrices.
//   * GSL gsl_combination_next order -> lexicographic k-subsets.
//   * Fortran stdlib gauss_legendre_lobatto -> Newton iteration on P'_{n-1}.
//   * FFTW zero-padded convolution -> the direct Toeplitz sum it equals.
//
// Extensions the reference lacks (parity unpinned by reference tests):
//   * 1D FEDVR kinetic operator on grid.linear.fedvr, built from the radial
//     template src/SysKinetic/Ylm/Laplacian/Fedvr/S_SysKinetic_Ylm_Laplacian_Fedvr.f90:49-95
//     with nLocals = order+1 points per element.
//   * dense soft-Yukawa interaction V(x_i,x_j) on non-uniform grids.
//   * 1D length-gauge laser E(t)*x, from
//     src/SysPotential/Ylm/CoulombLaser/S_SysPotential_Ylm_CoulombLaser.f90:60-83,
//     or a piecewise-constant sampled field.
//
// Build: see oracle/Makefile (g++ -O3 -fopenmp -shared).

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef std::complex<double> cd;
static const cd IU(0.0, 1.0);
static const double PI = 3.14159265358979323846264338327950288;

// ---------------------------------------------------------------------------
// Specification struct shared with the Python test harness (oracle/oracle.py).
// ---------------------------------------------------------------------------
extern "C" {
typedef struct {
  int grid_kind;            // 0: grid.linear.const + finite differences, 1: FEDVR
  double xmin, xmax;
  int n_points;             // const grid
  int n_elements, n_locals; // FEDVR: points per element (order + 1)
  int xmin_excluded, xmax_excluded;
  int n_bt;
  int n_bodies[4];
  int n_orbs[4];
  double mass[4];
  char stats[4];            // 'f' or 'b' (bosons unsupported here)
  int restricted;
  double reg_eps;
  int n_nuclei;
  double nuc_pos[8], nuc_charge[8], nuc_s1[8], nuc_s2[8], nuc_damp[8];
  int has_interaction;
  double int_strength, int_s1, int_s2, int_damp;
  int int_kind;             // 0: Toeplitz K(|i-j|dx) (uniform grid), 1: dense K(|x_i-x_j|)
  int laser_kind;           // 0 none, 1 sin^2 pulse, 2 sampled piecewise constant
  double E0, omega, n_cycles, cep, t_start;
  const double* field_samples;
  int n_samples;
  double sample_dt, sample_t0;
  int method;               // 0 MCTDHX, 1 TDCI (static orbitals)
  int n_threads;            // OpenMP threads (0 = runtime default)
} orc_spec;
}

// ---------------------------------------------------------------------------
// Eigen solvers (restating LAPACK ZHEEV/DSYEV results by the Jacobi method).
// A is column-major n x n; on return evals ascending, evecs column-major.
// ---------------------------------------------------------------------------
static void jacobi_herm(int n, const cd* Ain, double* evals, cd* evecs) {
  std::vector<cd> A(Ain, Ain + (size_t)n * n);
  auto a = [&](int i, int j) -> cd& { return A[i + (size_t)n * j]; };
  std::vector<cd> V((size_t)n * n, 0.0);
  for (int i = 0; i < n; i++) V[i + (size_t)n * i] = 1.0;
  for (int i = 0; i < n; i++) a(i, i) = cd(a(i, i).real(), 0.0);
  for (int sweep = 0; sweep < 100; sweep++) {
    double off = 0.0, diag = 0.0;
    for (int j = 0; j < n; j++)
      for (int i = 0; i < n; i++) {
        if (i != j) off += std::norm(a(i, j));
        else diag += std::norm(a(i, j));
      }
    if (off <= 1e-28 * (diag + off) || off == 0.0) break;  // rounding floor is ~1e-32
    for (int p = 0; p < n - 1; p++)
      for (int q = p + 1; q < n; q++) {
        cd b = a(p, q);
        double g = std::abs(b);
        if (g == 0.0) continue;
        cd ph = b / g;  // e^{i theta}
        double app = a(p, p).real(), aqq = a(q, q).real();
        double tau = (aqq - app) / (2.0 * g);
        double t = (tau >= 0 ? 1.0 : -1.0) / (std::fabs(tau) + std::sqrt(1.0 + tau * tau));
        double c = 1.0 / std::sqrt(1.0 + t * t), s = t * c;
        cd phc = std::conj(ph);
        // columns: A <- A U, U = [[c, s],[-s e^{-i th}, c e^{-i th}]]
        for (int k = 0; k < n; k++) {
          cd akp = a(k, p), akq = a(k, q);
          a(k, p) = akp * c - akq * s * phc;
          a(k, q) = akp * s + akq * c * phc;
        }
        // rows: A <- U^H A
        for (int k = 0; k < n; k++) {
          cd apk = a(p, k), aqk = a(q, k);
          a(p, k) = c * apk - s * ph * aqk;
          a(q, k) = s * apk + c * ph * aqk;
        }
        a(p, q) = 0.0;
        a(q, p) = 0.0;
        a(p, p) = cd(a(p, p).real(), 0.0);
        a(q, q) = cd(a(q, q).real(), 0.0);
        for (int k = 0; k < n; k++) {
          cd vkp = V[k + (size_t)n * p], vkq = V[k + (size_t)n * q];
          V[k + (size_t)n * p] = vkp * c - vkq * s * phc;
          V[k + (size_t)n * q] = vkp * s + vkq * c * phc;
        }
      }
  }
  std::vector<int> idx(n);
  for (int i = 0; i < n; i++) idx[i] = i;
  std::stable_sort(idx.begin(), idx.end(), [&](int i, int j) { return a(i, i).real() < a(j, j).real(); });
  for (int k = 0; k < n; k++) {
    evals[k] = a(idx[k], idx[k]).real();
    for (int i = 0; i < n; i++) evecs[i + (size_t)n * k] = V[i + (size_t)n * idx[k]];
  }
}

static void jacobi_sym(int n, const double* Ain, double* evals, double* evecs) {
  std::vector<double> A(Ain, Ain + (size_t)n * n);
  auto a = [&](int i, int j) -> double& { return A[i + (size_t)n * j]; };
  std::vector<double> V((size_t)n * n, 0.0);
  for (int i = 0; i < n; i++) V[i + (size_t)n * i] = 1.0;
  for (int sweep = 0; sweep < 100; sweep++) {
    double off = 0.0, diag = 0.0;
    for (int j = 0; j < n; j++)
      for (int i = 0; i < n; i++) {
        if (i != j) off += a(i, j) * a(i, j);
        else diag += a(i, j) * a(i, j);
      }
    if (off <= 1e-28 * (diag + off) || off == 0.0) break;  // rounding floor is ~1e-32
    for (int p = 0; p < n - 1; p++)
      for (int q = p + 1; q < n; q++) {
        double g = a(p, q);
        if (g == 0.0) continue;
        double tau = (a(q, q) - a(p, p)) / (2.0 * g);
        double t = (tau >= 0 ? 1.0 : -1.0) / (std::fabs(tau) + std::sqrt(1.0 + tau * tau));
        double c = 1.0 / std::sqrt(1.0 + t * t), s = t * c;
        for (int k = 0; k < n; k++) {
          double akp = a(k, p), akq = a(k, q);
          a(k, p) = akp * c - akq * s;
          a(k, q) = akp * s + akq * c;
        }
        for (int k = 0; k < n; k++) {
          double apk = a(p, k), aqk = a(q, k);
          a(p, k) = c * apk - s * aqk;
          a(q, k) = s * apk + c * aqk;
        }
        a(p, q) = 0.0;
        a(q, p) = 0.0;
        for (int k = 0; k < n; k++) {
          double vkp = V[k + (size_t)n * p], vkq = V[k + (size_t)n * q];
          V[k + (size_t)n * p] = vkp * c - vkq * s;
          V[k + (size_t)n * q] = vkp * s + vkq * c;
        }
      }
  }
  std::vector<int> idx(n);
  for (int i = 0; i < n; i++) idx[i] = i;
  std::stable_sort(idx.begin(), idx.end(), [&](int i, int j) { return a(i, i) < a(j, j); });
  for (int k = 0; k < n; k++) {
    evals[k] = a(idx[k], idx[k]);
    for (int i = 0; i < n; i++) evecs[i + (size_t)n * k] = V[i + (size_t)n * idx[k]];
  }
}

// ---------------------------------------------------------------------------
// Gauss-Legendre-Lobatto nodes/weights on [a,b] (restates stdlib
// gauss_legendre_lobatto used at src/Utils/M_Utils_Fedvr.f90:127).
// Interior nodes are roots of P'_{n-1}, found by Newton iteration from
// Chebyshev-Gauss-Lobatto guesses; w_i = 2 / (n (n-1) P_{n-1}(x_i)^2).
// ---------------------------------------------------------------------------
static void legendre_p(int n, double x, double* p, double* dp) {
  double p0 = 1.0, p1 = x;
  if (n == 0) { *p = 1.0; *dp = 0.0; return; }
  for (int k = 2; k <= n; k++) {
    double p2 = ((2.0 * k - 1.0) * x * p1 - (k - 1.0) * p0) / k;
    p0 = p1; p1 = p2;
  }
  *p = p1;
  // (1-x^2) P_n' = n (P_{n-1} - x P_n)
  *dp = (std::fabs(1.0 - x * x) > 0) ? n * (p0 - x * p1) / (1.0 - x * x) : 0.0;
}

static void gll(int npts, double a, double b, double* x, double* w) {
  int n = npts - 1;  // polynomial degree
  std::vector<double> xr(npts);
  for (int i = 0; i < npts; i++) {
    if (i == 0) { xr[i] = -1.0; continue; }
    if (i == n) { xr[i] = 1.0; continue; }
    double xi = -std::cos(PI * i / n);
    for (int it = 0; it < 100; it++) {
      double p, dp;
      legendre_p(n, xi, &p, &dp);
      // P'' from the Legendre ODE: (1-x^2) P'' = 2x P' - n(n+1) P
      double d2p = (2.0 * xi * dp - n * (n + 1.0) * p) / (1.0 - xi * xi);
      double dx = dp / d2p;
      xi -= dx;
      if (std::fabs(dx) < 1e-16) break;
    }
    xr[i] = xi;
  }
  for (int i = 0; i < npts; i++) {
    double p, dp;
    legendre_p(n, xr[i], &p, &dp);
    double wr = 2.0 / (n * (n + 1.0) * p * p);
    x[i] = 0.5 * (b - a) * xr[i] + 0.5 * (a + b);
    w[i] = 0.5 * (b - a) * wr;
  }
}

// ---------------------------------------------------------------------------
// Oracle state.
// ---------------------------------------------------------------------------
struct Excitations {  // src/ConfigList/M_ConfigList.f90:112-128
  int maxConn = 0;
  std::vector<int> nConnected;   // (nConf)
  std::vector<int> excitedC;     // (maxConn, nConf) column-major, 1-based config index
  std::vector<int> orbCode;      // 1-based packed orbital code
  std::vector<double> factor;    // +-1
};

struct ConfigListE {
  int bodyTarget;  // 0-based body type
  int nConf;
  std::vector<int64_t> code;     // codeFromConfig
  Excitations singles, doubles;
};

struct Oracle {
  orc_spec s;
  // grid
  int nG = 0;
  std::vector<double> x, w;
  double dxConst = 0.0;
  // FEDVR
  int nE = 0, nLoc = 0;
  std::vector<int> elStart, elEnd;  // 0-based inclusive
  std::vector<double> elSize;
  std::vector<double> Kref;         // nLoc x nLoc column-major (secondOrderMatrix)
  std::vector<double> Dref;         // first order
  // potential (time independent part)
  std::vector<double> V0;
  // interaction
  std::vector<double> kernelVals;   // Toeplitz kernel K(k dx)
  std::vector<double> Vdense;       // dense nG x nG (column-major, symmetric)
  // method
  int nBt = 0, nO = 0, nOS = 0, nC = 0;
  std::vector<int> btOfOrb, orbStart, orbEnd;  // 0-based
  std::vector<ConfigListE> cl;
  // TDCI static data
  std::vector<cd> tdciOrbs, tdciH1, tdciH2, tdciH2Lin;
  std::string err;
};

// ---------------------------------------------------------------------------
// Binomial (src/Utils/M_Utils_SfGslLib.f90:95-121) and lexicographic rank
// (src/Utils/M_Utils_Combinatorics.f90:43-73).
// ---------------------------------------------------------------------------
static long long binom(int n, int k) {
  if (n == k) return 1;
  if (k == 0) return 1;
  if (n > k) {
    if (k < 0) return 0;
    long double r = 1.0;
    for (int i = 1; i <= k; i++) r = r * (n - k + i) / i;
    return (long long)std::llround((double)r);
  }
  if (n < k && n >= 0) return 0;
  return 0;
}

static int index_of_combi(int n, const int* combi, int k) {  // 1-based combi entries
  long long res = 1;
  int s = 0;
  for (int i = 1; i <= k; i++) {
    int e = combi[i - 1];
    if (i > 1) s = combi[i - 2];
    if (s + 1 < e) res += binom(n - s, k - i + 1) - binom(n - e + 1, k - i + 1);
  }
  return (int)res;
}

// src/ConfigList/AllActive/Fermions/S_ConfigList_AllActive_Fermions.f90:232-334
static int excite_configuration(const ConfigListE& c, const int* nOrbsBt, const int* nBodiesBt, double* factor,
                                const int* creates, int nCreates, const int* destroys, int nDestroys, int iC) {
  int nOBt = nOrbsBt[c.bodyTarget], nBBt = nBodiesBt[c.bodyTarget];
  *factor = 1.0;
  int occ[64];
  int64_t code = c.code[iC - 1];
  for (int i = 1; i <= nOBt; i++) occ[i] = ((code >> (i - 1)) & 1) ? 1 : 0;
  for (int i = 0; i < nDestroys; i++) {
    int d = destroys[i];
    if (occ[d] == 0) return 0;
    for (int j = 1; j < d; j++)
      if (occ[j] == 1) *factor = -*factor;
    occ[d] -= 1;
  }
  for (int i = 0; i < nCreates; i++) {
    int cr = creates[nCreates - 1 - i];
    if (occ[cr] == 1) return 0;
    for (int j = 1; j < cr; j++)
      if (occ[j] == 1) *factor = -*factor;
    occ[cr] += 1;
  }
  int i1[64];
  int i = 0, sum = 1;
  while (sum <= nBBt) {
    i++;
    if (occ[i] == 0) continue;
    i1[sum - 1] = i;
    sum += occ[i];
  }
  return index_of_combi(nOBt, i1, nBBt);
}

// Fermion Setup: src/ConfigList/AllActive/Fermions/S_ConfigList_AllActive_Fermions.f90:147-199
// Singles: src/ConfigList/AllActive/S_ConfigList_AllActive.f90:141-229
// Doubles: src/ConfigList/AllActive/S_ConfigList_AllActive.f90:250-349
static void setup_configlist(Oracle& o, int bt) {
  ConfigListE c;
  c.bodyTarget = bt;
  int M = o.s.n_orbs[bt], N = o.s.n_bodies[bt];
  // nConfigurations = sum_k C(M-N,k) C(N,k), k = 0..nExcitations (= N): equals C(M,N)
  long long nconf = 0;
  for (int k = 0; k <= N; k++) nconf += binom(M - N, k) * binom(N, k);
  c.nConf = (int)nconf;
  // lexicographic k-subsets (GSL combination order)
  std::vector<int> comb(N);
  for (int i = 0; i < N; i++) comb[i] = i;
  c.code.assign(c.nConf, 0);
  for (int iC = 0; iC < c.nConf; iC++) {
    int64_t code = 0;
    for (int j = 0; j < N; j++) code |= (int64_t)1 << comb[j];
    c.code[iC] = code;
    int one_based[64] = {0};
    for (int j = 0; j < N; j++) one_based[j] = comb[j] + 1;
    if (index_of_combi(M, one_based, N) != iC + 1) { o.err = "index calc failed"; }
    // gsl_combination_next
    int i = N - 1;
    while (i >= 0 && comb[i] == M - N + i) i--;
    if (i < 0) break;
    comb[i]++;
    for (int j = i + 1; j < N; j++) comb[j] = comb[j - 1] + 1;
  }
  int shift = 0;
  for (int b = 0; b < bt; b++) shift += o.s.n_orbs[b];
  int nO = o.nO;
  // singles
  {
    Excitations& e = c.singles;
    e.nConnected.assign(c.nConf, 0);
    for (int iC = 1; iC <= c.nConf; iC++) {
      int k = 0;
      for (int j1 = 1; j1 <= M; j1++)
        for (int i1 = 1; i1 <= M; i1++) {
          double f;
          if (excite_configuration(c, o.s.n_orbs, o.s.n_bodies, &f, &i1, 1, &j1, 1, iC) == 0) continue;
          k++;
        }
      e.nConnected[iC - 1] = k;
    }
    e.maxConn = *std::max_element(e.nConnected.begin(), e.nConnected.end());
    e.excitedC.assign((size_t)e.maxConn * c.nConf, 0);
    e.orbCode.assign((size_t)e.maxConn * c.nConf, 0);
    e.factor.assign((size_t)e.maxConn * c.nConf, 0.0);
    for (int iC = 1; iC <= c.nConf; iC++) {
      int k = 0;
      for (int j1 = 1; j1 <= M; j1++)
        for (int i1 = 1; i1 <= M; i1++) {
          double f;
          int iCNew = excite_configuration(c, o.s.n_orbs, o.s.n_bodies, &f, &i1, 1, &j1, 1, iC);
          if (iCNew == 0) continue;
          k++;
          int orbCode = 1;
          orbCode = (orbCode - 1) * nO + (i1 + shift);
          orbCode = (orbCode - 1) * nO + (j1 + shift);
          size_t at = (size_t)(k - 1) + (size_t)e.maxConn * (iC - 1);
          e.orbCode[at] = orbCode;
          e.excitedC[at] = iCNew;
          e.factor[at] = f;
        }
    }
  }
  // doubles
  {
    Excitations& e = c.doubles;
    e.nConnected.assign(c.nConf, 0);
    for (int pass = 0; pass < 2; pass++) {
      if (pass == 1) {
        e.maxConn = *std::max_element(e.nConnected.begin(), e.nConnected.end());
        e.excitedC.assign((size_t)e.maxConn * c.nConf, 0);
        e.orbCode.assign((size_t)e.maxConn * c.nConf, 0);
        e.factor.assign((size_t)e.maxConn * c.nConf, 0.0);
      }
      for (int iC = 1; iC <= c.nConf; iC++) {
        int k = 0;
        for (int j2 = 1; j2 <= M; j2++)
          for (int j1 = 1; j1 <= j2; j1++)
            for (int i2 = 1; i2 <= M; i2++)
              for (int i1 = 1; i1 <= i2; i1++) {
                int cr[2] = {i1, i2}, de[2] = {j1, j2};
                double f;
                int iCNew = excite_configuration(c, o.s.n_orbs, o.s.n_bodies, &f, cr, 2, de, 2, iC);
                if (iCNew == 0) continue;
                k++;
                if (pass == 1) {
                  int orbCode = 1;
                  orbCode = (orbCode - 1) * nO + (i1 + shift);
                  orbCode = (orbCode - 1) * nO + (j1 + shift);
                  orbCode = (orbCode - 1) * nO + (i2 + shift);
                  orbCode = (orbCode - 1) * nO + (j2 + shift);
                  size_t at = (size_t)(k - 1) + (size_t)e.maxConn * (iC - 1);
                  e.orbCode[at] = orbCode;
                  e.excitedC[at] = iCNew;
                  e.factor[at] = f;
                }
              }
        if (pass == 0) e.nConnected[iC - 1] = k;
      }
    }
  }
  o.cl.push_back(std::move(c));
}

// ---------------------------------------------------------------------------
// Grid (src/Grid/Linear/Const/S_Grid_Linear_Const.f90:34-52,
// src/Utils/M_Utils_Fedvr.f90:76-149) and FEDVR derivative context
// (src/Utils/M_Utils_DerivativeFedvr.f90:29-76, 160-181).
// ---------------------------------------------------------------------------
static double lagrange_derivative(const double* xr, int iLocal, int iNode, int n) {
  double res;
  if (iLocal == iNode) {
    res = 0.0;
    for (int k = 0; k < n; k++)
      if (k != iLocal) res += 1.0 / (xr[iNode] - xr[k]);
  } else {
    res = 1.0 / (xr[iLocal] - xr[iNode]);
    for (int k = 0; k < n; k++)
      if (k != iLocal && k != iNode) res *= (xr[iNode] - xr[k]) / (xr[iLocal] - xr[k]);
  }
  return res;
}

static void setup_grid(Oracle& o) {
  const orc_spec& s = o.s;
  if (s.grid_kind == 0) {
    o.nG = s.n_points;
    o.x.resize(o.nG);
    o.w.resize(o.nG);
    double dx = (s.xmax - s.xmin) / (o.nG - 1);
    for (int i = 0; i < o.nG; i++) {
      o.w[i] = dx;
      o.x[i] = s.xmin + o.w[i] * i;
    }
    o.dxConst = dx;
  } else {
    int nE = s.n_elements, nL = s.n_locals;
    o.nE = nE; o.nLoc = nL;
    double es = (s.xmax - s.xmin) / nE;
    int np = nE * (nL - 1) + 1;
    if (s.xmin_excluded) np--;
    if (s.xmax_excluded) np--;
    o.nG = np;
    o.x.assign(np, 0.0);
    o.w.assign(np, 0.0);
    o.elStart.resize(nE);
    o.elEnd.resize(nE);
    o.elSize.assign(nE, es);
    std::vector<double> ep(nL), ew(nL);
    int iGrid = 0;  // 1-based as in the reference
    for (int iE = 1; iE <= nE; iE++) {
      double lb = s.xmin + (iE - 1) * es, rb = s.xmin + iE * es;
      gll(nL, lb, rb, ep.data(), ew.data());
      int iStart = 0;
      for (int iL = 1; iL <= nL; iL++) {
        if (iE == 1 && iL == 1 && s.xmin_excluded) continue;
        if (iE == nE && iL == nL && s.xmax_excluded) continue;
        if (iE == 1 || iL != 1) iGrid++;
        if (iStart == 0) iStart = iGrid;
        o.x[iGrid - 1] = ep[iL - 1];
        o.w[iGrid - 1] += ew[iL - 1];
      }
      o.elStart[iE - 1] = iStart - 1;
      o.elEnd[iE - 1] = iGrid - 1;
    }
    std::vector<double> xr(nL), wr(nL);
    gll(nL, -0.5, 0.5, xr.data(), wr.data());
    o.Dref.assign((size_t)nL * nL, 0.0);
    o.Kref.assign((size_t)nL * nL, 0.0);
    for (int i = 0; i < nL; i++)
      for (int j = 0; j < nL; j++) o.Dref[i + (size_t)nL * j] = lagrange_derivative(xr.data(), j, i, nL);
    for (int i = 0; i < nL; i++)
      for (int j = 0; j < nL; j++)
        for (int k = 0; k < nL; k++)
          o.Kref[i + (size_t)nL * j] -= wr[k] * o.Dref[k + (size_t)nL * i] * o.Dref[k + (size_t)nL * j];
  }
}

// ApplyDerivativeOperator (src/Utils/M_Utils_DerivativeFedvr.f90:115-152), dxPower = 1
static void fedvr_second_derivative(const Oracle& o, const cd* f, cd* res) {
  int nL = o.nLoc, nE = o.nE;
  for (int i = 0; i < o.nG; i++) res[i] = 0.0;
  for (int iE = 0; iE < nE; iE++) {
    int iS = o.elStart[iE], iEn = o.elEnd[iE];
    int l0 = 0, l1 = nL - 1;
    if (o.s.xmin_excluded && iE == 0) l0 = 1;
    if (o.s.xmax_excluded && iE == nE - 1) l1 = nL - 2;
    double dx = o.elSize[iE];
    int m = l1 - l0 + 1;
    (void)iEn;
    for (int a = 0; a < m; a++) {
      cd acc = 0.0;
      for (int b = 0; b < m; b++) acc += o.Kref[(a + l0) + (size_t)nL * (b + l0)] * f[iS + b];
      res[iS + a] += acc / dx;
    }
  }
  for (int i = 0; i < o.nG; i++) res[i] /= o.w[i];
}

static void fedvr_first_derivative(const Oracle& o, const cd* f, cd* res) {
  int nL = o.nLoc, nE = o.nE;
  std::vector<double> xr(nL), wr(nL);
  gll(nL, -0.5, 0.5, xr.data(), wr.data());
  for (int i = 0; i < o.nG; i++) res[i] = 0.0;
  for (int iE = 0; iE < nE; iE++) {
    int iS = o.elStart[iE];
    int l0 = 0, l1 = nL - 1;
    if (o.s.xmin_excluded && iE == 0) l0 = 1;
    if (o.s.xmax_excluded && iE == nE - 1) l1 = nL - 2;
    int m = l1 - l0 + 1;
    for (int a = 0; a < m; a++) {
      cd acc = 0.0;
      for (int b = 0; b < m; b++) acc += wr[a + l0] * o.Dref[(a + l0) + (size_t)nL * (b + l0)] * f[iS + b];
      res[iS + a] += acc;
    }
  }
  for (int i = 0; i < o.nG; i++) res[i] /= o.w[i];
}

// DerivativeFinDiff_Do2ndDerivativeZeroEnds (src/Utils/M_Utils_DerivativeFinDiff.f90:179-198)
static void findiff_second_derivative_zero_ends(const Oracle& o, const cd* f, cd* res) {
  const double c0 = -205.0 / 72.0, c1 = 8.0 / 5.0, c2 = -1.0 / 5.0, c3 = 8.0 / 315.0, c4 = -1.0 / 560.0;
  int n = o.nG;
  double dxSq = o.dxConst * o.dxConst;
  auto F = [&](int i) -> cd { return (i >= 0 && i < n) ? f[i] : cd(0.0); };
  for (int i = 0; i < n; i++) {
    cd v = c0 * f[i] + c1 * (F(i + 1) + F(i - 1)) + c2 * (F(i + 2) + F(i - 2)) + c3 * (F(i + 3) + F(i - 3)) +
           c4 * (F(i + 4) + F(i - 4));
    res[i] = v / dxSq;
  }
}

// SysKinetic_MultiplyWithKineticOp: FinDiff
// (src/SysKinetic/Linear/Laplacian/FinDiff/S_SysKinetic_Linear_Laplacian_FinDiff.f90:64-94)
// or the 1D FEDVR extension (pattern of S_SysKinetic_Ylm_Laplacian_Fedvr.f90:49-95 without r-transform).
static void kinetic_apply(const Oracle& o, const cd* orb, cd* dOrb, int bt) {
  std::vector<cd> d2(o.nG);
  if (o.s.grid_kind == 0) findiff_second_derivative_zero_ends(o, orb, d2.data());
  else fedvr_second_derivative(o, orb, d2.data());
  for (int i = 0; i < o.nG; i++) dOrb[i] = -0.5 * d2[i] / o.s.mass[bt];
}

// Laser field amplitude (pattern of S_SysPotential_Ylm_CoulombLaser.f90:60-83)
static double field_amplitude(const Oracle& o, double t) {
  const orc_spec& s = o.s;
  if (s.laser_kind == 1) {
    if (s.omega <= 0.0) return 0.0;
    double duration = 2.0 * PI * s.n_cycles / s.omega;
    double tRel = t - s.t_start;
    if (tRel < 0.0 || tRel > duration) return 0.0;
    double env = std::sin(PI * tRel / duration);
    env = env * env;
    double carrier = std::cos(s.omega * (tRel - 0.5 * duration) + s.cep);
    return s.E0 * env * carrier;
  } else if (s.laser_kind == 2) {
    double u = (t - s.sample_t0) / s.sample_dt;
    long n = (long)std::floor(u + 1e-9);
    if (n < 0 || n >= s.n_samples) return 0.0;
    return s.field_samples[n];
  }
  return 0.0;
}

// FillExternalPotential (src/SysPotential/Linear/SoftYukawa/StdImpl/S_SysPotential_Linear_SoftYukawa_StdImpl.f90:82-113)
static void setup_potential(Oracle& o) {
  o.V0.assign(o.nG, 0.0);
  for (int n = 0; n < o.s.n_nuclei; n++)
    for (int i = 0; i < o.nG; i++) {
      double d = std::fabs(o.x[i] - o.s.nuc_pos[n]);
      o.V0[i] -= o.s.nuc_charge[n] * std::exp(-d * o.s.nuc_damp[n]) /
                 (std::sqrt(d * d + o.s.nuc_s1[n] * o.s.nuc_s1[n]) + o.s.nuc_s2[n]);
    }
}

// SysInteraction_Linear_SoftYukawa_Interaction (S_SysInteraction_Linear_SoftYukawa.f90:67-73)
static double int_kernel(const Oracle& o, double d) {
  return o.s.int_strength * std::exp(-d * o.s.int_damp) / (std::sqrt(d * d + o.s.int_s1 * o.s.int_s1) + o.s.int_s2);
}

static void setup_interaction(Oracle& o) {
  if (!o.s.has_interaction) return;
  if (o.s.int_kind == 0) {
    // ConvolutionIntegral_CreateCtx (src/Utils/M_Utils_ConvolutionIntegral.f90:38-57), dx = x(2)-x(1)
    double dx = o.x[1] - o.x[0];
    o.kernelVals.resize(o.nG);
    for (int k = 0; k < o.nG; k++) o.kernelVals[k] = int_kernel(o, (double)k * dx);
  } else {
    o.Vdense.resize((size_t)o.nG * o.nG);
    for (int j = 0; j < o.nG; j++)
      for (int i = 0; i < o.nG; i++) o.Vdense[i + (size_t)o.nG * j] = int_kernel(o, std::fabs(o.x[i] - o.x[j]));
  }
}

// FillInteractionSrc (src/SysInteraction/Linear/S_SysInteraction_Linear.f90:57-72)
// + FillInteractionPotential: ConvolutionIntegral_Apply (M_Utils_ConvolutionIntegral.f90:71-107)
static void interaction_potential(const Oracle& o, const cd* orbConj, const cd* orb, cd* pot) {
  int n = o.nG;
  std::vector<cd> src(n);
  for (int i = 0; i < n; i++) src[i] = std::conj(orbConj[i]) * orb[i] * o.w[i];
  if (o.s.int_kind == 0) {
    for (int i = 0; i < n; i++) {
      cd acc = 0.0;
      for (int j = 0; j < n; j++) acc += o.kernelVals[std::abs(i - j)] * src[j];
      pot[i] = acc;
    }
  } else {
    for (int i = 0; i < n; i++) {
      cd acc = 0.0;
      for (int j = 0; j < n; j++) acc += o.Vdense[i + (size_t)n * j] * src[j];
      pot[i] = acc;
    }
  }
}

// ---------------------------------------------------------------------------
// Method_Mb_OrbBased helpers (src/Method/Mb/OrbBased/S_Method_Mb_OrbBased.f90)
// ---------------------------------------------------------------------------
static inline cd grid_inner(const Oracle& o, const cd* a, const cd* b) {  // S_Grid_Linear.f90:53-61
  cd r = 0.0;
  for (int i = 0; i < o.nG; i++) r += std::conj(a[i]) * b[i] * o.w[i];
  return r;
}

static inline int bt_of(const Oracle& o, int i) { return o.btOfOrb[i]; }

// ApplyKineticOp :332-375
static void apply_kinetic_op(const Oracle& o, cd* dOrbs, const cd* orbs, double t) {
  (void)t;
  int nG = o.nG;
#pragma omp parallel for schedule(static)
  for (int i1 = 0; i1 < o.nOS; i1++) {
    std::vector<cd> tmp(nG);
    kinetic_apply(o, orbs + (size_t)nG * i1, tmp.data(), bt_of(o, i1));
    for (int g = 0; g < nG; g++) dOrbs[g + (size_t)nG * i1] += tmp[g];
  }
}

// ApplyPotentialOp :425-488 (body-type independent soft-Yukawa + length-gauge E(t) x)
static void apply_potential_op(const Oracle& o, cd* dOrbs, const cd* orbs, double t) {
  int nG = o.nG;
  double E = field_amplitude(o, t);
  std::vector<cd> pot(nG);
  for (int g = 0; g < nG; g++) pot[g] = o.V0[g] + E * o.x[g];
#pragma omp parallel for schedule(static)
  for (int i1 = 0; i1 < o.nOS; i1++)
    for (int g = 0; g < nG; g++) dOrbs[g + (size_t)nG * i1] += pot[g] * orbs[g + (size_t)nG * i1];
}

// ApplySingleBodyOp :976-1034
static void apply_single_body_op(const Oracle& o, cd* dOrbs, const cd* orbs, double t, cd* h1 /*nO x nO or null*/) {
  apply_kinetic_op(o, dOrbs, orbs, t);
  if (o.s.n_nuclei > 0 || o.s.laser_kind != 0) apply_potential_op(o, dOrbs, orbs, t);
  if (h1) {
    int nO = o.nO, nOS = o.nOS, nG = o.nG;
    for (size_t k = 0; k < (size_t)nO * nO; k++) h1[k] = 0.0;
    for (int j1 = 0; j1 < nOS; j1++)
      for (int i1 = 0; i1 < nOS; i1++) {
        if (bt_of(o, i1) != bt_of(o, j1)) continue;
        h1[i1 + (size_t)nO * j1] = grid_inner(o, orbs + (size_t)nG * i1, dOrbs + (size_t)nG * j1);
      }
    if (o.s.restricted)
      for (int j = 0; j < nOS; j++)
        for (int i = 0; i < nOS; i++) h1[(nOS + i) + (size_t)nO * (nOS + j)] = h1[i + (size_t)nO * j];
  }
}

// FillH1 :164-224
static void fill_h1(const Oracle& o, cd* h1, const cd* orbs, double t) {
  std::vector<cd> tmp((size_t)o.nG * o.nOS, 0.0);
  apply_single_body_op(o, tmp.data(), orbs, t, h1);
}

// ApplyInteractionOp :491-542 with MultiplyPotentialOnOrbRange :545-572 (body-type independent)
// ApplyInteractionOpPair :575-644 uses the conjugate symmetry for the swapped pair.
static void interaction_apply_pair(const Oracle& o, cd* outA, cd* outB, const cd* orbs, int i2, int j2) {
  int nG = o.nG;
  std::vector<cd> pot(nG);
  interaction_potential(o, orbs + (size_t)nG * i2, orbs + (size_t)nG * j2, pot.data());
  for (int i = 0; i < o.nOS; i++)
    for (int g = 0; g < nG; g++) {
      outA[g + (size_t)nG * i] += pot[g] * orbs[g + (size_t)nG * i];
      if (outB) outB[g + (size_t)nG * i] += std::conj(pot[g]) * orbs[g + (size_t)nG * i];
    }
}

static void duplicate_h2_spin_blocks(const Oracle& o, cd* h2) {
  int nO = o.nO, nOS = o.nOS;
  auto H = [&](int a, int b, int c, int d) -> cd& { return h2[a + (size_t)nO * (b + (size_t)nO * (c + (size_t)nO * d))]; };
  for (int d = 0; d < nOS; d++)
    for (int c = 0; c < nOS; c++)
      for (int b = 0; b < nOS; b++)
        for (int a = 0; a < nOS; a++) {
          cd v = H(a, b, c, d);
          H(nOS + a, b, nOS + c, d) = v;
          H(a, nOS + b, c, nOS + d) = v;
          H(nOS + a, nOS + b, nOS + c, nOS + d) = v;
        }
}

// FillH2 :227-293, FillH2Block :296-329
static void fill_h2(const Oracle& o, cd* h2, const cd* orbs, double t) {
  (void)t;
  int nO = o.nO, nOS = o.nOS, nG = o.nG;
  for (size_t k = 0; k < (size_t)nO * nO * nO * nO; k++) h2[k] = 0.0;
  if (!o.s.has_interaction) return;
  std::vector<cd> A((size_t)nG * nOS), B((size_t)nG * nOS);
  auto H = [&](int a, int b, int c, int d) -> cd& { return h2[a + (size_t)nO * (b + (size_t)nO * (c + (size_t)nO * d))]; };
  auto block = [&](const std::vector<cd>& tmp, int i2, int j2) {
    for (int j1 = 0; j1 < nOS; j1++)
      for (int i1 = 0; i1 < nOS; i1++) {
        if (bt_of(o, i1) != bt_of(o, j1)) continue;
        H(i1, i2, j1, j2) = 0.5 * grid_inner(o, orbs + (size_t)nG * i1, tmp.data() + (size_t)nG * j1);
      }
  };
  for (int j2 = 0; j2 < nOS; j2++)
    for (int i2 = j2; i2 < nOS; i2++) {
      if (bt_of(o, i2) != bt_of(o, j2)) continue;
      std::fill(A.begin(), A.end(), cd(0.0));
      if (i2 == j2) {
        interaction_apply_pair(o, A.data(), nullptr, orbs, i2, j2);
        block(A, i2, j2);
      } else {
        std::fill(B.begin(), B.end(), cd(0.0));
        interaction_apply_pair(o, A.data(), B.data(), orbs, i2, j2);
        block(A, i2, j2);
        block(B, j2, i2);
      }
    }
  if (o.s.restricted) duplicate_h2_spin_blocks(o, h2);
}

// ApplyCorrelationOp :647-805, AccumulateCorrelation :808-838, FillH2CorrelationBlock :841-872
static void apply_correlation_op(const Oracle& o, cd* dOrbs, const cd* orbs, const cd* rdm1, const cd* rdm2, double t,
                                 cd* h2 /* or null */) {
  (void)t;
  int nO = o.nO, nOS = o.nOS, nG = o.nG;
  if (h2)
    for (size_t k = 0; k < (size_t)nO * nO * nO * nO; k++) h2[k] = 0.0;
  size_t M = nOS;
  std::vector<cd> r1(M * M), r2(M * M * M * M);
  auto R1 = [&](int a, int b) { return rdm1[a + (size_t)nO * b]; };
  auto R2 = [&](int a, int b, int c, int d) { return rdm2[a + (size_t)nO * (b + (size_t)nO * (c + (size_t)nO * d))]; };
  if (nO == nOS) {
    for (size_t b = 0; b < M; b++)
      for (size_t a = 0; a < M; a++) r1[a + M * b] = R1(a, b);
    for (size_t d = 0; d < M; d++)
      for (size_t c = 0; c < M; c++)
        for (size_t b = 0; b < M; b++)
          for (size_t a = 0; a < M; a++) r2[a + M * (b + M * (c + M * d))] = R2(a, b, c, d);
  } else if (nO == 2 * nOS) {
    int S = nOS;
    for (size_t b = 0; b < M; b++)
      for (size_t a = 0; a < M; a++) r1[a + M * b] = R1(a, b) + R1(S + a, S + b);
    for (size_t d = 0; d < M; d++)
      for (size_t c = 0; c < M; c++)
        for (size_t b = 0; b < M; b++)
          for (size_t a = 0; a < M; a++)
            r2[a + M * (b + M * (c + M * d))] =
                R2(a, b, c, d) + R2(S + a, b, S + c, d) + R2(a, S + b, c, S + d) + R2(S + a, S + b, S + c, S + d);
  }
  // RdmDiagonalize_Rdm1 (src/Utils/M_Utils_RdmDiagonalize.f90:17-36)
  std::vector<double> occ(M);
  std::vector<cd> U(M * M);
  jacobi_herm((int)M, r1.data(), occ.data(), U.data());
  double reg = o.s.reg_eps;
  std::vector<cd> Mreg(M * M);
  for (size_t j1 = 0; j1 < M; j1++)
    for (size_t k1 = 0; k1 < M; k1++) {
      cd acc = 0.0;
      for (size_t j = 0; j < M; j++) acc += U[k1 + M * j] * (occ[j] / (occ[j] * occ[j] + reg)) * std::conj(U[j1 + M * j]);
      Mreg[k1 + M * j1] = acc;
    }
  std::vector<cd> R(M * M * M * M, 0.0);
  for (size_t j1 = 0; j1 < M; j1++)
    for (size_t k1 = 0; k1 < M; k1++) {
      cd m = Mreg[k1 + M * j1];
      for (size_t d = 0; d < M; d++)
        for (size_t b = 0; b < M; b++)
          for (size_t a = 0; a < M; a++) R[a + M * (b + M * (j1 + M * d))] += r2[a + M * (b + M * (k1 + M * d))] * m;
    }
  auto accumulate = [&](const std::vector<cd>& tmp, int k2, int l2) {
    for (int j1 = 0; j1 < nOS; j1++)
      for (int k1 = 0; k1 < nOS; k1++) {
        if (bt_of(o, j1) != bt_of(o, k1)) continue;
        cd r = R[k1 + M * (k2 + M * (j1 + M * l2))];
        for (int g = 0; g < nG; g++) dOrbs[g + (size_t)nG * j1] += tmp[g + (size_t)nG * k1] * r;
      }
  };
  auto h2block = [&](const std::vector<cd>& tmp, int k2, int l2) {
    for (int j1 = 0; j1 < nOS; j1++)
      for (int i1 = 0; i1 < nOS; i1++) {
        if (bt_of(o, i1) != bt_of(o, j1)) continue;
        h2[i1 + (size_t)nO * (l2 + (size_t)nO * (j1 + (size_t)nO * k2))] =
            0.5 * grid_inner(o, orbs + (size_t)nG * i1, tmp.data() + (size_t)nG * j1);
      }
  };
  if (o.s.has_interaction) {
    std::vector<cd> A((size_t)nG * nOS), B((size_t)nG * nOS);
    for (int l2 = 0; l2 < nOS; l2++)
      for (int k2 = l2; k2 < nOS; k2++) {
        if (bt_of(o, l2) != bt_of(o, k2)) continue;
        std::fill(A.begin(), A.end(), cd(0.0));
        if (k2 == l2) {
          interaction_apply_pair(o, A.data(), nullptr, orbs, l2, k2);
          accumulate(A, k2, l2);
          if (h2) h2block(A, k2, l2);
        } else {
          std::fill(B.begin(), B.end(), cd(0.0));
          interaction_apply_pair(o, A.data(), B.data(), orbs, l2, k2);
          accumulate(A, k2, l2);
          accumulate(B, l2, k2);
          if (h2) {
            h2block(A, k2, l2);
            h2block(B, l2, k2);
          }
        }
      }
  }
  if (h2 && o.s.restricted) duplicate_h2_spin_blocks(o, h2);
}

// ---------------------------------------------------------------------------
// Coeffs_Generic (src/Coeffs/Generic/S_Coeffs_Generic.f90)
// ---------------------------------------------------------------------------
static void configurations_from_index(const Oracle& o, int iCoeff /*1-based*/, int* conf) {  // :625-639
  int iTmp = iCoeff - 1;
  for (int b = 0; b < o.nBt; b++) {
    conf[b] = iTmp % o.cl[b].nConf + 1;
    iTmp /= o.cl[b].nConf;
  }
}

static void fill_h1_lin(const Oracle& o, const cd* h1, std::vector<cd>& h1Lin) {  // :440-464
  int nO = o.nO;
  h1Lin.assign((size_t)nO * nO + 1, 0.0);
  for (int j1 = 1; j1 <= nO; j1++)
    for (int i1 = 1; i1 <= nO; i1++) {
      int oc = (i1 - 1) * nO + j1;
      h1Lin[oc] = h1[(i1 - 1) + (size_t)nO * (j1 - 1)];
    }
}

static void fill_h2_lin(const Oracle& o, const cd* h2, std::vector<cd>& h2Lin) {  // :478-542
  int nO = o.nO;
  h2Lin.assign((size_t)nO * nO * nO * nO + 1, 0.0);
  auto H = [&](int a, int b, int c, int d) {
    return h2[(a - 1) + (size_t)nO * ((b - 1) + (size_t)nO * ((c - 1) + (size_t)nO * (d - 1)))];
  };
  for (int j2 = 1; j2 <= nO; j2++)
    for (int j1 = 1; j1 <= j2; j1++)
      for (int i2 = 1; i2 <= nO; i2++)
        for (int i1 = 1; i1 <= i2; i1++) {
          int b_j2 = o.btOfOrb[j2 - 1], b_j1 = o.btOfOrb[j1 - 1], b_i2 = o.btOfOrb[i2 - 1], b_i1 = o.btOfOrb[i1 - 1];
          if (b_i1 == b_i2 && b_j1 != b_j2) continue;
          if (b_i1 != b_i2 && b_j1 == b_j2) continue;
          int oc = 1;
          oc = (oc - 1) * nO + i1;
          oc = (oc - 1) * nO + j1;
          oc = (oc - 1) * nO + i2;
          oc = (oc - 1) * nO + j2;
          cd v = (H(i1, i2, j1, j2) - H(i1, i2, j2, j1) - H(i2, i1, j1, j2) + H(i2, i1, j2, j1));
          if (i1 == i2) v = 0.0;
          if (j1 == j2) v = 0.0;
          h2Lin[oc] = v;
        }
}

static void fill_rdm1_from_lin(const Oracle& o, const std::vector<cd>& lin, cd* rdm1) {  // :325-349
  int nO = o.nO;
  for (int j1 = 1; j1 <= nO; j1++)
    for (int i1 = 1; i1 <= nO; i1++) rdm1[(i1 - 1) + (size_t)nO * (j1 - 1)] = lin[(i1 - 1) * nO + j1];
}

static void fill_rdm2_from_lin(const Oracle& o, const std::vector<cd>& lin, cd* rdm2) {  // :362-434
  int nO = o.nO;
  size_t n4 = (size_t)nO * nO * nO * nO;
  for (size_t k = 0; k < n4; k++) rdm2[k] = 0.0;
  auto R = [&](int a, int b, int c, int d) -> cd& {
    return rdm2[(a - 1) + (size_t)nO * ((b - 1) + (size_t)nO * ((c - 1) + (size_t)nO * (d - 1)))];
  };
  for (int j2 = 1; j2 <= nO; j2++)
    for (int j1 = 1; j1 <= j2; j1++)
      for (int i2 = 1; i2 <= nO; i2++)
        for (int i1 = 1; i1 <= i2; i1++) {
          int b_j2 = o.btOfOrb[j2 - 1], b_j1 = o.btOfOrb[j1 - 1], b_i2 = o.btOfOrb[i2 - 1], b_i1 = o.btOfOrb[i1 - 1];
          if (b_i1 == b_i2 && b_j1 != b_j2) continue;
          if (b_i1 != b_i2 && b_j1 == b_j2) continue;
          int oc = 1;
          oc = (oc - 1) * nO + i1;
          oc = (oc - 1) * nO + j1;
          oc = (oc - 1) * nO + i2;
          oc = (oc - 1) * nO + j2;
          cd v = lin[oc];
          R(i1, i2, j1, j2) += v;
          R(i2, i1, j1, j2) -= v;
          R(i1, i2, j2, j1) -= v;
          R(i2, i1, j2, j1) += v;
        }
}

static int n_threads(const Oracle& o) {
#ifdef _OPENMP
  return o.s.n_threads > 0 ? o.s.n_threads : omp_get_max_threads();
#else
  (void)o;
  return 1;
#endif
}

// ApplyH1FillRdm1 :103-178
static void apply_h1_fill_rdm1(const Oracle& o, const cd* coeffs, cd* rdm1, cd* dCoeffs, const cd* h1) {
  int nO = o.nO, nT = n_threads(o);
  std::vector<cd> h1Lin;
  if (h1) fill_h1_lin(o, h1, h1Lin);
  std::vector<std::vector<cd>> part(nT);
#pragma omp parallel num_threads(nT)
  {
    int tid = 0;
#ifdef _OPENMP
    tid = omp_get_thread_num();
#endif
    std::vector<cd>& loc = part[tid];
    if (rdm1) loc.assign((size_t)nO * nO + 1, 0.0);
    int conf[8];
#pragma omp for schedule(static)
    for (int iCoeff = 1; iCoeff <= o.nC; iCoeff++) {
      int iTmp = 1;
      configurations_from_index(o, iCoeff, conf);
      for (int b = 0; b < o.nBt; b++) {
        const Excitations& e = o.cl[b].singles;
        int c = conf[b];
        for (int k = 0; k < e.nConnected[c - 1]; k++) {
          size_t at = (size_t)k + (size_t)e.maxConn * (c - 1);
          int oc = e.orbCode[at];
          double f = e.factor[at];
          int jC = e.excitedC[at];
          jC = (jC - c);
          jC = iCoeff + jC * iTmp;
          if (dCoeffs && h1) dCoeffs[iCoeff - 1] += f * h1Lin[oc] * coeffs[jC - 1];
          if (rdm1) loc[oc] += f * std::conj(coeffs[jC - 1]) * coeffs[iCoeff - 1];
        }
        iTmp *= o.cl[b].nConf;
      }
    }
  }
  if (rdm1) {
    std::vector<cd> lin((size_t)nO * nO + 1, 0.0);
    for (int t = 0; t < nT; t++)
      if (!part[t].empty())
        for (size_t k = 0; k < lin.size(); k++) lin[k] += part[t][k];
    fill_rdm1_from_lin(o, lin, rdm1);
  }
}

// ApplyH2FillRdm2 :197-319
static void apply_h2_fill_rdm2(const Oracle& o, const cd* coeffs, cd* rdm2, cd* dCoeffs, const cd* h2,
                               const std::vector<cd>* h2LinCached = nullptr) {
  int nO = o.nO, nT = n_threads(o);
  size_t n4 = (size_t)nO * nO * nO * nO;
  std::vector<cd> h2LinOwn;
  if (h2 && !h2LinCached) fill_h2_lin(o, h2, h2LinOwn);
  const std::vector<cd>& h2Lin = h2LinCached ? *h2LinCached : h2LinOwn;
  std::vector<std::vector<cd>> part(nT);
#pragma omp parallel num_threads(nT)
  {
    int tid = 0;
#ifdef _OPENMP
    tid = omp_get_thread_num();
#endif
    std::vector<cd>& loc = part[tid];
    if (rdm2) loc.assign(n4 + 1, 0.0);
    int conf[8];
#pragma omp for schedule(static)
    for (int iCoeff = 1; iCoeff <= o.nC; iCoeff++) {
      int iTmp = 1;
      configurations_from_index(o, iCoeff, conf);
      cd dacc = 0.0;
      for (int b1 = 0; b1 < o.nBt; b1++) {
        int c1 = conf[b1];
        const Excitations& d = o.cl[b1].doubles;
        for (int k = 0; k < d.nConnected[c1 - 1]; k++) {
          size_t at = (size_t)k + (size_t)d.maxConn * (c1 - 1);
          int oc = d.orbCode[at];
          double f = d.factor[at];
          int jC = d.excitedC[at];
          jC = (jC - c1);
          jC = iCoeff + jC * iTmp;
          if (dCoeffs && h2) dacc += f * h2Lin[oc] * coeffs[jC - 1];
          if (rdm2) loc[oc] += f * std::conj(coeffs[jC - 1]) * coeffs[iCoeff - 1];
        }
        if (b1 == o.nBt - 1) continue;
        const Excitations& s1 = o.cl[b1].singles;
        for (int k1 = 0; k1 < s1.nConnected[c1 - 1]; k1++) {
          size_t at1 = (size_t)k1 + (size_t)s1.maxConn * (c1 - 1);
          int ocT = (s1.orbCode[at1] - 1) * nO * nO;
          double fT = s1.factor[at1];
          int jCT = s1.excitedC[at1];
          jCT = (jCT - c1);
          jCT = iCoeff + jCT * iTmp;
          int jTmp = iTmp * o.cl[b1].nConf;
          for (int b2 = b1 + 1; b2 < o.nBt; b2++) {
            int c2 = conf[b2];
            const Excitations& s2 = o.cl[b2].singles;
            for (int k2 = 0; k2 < s2.nConnected[c2 - 1]; k2++) {
              size_t at2 = (size_t)k2 + (size_t)s2.maxConn * (c2 - 1);
              int oc = ocT + s2.orbCode[at2];
              double f = fT * s2.factor[at2];
              int jC = s2.excitedC[at2];
              jC = (jC - c2);
              jC = jCT + jC * jTmp;
              if (dCoeffs && h2) dacc += f * h2Lin[oc] * coeffs[jC - 1];
              if (rdm2) loc[oc] += f * std::conj(coeffs[jC - 1]) * coeffs[iCoeff - 1];
            }
            jTmp *= o.cl[b2].nConf;
          }
        }
        iTmp *= o.cl[b1].nConf;
      }
      if (dCoeffs && h2) dCoeffs[iCoeff - 1] += dacc;
    }
  }
  if (rdm2) {
    std::vector<cd> lin(n4 + 1, 0.0);
    for (int t = 0; t < nT; t++)
      if (!part[t].empty())
        for (size_t k = 0; k < lin.size(); k++) lin[k] += part[t][k];
    fill_rdm2_from_lin(o, lin, rdm2);
  }
}

// Coeffs ProjectOnSubspace (src/Coeffs/S_Coeffs.f90:105-111)
static void coeffs_project(const Oracle& o, cd* dC, const cd* C) {
  cd ov = 0.0;
  for (int i = 0; i < o.nC; i++) ov += std::conj(C[i]) * dC[i];
  for (int i = 0; i < o.nC; i++) dC[i] -= ov * C[i];
}

// Grid_ProjectOnSubspace (src/Grid/S_Grid.f90:170-203) over columns [c0,c1)
static void grid_project(const Oracle& o, cd* dOrbs, const cd* orbs, int c0, int c1) {
  int nG = o.nG, n = c1 - c0;
  std::vector<cd> inp((size_t)n * n);
  for (int j = 0; j < n; j++)
    for (int i = 0; i < n; i++) inp[i + (size_t)n * j] = grid_inner(o, orbs + (size_t)nG * (c0 + i), dOrbs + (size_t)nG * (c0 + j));
  for (int j = 0; j < n; j++)
    for (int g = 0; g < nG; g++) {
      cd acc = 0.0;
      for (int i = 0; i < n; i++) acc += orbs[g + (size_t)nG * (c0 + i)] * inp[i + (size_t)n * j];
      dOrbs[g + (size_t)nG * (c0 + j)] -= acc;
    }
}

// Orbs_ProjectOnSubspace (src/Orbs/S_Orbs.f90:198-225)
static void orbs_project(const Oracle& o, cd* dOrbs, const cd* orbs) {
  if (o.s.restricted) { grid_project(o, dOrbs, orbs, 0, o.nOS); return; }
  for (int b = 0; b < o.nBt; b++) grid_project(o, dOrbs, orbs, o.orbStart[b], o.orbEnd[b] + 1);
}

// Grid_Orthonormalize (src/Grid/S_Grid.f90:120-151)
static int grid_orthonormalize(const Oracle& o, cd* f, int c0, int c1) {
  int nG = o.nG;
  for (int i1 = c0; i1 < c1; i1++) {
    for (int pass = 0; pass < 2; pass++)
      for (int j1 = c0; j1 < i1; j1++) {
        cd ov = grid_inner(o, f + (size_t)nG * j1, f + (size_t)nG * i1);
        for (int g = 0; g < nG; g++) f[g + (size_t)nG * i1] -= f[g + (size_t)nG * j1] * ov;
      }
    double nrm = grid_inner(o, f + (size_t)nG * i1, f + (size_t)nG * i1).real();
    if (!(nrm > 0.0)) return 1;
    double sq = std::sqrt(nrm);
    for (int g = 0; g < nG; g++) f[g + (size_t)nG * i1] /= sq;
  }
  return 0;
}

// Orbs_Orthonormalize (src/Orbs/S_Orbs.f90:145-173)
static int orbs_orthonormalize(const Oracle& o, cd* orbs) {
  if (o.s.restricted) return grid_orthonormalize(o, orbs, 0, o.nOS);
  for (int b = 0; b < o.nBt; b++)
    if (grid_orthonormalize(o, orbs, o.orbStart[b], o.orbEnd[b] + 1)) return 1;
  return 0;
}

// ---------------------------------------------------------------------------
// MCTDHX time derivatives (src/Method/Mb/OrbBased/Mctdhx/S_Method_Mb_OrbBased_Mctdhx.f90)
// which: 0 full (:101-149), 1 OrbsLin (:152-177), 2 CoeffsPlusOrbsNonLin (:180-226)
// TDCI (src/Method/Mb/OrbBased/Tdci/S_Method_Mb_OrbBased_Tdci.f90:75-107): which = 3
// ---------------------------------------------------------------------------
static void time_derivative(const Oracle& o, int which, cd* dState, const cd* state, double t) {
  int nC = o.nC, nO = o.nO;
  size_t nS = (size_t)nC + (size_t)o.nG * o.nOS;
  if (which == 3) {
    std::vector<cd> h1 = o.tdciH1;
    for (int i = 0; i < nC; i++) dState[i] = 0.0;
    // time-dependent one-body part is refreshed when a laser is present (Tdci:90-92)
    if (o.s.laser_kind != 0) fill_h1(o, h1.data(), o.tdciOrbs.data(), t);
    apply_h1_fill_rdm1(o, state, nullptr, dState, h1.data());
    // h2 is time independent: its folded form is computed once at set-up (same values as FillH2Lin per call)
    apply_h2_fill_rdm2(o, state, nullptr, dState, o.tdciH2.data(), &o.tdciH2Lin);
    for (int i = 0; i < nC; i++) dState[i] = -IU * dState[i];
    return;
  }
  for (size_t i = 0; i < nS; i++) dState[i] = 0.0;
  const cd* C = state;
  const cd* orbs = state + nC;
  cd* dC = dState;
  cd* dOrbs = dState + nC;
  if (which == 1) {
    apply_single_body_op(o, dOrbs, orbs, t, nullptr);
  } else {
    std::vector<cd> rdm1((size_t)nO * nO), rdm2((size_t)nO * nO * nO * nO), h1((size_t)nO * nO),
        h2((size_t)nO * nO * nO * nO);
    apply_h1_fill_rdm1(o, C, rdm1.data(), nullptr, nullptr);
    apply_h2_fill_rdm2(o, C, rdm2.data(), nullptr, nullptr);
    if (which == 0) apply_single_body_op(o, dOrbs, orbs, t, h1.data());
    else fill_h1(o, h1.data(), orbs, t);
    apply_correlation_op(o, dOrbs, orbs, rdm1.data(), rdm2.data(), t, h2.data());
    apply_h1_fill_rdm1(o, C, nullptr, dC, h1.data());
    apply_h2_fill_rdm2(o, C, nullptr, dC, h2.data());
    coeffs_project(o, dC, C);
    orbs_project(o, dOrbs, orbs);
  }
  for (size_t i = 0; i < nS; i++) dState[i] = -IU * dState[i];
}

// GetEnergy (S_Method_Mb_OrbBased.f90:132-161) + RdmObservables_Energy (src/Utils/M_Utils_RdmObservables.f90:17-52)
static double get_energy(const Oracle& o, const cd* state, double t) {
  int nO = o.nO, nC = o.nC;
  size_t n4 = (size_t)nO * nO * nO * nO;
  std::vector<cd> rdm1((size_t)nO * nO), rdm2(n4), h1((size_t)nO * nO), h2(n4);
  apply_h1_fill_rdm1(o, state, rdm1.data(), nullptr, nullptr);
  apply_h2_fill_rdm2(o, state, rdm2.data(), nullptr, nullptr);
  const cd* orbs = (o.s.method == 1) ? o.tdciOrbs.data() : state + nC;
  fill_h1(o, h1.data(), orbs, t);
  fill_h2(o, h2.data(), orbs, t);
  cd acc = 0.0;
  for (int k1 = 0; k1 < nO; k1++)
    for (int l1 = 0; l1 < nO; l1++) acc += h1[k1 + (size_t)nO * l1] * rdm1[l1 + (size_t)nO * k1];
  for (int k1 = 0; k1 < nO; k1++)
    for (int k2 = 0; k2 < nO; k2++)
      for (int l1 = 0; l1 < nO; l1++)
        for (int l2 = 0; l2 < nO; l2++)
          acc += h2[k1 + (size_t)nO * (k2 + (size_t)nO * (l1 + (size_t)nO * l2))] *
                 rdm2[l1 + (size_t)nO * (l2 + (size_t)nO * (k1 + (size_t)nO * k2))];
  return acc.real();
}

// ---------------------------------------------------------------------------
// Integrators
// ---------------------------------------------------------------------------
typedef void (*td_fn)(const Oracle&, int, cd*, const cd*, double);

static void deriv(const Oracle& o, int which, bool imag, cd* d, const cd* s, double t) {
  time_derivative(o, which, d, s, t);
  if (imag) {  // Actions_ImagTimeDerivative (src/Utils/M_Utils_Actions.f90:66-78)
    size_t nS = (o.s.method == 1) ? (size_t)o.nC : (size_t)o.nC + (size_t)o.nG * o.nOS;
    for (size_t i = 0; i < nS; i++) d[i] = -IU * d[i];
  }
}

static size_t state_size(const Oracle& o) {
  return (o.s.method == 1) ? (size_t)o.nC : (size_t)o.nC + (size_t)o.nG * o.nOS;
}

// RK4 (src/IntegratorList/Rk/O4Expl/S_IntegratorList_Rk_O4Expl.f90:90-141)
static void rk4(const Oracle& o, int which, bool imag, cd* state, double t0, double t1) {
  size_t nS = state_size(o);
  std::vector<cd> d(nS), inc(nS), tmp(nS);
  double dt = t1 - t0, dt2 = dt / 2.0, dt3 = dt / 3.0, dt6 = dt / 6.0;
  deriv(o, which, imag, d.data(), state, t0);
  for (size_t i = 0; i < nS; i++) { inc[i] = d[i] * dt6; tmp[i] = state[i] + d[i] * dt2; }
  double tp = t0 + dt2;
  deriv(o, which, imag, d.data(), tmp.data(), tp);
  for (size_t i = 0; i < nS; i++) { inc[i] = inc[i] + d[i] * dt3; tmp[i] = state[i] + d[i] * dt2; }
  deriv(o, which, imag, d.data(), tmp.data(), tp);
  for (size_t i = 0; i < nS; i++) { inc[i] = inc[i] + d[i] * dt3; tmp[i] = state[i] + d[i] * dt; }
  tp = t0 + dt;
  deriv(o, which, imag, d.data(), tmp.data(), tp);
  for (size_t i = 0; i < nS; i++) inc[i] = inc[i] + d[i] * dt6;
  for (size_t i = 0; i < nS; i++) state[i] = state[i] + inc[i];
}

// Forward Euler (src/IntegratorList/Rk/O1Expl/S_IntegratorList_Rk_O1Expl.f90:50-72)
static void euler(const Oracle& o, int which, bool imag, cd* state, double t0, double t1) {
  size_t nS = state_size(o);
  std::vector<cd> d(nS);
  cd dt(t1 - t0, 0.0);
  deriv(o, which, imag, d.data(), state, t0);
  for (size_t i = 0; i < nS; i++) state[i] = state[i] + d[i] * dt;
}

struct SilParams {
  int krylovDim;
  double tol;
  int maxRestarts;
  const double* metric;  // null: Euclidean
};

// Short iterative Lanczos (src/IntegratorList/Sil/S_IntegratorList_Sil.f90:114-310)
static int sil(const Oracle& o, int which, cd* state, double t0, double t1, const SilParams& p, int* warnings) {
  const double zeroThreshold = 1.0e-14;
  if (std::fabs(t1 - t0) <= zeroThreshold) return 0;
  size_t nS = state_size(o);
  int maxDim = std::max(1, std::min(p.krylovDim, (int)nS));
  std::vector<cd> work(state, state + nS), trial(nS), basis(nS * maxDim), der(nS), w(nS);
  std::vector<cd> phi(maxDim);
  std::vector<double> alpha(maxDim), beta(maxDim);
  auto mdot = [&](const cd* a, const cd* b) {
    cd r = 0.0;
    if (p.metric)
      for (size_t i = 0; i < nS; i++) r += std::conj(a[i]) * p.metric[i] * b[i];
    else
      for (size_t i = 0; i < nS; i++) r += std::conj(a[i]) * b[i];
    return r;
  };
  auto expSub = [&](double dt, int m, double* errEst) {
    std::vector<double> T((size_t)m * m, 0.0), ev(m), U((size_t)m * m);
    for (int j = 0; j < m; j++) T[j + (size_t)m * j] = alpha[j];
    for (int j = 0; j < m - 1; j++) { T[j + (size_t)m * (j + 1)] = beta[j]; T[(j + 1) + (size_t)m * j] = beta[j]; }
    jacobi_sym(m, T.data(), ev.data(), U.data());
    for (int i = 0; i < m; i++) {
      cd acc = 0.0;
      for (int j = 0; j < m; j++) acc += U[i + (size_t)m * j] * (U[0 + (size_t)m * j] * std::exp(-IU * dt * ev[j]));
      phi[i] = acc;
    }
    *errEst = beta[m - 1] * std::abs(phi[m - 1]);
  };
  auto lanczos = [&](double tBase, double dt, double* errEst, bool* converged) {
    double nrm = std::sqrt(mdot(work.data(), work.data()).real());
    if (nrm <= zeroThreshold) {
      trial = work;
      *errEst = 0.0;
      *converged = true;
      return;
    }
    for (size_t i = 0; i < nS; i++) basis[i] = work[i] / nrm;
    double tEval = tBase + 0.5 * dt;
    int mDim = maxDim;
    for (int j = 1; j <= maxDim; j++) {
      cd* v = &basis[nS * (j - 1)];
      time_derivative(o, which, der.data(), v, tEval);
      for (size_t i = 0; i < nS; i++) w[i] = IU * der[i];
      if (j > 1)
        for (size_t i = 0; i < nS; i++) w[i] -= beta[j - 2] * basis[nS * (j - 2) + i];
      alpha[j - 1] = mdot(v, w.data()).real();
      for (size_t i = 0; i < nS; i++) w[i] -= alpha[j - 1] * v[i];
      for (int k = 1; k <= j; k++) {
        cd c = mdot(&basis[nS * (k - 1)], w.data());
        for (size_t i = 0; i < nS; i++) w[i] -= c * basis[nS * (k - 1) + i];
      }
      beta[j - 1] = std::sqrt(mdot(w.data(), w.data()).real());
      bool breakdown = beta[j - 1] <= zeroThreshold;
      expSub(dt, j, errEst);
      if (breakdown) *errEst = 0.0;
      *converged = *errEst <= p.tol;
      if (*converged || breakdown || j == maxDim) {
        mDim = j;
        break;
      }
      for (size_t i = 0; i < nS; i++) basis[nS * j + i] = w[i] / beta[j - 1];
    }
    for (size_t i = 0; i < nS; i++) {
      cd acc = 0.0;
      for (int j = 0; j < mDim; j++) acc += basis[nS * j + i] * phi[j];
      trial[i] = nrm * acc;
    }
  };
  double tCur = t0, rem = t1 - t0;
  while (std::fabs(rem) > zeroThreshold) {
    double dtS = rem;
    int restarts = 0;
    double errEst = 0.0;
    bool conv = false;
    for (;;) {
      lanczos(tCur, dtS, &errEst, &conv);
      if (conv) break;
      if (std::fabs(dtS) <= zeroThreshold || restarts >= p.maxRestarts) break;
      dtS = 0.5 * dtS;
      restarts++;
    }
    if (!conv && warnings) (*warnings)++;
    work = trial;
    tCur = tCur + dtS;
    rem = rem - dtS;
  }
  for (size_t i = 0; i < nS; i++) state[i] = work[i];
  return 0;
}

// ---------------------------------------------------------------------------
// C API
// ---------------------------------------------------------------------------
extern "C" {

void* orc_create(const orc_spec* spec) {
  Oracle* o = new Oracle();
  o->s = *spec;
  if (o->s.n_samples > 0 && spec->field_samples) {
    double* cp = new double[o->s.n_samples];
    std::memcpy(cp, spec->field_samples, sizeof(double) * o->s.n_samples);
    o->s.field_samples = cp;
  } else {
    o->s.field_samples = nullptr;
  }
  setup_grid(*o);
  setup_potential(*o);
  setup_interaction(*o);
  o->nBt = spec->n_bt;
  o->nO = 0;
  for (int b = 0; b < o->nBt; b++) {
    o->orbStart.push_back(o->nO);
    for (int i = 0; i < spec->n_orbs[b]; i++) o->btOfOrb.push_back(b);
    o->nO += spec->n_orbs[b];
    o->orbEnd.push_back(o->nO - 1);
  }
  o->nOS = spec->restricted ? spec->n_orbs[0] : o->nO;
  for (int b = 0; b < o->nBt; b++) setup_configlist(*o, b);
  o->nC = 1;
  for (int b = 0; b < o->nBt; b++) o->nC *= o->cl[b].nConf;
  return o;
}

void orc_destroy(void* h) {
  Oracle* o = (Oracle*)h;
  delete[] o->s.field_samples;
  delete o;
}

const char* orc_error(void* h) { return ((Oracle*)h)->err.c_str(); }

void orc_sizes(void* h, int* out) {  // nG, nO, nOS, nC, nBt
  Oracle* o = (Oracle*)h;
  out[0] = o->nG; out[1] = o->nO; out[2] = o->nOS; out[3] = o->nC; out[4] = o->nBt;
}

void orc_grid(void* h, double* x, double* w) {
  Oracle* o = (Oracle*)h;
  std::memcpy(x, o->x.data(), sizeof(double) * o->nG);
  std::memcpy(w, o->w.data(), sizeof(double) * o->nG);
}

void orc_gll(int n, double a, double b, double* x, double* w) { gll(n, a, b, x, w); }

int orc_configlist_sizes(void* h, int bt, int* out) {  // nConf, maxSingles, maxDoubles
  Oracle* o = (Oracle*)h;
  if (bt < 0 || bt >= o->nBt) return 1;
  out[0] = o->cl[bt].nConf;
  out[1] = o->cl[bt].singles.maxConn;
  out[2] = o->cl[bt].doubles.maxConn;
  return 0;
}

// kind 0: singles, 1: doubles.  Arrays (maxConn, nConf) column-major.
int orc_configlist_tables(void* h, int bt, int kind, int64_t* codes, int* nConnected, int* excitedC, int* orbCode,
                          double* factor) {
  Oracle* o = (Oracle*)h;
  if (bt < 0 || bt >= o->nBt) return 1;
  const ConfigListE& c = o->cl[bt];
  const Excitations& e = kind == 0 ? c.singles : c.doubles;
  if (codes) std::memcpy(codes, c.code.data(), sizeof(int64_t) * c.nConf);
  std::memcpy(nConnected, e.nConnected.data(), sizeof(int) * c.nConf);
  std::memcpy(excitedC, e.excitedC.data(), sizeof(int) * e.excitedC.size());
  std::memcpy(orbCode, e.orbCode.data(), sizeof(int) * e.orbCode.size());
  std::memcpy(factor, e.factor.data(), sizeof(double) * e.factor.size());
  return 0;
}

void orc_kinetic_apply(void* h, const cd* orb, cd* out, int bt) { kinetic_apply(*(Oracle*)h, orb, out, bt); }
void orc_fedvr_second_derivative(void* h, const cd* f, cd* out) { fedvr_second_derivative(*(Oracle*)h, f, out); }
void orc_fedvr_first_derivative(void* h, const cd* f, cd* out) { fedvr_first_derivative(*(Oracle*)h, f, out); }
double orc_field(void* h, double t) { return field_amplitude(*(Oracle*)h, t); }
void orc_potential(void* h, double* v) { std::memcpy(v, ((Oracle*)h)->V0.data(), sizeof(double) * ((Oracle*)h)->nG); }

void orc_apply_single_body_op(void* h, cd* dOrbs, const cd* orbs, double t, cd* h1) {
  apply_single_body_op(*(Oracle*)h, dOrbs, orbs, t, h1);
}
void orc_fill_h1(void* h, cd* h1, const cd* orbs, double t) { fill_h1(*(Oracle*)h, h1, orbs, t); }
void orc_fill_h2(void* h, cd* h2, const cd* orbs, double t) { fill_h2(*(Oracle*)h, h2, orbs, t); }
void orc_interaction_potential(void* h, const cd* orbConj, const cd* orb, cd* pot) {
  interaction_potential(*(Oracle*)h, orbConj, orb, pot);
}
void orc_apply_correlation_op(void* h, cd* dOrbs, const cd* orbs, const cd* rdm1, const cd* rdm2, double t, cd* h2) {
  apply_correlation_op(*(Oracle*)h, dOrbs, orbs, rdm1, rdm2, t, h2);
}
void orc_apply_h1_fill_rdm1(void* h, const cd* C, cd* rdm1, cd* dC, const cd* h1) {
  apply_h1_fill_rdm1(*(Oracle*)h, C, rdm1, dC, h1);
}
void orc_apply_h2_fill_rdm2(void* h, const cd* C, cd* rdm2, cd* dC, const cd* h2) {
  apply_h2_fill_rdm2(*(Oracle*)h, C, rdm2, dC, h2);
}
void orc_project_coeffs(void* h, cd* dC, const cd* C) { coeffs_project(*(Oracle*)h, dC, C); }
void orc_project_orbs(void* h, cd* dOrbs, const cd* orbs) { orbs_project(*(Oracle*)h, dOrbs, orbs); }
int orc_orthonormalize(void* h, cd* orbs) { return orbs_orthonormalize(*(Oracle*)h, orbs); }
void orc_normalize(void* h, cd* C) {  // Coeffs_Normalize (src/Coeffs/S_Coeffs.f90:84-94)
  Oracle* o = (Oracle*)h;
  double s = 0.0;
  for (int i = 0; i < o->nC; i++) s += std::norm(C[i]);
  double nrm = std::sqrt(s);
  for (int i = 0; i < o->nC; i++) C[i] /= nrm;
}
void orc_time_derivative(void* h, int which, cd* dState, const cd* state, double t) {
  time_derivative(*(Oracle*)h, which, dState, state, t);
}
double orc_energy(void* h, const cd* state, double t) { return get_energy(*(Oracle*)h, state, t); }

void orc_eig_herm(int n, const cd* A, double* ev, cd* U) { jacobi_herm(n, A, ev, U); }
void orc_eig_sym(int n, const double* A, double* ev, double* U) { jacobi_sym(n, A, ev, U); }

// TDCI setup (Tdci Setup :40-72): static orbitals and their h1/h2
void orc_tdci_set_orbitals(void* h, const cd* orbs) {
  Oracle* o = (Oracle*)h;
  size_t n = (size_t)o->nG * o->nOS;
  o->tdciOrbs.assign(orbs, orbs + n);
  o->tdciH1.assign((size_t)o->nO * o->nO, 0.0);
  o->tdciH2.assign((size_t)o->nO * o->nO * o->nO * o->nO, 0.0);
  fill_h1(*o, o->tdciH1.data(), o->tdciOrbs.data(), 0.0);
  fill_h2(*o, o->tdciH2.data(), o->tdciOrbs.data(), 0.0);
  fill_h2_lin(*o, o->tdciH2.data(), o->tdciH2Lin);
}

// which: integrator target derivative; integrator: 0 euler, 1 rk4; imag: imaginary time
void orc_integrate_rk(void* h, int integrator, int which, int imag, cd* state, double t0, double t1) {
  Oracle* o = (Oracle*)h;
  if (integrator == 0) euler(*o, which, imag != 0, state, t0, t1);
  else rk4(*o, which, imag != 0, state, t0, t1);
}

int orc_integrate_sil(void* h, int which, cd* state, double t0, double t1, int krylovDim, double tol, int maxRestarts,
                      const double* metric) {
  Oracle* o = (Oracle*)h;
  SilParams p{krylovDim, tol, maxRestarts, metric};
  int warn = 0;
  sil(*o, which, state, t0, t1, p, &warn);
  return warn;
}

// Strang split (src/Propagator/SplitStep/Order2/S_Propagator_SplitStep_Order2.f90:52-77):
// A = SIL on OrbsLin (or RK4 if krylovDim <= 0), B = RK4 on CoeffsPlusOrbsNonLin.
int orc_propagate_split2(void* h, cd* state, double t0, double t1, int krylovDim, double tol, int maxRestarts,
                         const double* metric) {
  Oracle* o = (Oracle*)h;
  double dt = t1 - t0, time1 = t0, time2 = time1 + 0.5 * dt;
  int warn = 0;
  SilParams p{krylovDim, tol, maxRestarts, metric};
  if (krylovDim > 0) sil(*o, 1, state, time1, time1 + 0.5 * dt, p, &warn);
  else rk4(*o, 1, false, state, time1, time1 + 0.5 * dt);
  rk4(*o, 2, false, state, time1, time1 + 1.0 * dt);
  if (krylovDim > 0) sil(*o, 1, state, time2, time2 + 0.5 * dt, p, &warn);
  else rk4(*o, 1, false, state, time2, time2 + 0.5 * dt);
  return warn;
}

// Imaginary-time relaxation driver, as in
// test/simulationTests/He1d/T_He1d_04_ImagTimePropagationMctdhx.f90:82-99:
// Euler on the imaginary-time derivative, then Coeffs_Normalize and
// Orbs_Orthonormalize after every step; stop when |dE| <= convThresh.
double orc_relax(void* h, cd* state, double dt, int nInner, double convThresh, int maxOuter, int* nOuterOut) {
  Oracle* o = (Oracle*)h;
  double eNew = 0.0, eOld = 0.0, conv = 1.0, time = 0.0;
  int outer = 0;
  while (std::fabs(conv) > convThresh && outer < maxOuter) {
    outer++;
    for (int k = 0; k < nInner; k++) {
      euler(*o, 0, true, state, time, time + dt);
      time = time + dt;
      orc_normalize(h, state);
      orbs_orthonormalize(*o, state + o->nC);
    }
    eOld = eNew;
    eNew = get_energy(*o, state, time);
    conv = eNew - eOld;
  }
  if (nOuterOut) *nOuterOut = outer;
  return eNew;
}

}  // extern "C"
