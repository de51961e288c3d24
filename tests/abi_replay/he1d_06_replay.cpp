// he1d_06_replay.cpp -- a host program that drives the C ABI (include/cody_gpu.h)
// in the call order of the reference's He1d chain, the way a Fortran host
// bound through ISO_C_BINDING would:
//
//   T_He1d_04_ImagTimePropagationMctdhx.f90:46-99   Fabricate + Setup (one context),
//       harmonic initial orbitals (OrbsInit harmonic), unary coefficients,
//       imaginary-time relaxation (Euler + Coeffs_Normalize + Orbs_Orthonormalize
//       until |dE| <= 1e-12), Orbs_Save / Coeffs_Save of the result;
//   T_He1d_06_TimePropagationMctdhxSil.f90:46-140  a new context that loads the
//       saved orbitals and coefficients (orbsInit.load, coeffsInit.load),
//       start energy and norm, then the output loop: nTimeSteps = 2 split steps
//       (SIL krylovDim 24, tolerance 1e-12, maxRestarts 8 on OrbsLin; RK4 on
//       NonLin) of outputStep / 2 until endTime = 1e-3, GetEnergy after each
//       output step; the checks of :130-140.
//
// Usage: he1d_06_replay <scratch dir> <golden E_He1d_04> <golden E_He1d_05/06>
// Exit status 0 when every check passes.
#include <cstddef>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "cody_gpu.h"

static int check(int rc, const cgpu_ctx* c, const char* what) {
  if (rc != CGPU_OK) {
    std::fprintf(stderr, "%s failed (%d): %s\n", what, rc, c ? cgpu_last_error(c) : cgpu_last_global_error());
    std::exit(2);
  }
  return rc;
}

// He1d JSON: 21-point grid on [-20, 20], V = -2 / (|x| + 1), W = 1 / (|x - x'| + 1),
// two body types of one fermion, 4 + 4 orbitals, unrestricted.
static cgpu_desc he1d_desc() {
  cgpu_desc d = {};
  d.grid_kind = CGPU_GRID_CONST;
  d.xmin = -20.0;
  d.xmax = 20.0;
  d.n_points = 21;
  d.n_body_types = 2;
  d.n_bodies[0] = d.n_bodies[1] = 1;
  d.n_orbs[0] = d.n_orbs[1] = 4;
  d.body_mass[0] = d.body_mass[1] = 1.0;
  d.restricted = 0;
  d.regularization = 1e-10;
  d.n_nuclei = 1;
  d.nuc_position[0] = 0.0;
  d.nuc_charge[0] = 2.0;
  d.nuc_softening1[0] = 0.0;
  d.nuc_softening2[0] = 1.0;
  d.has_interaction = 1;
  d.int_strength = 1.0;
  d.int_softening1 = 0.0;
  d.int_softening2 = 1.0;
  d.int_kind = CGPU_INT_TOEPLITZ;
  d.laser_kind = CGPU_LASER_NONE;
  d.method = CGPU_METHOD_MCTDHX;
  d.precision = CGPU_PREC_FP64;
  d.max_krylov = 24;
  return d;
}

static double norm(const std::vector<cgpu_complex>& s) {
  double a = 0.0;
  for (const cgpu_complex& z : s) a += z.re * z.re + z.im * z.im;
  return std::sqrt(a);
}

int main(int argc, char** argv) {
  if (argc != 4) {
    std::fprintf(stderr, "usage: %s <scratch dir> <E_He1d_04> <E_He1d_05/06>\n", argv[0]);
    return 2;
  }
  const char* dir = argv[1];
  const double g04 = std::atof(argv[2]), g06 = std::atof(argv[3]);
  int fails = 0;

  // ---- T_He1d_04: Fabricate + Setup, harmonic start, relaxation, save -----
  cgpu_desc d = he1d_desc();
  cgpu_ctx* c = nullptr;
  check(cgpu_ctx_create(&d, &c), nullptr, "cgpu_ctx_create");
  int sz[6];
  check(cgpu_sizes(c, sz), c, "cgpu_sizes");
  const int nG = sz[0], nOS = sz[2], nC = sz[3], nS = sz[5];
  std::vector<double> x(nG), w(nG);
  check(cgpu_grid(c, x.data(), w.data()), c, "cgpu_grid");
  // OrbsInit harmonic (src/OrbsInit/Linear/Harmonic/S_OrbsInit_Linear_Harmonic.f90:52-80):
  // H_n(xi) exp(-xi^2) per body type, n = 0..3
  std::vector<cgpu_complex> orbs((size_t)nG * nOS);
  for (int o = 0; o < nOS; o++) {
    const int n = o % 4;
    for (int g = 0; g < nG; g++) {
      const double xi = x[g];
      double h0 = 1.0, h1 = 2.0 * xi;
      double hn = n == 0 ? h0 : h1;
      for (int k = 1; k < n; k++) {
        const double h2 = 2.0 * xi * h1 - 2.0 * k * h0;
        h0 = h1;
        h1 = h2;
        hn = h2;
      }
      orbs[(size_t)o * nG + g] = {hn * std::exp(-xi * xi), 0.0};
    }
  }
  check(cgpu_orthonormalize_orbs(c, orbs.data()), c, "cgpu_orthonormalize_orbs");
  std::vector<cgpu_complex> state(nS, cgpu_complex{0.0, 0.0});
  state[0] = {1.0, 0.0};  // CoeffsInit unary
  for (size_t k = 0; k < orbs.size(); k++) state[nC + k] = orbs[k];
  double e04 = 0.0;
  int rounds = 0;
  check(cgpu_relax(c, state.data(), 0.01, 10, 1e-12, 1000, &e04, &rounds), c, "cgpu_relax");
  check(cgpu_state_upload(c, state.data()), c, "cgpu_state_upload");
  check(cgpu_save_restart(c, dir, 0), c, "cgpu_save_restart");
  std::printf("He1d_04: relaxed energy %.16f after %d rounds (golden %.16f)\n", e04, rounds, g04);
  if (!(std::fabs(e04 - g04) < 1e-7)) fails++;
  check(cgpu_ctx_destroy(c), nullptr, "cgpu_ctx_destroy");

  // ---- T_He1d_06: a new run that loads the saved state ---------------------
  check(cgpu_ctx_create(&d, &c), nullptr, "cgpu_ctx_create");
  check(cgpu_load_restart(c, dir), c, "cgpu_load_restart");
  check(cgpu_state_download(c, state.data()), c, "cgpu_state_download");
  const double startTime = 0.0, endTime = 0.001, outputStep = 0.00002;
  const int nTimeSteps = 2;
  double startEnergy = 0.0;
  check(cgpu_energy(c, state.data(), startTime, &startEnergy), c, "cgpu_energy");
  const double startNorm = norm(state);
  double t = startTime, energy = startEnergy;
  const double timeStep = outputStep / nTimeSteps;
  int iStep = 0;
  while (t < endTime) {
    iStep++;
    for (int k = 0; k < nTimeSteps; k++) {
      check(cgpu_propagate_split2(c, state.data(), t, t + timeStep, 24, 1e-12, 8, 0), c, "cgpu_propagate_split2");
      t = t + timeStep;
    }
    check(cgpu_energy(c, state.data(), t, &energy), c, "cgpu_energy");
  }
  const double finalNorm = norm(state);
  std::printf("He1d_06: %d output steps, start energy %.16f, final energy %.16f (golden %.16f)\n", iStep, startEnergy,
              energy, g06);
  std::printf("He1d_06: start norm %.16f, final norm %.16f\n", startNorm, finalNorm);
  if (!(std::fabs(energy - startEnergy) < 1e-6)) fails++;  // :130 energy conserved
  if (!(std::fabs(energy - g06) < 1e-7)) fails++;          // :135 final energy vs reference
  if (!(std::fabs(finalNorm - startNorm) < 1e-10)) fails++;  // :139 norm conserved
  // the golden energy drift of the SIL+RK4 chain
  if (!(std::fabs((energy - startEnergy) - (g06 - g04)) < 1e-10)) fails++;
  check(cgpu_ctx_destroy(c), nullptr, "cgpu_ctx_destroy");
  std::printf("%s (%d failed checks)\n", fails ? "FAIL" : "OK", fails);
  return fails ? 1 : 0;
}
