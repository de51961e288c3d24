/* cody_gpu.h -- C ABI of the GB300 engine for CodyFortran's MCTDHX/TDCI hot path.
 *
 * Every entry point returns an int status (CGPU_OK = 0).  On failure the
 * message is available from cgpu_last_error(ctx) (or cgpu_last_global_error()
 * when no context exists); the reference's equivalent is `error stop "<msg>"`.
 *
 * Array arguments are HOST pointers in the reference's layouts (Fortran
 * column-major, complex(R64) = two doubles):
 *   state   : [C(nC) | orbs(nG, nOS)]   (Method_state,
 *             src/Method/Mb/OrbBased/Mctdhx/S_Method_Mb_OrbBased_Mctdhx.f90:229-249)
 *   orbs    : (nG, nOS)
 *   rdm1/h1 : (nO, nO);  rdm2/h2 : (nO, nO, nO, nO)
 * The device copies are owned by the context.  The "resident" entry points
 * keep the state on the GPU between calls.
 *
 * One context = one system, one CUDA stream.  A context is not reentrant:
 * one host thread calls in at a time (the reference's module state is global,
 * src/Orbs/M_Orbs.f90:25-29).
 */
#ifndef CODY_GPU_H
#define CODY_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CGPU_OK 0
#define CGPU_ERR_ARG 1
#define CGPU_ERR_CUDA 2
#define CGPU_ERR_NUMERIC 3
#define CGPU_ERR_UNSUPPORTED 4

#define CGPU_GRID_CONST 0 /* grid.linear.const + 8th-order finite differences */
#define CGPU_GRID_FEDVR 1 /* grid.linear.fedvr + 1D FEDVR kinetic operator      */

#define CGPU_INT_TOEPLITZ 0 /* K(|i-j| dx), dx = x(2)-x(1): the reference's uniform-grid kernel */
#define CGPU_INT_DENSE 1    /* K(|x_i - x_j|): valid on any grid                            */

#define CGPU_LASER_NONE 0
#define CGPU_LASER_SIN2 1    /* E(t) = E0 sin^2(pi tau/T) cos(w (tau - T/2) + cep), T = 2 pi n/w */
#define CGPU_LASER_SAMPLED 2 /* E(t) = E_n on [t0 + n dt, t0 + (n+1) dt)                       */

#define CGPU_METHOD_MCTDHX 0
#define CGPU_METHOD_TDCI 1

#define CGPU_PREC_FP64 0
/* Mixed: the pair-potential, correlation and h2 contractions on tcgen05 tensor cores with
 * split-bf16 operands (hi + lo, three products) and FP32 accumulation; RDMs, rho^-1,
 * projectors, Lanczos, energy and norm in FP64. */
#define CGPU_PREC_MIXED 1
/* As CGPU_PREC_MIXED with three-way split operands (hi + mid + lo, six products). */
#define CGPU_PREC_MIXED_X6 2
/* Fixed-point split form: every operand row carried as bf16 digit slices under one power
 * of two per row, holding 30 bits of the row maximum (5 base-64 slices for the contractions
 * over the grid, 4 base-256 slices for the one over orbital pairs); slice products of one
 * level summed exactly in their own FP32 tensor-memory accumulator, levels combined in
 * 64-bit integers: the contractions equal the products of the truncated operands. */
#define CGPU_PREC_MIXED_FX 3
/* As CGPU_PREC_MIXED_FX with 36 bits (6 base-64 slices, 5 base-256 slices). */
#define CGPU_PREC_MIXED_FX6 4

/* Time-derivative selectors (the TimeDerivative procedure pointers). */
#define CGPU_TD_FULL 0   /* Method_TimeDerivative (Mctdhx :101-149)                        */
#define CGPU_TD_ORBS_LIN 1   /* TimeDerivativeOrbsLin (Mctdhx :152-177)                    */
#define CGPU_TD_NONLIN 2 /* TimeDerivativeCoeffsPlusOrbsNonLin (Mctdhx :180-226)           */
#define CGPU_TD_TDCI 3   /* Tdci TimeDerivative (src/Method/Mb/OrbBased/Tdci/S_Method_Mb_OrbBased_Tdci.f90:75-107) */

typedef struct cgpu_ctx cgpu_ctx;

typedef struct {
  double re, im;
} cgpu_complex;

/* The configuration tree of one run (grid, sysKinetic, sysPotential,
 * sysInteraction, method.mb, orbs); the keys it mirrors are listed beside
 * each field. */
typedef struct {
  int grid_kind;                 /* grid.linear.const | grid.linear.fedvr                     */
  double xmin, xmax;             /* grid.linear.xmin/xmax (src/Grid/Linear/S_Grid_Linear.f90:29-30) */
  int n_points;                  /* grid.linear.const.nPoints                                */
  int n_elements, n_locals;      /* FEDVR elements and GLL points per element (order + 1)    */
  int xmin_excluded, xmax_excluded;
  int n_body_types;              /* method.mb.nBodyTypes                                      */
  int n_bodies[4];               /* method.mb.nBodies                                        */
  int n_orbs[4];                 /* method.mb.orbBased.nOrbs                                 */
  double body_mass[4];           /* sysKinetic.linear.laplacian.bodyMass                     */
  int restricted;                /* orbs.restrictedQ                                         */
  double regularization;         /* method.mb.orbBased.regularizationParameter (1e-10)       */
  int n_nuclei;                  /* sysPotential.linear.softYukawa.*                         */
  double nuc_position[8], nuc_charge[8], nuc_softening1[8], nuc_softening2[8], nuc_dampening[8];
  int has_interaction;           /* sysInteraction.linear.softYukawa present                 */
  double int_strength, int_softening1, int_softening2, int_dampening;
  int int_kind;                  /* CGPU_INT_*                                               */
  int laser_kind;                /* CGPU_LASER_*                                             */
  double laser_E0, laser_omega, laser_n_cycles, laser_cep, laser_t_start;
  const double* field_samples;   /* CGPU_LASER_SAMPLED: copied at creation                   */
  int n_field_samples;
  double field_dt, field_t0;
  int method;                    /* CGPU_METHOD_*                                            */
  int precision;                 /* CGPU_PREC_*                                              */
  int max_krylov;                /* largest Krylov dimension the context will be asked for   */
  int krylov_window;             /* 0: each Lanczos vector is orthogonalised against the whole
                                    basis (the reference's loop); 1: the three-term recurrence
                                    (w = H v_j - beta v_{j-1} - alpha v_j); k > 1: Gram-Schmidt
                                    against the last k basis vectors; the same for every
                                    trajectory of a batch                                       */
} cgpu_desc;

/* ---- context (Fabricate + Setup) ---------------------------------------- */
/* Replaces the *_Fabricate / *_Setup chain of the hot path: Grid_Setup
 * (src/Grid/Linear/Const/S_Grid_Linear_Const.f90:34-52, src/Utils/M_Utils_Fedvr.f90:76-149),
 * SysKinetic_Setup, SysPotential/SysInteraction setup, ConfigList_Setup
 * (src/ConfigList/AllActive/S_ConfigList_AllActive.f90:105-349) and the
 * Method_state allocation (Mctdhx :40-68). */
int cgpu_ctx_create(const cgpu_desc* desc, cgpu_ctx** out);
int cgpu_ctx_destroy(cgpu_ctx* ctx);
const char* cgpu_last_error(const cgpu_ctx* ctx);
const char* cgpu_last_global_error(void);
/* Page-locked host memory for the state buffers of the upload / download /
 * propagate entry points: their host<->device copies then run as direct DMA
 * at the link rate instead of through the CUDA driver's pageable staging.  An
 * addition of the GPU boundary (the reference keeps its states in ordinary
 * host arrays).  bytes == 0 gives *out = NULL; cgpu_host_free(NULL) is a no-op. */
int cgpu_host_alloc(size_t bytes, void** out);
int cgpu_host_free(void* ptr);
/* Makes device the calling thread's CUDA device for the contexts and batches
 * it creates afterwards (one process per GPU passes its local rank).  An
 * addition of the GPU boundary. */
int cgpu_select_device(int device);
/* out[0..5] = nG, nO (spin-orbitals), nOS (stored orbitals), nC, nBodyTypes, nState */
int cgpu_sizes(const cgpu_ctx* ctx, int* out);
/* Grid_Linear_xCoord / Grid_Linear_weights */
int cgpu_grid(const cgpu_ctx* ctx, double* x, double* w);
/* The device-built ConfigList tables of body type bt, copied to the host in the
 * reference layout (src/ConfigList/M_ConfigList.f90:112-128): kind 0 singles,
 * 1 doubles; arrays sized (maxConn, nConf) column-major; factor as +-1.0.
 * Pass NULL arrays to query only max_conn / n_conf. */
int cgpu_configlist_tables(cgpu_ctx* ctx, int bt, int kind, int* n_conf, int* max_conn, int64_t* codes,
                           int* n_connected, int* excited_c, int* orb_code, double* factor);
int cgpu_synchronize(cgpu_ctx* ctx);
/* Number of CUDA kernels this context launched since the last reset. */
long cgpu_launch_count(cgpu_ctx* ctx, int reset);

/* ---- equation of motion (Method / Method_Mb_OrbBased pointers) ---------- */
/* I_Method_TimeDerivative (src/Method/M_Method.f90:82-90) with the selector
 * CGPU_TD_* choosing among Mctdhx TimeDerivative / OrbsLin / NonLin and Tdci. */
int cgpu_time_derivative(cgpu_ctx* ctx, int which, cgpu_complex* d_state, const cgpu_complex* state, double time);
/* ApplySingleBodyOp (src/Method/Mb/OrbBased/S_Method_Mb_OrbBased.f90:976-1034):
 * d_orbs += (T + V(t)) orbs; h1 (nO, nO) filled when non-NULL. */
int cgpu_apply_single_body_op(cgpu_ctx* ctx, cgpu_complex* d_orbs, const cgpu_complex* orbs, double time,
                              cgpu_complex* h1);
/* FillH1 (S_Method_Mb_OrbBased.f90:164-224) */
int cgpu_fill_h1(cgpu_ctx* ctx, cgpu_complex* h1, const cgpu_complex* orbs, double time);
/* FillH2 (S_Method_Mb_OrbBased.f90:227-293) */
int cgpu_fill_h2(cgpu_ctx* ctx, cgpu_complex* h2, const cgpu_complex* orbs, double time);
/* ApplyCorrelationOp (S_Method_Mb_OrbBased.f90:647-805): d_orbs += rho^-1 rho2 W orbs;
 * h2 (nO^4) filled when non-NULL. */
int cgpu_apply_correlation_op(cgpu_ctx* ctx, cgpu_complex* d_orbs, const cgpu_complex* orbs,
                              const cgpu_complex* rdm1, const cgpu_complex* rdm2, double time, cgpu_complex* h2);
/* Method_GetEnergy (S_Method_Mb_OrbBased.f90:132-161) of the given state. */
int cgpu_energy(cgpu_ctx* ctx, const cgpu_complex* state, double time, double* energy);

/* ---- Sys* operators on one orbital (single-system contexts) -------------- */
/* The procedure pointers a configuration binds when it moves only sysKinetic,
 * sysPotential or sysInteraction to the GPU; nG-point host arrays.  Body
 * types are 1-based as in Fortran; 0 stands for an absent optional bt_. */
/* I_SysKinetic_MultiplyWithKineticOp (src/SysKinetic/M_SysKinetic.f90:141-160):
 * d_orb = T orb with the mass of body type bt (FEDVR or finite differences). */
int cgpu_sys_kinetic_multiply(cgpu_ctx* ctx, cgpu_complex* d_orb, const cgpu_complex* orb, double time, int bt);
/* I_SysPotential_FillExternalPotential (src/SysPotential/M_SysPotential.f90:71-84):
 * potential = V(x) + E(t) x on the grid (soft-Yukawa nuclei; the 1D
 * length-gauge laser is carried by the external potential). */
int cgpu_sys_potential_fill(cgpu_ctx* ctx, cgpu_complex* potential, double time, int bt);
/* I_SysPotential_MultiplyWithExternalPotential (src/SysPotential/M_SysPotential.f90:89-101):
 * d_orb = potential * orb point by point. */
int cgpu_sys_potential_multiply(cgpu_ctx* ctx, cgpu_complex* d_orb, const cgpu_complex* potential,
                                const cgpu_complex* orb);
/* I_SysInteraction_FillInteractionSrc (src/SysInteraction/M_SysInteraction.f90:114-128;
 * src/SysInteraction/Linear/S_SysInteraction_Linear.f90:57-72): src = conj(orb_conjg) orb w. */
int cgpu_sys_interaction_src(cgpu_ctx* ctx, cgpu_complex* src, const cgpu_complex* orb_conjg, const cgpu_complex* orb);
/* I_SysInteraction_FillInteractionPotential (src/SysInteraction/M_SysInteraction.f90:94-111):
 * potential(x_i) = sum_j K(x_i, x_j) src_j with the context's interaction
 * kernel (CGPU_INT_TOEPLITZ or CGPU_INT_DENSE). */
int cgpu_sys_interaction_potential(cgpu_ctx* ctx, cgpu_complex* potential, const cgpu_complex* src, double time,
                                   int bt1, int bt2);
/* I_SysInteraction_MultiplyWithInteractionPotential (src/SysInteraction/M_SysInteraction.f90:145-157):
 * res = potential * orb point by point. */
int cgpu_sys_interaction_multiply(cgpu_ctx* ctx, cgpu_complex* res, const cgpu_complex* potential,
                                  const cgpu_complex* orb);

/* ---- CI vector (Coeffs pointers) ---------------------------------------- */
/* I_Coeffs_ApplyH1FillRdm1 (src/Coeffs/M_Coeffs.f90:119-135; Generic :103-178).
 * NULL optional arguments select the mode, as the Fortran optionals do. */
int cgpu_ci_apply_h1_fill_rdm1(cgpu_ctx* ctx, const cgpu_complex* coeffs, cgpu_complex* rdm1,
                               cgpu_complex* d_coeffs, const cgpu_complex* h1);
/* I_Coeffs_ApplyH2FillRdm2 (src/Coeffs/M_Coeffs.f90:139-156; Generic :197-319). */
int cgpu_ci_apply_h2_fill_rdm2(cgpu_ctx* ctx, const cgpu_complex* coeffs, cgpu_complex* rdm2,
                               cgpu_complex* d_coeffs, const cgpu_complex* h2);
/* Coeffs_ProjectOnSubspace (src/Coeffs/S_Coeffs.f90:105-111) */
int cgpu_project_coeffs(cgpu_ctx* ctx, cgpu_complex* d_coeffs, const cgpu_complex* coeffs);
/* Coeffs_Normalize (src/Coeffs/S_Coeffs.f90:84-94) */
int cgpu_normalize_coeffs(cgpu_ctx* ctx, cgpu_complex* coeffs);

/* ---- orbitals (Orbs / Grid pointers) ------------------------------------ */
/* Orbs_ProjectOnSubspace (src/Orbs/S_Orbs.f90:198-225 -> src/Grid/S_Grid.f90:170-203) */
int cgpu_project_orbs(cgpu_ctx* ctx, cgpu_complex* d_orbs, const cgpu_complex* orbs);
/* Orbs_Orthonormalize (src/Orbs/S_Orbs.f90:145-173 -> src/Grid/S_Grid.f90:120-151) */
int cgpu_orthonormalize_orbs(cgpu_ctx* ctx, cgpu_complex* orbs);

/* ---- integrators and propagator ----------------------------------------- */
/* Rk O4Expl Integrate (src/IntegratorList/Rk/O4Expl/S_IntegratorList_Rk_O4Expl.f90:90-141) */
int cgpu_integrate_rk4(cgpu_ctx* ctx, int which, cgpu_complex* state, double t0, double t1);
/* Rk O1Expl Integrate (src/IntegratorList/Rk/O1Expl/S_IntegratorList_Rk_O1Expl.f90:50-72);
 * imag != 0 wraps the derivative as Actions_ImagTimeDerivative (src/Utils/M_Utils_Actions.f90:66-78). */
int cgpu_integrate_euler(cgpu_ctx* ctx, int which, int imag, cgpu_complex* state, double t0, double t1);
/* Sil Integrate (src/IntegratorList/Sil/S_IntegratorList_Sil.f90:114-310).  metric:
 * NULL = Euclidean; otherwise nState weights (metricWeights).  *warnings counts
 * sub-steps that did not reach the tolerance (the reference prints a warning). */
int cgpu_integrate_sil(cgpu_ctx* ctx, int which, cgpu_complex* state, double t0, double t1, int krylov_dim,
                       double tolerance, int max_restarts, const double* metric, int* warnings);
/* SplitStep Order2 Propagate (src/Propagator/SplitStep/Order2/S_Propagator_SplitStep_Order2.f90:52-77):
 * integratorList(1) = SIL on OrbsLin (RK4 when krylov_dim <= 0), integratorList(2) = RK4 on NonLin.
 * use_metric != 0 sets the SIL metric to [1 on C | grid weights on orbitals]. */
int cgpu_propagate_split2(cgpu_ctx* ctx, cgpu_complex* state, double t0, double t1, int krylov_dim,
                          double tolerance, int max_restarts, int use_metric);

/* ---- resident state (GPU-native driver loop) ---------------------------- */
int cgpu_state_upload(cgpu_ctx* ctx, const cgpu_complex* state);
int cgpu_state_download(cgpu_ctx* ctx, cgpu_complex* state);
/* n_steps Strang steps of size dt from t0 on the resident state, fixed-order
 * SIL (krylov_dim, tolerance 0, no restarts).  use_graph != 0 replays one
 * captured CUDA graph per step. */
int cgpu_propagate_resident(cgpu_ctx* ctx, double t0, double dt, int n_steps, int krylov_dim, int use_metric,
                            int use_graph);
int cgpu_energy_resident(cgpu_ctx* ctx, double time, double* energy);

/* Same as cgpu_propagate_resident, timed with CUDA events recorded on the
 * context's stream around the n_steps; *elapsed_ms receives the device time. */
int cgpu_propagate_resident_timed(cgpu_ctx* ctx, double t0, double dt, int n_steps, int krylov_dim, int use_metric,
                                  int use_graph, double* elapsed_ms);

/* ---- profiling ----------------------------------------------------------- */
/* Kernel families whose launches can be bracketed by CUDA events. */
#define CGPU_KERNEL_PAIR_POTENTIALS 1 /* W = V S (interaction potentials of all orbital pairs) */
#define CGPU_KERNEL_CORRELATION 2     /* rho^-1 rho2 W phi contraction                        */
#define CGPU_KERNEL_H2 3              /* h2 = 1/2 S^T W                                        */
#define CGPU_KERNEL_CI_APPLY 4        /* H1/H2 application to the CI vector                    */
#define CGPU_KERNEL_CI_RDM 5          /* one- and two-body RDM accumulation                    */
#define CGPU_KERNEL_ONEBODY 6         /* banded kinetic + potential + laser apply              */
#define CGPU_KERNEL_LANCZOS 7         /* Krylov reorthogonalisation / update                   */
#define CGPU_KERNEL_RDM_INVERSE 8     /* regularised rho^-1 and the correlation matrix R'      */
#define CGPU_KERNEL_PROJECTORS 9      /* Gram matrices: h1, (1-P) on orbitals, P on coefficients */
#define CGPU_KERNEL_FOLD 10           /* h1/h2 folding into the CI code layout                 */
#define CGPU_KERNEL_VECTOR 11         /* state-vector updates: RK stages, Lanczos start/combine, copies */
/* Start recording events around every launch of `kernel` (0 disables). */
int cgpu_profile_begin(cgpu_ctx* ctx, int kernel);
/* Stop; *launches and *total_ms receive the bracketed launches and their summed device time. */
int cgpu_profile_end(cgpu_ctx* ctx, long* launches, double* total_ms);

/* ---- TDCI ---------------------------------------------------------------- */
/* Tdci Setup (src/Method/Mb/OrbBased/Tdci/S_Method_Mb_OrbBased_Tdci.f90:40-72):
 * fix the orbitals and fill h1/h2 once. */
int cgpu_tdci_set_orbitals(cgpu_ctx* ctx, const cgpu_complex* orbs);

/* ---- observables and relaxation ------------------------------------------ */
/* Observables of the resident state at `time` (GetEnergy and the RDM
 * observables the printers use, src/Utils/M_Utils_RdmObservables.f90:17-52,
 * src/Utils/M_Utils_PrinterObservableLinear.f90:25-103):
 * out[0] = energy, out[1] = ||C||, out[2] = <x> (dipole, sum rho1 x), then the
 * nOS natural occupations (eigenvalues of the spin-summed rho1, descending;
 * zero for TDCI contexts).  out has 3 + nOS entries. */
int cgpu_observables(cgpu_ctx* ctx, double time, double* out);
/* Imaginary-time relaxation of a host state (T_He1d_04_ImagTimePropagationMctdhx.f90:82-99):
 * n_inner Euler steps, each followed by Coeffs_Normalize and Orbs_Orthonormalize,
 * then GetEnergy; repeated until |dE| <= conv_thresh or max_outer rounds.
 * Replaces state; returns the final energy and the number of rounds. */
int cgpu_relax(cgpu_ctx* ctx, cgpu_complex* state, double dt, int n_inner, double conv_thresh, int max_outer,
               double* energy, int* n_outer);

/* Restart files of the resident state in the reference's raw format
 * (src/Utils/M_Utils_DataStorage.f90:20-106): coeffs.in, orbBB_II.in per
 * stored orbital (src/Orbs/S_Orbs.f90:251-276) and, with with_rdm2,
 * rdm2BtXX_YY.in (src/Coeffs/S_Coeffs.f90:177-214), under the directory `dir`. */
int cgpu_save_restart(cgpu_ctx* ctx, const char* dir, int with_rdm2);
int cgpu_load_restart(cgpu_ctx* ctx, const char* dir);

/* Cosine absorber (src/Absorber/Linear/Cosinus/S_Absorber_Linear_Cosinus.f90:75-128):
 * mask 1 for |x| < onset, cos(pi/2 xi)^(1/order) beyond, xi = (|x| - onset) /
 * (x_last - onset).  cgpu_absorber_apply multiplies the resident orbitals by it
 * once (Absorber_ApplyAbsorber); with apply_each_step the resident / graph
 * propagations apply it after every step. */
int cgpu_absorber_setup(cgpu_ctx* ctx, double onset, double order, int apply_each_step);
int cgpu_absorber_apply(cgpu_ctx* ctx);

/* ---- pulse gradient (adjoint) ------------------------------------------- */
/* No counterpart in the reference.  For a TDCI context (orbitals set with
 * cgpu_tdci_set_orbitals, at most 64 configurations): propagates c0 over
 * n_steps RK4 steps of dt with the field constant over step n (field[n]), and
 * returns objective = 1 - |overlap|^2, overlap = c0^H C_N, the final
 * coefficients c_final (may be NULL) and, if d_objective is not NULL, the
 * exact gradient of the discrete map d objective / d field[n] from the
 * adjoint sweep (states checkpointed every `checkpoint` steps, 0 = 64).
 * The context's one-body integrals are restored to t = 0 afterwards. */
int cgpu_tdci_adjoint(cgpu_ctx* ctx, const cgpu_complex* c0, const double* field, int n_steps, double dt,
                      int checkpoint, double* objective, double* overlap, cgpu_complex* c_final,
                      double* d_objective);

/* MCTDHF pulse gradient, as an explicit forward / backward pair.  No
 * counterpart in the reference.  For a single FP64 MCTDHX context that is
 * restricted, with two body types of one particle each (the two-electron
 * problem of the 1D helium model, M <= 16 spatial orbitals):
 * cgpu_mc_adjoint_forward propagates state0 over n_steps Strang steps of dt
 * (fixed-order SIL of krylov_dim <= 32 with the metric [1 | w] on OrbsLin,
 * RK4 on NonLin: the map of cgpu_propagate_split2) with the piecewise-
 * constant field E(t) = field[floor(t / dt)] (zero from n_steps dt on) in the
 * length gauge, in place of the context's laser.  It returns
 * objective = 1 - |<ref|Psi_N>|^2 with the MCTDHF overlap
 * sum conj(C_ref[a,b]) (S C S^T)[a,b], S = phi_ref^H W phi (ref_state NULL =
 * state0), overlap[2] = <ref|Psi_N>, and state_final (may be NULL), and keeps
 * the state every `checkpoint` steps (0 = 64) on the device.
 * cgpu_mc_adjoint_backward then returns d_objective[n] = d objective / d field[n]
 * for every n: the exact gradient of the discrete map, from the co-state
 * propagated backward through the Krylov, RK4 and Lanczos steps, each segment
 * of `checkpoint` steps recomputed from its checkpoint. */
int cgpu_mc_adjoint_forward(cgpu_ctx* ctx, const cgpu_complex* state0, const cgpu_complex* ref_state,
                            const double* field, int n_steps, double dt, int krylov_dim, int checkpoint,
                            double* objective, double* overlap, cgpu_complex* state_final);
int cgpu_mc_adjoint_backward(cgpu_ctx* ctx, double* d_objective);

/* ---- batched trajectories ------------------------------------------------ */
/* No counterpart in the reference, whose module-global state allows one
 * trajectory per process (src/Method/M_Method.f90:47).  A batch holds n
 * independent systems of any sizes (pulse scans, uneven grids and orbital
 * counts) with the same body-type layout, method and precision.  Every kernel
 * of the step covers all systems in one launch, and cgpu_batch_propagate
 * replays the fixed-order Strang step (as cgpu_propagate_resident) as one
 * CUDA graph per time step. */
typedef struct cgpu_batch cgpu_batch;
int cgpu_batch_create(const cgpu_desc* descs, int n, cgpu_batch** out);
int cgpu_batch_destroy(cgpu_batch* batch);
int cgpu_batch_size(const cgpu_batch* batch);
/* cgpu_sizes / cgpu_grid of system i */
int cgpu_batch_sizes(const cgpu_batch* batch, int i, int* sizes6);
int cgpu_batch_grid(const cgpu_batch* batch, int i, double* x, double* w);
/* All states, concatenated in system order (nS_i entries each, layout
 * [C | orbitals] as cgpu_state_upload). */
int cgpu_batch_upload(cgpu_batch* batch, const cgpu_complex* states);
/* cgpu_save_restart / cgpu_load_restart for every trajectory of a batch: the
 * files of trajectory i (the same raw format: coeffs.in, orbBB_KK.in, with
 * with_rdm2 the rdm2BtXX_YY.in blocks) under <dir>/traj<i, 5 digits>/; save
 * creates the subdirectories, dir itself must exist. */
int cgpu_batch_save_restart(cgpu_batch* batch, const char* dir, int with_rdm2);
int cgpu_batch_load_restart(cgpu_batch* batch, const char* dir);
int cgpu_batch_download(cgpu_batch* batch, cgpu_complex* states);
/* n_steps steps of size dt; system i starts at t0[i].  *elapsed_ms (may be
 * NULL) receives the device time from CUDA events around the launches. */
int cgpu_batch_propagate(cgpu_batch* batch, const double* t0, double dt, int n_steps, int krylov_dim,
                         int use_metric, double* elapsed_ms);
/* energies[i] = GetEnergy of system i at time t[i] */
int cgpu_batch_energies(cgpu_batch* batch, const double* t, double* energies);
/* cgpu_observables of every system at t[i]: out[i * (3 + nOSmax) + ...],
 * nOSmax the largest orbital count of the batch (cgpu_batch_sizes). */
int cgpu_batch_observables(cgpu_batch* batch, const double* t, double* out);
/* The absorber for every system of the batch (each with its own grid). */
int cgpu_batch_absorber_setup(cgpu_batch* batch, double onset, double order, int apply_each_step);
/* Kernels launched per step (all systems); launches so far (reset if nonzero). */
long cgpu_batch_kernels_per_step(const cgpu_batch* batch);
/* As cgpu_profile_begin / cgpu_profile_end, for the launches of a batch step. */
int cgpu_batch_profile_begin(cgpu_batch* batch, int kernel);
int cgpu_batch_profile_end(cgpu_batch* batch, long* launches, double* total_ms);
long cgpu_batch_launch_count(cgpu_batch* batch, int reset);
/* Fixed-point form: the number of shared interaction matrices (root grids in which every
 * trajectory's grid is a contiguous piece), 0 when each trajectory keeps its own. */
int cgpu_batch_shared_interactions(const cgpu_batch* batch);

/* ---- tile autotuner ------------------------------------------------------ */
/* No counterpart in the reference.  The tile table of a context or batch:
 * tiles[0..8] = for the fixed-point contractions W = V S, Z = W R'' and
 * h2 = S^T W in turn: N-tile width, compact flag (two CTAs per SM), K splits
 * (zero outside CGPU_PREC_MIXED_FX / _FX6); tiles[9] = blocks per trajectory
 * of the Lanczos reductions.  The set-up heuristics choose the initial table.
 * cgpu_autotune times the candidates on the resident states (upload them
 * first) with CUDA events on the context's stream and applies the fastest:
 * every instantiated tile configuration and feasible K split of each
 * contraction, and half / one / two times the heuristic's Lanczos blocks.
 * cache_path (may be NULL) is a JSON-lines file of winners keyed by the
 * precision, device, Krylov order and window and the trajectories' sizes:
 * CGPU_TUNE_CACHED applies the cached entry of this shape if there is one and
 * otherwise tunes and adds it; CGPU_TUNE_FORCE always tunes and replaces it.
 * report (may be NULL) receives a JSON object with the source ("tuned" or
 * "cache"), the key, the timed candidates [tile..., ms] and the chosen table.
 * The tile choice leaves the fixed-point contractions' results unchanged (exact
 * digit sums); K splits and Lanczos blocks change FP64 summation orders only.
 * A changed table is used from the next step on (a captured step graph is
 * re-captured). */
#define CGPU_TUNE_CACHED 0
#define CGPU_TUNE_FORCE 1
int cgpu_autotune(cgpu_ctx* ctx, const char* cache_path, int mode, char* report, int report_len);
int cgpu_get_tiles(const cgpu_ctx* ctx, int* tiles);
/* Applies a table (validated against the instantiated configurations, the
 * digits' exact range and the partial buffers; CGPU_ERR_ARG otherwise). */
int cgpu_set_tiles(cgpu_ctx* ctx, const int* tiles);
int cgpu_batch_autotune(cgpu_batch* batch, const char* cache_path, int mode, char* report, int report_len);
int cgpu_batch_get_tiles(const cgpu_batch* batch, int* tiles);
int cgpu_batch_set_tiles(cgpu_batch* batch, const int* tiles);

/* ---- no-allocation variant ---------------------------------------------- */
/* No counterpart in the reference.  Weighted Gram matrix of two orbital sets,
 *   gram(i,j) = sum_g conj(a[g + n_grid*i]) * b[g + n_grid*j] * weights[g],
 * (column-major n_cols x n_cols), the matrix that Grid_InnerProduct builds in
 * FillH1 and the (1-P) projector.  It is for callers that cannot call
 * cudaMalloc when they need it: a host program whose device memory belongs
 * to another component, or code running where allocation is not allowed.
 * It allocates nothing: a, b, weights and gram are the caller's DEVICE
 * pointers, and the per-block partial sums live in a fixed 1 MiB __device__
 * array inside the library, which every GPU that loads the library holds
 * until exit.  Limits: 1 <= n_cols <= 32, n_grid >= 1; larger sizes are
 * rejected with CGPU_ERR_ARG and a message in cgpu_last_global_error().
 * The first call on each device looks up that array's device address (with
 * the device current) and keeps it for the life of the process; make that
 * first call before any stream capture.  Calls after cudaDeviceReset (or any
 * other teardown of the device's primary context) are not supported.  A CUDA
 * error already pending on the calling thread is reported (CGPU_ERR_CUDA) and
 * left pending; nothing is launched then.
 * The kernels run asynchronously on `stream` (a cudaStream_t, NULL = legacy
 * default stream).  All calls share the one array: calls that overlap on the
 * GPU (concurrent streams) race on it and must be serialised by the caller. */
int cgpu_weighted_gram_noalloc(const cgpu_complex* a, const cgpu_complex* b, const double* weights, int n_grid,
                               int n_cols, cgpu_complex* gram, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* CODY_GPU_H */
