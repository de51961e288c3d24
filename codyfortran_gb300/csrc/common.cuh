// common.cuh -- shared types and kernel launchers of the GB300 MCTDHX/TDCI engine.
//
// A context holds nb >= 1 independent trajectories ("systems").  The device
// buffers of trajectory b sit at byte offset b * bs from those of trajectory 0
// (one arena, the same layout in every block, sized for the largest system),
// every kernel takes its trajectory from blockIdx.z and its sizes from the
// TrajShape table, so one launch advances all trajectories.  A plain context
// is the case nb = 1.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <array>
#include <string>
#include <vector>

#include "../../include/cody_gpu.h"
#include "dfloat.cuh"

// ---------------------------------------------------------------------------
// Complex arithmetic on double2 (layout-compatible with Fortran complex(R64)).
// ---------------------------------------------------------------------------
typedef double2 z_t;

__host__ __device__ __forceinline__ z_t zmk(double r, double i) { return make_double2(r, i); }
__host__ __device__ __forceinline__ z_t zadd(z_t a, z_t b) { return make_double2(a.x + b.x, a.y + b.y); }
__host__ __device__ __forceinline__ z_t zsub(z_t a, z_t b) { return make_double2(a.x - b.x, a.y - b.y); }
__host__ __device__ __forceinline__ z_t zmul(z_t a, z_t b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__host__ __device__ __forceinline__ z_t zconj(z_t a) { return make_double2(a.x, -a.y); }
__host__ __device__ __forceinline__ z_t zscale(z_t a, double s) { return make_double2(a.x * s, a.y * s); }
// conj(a) * b
__host__ __device__ __forceinline__ z_t zcmul(z_t a, z_t b) {
  return make_double2(a.x * b.x + a.y * b.y, a.x * b.y - a.y * b.x);
}
// a += b * c
__host__ __device__ __forceinline__ void zfma(z_t& a, z_t b, z_t c) {
  a.x = fma(b.x, c.x, fma(-b.y, c.y, a.x));
  a.y = fma(b.x, c.y, fma(b.y, c.x, a.y));
}
// a with its sign flipped when neg (integer operation on the sign bits, no FP64 instruction)
__device__ __forceinline__ z_t zsign(z_t a, bool neg) {
  long long m = neg ? (long long)0x8000000000000000ULL : 0LL;
  return make_double2(__longlong_as_double(__double_as_longlong(a.x) ^ m),
                      __longlong_as_double(__double_as_longlong(a.y) ^ m));
}

// ---- element formulas shared by the nO^4 layout kernels and their fused forms

// Body-type rule of FillH2Lin / FillRdm2FromRdm2Lin.
__device__ __forceinline__ bool bt_rule_ok(const int* btOf, int i1, int i2, int j1, int j2) {
  int bi1 = btOf[i1], bi2 = btOf[i2], bj1 = btOf[j1], bj2 = btOf[j2];
  if (bi1 == bi2 && bj1 != bj2) return false;
  if (bi1 != bi2 && bj1 == bj2) return false;
  return true;
}

// rdm2(a, b, c, d) (index a + n (b + n (c + n d))) from rdm2Lin (FillRdm2FromRdm2Lin).
__device__ __forceinline__ z_t rdm2_from_lin(const z_t* __restrict__ lin, const int* __restrict__ btOf, size_t n, int a,
                                             int b, int c, int d) {
  auto L = [&](int i1, int j1, int i2, int j2) { return lin[(((size_t)i1 * n + j1) * n + i2) * n + j2 + 1]; };
  z_t s = make_double2(0.0, 0.0);
  if (a <= b && c <= d && bt_rule_ok(btOf, a, b, c, d)) s = zadd(s, L(a, c, b, d));
  if (b <= a && c <= d && bt_rule_ok(btOf, b, a, c, d)) s = zsub(s, L(b, c, a, d));
  if (a <= b && d <= c && bt_rule_ok(btOf, a, b, d, c)) s = zsub(s, L(a, d, b, c));
  if (b <= a && d <= c && bt_rule_ok(btOf, b, a, d, c)) s = zadd(s, L(b, d, a, c));
  return s;
}

// h2(i1, l2, j1, k2) (index i1 + N (l2 + N (j1 + N k2))) from the spatial H2s.
__device__ __forceinline__ z_t h2_from_h2s(const z_t* __restrict__ H2s, const int* __restrict__ btOf, int restricted,
                                           int n, int i1, int l2, int j1, int k2) {
  if (restricted) {
    int s1 = i1 / n, s2 = l2 / n, s3 = j1 / n, s4 = k2 / n;
    if (s1 == s3 && s2 == s4) {
      int a = i1 % n, b = l2 % n, c = j1 % n, d = k2 % n;
      return H2s[(size_t)(a * n + c) * n * n + (b * n + d)];
    }
    return make_double2(0.0, 0.0);
  }
  if (btOf[i1] == btOf[j1] && btOf[l2] == btOf[k2]) return H2s[(size_t)(i1 * n + j1) * n * n + (l2 * n + k2)];
  return make_double2(0.0, 0.0);
}

// h2Lin(orbCode) (FillH2Lin, fermions) with H(a, b, c, d) = h2(a, b, c, d).
template <class H>
__device__ __forceinline__ z_t h2lin_value(const int* __restrict__ btOf, int i1, int j1, int i2, int j2, H h) {
  z_t v = make_double2(0.0, 0.0);
  if (i1 <= i2 && j1 <= j2 && bt_rule_ok(btOf, i1, i2, j1, j2) && i1 != i2 && j1 != j2)
    v = zadd(zsub(zsub(h(i1, i2, j1, j2), h(i1, i2, j2, j1)), h(i2, i1, j1, j2)), h(i2, i1, j2, j1));
  return v;
}

// ---- double-float arithmetic: dfloat.cuh; the warp sum of an accumulator here.
__device__ __forceinline__ zdf_acc zdf_warp_sum(zdf_acc a) {
  for (int o = 16; o > 0; o >>= 1) {
    const float rs = __shfl_xor_sync(0xffffffffu, a.rs, o), rc = __shfl_xor_sync(0xffffffffu, a.rc, o);
    const float is = __shfl_xor_sync(0xffffffffu, a.is, o), ic = __shfl_xor_sync(0xffffffffu, a.ic, o);
    df_acc(a.rs, a.rc, rs, rc);
    df_acc(a.is, a.ic, is, ic);
  }
  return a;
}

// a += conj(b) * c
__host__ __device__ __forceinline__ void zcfma(z_t& a, z_t b, z_t c) {
  a.x = fma(b.x, c.x, fma(b.y, c.y, a.x));
  a.y = fma(b.x, c.y, fma(-b.y, c.x, a.y));
}
// multiply by -i
__host__ __device__ __forceinline__ z_t zmi(z_t a) { return make_double2(a.y, -a.x); }
// multiply by +i
__host__ __device__ __forceinline__ z_t zpi(z_t a) { return make_double2(-a.y, a.x); }

// out[k] = sum_{b < nBlk} part[b*stride + k] for k < nk, computed by the whole
// block (warp per k, lanes over b, fixed order: every block that calls it with
// the same arguments gets bit-identical sums).  Ends with __syncthreads().
__device__ __forceinline__ void sum_partials(const double2* __restrict__ part, int nBlk, int stride, int nk,
                                             double2* out) {
  int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int k = wid; k < nk; k += nw) {
    double2 s = make_double2(0.0, 0.0);
    for (int b = lane; b < nBlk; b += 32) {
      double2 p = part[(size_t)b * stride + k];
      s.x += p.x;
      s.y += p.y;
    }
    for (int o = 16; o > 0; o >>= 1) {
      s.x += __shfl_xor_sync(0xffffffffu, s.x, o);
      s.y += __shfl_xor_sync(0xffffffffu, s.y, o);
    }
    if (lane == 0) out[k] = s;
  }
  __syncthreads();
}

#define CODY_MAX_BT 4
#define CODY_MAX_ORBS 64
#define CODY_MAX_KRYLOV 64

// ---------------------------------------------------------------------------
// Per-body-type configuration tables (ConfigList), generated on the device.
// Layout as the reference: (maxConn, nConf) column-major, 1-based indices.
// ---------------------------------------------------------------------------
struct CiTables {
  int nOrbs, nBodies, nConf, maxS, maxD, shift;
  int64_t* codes;      // codeFromConfig
  int* sN;             // singles nConnected
  int* sExc;           // singles excitedC
  int* sCode;          // singles orbCode
  int8_t* sFac;        // singles factor (+-1)
  int* dN;
  int* dExc;
  int* dCode;
  int8_t* dFac;
  int* rankTab;        // (nBodies+1) x (nOrbs+1) additive rank table
  // the same excitations grouped by orbital code (for the RDM gathers):
  // code q has value xCode[q] and edges [xStart[q], xStart[q+1]) with
  // source / target configuration (0-based) and sign
  int nSc, nDc;        // distinct singles / doubles codes
  int *sxCode, *sxStart, *sxSrc, *sxDst;
  int8_t* sxFac;
  int *dxCode, *dxStart, *dxSrc, *dxDst;
  int8_t* dxFac;
};

// Device view of the CI layout for the traversal kernels.
struct CiView {
  int nBt, nO, nC;
  int stride[CODY_MAX_BT];
  int nConf[CODY_MAX_BT];
  int maxS[CODY_MAX_BT], maxD[CODY_MAX_BT];
  const int* sN[CODY_MAX_BT];
  const int* sExc[CODY_MAX_BT];
  const int* sCode[CODY_MAX_BT];
  const int8_t* sFac[CODY_MAX_BT];
  const int* dN[CODY_MAX_BT];
  const int* dExc[CODY_MAX_BT];
  const int* dCode[CODY_MAX_BT];
  const int8_t* dFac[CODY_MAX_BT];
  // code-major excitation lists (CiTables::sx*, dx*)
  int nSc[CODY_MAX_BT], nDc[CODY_MAX_BT];
  const int *sxCode[CODY_MAX_BT], *sxStart[CODY_MAX_BT], *sxSrc[CODY_MAX_BT], *sxDst[CODY_MAX_BT];
  const int8_t* sxFac[CODY_MAX_BT];
  const int *dxCode[CODY_MAX_BT], *dxStart[CODY_MAX_BT], *dxSrc[CODY_MAX_BT], *dxDst[CODY_MAX_BT];
  const int8_t* dxFac[CODY_MAX_BT];
};

struct MixedBufs;  // mixed-precision operand layout (k_mixed.cu)
struct McAdjoint;  // MCTDHF pulse-gradient buffers (k_adjoint_mc.cu)

// Laser parameters as the device sees them (E(t) is evaluated in the kernels so
// that a captured step can be replayed at any time).
struct LaserDev {
  int kind;
  double E0, omega, nCycles, cep, tStart, sampleDt, sampleT0;
  int nSamples;
  const double* samples;
};

// Sizes and parameters of one trajectory, as the kernels read them.
struct TrajShape {
  int nG, nOS, nO, nC, nS, nGO, nPairs, band, restricted, hasPot, nBt;
  int nCpad;                 // offset of the orbitals in a state vector (the context's largest nC)
  int nGroups;               // (1-P) projector groups: one when restricted, else one per body type
  int grpStart[CODY_MAX_BT], grpSize[CODY_MAX_BT];
  int Kg, Kp;                // mixed form: K of the grid / pair contractions padded to 64 (Kg includes gShift)
  int vRow, gShift;          // fixed-point form with shared interaction matrices: first grid point of this
                             // trajectory in its root grid, and its offset within a 64-wide K tile
  int vRoot, vExp;           // the root grid (plane of the shared slices) and the offset of the
                             // trajectory's first row in the shared row-exponent array
  double regEps;
  LaserDev laser;
  CiView view;
};

// Pointer p of trajectory 0 moved to the trajectory of this block.
template <class T>
__device__ __forceinline__ T* bat(T* p, size_t bs) {
  return p ? (T*)((char*)p + (size_t)blockIdx.z * bs) : p;
}

// Pointer p of trajectory b (for kernels that fold more than the trajectory into blockIdx.z).
template <class T>
__device__ __forceinline__ T* batn(T* p, size_t bs, int b) {
  return p ? (T*)((char*)p + (size_t)b * bs) : p;
}

// A state vector is [C (nC) | unused up to nCpad | orbitals (nG x nOS)]; the
// vector kernels walk its nS = nC + nG nOS entries through these maps.
enum { VSEL_STATE = 0, VSEL_COEFFS = 1 };
__device__ __forceinline__ size_t vlen(const TrajShape& S, int sel) {
  return sel == VSEL_STATE ? (size_t)S.nS : (size_t)S.nC;
}
__device__ __forceinline__ size_t vidx(const TrajShape& S, size_t i) {
  return i < (size_t)S.nC ? i : i + (size_t)(S.nCpad - S.nC);
}

// Host-side data of one system (grid, operators, tables).
struct SysHost {
  int nG = 0, nO = 0, nOS = 0, nC = 0, nS = 0, nPairs = 0, band = 0, nBtK = 1;
  int nBodies[CODY_MAX_BT] = {0}, nOrbs[CODY_MAX_BT] = {0}, orbStart[CODY_MAX_BT] = {0};
  double mass[CODY_MAX_BT] = {0};
  double regEps = 1e-10;
  int hasPotential = 0;
  int laserKind = 0;
  double E0 = 0, omega = 0, nCycles = 0, cep = 0, tStart = 0, sampleDt = 1, sampleT0 = 0;
  std::vector<double> samples;
  double* samples_d = nullptr;
  std::vector<double> x, w, V0, band_h;
  std::vector<int> btOfOrb, pl, pk, pidx;
  int intToeplitz = 0;
  double intS = 0, intS1 = 0, intS2 = 0, intDamp = 0;
  CiTables tab[CODY_MAX_BT] = {};
  CiView view = {};
  // host copies for the work lists: connections per configuration, code-list starts
  std::vector<int> hsN[CODY_MAX_BT], hdN[CODY_MAX_BT], hsxStart[CODY_MAX_BT], hdxStart[CODY_MAX_BT];
};

// One block's share of a CI kernel: trajectory and task range [t0, t1).
struct CiWork {
  int traj, t0, t1;
};

// ---------------------------------------------------------------------------
// The context: nb systems, their device-resident operators, tables and work
// buffers, and one CUDA stream.  Not reentrant (one host thread at a time),
// like the reference's module-global state.  The size fields are the largest
// over the systems (they size grids and buffers); kernels read the true sizes
// of their trajectory from shape_d.
// ---------------------------------------------------------------------------
struct cgpu_ctx {
  // batch
  int nb = 1;
  size_t bs = 0;                  // bytes between the buffers of consecutive trajectories
  char* arena = nullptr;
  std::vector<SysHost> sys;
  std::vector<TrajShape> shape_h;
  TrajShape* shape_d = nullptr;
  // sizes (maxima over the systems; uniform: nBt, restricted, method, precision, hasInteraction)
  int nG = 0, nBt = 0, nO = 0, nOS = 0, nC = 0, nS = 0, nGO = 0, restricted = 0, method = 0, precision = 0;
  int band = 0, nBtK = 1, nPairs = 0;
  int minS = 0;                   // smallest state size (bounds the Krylov order)
  // CI work lists (blocks balanced by the number of terms; see ci_build_work)
  CiWork *applyWork_d = nullptr, *rdmWork_d = nullptr, *pairWork_d = nullptr;
  int nApplyWork = 0, nRdmWork = 0, nPairWork = 0;
  int ciSmem = 0;                 // bytes of shared memory for a CI vector (0: read it from global memory)
  int hasInteraction = 0, anyLaser = 0;
  // packed host states <-> the arena (batched upload / download)
  std::vector<long> stageOff;     // prefix sums of the systems' state sizes
  long* stageOff_d = nullptr;
  z_t* stage_d = nullptr;
  size_t stageCap = 0;
  double* tStage_d = nullptr;     // the nb step start times, contiguous, before k_set_step_times
  // device operators (trajectory 0; the others at multiples of bs)
  double *x_d = nullptr, *w_d = nullptr, *V0_d = nullptr, *T_d = nullptr, *Vint_d = nullptr, *metric_d = nullptr;
  double *metricW_d = nullptr, *metricOne_d = nullptr;  // [1 | w per orbital point] and all ones
  double *metricUser_d = nullptr;                      // caller-supplied SIL metric (single system)
  double *mask_d = nullptr;                            // absorber mask per grid point (1 = none)
  int absorbEachStep = 0, graphAbsorb = -1;
  int* btOfOrb_d = nullptr;
  int *pairL_d = nullptr, *pairK_d = nullptr, *pidx_d = nullptr;
  // CI
  z_t *h1Lin_d = nullptr, *h2Lin_d = nullptr, *rdm1Lin_d = nullptr, *rdm2Lin_d = nullptr;
  // fixed-point forms: the CI apply in double-float arithmetic, from double-float copies of h1Lin / h2Lin
  int ciDf = 0;
  // inside the NonLin time derivative: r2s from rdm2Lin and h2Lin from h2s
  // directly (the nO^4 rdm2 / h2 tensors are not formed)
  int fuseLayouts = 0;
  // SIL on OrbsLin with the three-term recurrence: the double-float one-body
  // apply emits the recurrence's first-pass partials (launch_onebody_lz)
  int fuseOrbsLinLz = 1;
  int numSms = 148;  // streaming multiprocessors of the device
  float4 *h1Df_d = nullptr, *h2Df_d = nullptr;
  float2* Tdf_d = nullptr;  // double-float copy of the kinetic band (static)
  z_t *rdm1_d = nullptr, *rdm2_d = nullptr, *h1_d = nullptr, *h2_d = nullptr;
  // mean-field
  z_t *S_d = nullptr, *W_d = nullptr;         // (nG, nPairs) row-major by grid point
  z_t *Sfull_d = nullptr, *Wfull_d = nullptr; // (nG, nOS*nOS) row-major by grid point; Wfull has a Z half
  z_t *Rp_d = nullptr;                        // (nOS^2, nOS^2) correlation matrix
  z_t *h2s_d = nullptr;                       // (nOS^2, nOS^2) spatial h2 block
  z_t *Mreg_d = nullptr;                      // (nOS, nOS)
  z_t *Uprev_d = nullptr;                     // (nOS, nOS) natural orbitals of the previous rho^-1 call
  z_t *r1s_d = nullptr;                       // spin-summed spatial rdm1
  z_t *r2s_d = nullptr;                       // spin-summed spatial rdm2 (nOS^2 x nOS^2)
  // reductions / scratch
  z_t* partial_d = nullptr;
  size_t partialCap = 0;                      // complex entries per trajectory
  int lzBlocks = 148;                         // blocks per trajectory of the Lanczos reductions
  int lzBlocksHeur = 148, lzBlocksCap = 148;  // the set-up heuristic's count and the most the partials hold
  int lzElems = 1;                            // state entries per thread and chunk in those blocks
  int redBlocks = 148;                        // blocks per trajectory of the Gram reductions
  z_t *gram_d = nullptr;                      // (nOS, nOS)
  z_t *orbTmp_d = nullptr;                    // (nG, nOS)
  double* scal_d = nullptr;                   // misc device scalars
  // state and integrators
  z_t *state_d = nullptr, *dstate_d = nullptr, *rkInc_d = nullptr, *rkTmp_d = nullptr, *rkStage_d = nullptr;
  z_t *basis_d = nullptr, *lw_d = nullptr, *trial_d = nullptr, *work_d = nullptr;
  int maxKrylov = 0;
  int krylovWindow = 0;                       // 0: full re-orthogonalisation; k: last k basis vectors
  // fixed-point form: every trajectory's grid a contiguous piece of one of a few root grids (same
  // interaction): one shared interaction matrix per root, rows/columns from fxVRow
  int fxShared = 0, fxKgMax = 0;
  std::vector<int> fxVRow, fxVRoot, fxRoots;  // per trajectory: row offset, root index; per root: trajectory
  double* lz_d = nullptr;   // Lanczos scalars: alpha, beta, dots, phi, flags
  double* lz_h = nullptr;   // pinned mirror (trajectory 0)
  // TDCI static data
  z_t* tdciOrbs_d = nullptr;
  // stream / graph
  cudaStream_t stream = nullptr;
  cudaGraphExec_t stepGraph = nullptr;
  double graphDt = 0;
  int graphKrylov = 0, graphMetric = -1, graphKernels = 0, graphProf = 0;
  size_t graphProfUsed = 0;
  // device-side time: kernels evaluate E(*timeBase + offset).  Outside a graph
  // capture the base is a device zero and the offset the absolute time; inside
  // one the base is the step-start time stepT_d that the graph advances.
  double* zero_d = nullptr;
  double* stepT_d = nullptr;
  int inCapture = 0;
  int useStepTime = 0;  // outside a capture: E(*stepT_d + t) per trajectory instead of E(t)
  double captureT0 = 0.0;
  z_t* warm_d = nullptr;
  std::string lastError;
  long launches = 0;  // kernels launched by this context (since the last reset)
  MixedBufs* mixed = nullptr;
  z_t* sysTmp_d = nullptr;  // three nG-point vectors of the Sys* entry points (first use)
  McAdjoint* mcAdj = nullptr;  // MCTDHF pulse gradient: checkpoints and work buffers (first use)
  // profiling: CUDA events around every launch of one kernel family
  int profTarget = 0;
  std::vector<cudaEvent_t> profEvents;  // start/stop pairs
  size_t profUsed = 0;
};

// Records CUDA events on the context stream around the launches of kernel
// family `id` while profiling of that family is enabled.
struct ProfScope {
  cgpu_ctx* c;
  bool on;
  ProfScope(cgpu_ctx* ctx, int id) : c(ctx), on(ctx->profTarget == id) {
    if (on) record();
  }
  ~ProfScope() {
    if (on) record();
  }
  void record() {
    if (c->profUsed >= c->profEvents.size()) {
      cudaEvent_t e;
      cudaEventCreate(&e);
      c->profEvents.push_back(e);
    }
    // inside a stream capture only an external record becomes an event-record node
    if (c->inCapture) cudaEventRecordWithFlags(c->profEvents[c->profUsed++], c->stream, cudaEventRecordExternal);
    else cudaEventRecord(c->profEvents[c->profUsed++], c->stream);
  }
};

// Launch configuration helpers: x-extent for n items per trajectory, z = nb.
inline dim3 bgrid(const cgpu_ctx* c, size_t x, unsigned y = 1) { return dim3((unsigned)(x < 1 ? 1 : x), y, c->nb); }
inline unsigned ceil_div(size_t a, size_t b) { return (unsigned)((a + b - 1) / b); }
// Blocks per trajectory of a grid-stride element-wise kernel over at most nmax
// items: enough for ~8k resident blocks in total, never more than the items need.
inline unsigned ew_blocks(const cgpu_ctx* c, size_t nmax, unsigned threads = 256) {
  size_t need = (nmax + threads - 1) / threads;
  size_t cap = (size_t)(c->nb > 1 ? (8192 / c->nb > 4 ? 8192 / c->nb : 4) : 8192);
  return (unsigned)(need < 1 ? 1 : (need < cap ? need : cap));
}
// Per-trajectory element counts stay below 2^32, so the loops index in 32 bits.
#define GRID_STRIDE(e, n) \
  for (unsigned e = blockIdx.x * blockDim.x + threadIdx.x; e < (unsigned)(n); e += gridDim.x * blockDim.x)

// Zero / copy `bytes` at p in every trajectory (strided by bs).
void batch_zero(cgpu_ctx* c, void* p, size_t bytes);
void batch_copy(cgpu_ctx* c, void* dst, const void* src, size_t bytes);

// ---------------------------------------------------------------------------
// Launchers (defined in the k_*.cu translation units).  Pointers name the
// buffers of trajectory 0; every launch covers all trajectories.
// ---------------------------------------------------------------------------
// Per-trajectory scalar slots in scal_d (64 doubles): MGS status (int), energy,
// norm, dipole, laser field, natural occupations (up to 32).
#define CODY_SCAL_STATUS 0
#define CODY_SCAL_ENERGY 8
#define CODY_SCAL_NORM 9
#define CODY_SCAL_DIPOLE 10
#define CODY_SCAL_FIELD 16
#define CODY_SCAL_OCC 24

// k_onebody.cu
void launch_onebody(cgpu_ctx* c, z_t* out, const z_t* orbs, double t, z_t alpha, int accumulate);
void launch_field(cgpu_ctx* c, double* E, double t);  // E(t) of every trajectory into its slot E
// The OrbsLin apply of Lanczos iteration j (three-term recurrence, double-float
// one-body operator) into c->lw_d, fused with the recurrence's first pass:
// partials of alpha_j and ||w'||^2 at c->partial_d (layout of k_lz3_dot).
// Returns the partial blocks per trajectory, or 0 when the fused form does not
// apply (the caller then runs the plain derivative and pass).
int launch_onebody_lz(cgpu_ctx* c, int j, double t);
// k_sys.cu: one orbital of a single-system context (the Sys* procedure pointers)
void sys_kinetic(cgpu_ctx* c, z_t* out, const z_t* in, int btBlock);
void sys_potential(cgpu_ctx* c, z_t* V, double t);
void sys_multiply(cgpu_ctx* c, z_t* out, const z_t* a, const z_t* b);
void sys_interaction_src(cgpu_ctx* c, z_t* src, const z_t* a, const z_t* b);
void sys_interaction_potential(cgpu_ctx* c, z_t* W, const z_t* src);
void launch_project_orbs(cgpu_ctx* c, z_t* dOrbs, const z_t* orbs);
void launch_project_coeffs(cgpu_ctx* c, z_t* dC, const z_t* C);
void launch_fill_h1_from(cgpu_ctx* c, const z_t* orbs, const z_t* hOrbs, z_t* h1);
void launch_axpby(cgpu_ctx* c, z_t* y, const z_t* x, z_t a, z_t b, int sel);  // y = a x + b y
void launch_rk_stage(cgpu_ctx* c, z_t* inc, z_t* tmp, const z_t* state, const z_t* d, double wInc, double wTmp,
                     int first);
void launch_scale(cgpu_ctx* c, z_t* y, z_t a, int sel);
void launch_orthonormalize(cgpu_ctx* c, z_t* orbs, int col0, int nCols, int resetStatus = 1);
void launch_norm_dipole(cgpu_ctx* c, const z_t* state);  // after the RDMs of state: norm and <x> slots
void launch_normalize_coeffs(cgpu_ctx* c, z_t* C);
void launch_energy(cgpu_ctx* c, double* out_d);
void launch_set_scalar(cgpu_ctx* c, double* p, double v);
void launch_absorber_setup(cgpu_ctx* c, double onset, double order);
void launch_absorber_apply(cgpu_ctx* c, z_t* orbs);
void launch_add_scalar(cgpu_ctx* c, double* p, double v);
size_t gram_partial_need(const cgpu_ctx* c, int n);
// k_ci.cu
void ci_build_tables(cgpu_ctx* c, SysHost& s);
void ci_build_work(cgpu_ctx* c);
void launch_ci_rdm(cgpu_ctx* c, const z_t* C, int want1, int want2);
void launch_ci_apply(cgpu_ctx* c, const z_t* C, z_t* dC, int useH1, int useH2);
void launch_fold_h1(cgpu_ctx* c);
void launch_fold_h2(cgpu_ctx* c);
// k_mf.cu
void launch_pair_potentials(cgpu_ctx* c, const z_t* orbs);
void launch_correlation(cgpu_ctx* c, z_t* dOrbs, const z_t* orbs, int wantH2);
void launch_fill_h2(cgpu_ctx* c, const z_t* orbs);
void launch_rdm_inverse(cgpu_ctx* c);
void launch_corr_epilogue(cgpu_ctx* c, z_t* dOrbs, const z_t* orbs, const z_t* Z);
void launch_h2_layout(cgpu_ctx* c);
void launch_build_vint(cgpu_ctx* c);
size_t zgemm_partial_need(const cgpu_ctx* c);
// k_mixed.cu
size_t mixed_layout(cgpu_ctx* c, char* base, size_t off);  // sizes (base == nullptr) or places the buffers
void mixed_init(cgpu_ctx* c);
void mixed_free(cgpu_ctx* c);
int mixed_error(cgpu_ctx* c);
void launch_correlation_mixed(cgpu_ctx* c, z_t* dOrbs, const z_t* orbs, int wantH2);
// Tile tuner hooks of the fixed-point contractions.  A tile table t[9] holds,
// for W = V S, Z = W R'' and h2 = S^T W in turn: N-tile width, compact (two
// CTAs per SM) flag, K splits.  fx_tiles_get returns false outside the
// fixed-point forms; fx_tiles_set validates and rebuilds the tile lists;
// fx_time_contraction times GEMM g (with its K-split reduction) on the
// operands in the arena, ms per launch.
bool fx_tiles_get(const cgpu_ctx* c, int* t);
void fx_tiles_set(cgpu_ctx* c, const int* t);
void fx_tile_candidates(const cgpu_ctx* c, int g, std::vector<std::array<int, 3>>& out);
double fx_time_contraction(cgpu_ctx* c, int g, int reps);
// ctx.cu: device ms of the Lanczos family over one fixed-order SIL half step
// (OrbsLin, krylov vectors) on a scratch copy of the resident states; drops the
// captured step graph (tile and block choices are baked into it).
double time_sil_lanczos(cgpu_ctx* c, int krylov);
void drop_step_graph(cgpu_ctx* c);
// ctx.cu: the time derivative `which` of every trajectory's state `in` into `out`.
void td_device_public(cgpu_ctx* c, int which, z_t* out, const z_t* in, double t);
// autotune.cu: the tile table t[10] (fx_tiles_get's nine entries, zero outside
// the fixed-point forms, then the Lanczos blocks per trajectory), and the tuner.
void tiles_get(const cgpu_ctx* c, int* t);
void tiles_set(cgpu_ctx* c, const int* t);
void autotune_run(cgpu_ctx* c, const char* cachePath, int force, std::string& report);
// k_adjoint_mc.cu: the MCTDHF pulse gradient (host states, field[nT]); the
// forward keeps checkpoints in the context for the backward sweep.
void mc_adjoint_forward(cgpu_ctx* c, const z_t* state0_h, const z_t* ref_h, const double* field_h, int nT, double dt,
                        int K, int checkpoint, double* J, double* overlap, z_t* final_h);
void mc_adjoint_backward(cgpu_ctx* c, double* grad_h);
void mc_adjoint_free(cgpu_ctx* c);
// k_adjoint.cu
void adjoint_tdci(cgpu_ctx* c, const z_t* C0_h, const double* E_h, int nT, double dt, int K, double* J,
                  double* aOut, z_t* CN_h, double* grad_h);
// k_lanczos.cu
// The SIL kernels work on c->basis_d, c->lw_d (H v_j), c->work_d (start vector),
// c->metric_d (current metric) and the scalar block c->lz_d.
void launch_lanczos_start(cgpu_ctx* c, const z_t* v);
// pass1Blocks > 0: the three-term pass-1 partials (alpha, ||w'||^2) were
// emitted by launch_onebody_lz with that many blocks per trajectory
void launch_lanczos_update(cgpu_ctx* c, int j, int maxDim, int pass1Blocks = 0);
void launch_lanczos_tail(cgpu_ctx* c, int j, double dt, int evalExp);  // j = 0: use the device mDim
void launch_lanczos_combine(cgpu_ctx* c, z_t* out, const z_t* start);
void launch_lz_set(cgpu_ctx* c, int idx, double v);
size_t lanczos_partial_need(const cgpu_ctx* c);
#define CODY_LZ_BETA 64
#define CODY_LZ_S 400
#define CODY_LZ_ERR 385
#define CODY_LZ_MDIM 386
#define CODY_LZ_DONE 387
#define CODY_LZ_BREAKJ 390

// error helpers
#define CODY_CUDA(call)                                                                              \
  do {                                                                                                \
    cudaError_t e_ = (call);                                                                          \
    if (e_ != cudaSuccess) throw std::string(#call) + ": " + cudaGetErrorString(e_);                  \
  } while (0)

#define CODY_LAUNCHED(c) \
  do {                   \
    (c)->launches++;     \
    CODY_CUDA(cudaGetLastError()); \
  } while (0)

#define TRAJ_ARGS const TrajShape* __restrict__ shp, size_t bs
#define TRAJ_PASS(c) (c)->shape_d, (c)->bs
