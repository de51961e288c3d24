// k_sys.cu -- the per-orbital operators of the Sys* procedure pointers, for a
// Fortran configuration that moves only sysKinetic, sysPotential or
// sysInteraction to the GPU and keeps the rest of the method on the host:
//   SysKinetic_MultiplyWithKineticOp            (src/SysKinetic/M_SysKinetic.f90:141-160)
//   SysPotential_FillExternalPotential / Multiply (src/SysPotential/M_SysPotential.f90:71-101)
//   SysInteraction_FillInteractionSrc / FillInteractionPotential / Multiply
//                                                (src/SysInteraction/M_SysInteraction.f90:94-157)
// They work on one orbital (nG points) of a single-system context, with the
// context's device operators: the banded kinetic rows (FEDVR element blocks
// or the 8th-order finite-difference stencil, scaled by the body mass), the
// nuclear potential V0 plus the 1D length-gauge laser E(t) x, and the
// interaction matrix K(x_i, x_j).
#include "common.cuh"

namespace {

constexpr int SYS_THREADS = 256;

// out = T in for one orbital: the band of body-type block Tb (nd diagonals).
__global__ void k_sys_kinetic(z_t* __restrict__ out, const z_t* __restrict__ in, const double* __restrict__ Tb, int nG,
                              int band) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= nG) return;
  const int nd = 2 * band + 1;
  z_t acc = zmk(0.0, 0.0);
  for (int d = 0; d < nd; d++) {
    const int gg = g - band + d;
    if (gg < 0 || gg >= nG) continue;
    const double c = Tb[(size_t)d * nG + g];
    acc.x = fma(c, in[gg].x, acc.x);
    acc.y = fma(c, in[gg].y, acc.y);
  }
  out[g] = acc;
}

// V(x, t) = V0(x) + E(t) x as complex values.
__global__ void k_sys_potential(z_t* __restrict__ V, const double* __restrict__ V0, const double* __restrict__ x,
                                const double* __restrict__ E, int nG) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g < nG) V[g] = zmk(fma(*E, x[g], V0[g]), 0.0);
}

// out = a * b point by point.
__global__ void k_sys_mul(z_t* __restrict__ out, const z_t* __restrict__ a, const z_t* __restrict__ b, int nG) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g < nG) out[g] = zmul(a[g], b[g]);
}

// src = conj(a) b w (FillInteractionSrc of the linear grids).
__global__ void k_sys_src(z_t* __restrict__ src, const z_t* __restrict__ a, const z_t* __restrict__ b,
                          const double* __restrict__ w, int nG) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g < nG) src[g] = zscale(zcmul(a[g], b[g]), w[g]);
}

// W(x_i) = sum_j K(x_i, x_j) src_j: one warp per row, fixed-order lane sums.
__global__ void k_sys_interaction(z_t* __restrict__ W, const double* __restrict__ K, const z_t* __restrict__ src,
                                  int nG) {
  const int row = blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5), lane = threadIdx.x & 31;
  if (row >= nG) return;
  const double* Kr = K + (size_t)row * nG;
  z_t s = zmk(0.0, 0.0);
  for (int j = lane; j < nG; j += 32) {
    s.x = fma(Kr[j], src[j].x, s.x);
    s.y = fma(Kr[j], src[j].y, s.y);
  }
  for (int o = 16; o > 0; o >>= 1) {
    s.x += __shfl_xor_sync(0xffffffffu, s.x, o);
    s.y += __shfl_xor_sync(0xffffffffu, s.y, o);
  }
  if (lane == 0) W[row] = s;
}

unsigned blocks(int n) { return (unsigned)((n + SYS_THREADS - 1) / SYS_THREADS); }

}  // namespace

void sys_kinetic(cgpu_ctx* c, z_t* out, const z_t* in, int btBlock) {
  k_sys_kinetic<<<blocks(c->nG), SYS_THREADS, 0, c->stream>>>(out, in, c->T_d + (size_t)btBlock * (2 * c->band + 1) *
                                                                                   c->nG,
                                                               c->nG, c->band);
  CODY_LAUNCHED(c);
}

void sys_potential(cgpu_ctx* c, z_t* V, double t) {
  double* E = c->scal_d + CODY_SCAL_FIELD;
  launch_field(c, E, t);
  k_sys_potential<<<blocks(c->nG), SYS_THREADS, 0, c->stream>>>(V, c->V0_d, c->x_d, E, c->nG);
  CODY_LAUNCHED(c);
}

void sys_multiply(cgpu_ctx* c, z_t* out, const z_t* a, const z_t* b) {
  k_sys_mul<<<blocks(c->nG), SYS_THREADS, 0, c->stream>>>(out, a, b, c->nG);
  CODY_LAUNCHED(c);
}

void sys_interaction_src(cgpu_ctx* c, z_t* src, const z_t* a, const z_t* b) {
  k_sys_src<<<blocks(c->nG), SYS_THREADS, 0, c->stream>>>(src, a, b, c->w_d, c->nG);
  CODY_LAUNCHED(c);
}

void sys_interaction_potential(cgpu_ctx* c, z_t* W, const z_t* src) {
  k_sys_interaction<<<(unsigned)((c->nG + 7) / 8), 256, 0, c->stream>>>(W, c->Vint_d, src, c->nG);
  CODY_LAUNCHED(c);
}
