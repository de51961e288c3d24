// noalloc.cu -- weighted Gram matrix without any device allocation.
//
// Some callers cannot call cudaMalloc at the point where they need this
// reduction.  Examples: a Fortran host program whose device memory pool is
// owned and pre-sized by another component, or code that runs while device
// allocation is forbidden (inside a region being recorded into a CUDA graph,
// or in a real-time loop that must not touch the allocator).  They still own
// their input and output buffers, but they cannot give the library a
// temporary one.  This entry point therefore keeps its per-block partial sums
// in a file-scope __device__ array.  The array is part of the module image:
// every GPU that loads the library holds it (1 MiB) until the process exits.
//
// Computed quantity (the Grid_InnerProduct matrix of two orbital sets):
//   gram(i, j) = sum_g conj(a[g + n_grid*i]) * b[g + n_grid*j] * weights[g],
//   for 0 <= i, j < n_cols, stored column-major (n_cols x n_cols).
#include <mutex>

#include "common.cuh"

#define CGPU_GRAM_NOALLOC_MAX_COLS 32
#define CGPU_GRAM_NOALLOC_BLOCKS 64
#define CGPU_GRAM_NOALLOC_CHUNK 32

// Partial sums of at most CGPU_GRAM_NOALLOC_BLOCKS blocks, each n_cols^2 entries.
static __device__ __align__(256) double2
    g_gram_scratch[CGPU_GRAM_NOALLOC_BLOCKS * CGPU_GRAM_NOALLOC_MAX_COLS * CGPU_GRAM_NOALLOC_MAX_COLS];

void cody_record_global_error(const std::string& msg);

namespace {

constexpr int kMaxDevices = 64;
std::mutex g_scratchMutex;
void* g_scratchAddr[kMaxDevices] = {nullptr};  // device address of g_gram_scratch, per device ordinal

// The host-side name g_gram_scratch is only a stand-in for the device array;
// its device address is looked up once per device, with that device current,
// and kept for the life of the process.  A host that destroys and re-creates
// the device's primary context (cudaDeviceReset) reloads the module at a new
// address: calls after such a reset are not supported.
cudaError_t scratch_address(void** out) {
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(g_scratchMutex);
  if (!g_scratchAddr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_gram_scratch);
    if (e != cudaSuccess) return e;
    g_scratchAddr[dev] = p;
  }
  *out = g_scratchAddr[dev];
  return cudaSuccess;
}

__global__ void k_gram_noalloc_partial(double2* __restrict__ part, const double2* __restrict__ A,
                                       const double2* __restrict__ B, const double* __restrict__ w, int nG, int n,
                                       int chunk) {
  extern __shared__ double2 sh[];
  double2* sa = sh;
  double2* sb = sh + chunk * n;
  int nn = n * n;
  double2 acc[4];
  for (int q = 0; q < 4; q++) acc[q] = make_double2(0.0, 0.0);
  for (int c0 = blockIdx.x * chunk; c0 < nG; c0 += gridDim.x * chunk) {
    __syncthreads();
    for (int t = threadIdx.x; t < chunk * n; t += blockDim.x) {
      int col = t / chunk, r = t % chunk;
      int g = c0 + r;
      double2 a = make_double2(0.0, 0.0), b = make_double2(0.0, 0.0);
      if (g < nG) {
        a = A[(size_t)nG * col + g];
        b = B[(size_t)nG * col + g];
        b = make_double2(b.x * w[g], b.y * w[g]);
      }
      sa[r * n + col] = a;
      sb[r * n + col] = b;
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < 4; q++) {
      int e = threadIdx.x + q * blockDim.x;
      if (e >= nn) break;
      int ii = e % n, jj = e / n;
      double2 s = acc[q];
      for (int r = 0; r < chunk; r++) {
        double2 a = sa[r * n + ii], b = sb[r * n + jj];
        s.x += a.x * b.x + a.y * b.y;
        s.y += a.x * b.y - a.y * b.x;
      }
      acc[q] = s;
    }
  }
#pragma unroll
  for (int q = 0; q < 4; q++) {
    int e = threadIdx.x + q * blockDim.x;
    if (e >= nn) break;
    part[(size_t)blockIdx.x * nn + e] = acc[q];
  }
}

__global__ void k_gram_noalloc_final(double2* __restrict__ G, const double2* __restrict__ part, int nBlk, int n) {
  int e = blockIdx.x * blockDim.x + threadIdx.x;
  int nn = n * n;
  if (e >= nn) return;
  double2 s = make_double2(0.0, 0.0);
  for (int b = 0; b < nBlk; b++) {
    double2 p = part[(size_t)b * nn + e];
    s.x += p.x;
    s.y += p.y;
  }
  G[e] = s;
}

int fail_noalloc(const std::string& msg, int code) {
  cody_record_global_error(msg);
  return code;
}

}  // namespace

extern "C" int cgpu_weighted_gram_noalloc(const cgpu_complex* a, const cgpu_complex* b, const double* weights,
                                          int n_grid, int n_cols, cgpu_complex* gram, void* stream) {
  if (!a || !b || !weights || !gram) return fail_noalloc("cgpu_weighted_gram_noalloc: null device pointer", CGPU_ERR_ARG);
  if (n_grid < 1) return fail_noalloc("cgpu_weighted_gram_noalloc: n_grid must be >= 1", CGPU_ERR_ARG);
  if (n_cols < 1 || n_cols > CGPU_GRAM_NOALLOC_MAX_COLS)
    return fail_noalloc("cgpu_weighted_gram_noalloc: n_cols must be in 1..32 (the fixed scratch holds 64 blocks of "
                        "32x32 partial sums)",
                        CGPU_ERR_ARG);
  void* scratch = nullptr;
  cudaError_t e = scratch_address(&scratch);
  if (e != cudaSuccess)
    return fail_noalloc(std::string("cgpu_weighted_gram_noalloc: cudaGetSymbolAddress: ") + cudaGetErrorString(e),
                        CGPU_ERR_CUDA);
  // An error left by earlier, unrelated work on this thread is reported as
  // such and left in place for its owner (cudaGetLastError below would clear it).
  e = cudaPeekAtLastError();
  if (e != cudaSuccess)
    return fail_noalloc(std::string("cgpu_weighted_gram_noalloc: a CUDA error was pending before the call: ") +
                            cudaGetErrorString(e),
                        CGPU_ERR_CUDA);
  cudaStream_t s = (cudaStream_t)stream;
  int chunk = CGPU_GRAM_NOALLOC_CHUNK;
  if (chunk * n_cols > 1024) chunk = 1024 / n_cols;
  int nBlk = (n_grid + chunk - 1) / chunk;
  if (nBlk > CGPU_GRAM_NOALLOC_BLOCKS) nBlk = CGPU_GRAM_NOALLOC_BLOCKS;
  size_t sh = 2 * sizeof(double2) * chunk * n_cols;
  // Every scratch slot the final kernel reads is written by the partial kernel
  // of the same call, so nothing in the array has to start at zero.
  k_gram_noalloc_partial<<<nBlk, 256, sh, s>>>((double2*)scratch, (const double2*)a, (const double2*)b, weights,
                                                n_grid, n_cols, chunk);
  int nn = n_cols * n_cols;
  k_gram_noalloc_final<<<(nn + 127) / 128, 128, 0, s>>>((double2*)gram, (const double2*)scratch, nBlk, n_cols);
  e = cudaGetLastError();
  if (e != cudaSuccess)
    return fail_noalloc(std::string("cgpu_weighted_gram_noalloc: launch: ") + cudaGetErrorString(e), CGPU_ERR_CUDA);
  return CGPU_OK;
}
