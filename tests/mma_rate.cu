// Issue-rate probe of tcgen05.mma (kind::f16, bf16 operands from shared
// memory, FP32 accumulators in tensor memory, M = 128, K = 16 per instruction)
// on one SM: cycles per MMA for a range of N, for one accumulator and for
// accumulators taken in turn.  The fixed-point GEMM's tile widths are chosen
// against these rates.  Run by tests/test_gpu_mma_rate.py; prints one JSON line.
//
// One CTA of 128 threads; thread 0 issues; every wait is bounded, and the
// tensor memory is freed on every path.  The operand tiles are zero (the rate
// does not depend on the values).
#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>

namespace {

__device__ __forceinline__ uint32_t su32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// K-major, 128-byte swizzle, 8-row atoms of 1024 bytes
__device__ __forceinline__ uint64_t sw128(uint32_t saddr) {
  return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((uint64_t)1 << 16) | ((uint64_t)(1024 >> 4) << 32) |
         ((uint64_t)1 << 46) | ((uint64_t)2 << 61);
}

__device__ __forceinline__ void mma(uint32_t d, uint64_t a, uint64_t b, uint32_t id, uint32_t acc) {
  asm volatile("{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d),
               "l"(a), "l"(b), "r"(id), "r"(acc)
               : "memory");
}

// mode 0: every MMA into one accumulator; mode 1: two accumulators in turn
// (N columns apart); mode 2: groups of four MMAs (one per 16-wide K step) per
// accumulator, two accumulators in turn.
__global__ void k_rate(int N, int reps, int mode, long long* out) {
  extern __shared__ uint8_t smRaw[];
  uint8_t* sm = (uint8_t*)(((uintptr_t)smRaw + 1023) & ~(uintptr_t)1023);
  uint8_t* A = sm;          // 128 rows x 128 bytes
  uint8_t* B = sm + 16384;  // up to 256 rows x 128 bytes
  __shared__ __align__(8) uint64_t bar;
  __shared__ uint32_t slot;
  for (int i = threadIdx.x; i < (16384 + 32768) / 16; i += blockDim.x) ((int4*)sm)[i] = make_int4(0, 0, 0, 0);
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(su32(&bar)) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (threadIdx.x < 32) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 512;" ::"r"(su32(&slot)) : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = slot;
  if (threadIdx.x == 0) {
    const uint32_t id = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(128 >> 4) << 24);
    const uint64_t ad = sw128(su32(A)), bd = sw128(su32(B));
    const long long t0 = clock64();
    if (mode == 0) {
      for (int r = 0; r < reps; r++) mma(tmem, ad + 2 * (r & 3), bd + 2 * (r & 3), id, r > 0);
    } else if (mode == 1) {
      for (int r = 0; r < reps; r += 8)
        for (int k = 0; k < 4; k++) {
          mma(tmem, ad + 2 * k, bd + 2 * k, id, r > 0 || k > 0);
          mma(tmem + (uint32_t)N, ad + 2 * k, bd + 2 * k, id, r > 0 || k > 0);
        }
    } else {
      for (int r = 0; r < reps; r += 8)
        for (int g = 0; g < 2; g++)
          for (int k = 0; k < 4; k++) mma(tmem + (uint32_t)(g * N), ad + 2 * k, bd + 2 * k, id, r > 0 || k > 0);
    }
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(su32(&bar))
                 : "memory");
    uint32_t ok = 0;
    const long long tw = clock64();
    while (!ok && clock64() - tw < 2000000000LL)
      asm volatile(
          "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], 0;\n selp.u32 %0, 1, 0, p;\n}\n"
          : "=r"(ok)
          : "r"(su32(&bar))
          : "memory");
    out[0] = ok ? clock64() - t0 : -1;
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  if (threadIdx.x < 32) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 512;" ::"r"(tmem) : "memory");
}

}  // namespace

int main() {
  long long* d = nullptr;
  if (cudaMalloc(&d, 8) != cudaSuccess) return 1;
  const int smem = 16384 + 32768 + 1024, reps = 4096;
  cudaFuncSetAttribute(k_rate, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  struct Case {
    int mode, N;
  };
  const Case cases[] = {{0, 16},  {0, 32},  {0, 48},  {0, 64},  {0, 80}, {0, 96}, {0, 112}, {0, 128},
                        {0, 160}, {0, 192}, {0, 256}, {1, 80},  {1, 128}, {2, 80}, {2, 128}};
  std::printf("{\"peak_ops_per_cycle\": 8192, \"rows\": [");
  bool first = true;
  for (const Case& cs : cases) {
    long long c = 0;
    for (int rep = 0; rep < 2; rep++) k_rate<<<1, 128, smem>>>(cs.N, reps, cs.mode, d);  // the first warms up
    if (cudaDeviceSynchronize() != cudaSuccess) return 2;
    cudaMemcpy(&c, d, 8, cudaMemcpyDeviceToHost);
    if (c <= 0) return 3;
    const double per = (double)c / reps, ideal = cs.N * 128.0 * 16 * 2 / 8192;
    std::printf("%s{\"mode\": %d, \"n\": %d, \"cycles_per_mma\": %.2f, \"ideal\": %.2f, \"efficiency\": %.3f}",
                first ? "" : ", ", cs.mode, cs.N, per, ideal, ideal / per);
    first = false;
  }
  std::printf("]}\n");
  cudaFree(d);
  return 0;
}
