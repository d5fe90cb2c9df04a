// tcgen05_mma_rate.cu -- rate of single-CTA tcgen05.mma (M = 128, K = 32
// bytes: 16 f16 or 32 e4m3 elements) on operands resident in shared memory,
// as the tensor-core scans issue it. One CTA per SM; thread 0 issues `iters`
// groups of `per_group` MMAs into TMEM buffer (group & 1) * N, commits every
// `groups_per_commit` groups and waits for that commit (bounded wait), so the
// lines measure back-to-back issue (one commit at the end) against the
// commit -> wait -> issue chain of a scan whose next tile needs the
// accumulator buffer the MMA is filling. Prints one JSON line per setting:
// cycles per MMA (clock64 on the issuing thread) and the whole-GPU rate.
// Not part of the library: built and run on its own,
//   nvcc -gencode arch=compute_103a,code=sm_103a -O3 -std=c++17 \
//        -Iflashvector-gpu_gb300/csrc -o /tmp/tcgen05_mma_rate \
//        flashvector-gpu_gb300/microbench/tcgen05_mma_rate.cu -lcuda
#include <cstdio>
#include <cstdlib>
#include <vector>
#include "tc_ptx.cuh"
using namespace fv;

template <bool FP8, int N>
__global__ void __launch_bounds__(128, 1) mma_bench(int iters, int per_group, int groups_per_commit,
                                                    unsigned long long* out, uint32_t* status) {
  extern __shared__ uint8_t smem_raw[];
  uint8_t* sm = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
  uint8_t* sA = sm;              // 128 rows x 128 B
  uint8_t* sB = sm + 16384;      // 256 rows x 128 B
  __shared__ uint64_t bar;
  __shared__ uint32_t tmem_slot;
  __shared__ uint32_t abort_flag;
  for (int i = threadIdx.x; i < 49152 / 4; i += blockDim.x)
    reinterpret_cast<uint32_t*>(sm)[i] = 0x3C3A3836u ^ (uint32_t)(i * 2654435761u & 0x07070707u);
  if (threadIdx.x == 0) {
    tc::mbar_init(&bar, 1);
    abort_flag = 0;
    tc::fence_mbar_init();
  }
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  if (threadIdx.x < 32) {
    tc::tmem_alloc(&tmem_slot, 512);
    tc::tc_fence_before();
  }
  __syncthreads();
  tc::tc_fence_after();
  const uint32_t tmem = tmem_slot;
  if (threadIdx.x == 0) {
    constexpr uint32_t idesc = tc::idesc_f32acc(0, 0, 128, N);
    const uint32_t a_base = tc::smem_addr(sA), b_base = tc::smem_addr(sB);
    uint32_t phase = 0;
    const long long t0 = clock64();
    for (int g = 0; g < iters; ++g) {
      const uint32_t d = tmem + (uint32_t)(g & 1) * N;
      for (int kk = 0; kk < per_group; ++kk)
        tc::mma<FP8>(d, tc::sdesc_k_sw128(a_base + (kk & 3) * 32), tc::sdesc_k_sw128(b_base + (kk & 3) * 32), idesc,
                     kk != 0);
      if ((g + 1) % groups_per_commit == 0 || g + 1 == iters) {
        tc::mma_commit(&bar);
        if (!tc::mbar_wait(&bar, phase, (volatile uint32_t*)&abort_flag, status, 2000000000ull)) break;
        phase ^= 1;
      }
    }
    const long long t1 = clock64();
    out[blockIdx.x] = (unsigned long long)(t1 - t0);
  }
  __syncthreads();
  if (threadIdx.x < 32) {
    tc::tc_fence_after();
    tc::tmem_dealloc(tmem, 512);
  }
}

template <bool FP8, int N>
void run(const char* name, int iters, int per_group, int gpc, int sms, unsigned long long* d_out, uint32_t* d_status) {
  auto k = mma_bench<FP8, N>;
  const int smem = 49152 + 1024 + 64 * 1024;  // extra to keep one CTA per SM
  cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  k<<<sms, 128, smem>>>(iters, per_group, gpc, d_out, d_status);
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  cudaEventRecord(e0);
  k<<<sms, 128, smem>>>(iters, per_group, gpc, d_out, d_status);
  cudaEventRecord(e1);
  cudaError_t err = cudaDeviceSynchronize();
  float ms = 0;
  cudaEventElapsedTime(&ms, e0, e1);
  std::vector<unsigned long long> h(sms);
  cudaMemcpy(h.data(), d_out, sms * 8, cudaMemcpyDeviceToHost);
  uint32_t st = 0;
  cudaMemcpy(&st, d_status, 4, cudaMemcpyDeviceToHost);
  double avg = 0;
  for (auto v : h) avg += (double)v;
  avg /= sms;
  const double mmas = (double)iters * per_group;
  const double macs = 128.0 * N * (FP8 ? 32 : 16);
  printf("{\"name\": \"%s\", \"N\": %d, \"per_group\": %d, \"groups_per_commit\": %d, \"cycles_per_mma\": %.1f, "
         "\"mac_per_cycle\": %.0f, \"ms\": %.3f, \"tflops\": %.1f, \"status\": %u, \"err\": %d}\n",
         name, N, per_group, gpc, avg / mmas, macs * mmas / avg, ms, 2.0 * macs * mmas * sms / (ms * 1e-3) / 1e12, st,
         (int)err);
  fflush(stdout);
}

int main() {
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, 0);
  unsigned long long* d_out;
  uint32_t* d_status;
  cudaMalloc(&d_out, sms * 8);
  cudaMalloc(&d_status, 4);
  cudaMemset(d_status, 0, 4);
  const int iters = 20000;
  for (int gpc : {1, 2, 1000000}) {
    run<true, 256>("fp8", iters, 4, gpc, sms, d_out, d_status);
    run<true, 128>("fp8", iters, 4, gpc, sms, d_out, d_status);
    run<true, 64>("fp8", iters, 4, gpc, sms, d_out, d_status);
    run<false, 256>("f16", iters, 4, gpc, sms, d_out, d_status);
    run<false, 128>("f16", iters, 4, gpc, sms, d_out, d_status);
  }
  run<true, 256>("fp8", iters / 4, 16, 1, sms, d_out, d_status);
  run<false, 256>("f16", iters / 4, 16, 1, sms, d_out, d_status);
  return 0;
}
