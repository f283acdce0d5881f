// C ABI: the FP64 pipe rate probe (roofline denominator).
//
// Part of the abi.cu translation unit (included at its end): it uses that file's error
// helpers and is not compiled on its own.
#pragma once

// ---------------------------------------------------------------------------------------------
// FP64 pipe rate.
//
// The sweeps are bound by the FP64 pipe, whose rate on this part is far below the tensor
// cores' and is not among the measured peaks. This probe measures it: every thread of a
// full grid runs kProbeChains independent dependent chains of one FP64 instruction kind (DFMA,
// DADD or DMUL), so the pipe, not the 64-cycle dependent latency, is the limit. The result is
// thread-level FP64 instructions per second (a DFMA counts once, as in the sweeps' structural
// counts); the best of several timed launches is reported.
// ---------------------------------------------------------------------------------------------
namespace {

constexpr int kProbeChains = 8;
constexpr int kProbeIters = 2048;
constexpr int kProbeThreads = 256;
constexpr int kProbeCtasPerSm = 8;

__device__ double g_probe_sink;

__device__ __forceinline__ double probe_fma(double a, double b, double c) {
  double r;
  asm volatile("fma.rn.f64 %0, %1, %2, %3;" : "=d"(r) : "d"(a), "d"(b), "d"(c));
  return r;
}

// KIND 0 DFMA, 1 DADD, 2 DMUL, 3 a product issued as DFMA (x*a + m, m = -0 from a kernel
// argument), 4 a sum issued as DFMA (x*u + b, u = 1 from a kernel argument)
template <int KIND>
__global__ void __launch_bounds__(kProbeThreads) k_fp64_rate(double a, double b, double u,
                                                             double m) {
  double x[kProbeChains];
#pragma unroll
  for (int c = 0; c < kProbeChains; ++c) x[c] = 1.0 + 1e-3 * (threadIdx.x + c);
#pragma unroll 1
  for (int it = 0; it < kProbeIters; ++it) {
#pragma unroll
    for (int c = 0; c < kProbeChains; ++c) {
      if (KIND == 0) x[c] = __fma_rn(x[c], a, b);
      else if (KIND == 1) x[c] = __dadd_rn(x[c], b);
      else if (KIND == 2) x[c] = __dmul_rn(x[c], a);
      else if (KIND == 3) x[c] = probe_fma(x[c], a, m);
      else x[c] = probe_fma(x[c], u, b);
    }
  }
  double s = 0.0;
#pragma unroll
  for (int c = 0; c < kProbeChains; ++c) s += x[c];
  // never true for the chains above (every x stays near 1); the comparison keeps the work of
  // every thread from being optimised away
  if (s == -1.0) g_probe_sink = s;
}

}  // namespace

extern "C" {

CASADI_GB300_API int casadi_gb300_fp64_rate(int kind, int reps, double* instr_per_s) {
  if (!instr_per_s || kind < 0 || kind > 4 || reps < 1 || reps > 100)
    return fail(CASADI_GB300_ERR_ARG, "fp64_rate: kind 0..4, reps 1..100, result pointer");
  int dev = 0, sms = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
  e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return cuda_fail(e, "cudaDeviceGetAttribute");
  const int grid = sms * kProbeCtasPerSm;
  // a chain step keeps x finite and near 1 for every kind: x*a + b with a = 1 - 2^-20,
  // b = 2^-20; x + b grows by 2^-20 per step; x*a decays by that factor
  const double a = 1.0 - 0x1p-20, b = 0x1p-20;
  cudaStream_t s = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if ((e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking)) != cudaSuccess ||
      (e = cudaEventCreate(&e0)) != cudaSuccess || (e = cudaEventCreate(&e1)) != cudaSuccess) {
    if (s) cudaStreamDestroy(s);
    if (e0) cudaEventDestroy(e0);
    return cuda_fail(e, "fp64_rate set-up");
  }
  auto launch = [&]() {
    const double u = 1.0, m = -0.0;
    switch (kind) {
      case 0: k_fp64_rate<0><<<grid, kProbeThreads, 0, s>>>(a, b, u, m); break;
      case 1: k_fp64_rate<1><<<grid, kProbeThreads, 0, s>>>(a, b, u, m); break;
      case 2: k_fp64_rate<2><<<grid, kProbeThreads, 0, s>>>(a, b, u, m); break;
      case 3: k_fp64_rate<3><<<grid, kProbeThreads, 0, s>>>(a, b, u, m); break;
      default: k_fp64_rate<4><<<grid, kProbeThreads, 0, s>>>(a, b, u, m); break;
    }
    return cudaGetLastError();
  };
  float best_ms = 0.0f;
  e = launch();  // warm-up
  for (int r = 0; r < reps && e == cudaSuccess; ++r) {
    if ((e = cudaEventRecord(e0, s)) != cudaSuccess) break;
    if ((e = launch()) != cudaSuccess) break;
    if ((e = cudaEventRecord(e1, s)) != cudaSuccess) break;
    if ((e = cudaEventSynchronize(e1)) != cudaSuccess) break;
    float ms = 0.0f;
    if ((e = cudaEventElapsedTime(&ms, e0, e1)) != cudaSuccess) break;
    if (r == 0 || ms < best_ms) best_ms = ms;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaStreamDestroy(s);
  if (e != cudaSuccess) return cuda_fail(e, "fp64_rate launch");
  const double instr = static_cast<double>(grid) * kProbeThreads * kProbeIters * kProbeChains;
  *instr_per_s = instr / (best_ms * 1e-3);
  return 0;
}

}  // extern "C"
