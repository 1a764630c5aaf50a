// Measured FP64 issue rate of this GPU, the denominator of the FP64 roofline.
//
// The FP64 form of the PM step is bound by the FP64 pipe, not by HBM: GB300
// issues FP64 at a small fraction of its FP32 rate.  Its achieved FP64 rate is
// reported against the rate this probe measures on the same GPU: every thread
// runs independent chains of dependent FP64 fused multiply-adds (8 or 16 chains,
// 4 or 8 blocks of 256 threads per SM: the best of the four shapes), timed with
// CUDA events on the context's stream; then the same with FP64 additions, whose
// rate is reported beside it (the stencil kernels are mostly additions).
// The chains converge (a -> a b + c with 0 < b < 1), so no value overflows or
// turns subnormal; the sum is stored only if it equals a value it never takes,
// which keeps the compiler from removing the work without a store per thread.
#include "pm_common.cuh"

#include <algorithm>
#include <cstring>

namespace nyxpm {

namespace {

constexpr int kProbeThreads = 256;

__device__ double g_probe_sink;

// ADD: chains of dependent FP64 additions a -> a + c instead (c tiny: no overflow)
template <int CHAINS, bool ADD>
__global__ void __launch_bounds__(kProbeThreads) k_fp64_fma_probe(int iters, double b, double c,
                                                                   double never)
{
    double a[CHAINS];
#pragma unroll
    for (int t = 0; t < CHAINS; ++t) a[t] = 1e-3 * (threadIdx.x + t);
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int t = 0; t < CHAINS; ++t) a[t] = ADD ? a[t] + c : fma(a[t], b, c);
    }
    double s = 0.0;
#pragma unroll
    for (int t = 0; t < CHAINS; ++t) s = s + a[t];
    if (s == never) g_probe_sink = s;
}

}  // namespace

}  // namespace nyxpm

using namespace nyxpm;

extern "C" nyxpm_status nyxpm_measure_fp64_peak(nyxpm_ctx* c, double* tflops, double* add_tops)
{
    if (!c || !tflops) return NYXPM_INVALID_ARG;
    cudaSetDevice(c->p.device);
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) {
        cudaGetLastError();
        if (e0) cudaEventDestroy(e0);
        c->err = "cudaEventCreate";
        return NYXPM_CUDA_ERROR;
    }
    double best_fma = 0.0, best_add = 0.0;   // operations (FMAs or adds) per second
    nyxpm_status st = NYXPM_OK;
    for (int shape = 0; shape < 8 && st == NYXPM_OK; ++shape) {
        const int chains = shape & 1 ? 16 : 8;
        const int blocks = std::max(1, c->sm_count) * (shape & 2 ? 8 : 4);
        const bool add = (shape & 4) != 0;
        // about the same work per shape (~10 ms at 0.5 T operations/s)
        const int iters = (shape & 1 ? 4096 : 8192) / (shape & 2 ? 2 : 1);
        for (int rep = 0; rep < 4 && st == NYXPM_OK; ++rep) {   // the first run warms up
            cudaEventRecord(e0, c->stream);
            if (chains == 16 && add)
                k_fp64_fma_probe<16, true><<<blocks, kProbeThreads, 0, c->stream>>>(iters, 0.999999, 1e-300, -1.0);
            else if (chains == 16)
                k_fp64_fma_probe<16, false><<<blocks, kProbeThreads, 0, c->stream>>>(iters, 0.999999, 1e-7, -1.0);
            else if (add)
                k_fp64_fma_probe<8, true><<<blocks, kProbeThreads, 0, c->stream>>>(iters, 0.999999, 1e-300, -1.0);
            else
                k_fp64_fma_probe<8, false><<<blocks, kProbeThreads, 0, c->stream>>>(iters, 0.999999, 1e-7, -1.0);
            cudaEventRecord(e1, c->stream);
            c->launches += 1;
            st = check_launch(*c, "fp64 probe");
            if (st == NYXPM_OK && cudaEventSynchronize(e1) != cudaSuccess) st = check_launch(*c, "fp64 probe");
            float ms = 0.f;
            if (st == NYXPM_OK && rep > 0 && cudaEventElapsedTime(&ms, e0, e1) == cudaSuccess && ms > 0) {
                const double ops = (double)chains * (double)iters * (double)blocks * kProbeThreads;
                double& best = add ? best_add : best_fma;
                best = std::max(best, ops / (ms * 1e-3) / 1e12);
            }
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (st != NYXPM_OK) return st;
    if (!(best_fma > 0) || !(best_add > 0)) {
        c->err = "fp64 probe: no timing";
        return NYXPM_CUDA_ERROR;
    }
    *tflops = 2.0 * best_fma;
    if (add_tops) *add_tops = best_add;
    return NYXPM_OK;
}
