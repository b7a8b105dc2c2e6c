// calib.cu — the FP64 fused multiply-add rate of this GPU, measured by a microkernel: the
// denominator of the FP64 step's compute roofline (the FP64 path is bound by the FP64 pipe, not by
// HBM).  No counterpart in the reference.
#include <algorithm>

#include "rbtp_internal.cuh"

namespace {

constexpr int DFMA_CHAINS = 8;        // independent dependency chains per thread
constexpr int DFMA_THREADS = 256;

// Each thread advances DFMA_CHAINS independent chains x <- x * a + b for `iters` rounds; the
// chains hide the FMA latency, so the FP64 pipe is the only limit.  The result is stored only
// when it equals an impossible value, which keeps the work live without memory traffic.
__global__ void __launch_bounds__(DFMA_THREADS) k_dfma(double *sink, int iters, double a, double b)
{
    double x[DFMA_CHAINS];
#pragma unroll
    for (int k = 0; k < DFMA_CHAINS; ++k) x[k] = 1.0 + 1e-3 * k + 1e-9 * threadIdx.x;
    for (int it = 0; it < iters; ++it) {
#pragma unroll
        for (int k = 0; k < DFMA_CHAINS; ++k) x[k] = fma(x[k], a, b);
    }
    double s = 0.0;
#pragma unroll
    for (int k = 0; k < DFMA_CHAINS; ++k) s += x[k];
    if (s == -1.0) sink[0] = s;
}

}  // namespace

extern "C" int rbtp_fp64_fma_rate(double *flops_per_s)
{
    if (!flops_per_s) return RBTP_ERR_ARG;
    *flops_per_s = 0.0;
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
        cudaGetLastError();
        return RBTP_ERR_NODEVICE;
    }
    cudaStream_t st = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    double *sink = nullptr;
    cudaError_t e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreate(&e0);
    if (e == cudaSuccess) e = cudaEventCreate(&e1);
    if (e == cudaSuccess) e = cudaMalloc(&sink, sizeof(double));
    const int blocks = 8 * sms, iters = 4096;
    const double work = 2.0 * DFMA_CHAINS * (double)iters * blocks * DFMA_THREADS;   // flops per launch
    double best = 0.0;
    for (int rep = 0; rep < 5 && e == cudaSuccess; ++rep) {
        e = cudaEventRecord(e0, st);
        if (e == cudaSuccess) {
            k_dfma<<<blocks, DFMA_THREADS, 0, st>>>(sink, iters, 0.9999999, 1e-7);
            e = cudaGetLastError();
        }
        if (e == cudaSuccess) e = cudaEventRecord(e1, st);
        if (e == cudaSuccess) e = cudaEventSynchronize(e1);
        float ms = 0.0f;
        if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
        if (e == cudaSuccess && rep > 0 && ms > 0.0f) best = std::max(best, work / (ms * 1e-3));   // rep 0 warms up
    }
    if (sink) cudaFree(sink);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (st) cudaStreamDestroy(st);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return RBTP_ERR_CUDA;
    }
    *flops_per_s = best;
    return RBTP_OK;
}
