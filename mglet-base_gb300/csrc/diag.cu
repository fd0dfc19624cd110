// diag.cu -- measured FP64 roof of the device (the second roof of the
// plain form's roofline: GB300 issues FP64 at a small fraction of its FP32
// rate, so the FP64 kernels of the parity form can be bound by their FP64
// instructions rather than by HBM).
//
// Each thread runs kChains independent dependent chains of one FP64
// operation (DFMA, DADD or DMUL) for iters steps; the grid holds enough warps
// on every SM that the pipe, not the chain latency, limits the rate.  The
// result of every chain feeds a store guarded by a condition that never holds,
// so nothing is optimised away.  Timed with CUDA events on a private stream,
// best of several runs.
#include <algorithm>

#include "internal.h"

namespace mg {
namespace {

constexpr int kChains = 8;

template <int kOp>
__global__ void __launch_bounds__(256) k_fp64_roof(double* sink, int iters, double a, double b) {
    double x[kChains];
#pragma unroll
    for (int q = 0; q < kChains; ++q) x[q] = 1.0 + 1e-3 * (threadIdx.x + q);
    for (int it = 0; it < iters; ++it) {
#pragma unroll
        for (int q = 0; q < kChains; ++q) {
            if (kOp == 0) x[q] = fma(x[q], a, b);
            else if (kOp == 1) x[q] = __dadd_rn(x[q], b);
            else x[q] = __dmul_rn(x[q], a);
        }
    }
    double s = 0.0;
#pragma unroll
    for (int q = 0; q < kChains; ++q) s += x[q];
    if (s == -1.2345e300) sink[blockIdx.x] = s;
}

template <int kOp>
cudaError_t time_roof(cudaStream_t st, double* sink, int blocks, int iters, float* best_ms) {
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    *best_ms = 1e30f;
    for (int rep = 0; rep < 6; ++rep) {
        cudaEventRecord(e0, st);
        k_fp64_roof<kOp><<<blocks, 256, 0, st>>>(sink, iters, 0.9999999, 1e-9);
        cudaEventRecord(e1, st);
        cudaError_t e = cudaEventSynchronize(e1);
        if (e != cudaSuccess) return e;
        e = cudaGetLastError();
        if (e != cudaSuccess) return e;
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (rep > 0) *best_ms = std::min(*best_ms, ms);   // the first run warms up
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return cudaSuccess;
}

}  // namespace
}  // namespace mg

// out[0] DFMA, out[1] DADD, out[2] DMUL: thread instructions per second of
// the whole device (a DFMA counts as one instruction, two flops).
extern "C" int mglet_gpu_fp64_roof(int32_t device, double* out) {
    using namespace mg;
    if (!out) {
        set_error("fp64_roof: null output");
        return MGLET_ERR_ARG;
    }
    MG_CUDA(cudaSetDevice(device));
    int sms = 0;
    MG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
    cudaStream_t st;
    MG_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    double* sink = nullptr;
    const int blocks = sms * 8;            // 64 warps per SM
    const int iters = 2048;
    cudaError_t e = cudaMalloc(&sink, (size_t)blocks * sizeof(double));
    if (e != cudaSuccess) {
        cudaStreamDestroy(st);
        return cuda_fail(e, "fp64_roof: cudaMalloc");
    }
    float ms[3];
    e = time_roof<0>(st, sink, blocks, iters, &ms[0]);
    if (e == cudaSuccess) e = time_roof<1>(st, sink, blocks, iters, &ms[1]);
    if (e == cudaSuccess) e = time_roof<2>(st, sink, blocks, iters, &ms[2]);
    cudaFree(sink);
    cudaStreamDestroy(st);
    if (e != cudaSuccess) return cuda_fail(e, "fp64_roof");
    const double n = (double)blocks * 256 * kChains * iters;
    for (int q = 0; q < 3; ++q) out[q] = n / (ms[q] * 1e-3);
    return 0;
}
