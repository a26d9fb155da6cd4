// Peak-rate probes: the denominators of the roofline of the path kernels,
// which are bound by the SFU (MUFU) and FP32/INT issue pipes rather than by
// HBM or the tensor cores.  Each probe runs 8 independent dependency chains
// per thread on every SM and reports device-wide operations per second.
#include <mutex>

#include "sde_kernels.cuh"

using namespace sdegpu;

namespace {

constexpr int PROBE_CHAINS = 16;

__global__ void __launch_bounds__(BLOCK) probe_sfu(float *sink, int iters) {
    float v[PROBE_CHAINS];
#pragma unroll
    for (int c = 0; c < PROBE_CHAINS; ++c) v[c] = 0.25f + 1e-4f * (threadIdx.x + 7 * c);
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int c = 0; c < PROBE_CHAINS; ++c) {
            // the four SFU operations of a Box-Muller pair
            switch (c & 3) {
            case 0: v[c] = approx_lg2(v[c] + 1.5f); break;
            case 1: v[c] = approx_sin(v[c]); break;
            case 2: v[c] = approx_cos(v[c]); break;
            default: v[c] = approx_sqrt(v[c] + 0.5f); break;
            }
        }
    }
    float s = 0.f;
#pragma unroll
    for (int c = 0; c < PROBE_CHAINS; ++c) s += v[c];
    if (s == 123.456f) sink[0] = s;
}

__global__ void __launch_bounds__(BLOCK) probe_fma(float *sink, int iters) {
    float v[PROBE_CHAINS];
#pragma unroll
    for (int c = 0; c < PROBE_CHAINS; ++c) v[c] = 1e-4f * (threadIdx.x + c);
    const float m = 0.999f, a = 1e-3f;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int c = 0; c < PROBE_CHAINS; ++c) v[c] = fmaf(v[c], m, a);
    }
    float s = 0.f;
#pragma unroll
    for (int c = 0; c < PROBE_CHAINS; ++c) s += v[c];
    if (s == 123.456f) sink[0] = s;
}

__global__ void __launch_bounds__(BLOCK) probe_imulhi(unsigned *sink, int iters) {
    unsigned v[PROBE_CHAINS];
#pragma unroll
    for (int c = 0; c < PROBE_CHAINS; ++c) v[c] = threadIdx.x * 2654435761u + c;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int c = 0; c < PROBE_CHAINS; ++c) v[c] = __umulhi(v[c], 0xD2511F53u) + v[c];
    }
    unsigned s = 0;
#pragma unroll
    for (int c = 0; c < PROBE_CHAINS; ++c) s ^= v[c];
    if (s == 0x12345678u) sink[0] = s;
}

}  // namespace

extern "C" int32_t sde_peak_probe(int32_t which, double *ops_per_s) {
    if (!ops_per_s || which < 0 || which > 2) return SDE_ERR_INVALID;
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return SDE_ERR_NO_DEVICE;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return SDE_ERR_CUDA;
    void *sink = nullptr;
    if (cudaMalloc(&sink, 64) != cudaSuccess) return SDE_ERR_CUDA;
    cudaStream_t st;
    cudaStreamCreate(&st);
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    // 8 resident blocks of 256 threads per SM, 16 independent chains per
    // thread: enough operations in flight to cover the SFU latency
    const int blocks = sms * 8, iters = 2048;
    auto launch = [&]() {
        if (which == 0) probe_sfu<<<blocks, BLOCK, 0, st>>>((float *)sink, iters);
        else if (which == 1) probe_fma<<<blocks, BLOCK, 0, st>>>((float *)sink, iters);
        else probe_imulhi<<<blocks, BLOCK, 0, st>>>((unsigned *)sink, iters);
    };
    launch();  // warm-up
    float best = 1e30f;
    for (int r = 0; r < 5; ++r) {
        cudaEventRecord(e0, st);
        launch();
        cudaEventRecord(e1, st);
        cudaEventSynchronize(e1);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (ms < best) best = ms;
    }
    cudaError_t err = cudaGetLastError();
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaStreamDestroy(st);
    cudaFree(sink);
    if (err != cudaSuccess) return SDE_ERR_CUDA;
    const double ops = (double)blocks * BLOCK * iters * PROBE_CHAINS;
    *ops_per_s = ops / (best * 1e-3);
    return SDE_OK;
}
