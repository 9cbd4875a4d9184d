// sph_probe.cu -- the FP32 issue rate of this GPU, measured.
//
// The neighbour passes are bound by instruction issue, not by HBM, so their
// roofline needs the rate at which the SMs issue warp instructions.  This
// probe measures it: every thread runs eight independent chains of fused
// multiply-adds (inline PTX fma.rn.f32, so the count is the instruction
// count), enough warps per SM to hide the FMA latency, timed with CUDA
// events.  Result: warp FMA instructions per second over the whole GPU.
// No clock or other GPU setting is touched; the caller samples the clock.
#include "sph_state.h"

namespace sph {
namespace {

constexpr int kProbeThreads = 256;
constexpr int kProbeChains = 8;
constexpr int kProbeUnroll = 8;          // FMAs per chain per loop iteration

__device__ __forceinline__ float fma_ptx(float x, float a, float b)
{
    float y;
    asm volatile("fma.rn.f32 %0, %1, %2, %3;" : "=f"(y) : "f"(x), "f"(a), "f"(b));
    return y;
}

__global__ void __launch_bounds__(kProbeThreads) k_fma_issue(float* out, uint32_t iters, float a, float b)
{
    float x[kProbeChains];
#pragma unroll
    for (int c = 0; c < kProbeChains; ++c) x[c] = (float)(threadIdx.x + c) * 1e-3f;
    for (uint32_t it = 0; it < iters; ++it) {
#pragma unroll
        for (int u = 0; u < kProbeUnroll; ++u)
#pragma unroll
            for (int c = 0; c < kProbeChains; ++c) x[c] = fma_ptx(x[c], a, b);
    }
    float s = 0.f;
#pragma unroll
    for (int c = 0; c < kProbeChains; ++c) s += x[c];
    if (s == -1.f) out[blockIdx.x] = s;   // never true for these inputs; keeps the chains live
}

}  // namespace
}  // namespace sph

extern "C" SPH_API sph_status sph_probe_fp32_issue(int device, double* warp_fma_per_s, float* ms_out)
{
    using namespace sph;
    if (!warp_fma_per_s) {
        set_last_error("sph_probe_fp32_issue: null output");
        return SPH_ERR_INVALID_ARGUMENT;
    }
    CUDA_TRY(cudaSetDevice(device));
    cudaDeviceProp prop{};
    CUDA_TRY(cudaGetDeviceProperties(&prop, device));
    int per_sm = 0;
    CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_fma_issue, kProbeThreads, 0));
    if (per_sm < 1) per_sm = 1;
    const uint32_t blocks = (uint32_t)prop.multiProcessorCount * (uint32_t)per_sm;
    float* out = nullptr;
    sph_status st = dev_alloc(&out, blocks);
    if (st != SPH_OK) return st;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaStream_t s = nullptr;
    float ms = 0.f;
    const float a = 0.999999f, b = 1e-6f;
    auto fail = [&](cudaError_t e, const char* what) {
        set_last_error(std::string(what) + ": " + cudaGetErrorString(e));
        return SPH_ERR_CUDA;
    };
    cudaError_t e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreate(&e0);
    if (e == cudaSuccess) e = cudaEventCreate(&e1);
    uint32_t iters = 256;
    // warm-up, then grow the loop until one launch lasts at least 50 ms
    for (int round = 0; e == cudaSuccess && round < 12; ++round) {
        k_fma_issue<<<blocks, kProbeThreads, 0, s>>>(out, iters, a, b);
        e = cudaGetLastError();
        if (e != cudaSuccess) break;
        e = cudaEventRecord(e0, s);
        if (e != cudaSuccess) break;
        k_fma_issue<<<blocks, kProbeThreads, 0, s>>>(out, iters, a, b);
        if ((e = cudaGetLastError()) != cudaSuccess) break;
        if ((e = cudaEventRecord(e1, s)) != cudaSuccess) break;
        if ((e = cudaEventSynchronize(e1)) != cudaSuccess) break;
        if ((e = cudaEventElapsedTime(&ms, e0, e1)) != cudaSuccess) break;
        if (ms >= 50.f) break;
        iters *= 2;
    }
    sph_status result = SPH_OK;
    if (e != cudaSuccess) {
        result = fail(e, "sph_probe_fp32_issue");
    } else {
        const double warps = (double)blocks * (kProbeThreads / 32);
        const double fma_instr = warps * (double)iters * kProbeUnroll * kProbeChains;
        *warp_fma_per_s = fma_instr / (ms * 1e-3);
        if (ms_out) *ms_out = ms;
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (s) cudaStreamDestroy(s);
    cudaFree(out);
    return result;
}
