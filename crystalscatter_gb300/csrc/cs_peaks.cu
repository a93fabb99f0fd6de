// cs_peaks.cu — arithmetic pipe peaks of the current GPU, measured.
//
// The pixel kernels are bound by arithmetic (FP32 FMA, FP64 FMA and the
// special-function unit), not by memory, so their roofline is the issue rate
// of those pipes. Each kernel below runs eight independent dependent chains of
// one instruction per thread on a grid of every SM's resident warps, long
// enough (milliseconds) for the clock to settle; the rate is taken from CUDA
// events on the launching stream, best of a few launches. The instructions are
// issued through inline PTX so that the compiler neither fuses nor removes
// them:
//   FP32  fma.rn.f32        (2 flops) and fma.rn.f32x2 (packed pair, 4 flops)
//   FP64  fma.rn.f64        (2 flops)
//   MUFU  ex2.approx.ftz.f32 (1 operation; the exp2 of every FP32 Gaussian
//                             and closed form in the mixed kernels)
// No counterpart in the reference (measurement support).
#include <cuda_runtime.h>

#include "../../include/crystalscatter.h"

namespace {

constexpr int kChains = 8;

__global__ void __launch_bounds__(256) k_peak_ffma(float *out, int iters, float a, float b) {
    float x[kChains];
#pragma unroll
    for (int c = 0; c < kChains; c++) x[c] = (float)(threadIdx.x + c) * 1e-3f;
    for (int it = 0; it < iters; it++) {
#pragma unroll
        for (int u = 0; u < 4; u++) {
#pragma unroll
            for (int c = 0; c < kChains; c++) asm volatile("fma.rn.f32 %0, %0, %1, %2;" : "+f"(x[c]) : "f"(a), "f"(b));
        }
    }
    float s = 0.0f;
#pragma unroll
    for (int c = 0; c < kChains; c++) s += x[c];
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

// packed FP32 pairs (fma.rn.f32x2: two FMAs per instruction)
__global__ void __launch_bounds__(256) k_peak_ffma2(float *out, int iters, float a, float b) {
    unsigned long long x[kChains];
    const unsigned long long A = ((unsigned long long)__float_as_uint(a) << 32) | __float_as_uint(a);
    const unsigned long long B = ((unsigned long long)__float_as_uint(b) << 32) | __float_as_uint(b);
#pragma unroll
    for (int c = 0; c < kChains; c++)
        x[c] = ((unsigned long long)__float_as_uint((float)c * 1e-3f) << 32) | __float_as_uint((float)threadIdx.x * 1e-3f);
    for (int it = 0; it < iters; it++) {
#pragma unroll
        for (int u = 0; u < 4; u++) {
#pragma unroll
            for (int c = 0; c < kChains; c++) asm volatile("fma.rn.f32x2 %0, %0, %1, %2;" : "+l"(x[c]) : "l"(A), "l"(B));
        }
    }
    float s = 0.0f;
#pragma unroll
    for (int c = 0; c < kChains; c++) s += __uint_as_float((unsigned)x[c]) + __uint_as_float((unsigned)(x[c] >> 32));
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

__global__ void __launch_bounds__(256) k_peak_dfma(double *out, int iters, double a, double b) {
    double x[kChains];
#pragma unroll
    for (int c = 0; c < kChains; c++) x[c] = (double)(threadIdx.x + c) * 1e-3;
    for (int it = 0; it < iters; it++) {
#pragma unroll
        for (int u = 0; u < 4; u++) {
#pragma unroll
            for (int c = 0; c < kChains; c++) asm volatile("fma.rn.f64 %0, %0, %1, %2;" : "+d"(x[c]) : "d"(a), "d"(b));
        }
    }
    double s = 0.0;
#pragma unroll
    for (int c = 0; c < kChains; c++) s += x[c];
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

__global__ void __launch_bounds__(256) k_peak_mufu(float *out, int iters) {
    float x[kChains];
#pragma unroll
    for (int c = 0; c < kChains; c++) x[c] = -(float)(threadIdx.x + c) * 1e-4f;
    for (int it = 0; it < iters; it++) {
#pragma unroll
        for (int u = 0; u < 4; u++) {
#pragma unroll
            for (int c = 0; c < kChains; c++) asm volatile("ex2.approx.ftz.f32 %0, %0;" : "+f"(x[c]));
        }
    }
    float s = 0.0f;
#pragma unroll
    for (int c = 0; c < kChains; c++) s += x[c];
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

// best time (s) of `reps` launches of f on s
template <class F>
cudaError_t best_time(F f, cudaStream_t s, int reps, double &best) {
    cudaEvent_t a, b;
    cudaError_t e = cudaEventCreate(&a);
    if (e != cudaSuccess) return e;
    if ((e = cudaEventCreate(&b)) != cudaSuccess) {
        cudaEventDestroy(a);
        return e;
    }
    best = 1e30;
    f();  // warm-up (clock ramp, module load)
    for (int r = 0; r < reps && e == cudaSuccess; r++) {
        cudaEventRecord(a, s);
        f();
        cudaEventRecord(b, s);
        if ((e = cudaEventSynchronize(b)) != cudaSuccess) break;
        float ms = 0;
        cudaEventElapsedTime(&ms, a, b);
        if (ms * 1e-3 < best) best = ms * 1e-3;
    }
    if (e == cudaSuccess) e = cudaGetLastError();
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    return e;
}

}  // namespace

extern "C" int cs_measure_pipe_peaks(void *stream, double *out, int n) {
    if (!out || n < 4) return CS_ERR_PARAM;
    cudaStream_t s = (cudaStream_t)stream;
    int dev = 0, sms = 0, per_sm = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return CS_ERR_CUDA;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_peak_ffma, 256, 0);
    if (sms <= 0 || per_sm <= 0) return CS_ERR_CUDA;
    const int grid = sms * per_sm, block = 256;
    const double threads = (double)grid * block;
    const double per_thread = 4.0 * kChains;  // instructions per iteration
    void *buf = nullptr;
    if (cudaMalloc(&buf, sizeof(double) * (size_t)grid * block) != cudaSuccess) return CS_ERR_CUDA;
    const int it32 = 16384, it64 = 256, itmu = 2048;
    double t = 0;
    cudaError_t e = best_time([&] { k_peak_ffma<<<grid, block, 0, s>>>((float *)buf, it32, 0.999f, 1e-7f); }, s, 5, t);
    if (e == cudaSuccess) out[0] = threads * it32 * per_thread * 2.0 / t / 1e12;
    if (e == cudaSuccess)
        e = best_time([&] { k_peak_ffma2<<<grid, block, 0, s>>>((float *)buf, it32 / 2, 0.999f, 1e-7f); }, s, 5, t);
    if (e == cudaSuccess) out[1] = threads * (it32 / 2) * per_thread * 4.0 / t / 1e12;
    if (e == cudaSuccess)
        e = best_time([&] { k_peak_dfma<<<grid, block, 0, s>>>((double *)buf, it64, 0.999, 1e-7); }, s, 5, t);
    if (e == cudaSuccess) out[2] = threads * it64 * per_thread * 2.0 / t / 1e12;
    if (e == cudaSuccess) e = best_time([&] { k_peak_mufu<<<grid, block, 0, s>>>((float *)buf, itmu); }, s, 5, t);
    if (e == cudaSuccess) out[3] = threads * itmu * per_thread / t / 1e12;
    cudaFree(buf);
    return e == cudaSuccess ? CS_OK : CS_ERR_CUDA;
}
