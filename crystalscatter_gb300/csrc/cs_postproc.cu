// cs_postproc.cu — the r-phi transform of the training-data generator on the
// GPU (cs_rphi_device in include/crystalscatter.h).
//
// SasCalc_PostProc::generateRphi (Source/sc_postproc.cpp:53-334) resamples a
// detector image onto an s x s polar grid around the beam centre: for every
// radius step k (ir = 0, irstp, 2 irstp, ... accumulated in single
// precision while ir <= irmax) and angle row i = 0..s it averages umf
// bilinear samples at phi = (i - 1.5) phiber + (j - 0.5) phiber/umf, and
// writes the average (clamped at 0) to out[int(float(i s) + ir/irstp)].
// Here one thread computes one (k, i) average, in the reference's order of
// samples and neighbours; the radius steps come from the host (the float
// accumulation is sequential). Different (k, i) can land on the same output
// entry (a float column index that falls just below an integer), where the
// reference's later write wins: an atomicMax over the flat (k, i) index picks
// that last writer per entry, then the winners write in parallel. Scaling and clipping (scaleAndClipData,
// :764-823) follow on the device.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "../../include/crystalscatter.h"
#include "cs_launch.h"

namespace {

__global__ void k_rphi_steps(const double *__restrict__ d, int srcsx, int srcsy, int xc, int yc, int s,
                             double phiber, const float *__restrict__ irs, int nsteps, float irstp,
                             double *__restrict__ val, int *__restrict__ pos) {
    const int rows = s + 1;
    const long n = (long)nsteps * rows;
    for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < n; t += (long)gridDim.x * blockDim.x) {
        const int k = (int)(t / rows), i = (int)(t % rows);
        const float ir = irs[k];
        const double rad = ir;
        const int umf = max(1024 - (int)(1024. - phiber * rad), 1);
        double twt = 0.0, avg = 0.0;
        for (int j = 1; j <= umf; j++) {
            const double phi = (i - 1.5) * phiber + (j - 0.5) * phiber / umf;
            double sn, cn;
            sincos(phi, &sn, &cn);
            const double xs = xc + rad * cn;
            const double ys = yc + rad * sn;
            const int ix1 = (int)xs, iy1 = (int)ys;
            const int ix2 = ix1 + 1, iy2 = iy1 + 1;
            const double rex = xs - ix1, rey = ys - iy1;
            if (ix1 >= 0 && ix1 < srcsx && iy1 >= 0 && iy1 < srcsy) {
                const double wt = (1.0 - rex) * (1.0 - rey);
                twt = twt + wt;
                avg = avg + wt * d[ix1 + (long)srcsx * iy1];
            }
            if (ix2 >= 0 && ix2 < srcsx && iy1 >= 0 && iy1 < srcsy) {
                const double wt = (rex) * (1.0 - rey);
                twt = twt + wt;
                avg = avg + wt * d[ix2 + (long)srcsx * iy1];
            }
            if (ix1 >= 0 && ix1 < srcsx && iy2 >= 0 && iy2 < srcsy) {
                const double wt = (1.0 - rex) * (rey);
                twt = twt + wt;
                avg = avg + wt * d[ix1 + (long)srcsx * iy2];
            }
            if (ix2 >= 0 && ix2 < srcsx && iy2 >= 0 && iy2 < srcsy) {
                const double wt = (rex) * (rey);
                twt = twt + wt;
                avg = avg + wt * d[ix2 + (long)srcsx * iy2];
            }
        }
        if (twt > 0.0) avg = avg / twt;
        const float col = __fdiv_rn(ir, irstp);
        val[t] = avg;
        pos[t] = (int)__fadd_rn((float)(i * s), col);
    }
}

// Several (k, i) can name one output entry; the reference's sequential loops
// (k outer, i inner) leave the last one, i.e. the largest flat index t.
__global__ void k_rphi_last_writer(const int *__restrict__ pos, int n, int len, int *__restrict__ winner) {
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
        const int idx = pos[t];
        if (idx >= 0 && idx < len) atomicMax(winner + idx, t);
    }
}

__global__ void k_rphi_write(const double *__restrict__ val, const int *__restrict__ pos, int n, int len,
                             const int *__restrict__ winner, double *__restrict__ out) {
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
        const int idx = pos[t];
        if (idx >= 0 && idx < len && winner[idx] == t) out[idx] = val[t] < 0 ? 0.0 : val[t];
    }
}

// the running maximum from 0 (NaN never wins), one block
__global__ void k_rphi_max(const double *__restrict__ a, int n, double *__restrict__ m) {
    __shared__ double sm[1024];
    double v = 0.0;
    for (int t = threadIdx.x; t < n; t += blockDim.x)
        if (a[t] > v) v = a[t];
    sm[threadIdx.x] = v;
    __syncthreads();
    for (int h = blockDim.x / 2; h > 0; h >>= 1) {
        if (threadIdx.x < h && sm[threadIdx.x + h] > sm[threadIdx.x]) sm[threadIdx.x] = sm[threadIdx.x + h];
        __syncthreads();
    }
    if (threadIdx.x == 0) *m = sm[0];
}

__global__ void k_rphi_scale_clip(double *__restrict__ a, int n, const double *__restrict__ m, int flags) {
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
        double v = a[t];
        if (flags & CS_RPHI_SCALE) v = v / *m;
        if (flags & CS_RPHI_CLIP) {
            v = ((log(fabs(v) / 1e-20) / log(10.0)) + 6.0) / 6.0;
            if (v < 0) v = 0.0;
        }
        if (flags & CS_RPHI_CLIP40) {
            v = 1.0 - (1.0 - v) / (1.0 - 0.4);
            if (v < 0) v = 0.0;
        }
        a[t] = v;
    }
}

}  // namespace

extern "C" int cs_rphi_device(const double *d_img, int x0, int x1, int y0, int y1, int xcenter, int ycenter, int s,
                              int flags, double *d_out, void *stream) {
    if (!d_img || !d_out || s < 2 || x1 <= x0 || y1 <= y0) return CS_ERR_PARAM;
    // the reference shifts negative minimum coordinates to 0 (:64-79); a
    // positive minimum misplaces its pixel lookup and is rejected here
    if (x0 < 0) {
        x1 -= x0;
        xcenter -= x0;
        x0 = 0;
    }
    if (y0 < 0) {
        y1 -= y0;
        ycenter -= y0;
        y0 = 0;
    }
    if (x0 > 0 || y0 > 0) return CS_ERR_PARAM;
    const int srcsx = x1 - x0, srcsy = y1 - y0;
    const int phisteps = s;
    const double phiber = 2. * M_PI / phisteps;
    auto sq = [](double v) { return v * v; };
    double rmax = std::sqrt(sq(1. - xcenter) + sq(1. - ycenter));
    rmax = std::fmax(rmax, std::sqrt(sq((srcsx - 1.) - xcenter) + sq(1. - ycenter)));
    rmax = std::fmax(rmax, std::sqrt(sq((srcsx - 1.) - xcenter) + sq((srcsy - 1.) - ycenter)));
    rmax = std::fmax(rmax, std::sqrt(sq(1. - xcenter) + sq((srcsy - 1.) - ycenter)));
    const int irmax = (int)(rmax + 0.5);
    const float irstp = float(irmax) / float(s - 1);
    if (irmax <= 0) return CS_ERR_PARAM;  // the reference's radius loop never ends for irstp = 0
    std::vector<float> irs;
    for (float ir = 0; ir <= irmax; ir += irstp) irs.push_back(ir);
    const int nsteps = (int)irs.size();
    const long nl = (long)nsteps * (s + 1);
    if (nl > 0x7fffffffL || (long)s * s > 0x7fffffffL) return CS_ERR_SIZE;
    const int n = (int)nl;
    const int len = s * s;
    cudaStream_t st = (cudaStream_t)stream;
    float *d_irs = nullptr;
    double *d_val = nullptr;
    int *d_pos = nullptr, *d_win = nullptr;
    double *d_max = nullptr;
    cudaError_t e = cudaMallocAsync(&d_irs, sizeof(float) * nsteps, st);
    if (e == cudaSuccess) e = cudaMallocAsync(&d_val, sizeof(double) * n, st);
    if (e == cudaSuccess) e = cudaMallocAsync(&d_pos, sizeof(int) * n, st);
    if (e == cudaSuccess) e = cudaMallocAsync(&d_win, sizeof(int) * len, st);
    if (e == cudaSuccess) e = cudaMallocAsync(&d_max, sizeof(double), st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_irs, irs.data(), sizeof(float) * nsteps, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(d_out, 0, sizeof(double) * len, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(d_win, 0xff, sizeof(int) * len, st);  // -1: no writer
    if (e == cudaSuccess) {
        const int blocks = std::min((n + 127) / 128, 4096);
        k_rphi_steps<<<blocks, 128, 0, st>>>(d_img, srcsx, srcsy, xcenter, ycenter, s, phiber, d_irs, nsteps, irstp,
                                             d_val, d_pos);
        k_rphi_last_writer<<<blocks, 128, 0, st>>>(d_pos, n, len, d_win);
        k_rphi_write<<<blocks, 128, 0, st>>>(d_val, d_pos, n, len, d_win, d_out);
        if (flags & (CS_RPHI_SCALE | CS_RPHI_CLIP | CS_RPHI_CLIP40)) {
            k_rphi_max<<<1, 1024, 0, st>>>(d_out, len, d_max);
            k_rphi_scale_clip<<<(len + 255) / 256, 256, 0, st>>>(d_out, len, d_max, flags);
        }
        e = cudaGetLastError();
    }
    if (d_win) cudaFreeAsync(d_win, st);
    if (d_irs) cudaFreeAsync(d_irs, st);
    if (d_val) cudaFreeAsync(d_val, st);
    if (d_pos) cudaFreeAsync(d_pos, st);
    if (d_max) cudaFreeAsync(d_max, st);
    // the synchronisation also keeps the host vector of radius steps alive
    // until its upload has ended
    const cudaError_t es = cudaStreamSynchronize(st);
    if (e == cudaSuccess) e = es;
    return e == cudaSuccess ? CS_OK : CS_ERR_CUDA;
}
