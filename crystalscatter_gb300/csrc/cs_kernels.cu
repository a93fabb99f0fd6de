// cs_kernels.cu — dispatch of the FP64 drop-in kernels by key, quadrant
// mirroring and the fit reduction. The per-key kernels live in
// cs_fp64_kernels.cuh and are compiled one key per unit (cs_fp64_unit.cu).
#include <cuda_runtime.h>

#include <cstdint>

#include "cs_batch.cuh"
#include "cs_fp64_kernels.cuh"
#include "cs_fp64_unit.h"
#include "cs_launch.h"
#include "cs_mixed.h"


namespace cs {

// Quadrant mirroring of doCalculation (Source/sc_calc_generic_cpu.cpp:1246-1269).
// Q1: each computed pixel (ihex,i), ihex,i in [0,zmax), is copied to
// (-ihex,i), (-ihex,-i-1), (ihex,-i-1). Q2: (ihex,i) -> (-ihex,-i) for ihex in
// [0,zmax), i in (-zmax,zmax); the reference runs this copy sequentially and
// for ihex = 0 reads pixels it has already overwritten, which this kernel
// reproduces (row 0 becomes I(0,-|i|) on both sides).
__global__ void k_mirror(double *img, int zmax, int xmin, int xmax, int ymin, int q1) {
    const int xs = xmax - xmin;
    auto at = [&](int x, int y) -> double & { return img[(long)(x - xmin) + (long)xs * (long)(y - ymin)]; };
    const long total = (long)zmax * (q1 ? zmax : (2 * zmax - 1));
    for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < total; t += (long)gridDim.x * blockDim.x) {
        if (q1) {
            const int ihex = (int)(t % zmax), i = (int)(t / zmax);
            const double v = at(ihex, i);
            at(-ihex, i) = v;  // ihex = 0 rewrites the same value
            at(-ihex, -i - 1) = v;
            at(ihex, -i - 1) = v;
        } else {
            const int ihex = 1 + (int)(t % zmax);  // rows 1..zmax-1 (ihex = 0 handled below)
            const int i = -zmax + 1 + (int)(t / zmax);
            if (ihex < zmax) at(-ihex, -i) = at(ihex, i);
        }
    }
    if (!q1 && blockIdx.x == 0 && threadIdx.x == 0) {
        // row ihex = 0, sequential semantics: for i > 0 the value becomes I(0,-i)
        for (int i = 1; i < zmax; i++) at(0, i) = at(0, -i);
    }
}

// Deterministic sum of the FQS array: NaN pixels are counted and skipped,
// non-zero pixels counted (doFitCalculation, sc_calc_generic_cpu.cpp:1421-1434).
// Pass 1: one partial per block; pass 2: one block combines the partials.
__device__ __forceinline__ void fit_block_partial(const double *__restrict__ fqs, long n, double &s,
                                                  unsigned long long &c, unsigned long long &nn) {
    __shared__ double ss[32];
    __shared__ unsigned long long sc[32], sn[32];
    s = 0.0;
    c = 0;
    nn = 0;
    for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < n; t += (long)gridDim.x * blockDim.x) {
        const double v = fqs[t];
        if (isnan(v))
            nn++;
        else {
            if (v != 0) c++;
            s += v;
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        s += __shfl_down_sync(0xffffffffu, s, o);
        c += __shfl_down_sync(0xffffffffu, c, o);
        nn += __shfl_down_sync(0xffffffffu, nn, o);
    }
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 0) {
        ss[w] = s;
        sc[w] = c;
        sn[w] = nn;
    }
    __syncthreads();
    if (w == 0) {
        const int nw = blockDim.x >> 5;
        s = lane < nw ? ss[lane] : 0.0;
        c = lane < nw ? sc[lane] : 0;
        nn = lane < nw ? sn[lane] : 0;
        for (int o = 16; o > 0; o >>= 1) {
            s += __shfl_down_sync(0xffffffffu, s, o);
            c += __shfl_down_sync(0xffffffffu, c, o);
            nn += __shfl_down_sync(0xffffffffu, nn, o);
        }
    }
}

__global__ void k_fit_reduce1(const double *__restrict__ fqs, long n, double *__restrict__ psum,
                              unsigned long long *__restrict__ pcnt, unsigned long long *__restrict__ pnan) {
    double s;
    unsigned long long c, nn;
    fit_block_partial(fqs, n, s, c, nn);
    if (threadIdx.x == 0) {
        psum[blockIdx.x] = s;
        pcnt[blockIdx.x] = c;
        pnan[blockIdx.x] = nn;
    }
}

// Batch form: blockIdx.y selects the set's FQS array (stride nbuf) and its row
// of partials; with the same gridDim.x every partial equals the single-set one.
__global__ void k_batch_fit_reduce1(const double *__restrict__ fqs, long nbuf, double *__restrict__ psum,
                                    unsigned long long *__restrict__ pcnt, unsigned long long *__restrict__ pnan) {
    double s;
    unsigned long long c, nn;
    fit_block_partial(fqs + (size_t)blockIdx.y * (size_t)nbuf, nbuf, s, c, nn);
    if (threadIdx.x == 0) {
        const size_t o = (size_t)blockIdx.y * gridDim.x + blockIdx.x;
        psum[o] = s;
        pcnt[o] = c;
        pnan[o] = nn;
    }
}

__global__ void k_fit_reduce2(const double *__restrict__ psum, const unsigned long long *__restrict__ pcnt,
                              const unsigned long long *__restrict__ pnan, int nb, double *__restrict__ out_sum,
                              unsigned long long *__restrict__ out_cnt, unsigned long long *__restrict__ out_nan) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    double s = 0.0;
    unsigned long long c = 0, nn = 0;
    for (int b = 0; b < nb; b++) {
        s += psum[b];
        c += pcnt[b];
        nn += pnan[b];
    }
    *out_sum = s;
    *out_cnt = c;
    *out_nan = nn;
}

__global__ void k_batch_fit_reduce2(const double *__restrict__ psum, const unsigned long long *__restrict__ pcnt,
                                    const unsigned long long *__restrict__ pnan, int nb, int nsets,
                                    double *__restrict__ out_sum, unsigned long long *__restrict__ out_cnt,
                                    unsigned long long *__restrict__ out_nan) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nsets) return;
    double s = 0.0;
    unsigned long long c = 0, nn = 0;
    for (int b = 0; b < nb; b++) {
        s += psum[(size_t)k * nb + b];
        c += pcnt[(size_t)k * nb + b];
        nn += pnan[(size_t)k * nb + b];
    }
    out_sum[k] = s;
    out_cnt[k] = c;
    out_nan[k] = nn;
}

// Per-pixel FQSVERGL of every set of a batch against the shared fit data: the
// masks and arithmetic of k_fit (doFitCalculation, KERNEL_PREWORK/POSTWORK
// with dofit), with the pixel value read from the set's computed image, which
// holds exactly the value k_fit computes for that pixel (the fit region is the
// whole calculated image). blockIdx.y = set.
__global__ void __launch_bounds__(256) k_batch_fqs(const cs::BatchSetDev *__restrict__ sets,
                                                   const double *__restrict__ img, const double *__restrict__ data,
                                                   double *__restrict__ fqs, long nfit, long nbuf) {
    const cs::BatchSetDev &S = sets[blockIdx.y];
    const cs_prepared &P = *S.prep;
    double *f = fqs + (size_t)blockIdx.y * (size_t)nbuf;
    const int xstride = P.xmax - P.xmin;
    for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < nfit; t += (long)gridDim.x * blockDim.x) {
        int x = (int)(t % P.fit_width);
        int y = (int)(t / P.fit_width);
        if (!cs64::check_fit_ranges(P, data, f, x, y)) continue;
        const long idx = (long)(x - P.xmin) + (long)xstride * (long)(y - P.ymin);
        if (idx < 0 || idx >= nbuf) continue;
        const double pixval = img[S.out_offset + idx];
        if (pixval > 0 && data[idx] > 0) {
            const double d = log(pixval) / log(10.) - log(data[idx]) / log(10.);
            f[idx] = d * d;
        } else
            f[idx] = 0.0;
    }
}

static int sm_count() {
    static int n = 0;
    if (n == 0) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        if (n <= 0) n = 1;
    }
    return n;
}

// Blocks for a grid-stride loop over n items: enough to cover them, capped at
// a multiple of the SM count (8 resident 256-thread blocks per SM).
static int grid_for(long n, int block) {
    const long need = (n + block - 1) / block;
    const long cap = (long)sm_count() * 8;
    long g = need < cap ? need : cap;
    return g < 1 ? 1 : (int)g;
}

namespace {
thread_local cudaError_t t_last_launch = cudaSuccess;
}

cudaError_t last_launch_error() { return t_last_launch; }

int launch_status() {
    t_last_launch = cudaGetLastError();
    return t_last_launch == cudaSuccess ? CS_OK : CS_ERR_CUDA;
}

bool key_supported(const cs_prepared &P) {
    switch (P.key) {
    case CS_KEY_SPHERE_NONE_ISO:
    case CS_KEY_SPHERE_GAUSS_FCC_GAUSS:
    case CS_KEY_CYL_NONE_GAUSS:
    case CS_KEY_CYL_NONE_ZDIR:
    case CS_KEY_CYL_GAUSS_BCT_ZDIR:
    case CS_KEY_CUBE_NONE_ISO:
    case CS_KEY_GENERIC:
        return true;
    default:
        return false;
    }
}

bool mixed_key(int key) {
    switch (key) {
    case CS_KEY_SPHERE_NONE_ISO:
    case CS_KEY_SPHERE_GAUSS_FCC_GAUSS:
    case CS_KEY_CYL_NONE_GAUSS:
    case CS_KEY_CYL_NONE_ZDIR:
    case CS_KEY_CYL_GAUSS_BCT_ZDIR:
        return true;
    default:
        return false;
    }
}

int launch_image(const DevSet &D, const cs_prepared &P, double *d_out, cudaStream_t s) {
    const int nx = P.zzmax - P.zzmin, ny = P.iimax - P.iimin;
    if (nx <= 0 || ny <= 0) return CS_OK;
    const int grid = grid_for((long)nx * (long)ny, 256);
    switch (P.key) {
#define CS_CASE(K) \
    case K: Fp64Unit<K>::image(D, P, d_out, grid, s); break;
        CS_FOR_EACH_KEY_FP64(CS_CASE)
#undef CS_CASE
    default: return CS_ERR_UNSUPPORTED;
    }
    if (P.expand && P.calc_quadrants != CS_RADQ4 && P.calc_quadrants != CS_RAD1D) launch_mirror(P, d_out, s);
    return launch_status();
}

void launch_mirror(const cs_prepared &P, double *d_out, cudaStream_t s) {
    const int q1 = P.calc_quadrants == CS_RADQ1;
    const long total = (long)P.zmax * (q1 ? P.zmax : 2 * P.zmax);
    k_mirror<<<grid_for(total, 256), 256, 0, s>>>(d_out, P.zmax, P.xmin, P.xmax, P.ymin, q1);
}

int launch_redo(const DevSet &D, const cs_prepared &P, double *d_out, const MixedScratch &S, cudaStream_t s) {
    const int grid = sm_count() * 4;
    switch (P.key) {
#define CS_CASE(K) \
    case K: Fp64Unit<K>::redo(D, P, d_out, S, grid, s); break;
        CS_FOR_EACH_KEY_FP64(CS_CASE)
#undef CS_CASE
    default: return CS_ERR_UNSUPPORTED;
    }
    return CS_OK;
}

int launch_fit(const DevSet &D, const cs_prepared &P, const double *d_data, double *d_fqs, long nbuf,
               FitReduce &R, cudaStream_t s) {
    const int grid = grid_for((long)P.fit_width * P.fit_height, 256);
    switch (P.key) {
#define CS_CASE(K) \
    case K: Fp64Unit<K>::fit(D, P, d_data, d_fqs, nbuf, grid, s); break;
        CS_FOR_EACH_KEY_FP64(CS_CASE)
#undef CS_CASE
    default: return CS_ERR_UNSUPPORTED;
    }
    const int nb = R.nblocks;
    k_fit_reduce1<<<nb, 256, 0, s>>>(d_fqs, nbuf, R.d_psum, R.d_pcnt, R.d_pnan);
    k_fit_reduce2<<<1, 32, 0, s>>>(R.d_psum, R.d_pcnt, R.d_pnan, nb, R.d_sum, R.d_cnt, R.d_nan);
    return launch_status();
}


// ---- batch launchers -------------------------------------------------------

int launch_batch_fp64(const BatchSetDev *d_sets, const BatchGroup &g, unsigned long long *d_counter,
                      const cs_chi_node *d_chi, double *d_out, int grid, cudaStream_t s) {
    if (g.tiles <= 0) return CS_OK;
    switch (g.key) {
#define CS_CASE(K) \
    case K: Fp64Unit<K>::batch(d_sets, g, d_counter, d_chi, d_out, grid, s); break;
        CS_FOR_EACH_KEY_FP64(CS_CASE)
#undef CS_CASE
    default: return CS_ERR_UNSUPPORTED;
    }
    return launch_status();
}

int launch_batch_redo(const BatchSetDev *d_sets, int key, const cs_chi_node *d_chi, double *d_out, const int *d_count,
                      const int2 *d_list, long cap, cudaStream_t s) {
    const int grid = sm_count() * 4;
    switch (key) {
#define CS_CASE(K) \
    case K: Fp64Unit<K>::batch_redo(d_sets, d_chi, d_out, d_count, d_list, cap, grid, s); break;
        CS_FOR_EACH_KEY_FP64(CS_CASE)
#undef CS_CASE
    default: return CS_ERR_UNSUPPORTED;
    }
    return launch_status();
}

int batch_blocks_per_sm_fp64(int key) {
    switch (key) {
#define CS_CASE(K) \
    case K: return Fp64Unit<K>::batch_blocks_per_sm();
        CS_FOR_EACH_KEY_FP64(CS_CASE)
#undef CS_CASE
    default: return 0;
    }
}


// FQS arrays and chi^2 per set of a batch whose images are in d_img.
int launch_batch_fit(const BatchSetDev *d_sets, int nsets, const double *d_img, const double *d_data, double *d_fqs,
                     long nfit, long nbuf, const BatchFitReduce &R, cudaStream_t s) {
    if (nsets <= 0) return CS_OK;
    t_last_launch = cudaMemsetAsync(d_fqs, 0, sizeof(double) * (size_t)nbuf * (size_t)nsets, s);
    if (t_last_launch != cudaSuccess) return CS_ERR_CUDA;
    const int gx = grid_for(nfit, 256);
    k_batch_fqs<<<dim3(gx, nsets), 256, 0, s>>>(d_sets, d_img, d_data, d_fqs, nfit, nbuf);
    k_batch_fit_reduce1<<<dim3(R.nblocks, nsets), 256, 0, s>>>(d_fqs, nbuf, R.d_psum, R.d_pcnt, R.d_pnan);
    k_batch_fit_reduce2<<<(nsets + 127) / 128, 128, 0, s>>>(R.d_psum, R.d_pcnt, R.d_pnan, R.nblocks, nsets, R.d_sum,
                                                            R.d_cnt, R.d_nan);
    return launch_status();
}

}  // namespace cs
