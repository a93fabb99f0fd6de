// cs_kernels.cu — pixel kernels, quadrant mirroring and the fit reduction.
//
// One thread computes one detector pixel; consecutive threads take
// consecutive ihex (the fastest image index), so the FP64 image store of a warp
// is one contiguous 256-byte segment. The reference launches one 16x16 block
// per image tile (Source/sc_calc_generic_gpu.cu:94-99); here the grid is a
// grid-stride loop sized to a multiple of the SM count so uneven per-pixel
// cost (series vs. asymptote vs. nested Romberg) does not leave SMs idle.
#include <cuda_runtime.h>

#include <cstdint>

#include "cs_batch.cuh"
#include "cs_fp64.cuh"
#include "cs_launch.h"
#include "cs_mixed.h"

namespace cs64 {

// Image kernel: pixel (ihex, i) over [zzmin,zzmax) x [iimin,iimax), written at
// IDX(ihex,i) = (ihex-xmin) + (xmax-xmin)*(i-ymin) (sc_calc_generic_gpu.h:575-578).
template <int KEY>
__global__ void __launch_bounds__(256) k_image(Ctx C, double *__restrict__ out, int nx, long npix) {
    const cs_prepared &P = *C.P;
    const int xstride = P.xmax - P.xmin;
    for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < npix; t += (long)gridDim.x * blockDim.x) {
        const int ihex = P.zzmin + (int)(t % nx);
        const int i = P.iimin + (int)(t / nx);
        double qx, qy, qz;
        convert_idx2q(P, ihex, i, qx, qy, qz);
        const double v = calc_pixel<KEY>(C, qx, qy, qz);
        out[(long)(ihex - P.xmin) + (long)xstride * (long)(i - P.ymin)] = v;
    }
}

// checkFitRanges, Source/sc_calc_generic_gpu.cu:293-347
__device__ __forceinline__ bool check_fit_ranges(const cs_prepared &P, const double *__restrict__ data,
                                                 double *__restrict__ fqs, int &x, int &y) {
    for (int i = 0; i < 4; i++) {
        if (P.nofit_x0[i] < 0) continue;
        if (x < P.nofit_x0[i]) continue;
        if (P.nofit_x1[i] < x) continue;
        if (y < P.nofit_y0[i]) continue;
        if (P.nofit_y1[i] < y) continue;
        fqs[x + (long)P.fit_width * y] = 0.0;
        return false;
    }
    if (P.fit_border > 0 || P.fit_bstop > 0) {
        if (x < P.xmin + P.fit_border || x >= P.xmax - P.fit_border || y < P.ymin + P.fit_border ||
            y >= P.ymax - P.fit_border) {
            fqs[x + (long)P.fit_width * y] = 0.0;
            return false;
        }
        if (x >= P.beamx0 - P.fit_bstop && x < P.beamx0 + P.fit_bstop && y >= P.beamy0 - P.fit_bstop &&
            y < P.beamy0 + P.fit_bstop) {
            fqs[x + (long)P.fit_width * y] = 0.0;
            return false;
        }
    } else if (P.fit_bstop == -1) {
        const long idx = x + (long)P.fit_width * y;
        if (data[idx] <= data[0]) {
            fqs[idx] = 0.0;
            return false;
        }
    }
    x += P.iimin;
    y += P.iimin;
    return true;
}

// Fit kernel: per-pixel FQSVERGL (Source/sc_globalConfig.h:32) into fqs,
// KERNEL_PREWORK/POSTWORK of Source/sc_calc_generic_gpu.cu:47-73 with dofit.
template <int KEY>
__global__ void __launch_bounds__(256) k_fit(Ctx C, const double *__restrict__ data, double *__restrict__ fqs,
                                             long nfit, long nbuf) {
    const cs_prepared &P = *C.P;
    const int xstride = P.xmax - P.xmin;
    for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < nfit; t += (long)gridDim.x * blockDim.x) {
        int x = (int)(t % P.fit_width);
        int y = (int)(t / P.fit_width);
        if (!check_fit_ranges(P, data, fqs, x, y)) continue;
        double qx, qy, qz;
        convert_idx2q(P, x, y, qx, qy, qz);
        const double pixval = calc_pixel<KEY>(C, qx, qy, qz);
        const long idx = (long)(x - P.xmin) + (long)xstride * (long)(y - P.ymin);
        if (idx < 0 || idx >= nbuf) continue;  // outside the fit buffer: the reference writes out of bounds
        if (pixval > 0 && data[idx] > 0) {
            const double d = log(pixval) / log(10.) - log(data[idx]) / log(10.);
            fqs[idx] = d * d;
        } else
            fqs[idx] = 0.0;
    }
}

// FP64 recomputation of the pixels that the mixed kernel flagged (list of
// linear pixel indices t of the calculated region, count on the device).
template <int KEY>
__global__ void __launch_bounds__(128) k_redo(Ctx C, double *__restrict__ out, int nx,
                                              const int *__restrict__ redo_count, const int *__restrict__ redo_list,
                                              int redo_cap) {
    const cs_prepared &P = *C.P;
    const int xstride = P.xmax - P.xmin;
    int n = *redo_count;
    if (n > redo_cap) n = redo_cap;
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
        const long t = redo_list[r];
        const int ihex = P.zzmin + (int)(t % nx);
        const int i = P.iimin + (int)(t / nx);
        double qx, qy, qz;
        convert_idx2q(P, ihex, i, qx, qy, qz);
        out[(long)(ihex - P.xmin) + (long)xstride * (long)(i - P.ymin)] = calc_pixel<KEY>(C, qx, qy, qz);
    }
}


// Persistent FP64 kernel over one group of a batch: tiles of CS_BATCH_TILE
// pixels from the group's counter, pixel arithmetic as k_image.
template <int KEY>
__global__ void __launch_bounds__(CS_BATCH_TILE) k_batch_fp64(const cs::BatchSetDev *__restrict__ sets, int set_begin,
                                                              int set_end, long tiles,
                                                              unsigned long long *__restrict__ counter,
                                                              const cs_chi_node *__restrict__ chi,
                                                              double *__restrict__ out) {
    int cur = set_begin;
    long tile;
    int k;
    while (cs::batch_next_tile(sets, set_begin, set_end, tiles, counter, cur, tile, k)) {
        const cs::BatchSetDev &S = sets[k];
        const long t = (tile - S.tile_begin) * CS_BATCH_TILE + threadIdx.x;
        if (t >= S.npix) continue;
        const cs_prepared &P = *S.prep;
        const Ctx C{S.prep, chi, S.delta};
        const int ihex = P.zzmin + (int)(t % S.nx);
        const int i = P.iimin + (int)(t / S.nx);
        double qx, qy, qz;
        convert_idx2q(P, ihex, i, qx, qy, qz);
        const double v = calc_pixel<KEY>(C, qx, qy, qz);
        out[S.out_offset + (long)(ihex - P.xmin) + (long)(P.xmax - P.xmin) * (long)(i - P.ymin)] = v;
    }
}

// FP64 recomputation of the guarded pixels of a batch group: list entries are
// (set, linear pixel of the set's calculated region).
template <int KEY>
__global__ void __launch_bounds__(128) k_batch_redo(const cs::BatchSetDev *__restrict__ sets,
                                                    const cs_chi_node *__restrict__ chi, double *__restrict__ out,
                                                    const int *__restrict__ redo_count,
                                                    const int2 *__restrict__ redo_list, long redo_cap) {
    long n = *redo_count;
    if (n > redo_cap) n = redo_cap;
    for (long r = blockIdx.x * (long)blockDim.x + threadIdx.x; r < n; r += (long)gridDim.x * blockDim.x) {
        const int2 e = redo_list[r];
        const cs::BatchSetDev &S = sets[e.x];
        const cs_prepared &P = *S.prep;
        const Ctx C{S.prep, chi, S.delta};
        const long t = e.y;
        const int ihex = P.zzmin + (int)(t % S.nx);
        const int i = P.iimin + (int)(t / S.nx);
        double qx, qy, qz;
        convert_idx2q(P, ihex, i, qx, qy, qz);
        out[S.out_offset + (long)(ihex - P.xmin) + (long)(P.xmax - P.xmin) * (long)(i - P.ymin)] =
            calc_pixel<KEY>(C, qx, qy, qz);
    }
}

}  // namespace cs64

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

template <int KEY>
static void launch_image_key(const DevSet &D, const cs_prepared &P, double *d_out, cudaStream_t s) {
    const int nx = P.zzmax - P.zzmin;
    const long npix = (long)nx * (long)(P.iimax - P.iimin);
    cs64::Ctx C{D.d_prep, D.d_chi, D.d_delta};
    cs64::k_image<KEY><<<grid_for(npix, 256), 256, 0, s>>>(C, d_out, nx, npix);
}

int launch_image(const DevSet &D, const cs_prepared &P, double *d_out, cudaStream_t s) {
    const int nx = P.zzmax - P.zzmin, ny = P.iimax - P.iimin;
    if (nx <= 0 || ny <= 0) return CS_OK;
    switch (P.key) {
    case CS_KEY_SPHERE_NONE_ISO: launch_image_key<CS_KEY_SPHERE_NONE_ISO>(D, P, d_out, s); break;
    case CS_KEY_SPHERE_GAUSS_FCC_GAUSS: launch_image_key<CS_KEY_SPHERE_GAUSS_FCC_GAUSS>(D, P, d_out, s); break;
    case CS_KEY_CYL_NONE_GAUSS: launch_image_key<CS_KEY_CYL_NONE_GAUSS>(D, P, d_out, s); break;
    case CS_KEY_CYL_NONE_ZDIR: launch_image_key<CS_KEY_CYL_NONE_ZDIR>(D, P, d_out, s); break;
    case CS_KEY_CYL_GAUSS_BCT_ZDIR: launch_image_key<CS_KEY_CYL_GAUSS_BCT_ZDIR>(D, P, d_out, s); break;
    case CS_KEY_CUBE_NONE_ISO: launch_image_key<CS_KEY_CUBE_NONE_ISO>(D, P, d_out, s); break;
    case CS_KEY_GENERIC: launch_image_key<CS_KEY_GENERIC>(D, P, d_out, s); break;
    default: return CS_ERR_UNSUPPORTED;
    }
    if (P.expand && P.calc_quadrants != CS_RADQ4 && P.calc_quadrants != CS_RAD1D) launch_mirror(P, d_out, s);
    return cudaGetLastError() == cudaSuccess ? CS_OK : CS_ERR_CUDA;
}

void launch_mirror(const cs_prepared &P, double *d_out, cudaStream_t s) {
    const int q1 = P.calc_quadrants == CS_RADQ1;
    const long total = (long)P.zmax * (q1 ? P.zmax : 2 * P.zmax);
    k_mirror<<<grid_for(total, 256), 256, 0, s>>>(d_out, P.zmax, P.xmin, P.xmax, P.ymin, q1);
}

template <int KEY>
static void launch_redo_key(const DevSet &D, const cs_prepared &P, double *d_out, const MixedScratch &S,
                            cudaStream_t s) {
    const int nx = P.zzmax - P.zzmin;
    cs64::Ctx C{D.d_prep, D.d_chi, D.d_delta};
    cs64::k_redo<KEY><<<sm_count() * 4, 128, 0, s>>>(C, d_out, nx, S.d_count, S.d_list, S.cap);
}

int launch_redo(const DevSet &D, const cs_prepared &P, double *d_out, const MixedScratch &S, cudaStream_t s) {
    switch (P.key) {
    case CS_KEY_SPHERE_NONE_ISO: launch_redo_key<CS_KEY_SPHERE_NONE_ISO>(D, P, d_out, S, s); break;
    case CS_KEY_SPHERE_GAUSS_FCC_GAUSS: launch_redo_key<CS_KEY_SPHERE_GAUSS_FCC_GAUSS>(D, P, d_out, S, s); break;
    case CS_KEY_CYL_NONE_GAUSS: launch_redo_key<CS_KEY_CYL_NONE_GAUSS>(D, P, d_out, S, s); break;
    case CS_KEY_CYL_NONE_ZDIR: launch_redo_key<CS_KEY_CYL_NONE_ZDIR>(D, P, d_out, S, s); break;
    case CS_KEY_CYL_GAUSS_BCT_ZDIR: launch_redo_key<CS_KEY_CYL_GAUSS_BCT_ZDIR>(D, P, d_out, S, s); break;
    case CS_KEY_CUBE_NONE_ISO: launch_redo_key<CS_KEY_CUBE_NONE_ISO>(D, P, d_out, S, s); break;
    case CS_KEY_GENERIC: launch_redo_key<CS_KEY_GENERIC>(D, P, d_out, S, s); break;
    default: return CS_ERR_UNSUPPORTED;
    }
    return CS_OK;
}

template <int KEY>
static void launch_fit_key(const DevSet &D, const cs_prepared &P, const double *d_data, double *d_fqs, long nbuf,
                           cudaStream_t s) {
    const long nfit = (long)P.fit_width * P.fit_height;
    cs64::Ctx C{D.d_prep, D.d_chi, D.d_delta};
    cs64::k_fit<KEY><<<grid_for(nfit, 256), 256, 0, s>>>(C, d_data, d_fqs, nfit, nbuf);
}

int launch_fit(const DevSet &D, const cs_prepared &P, const double *d_data, double *d_fqs, long nbuf,
               FitReduce &R, cudaStream_t s) {
    switch (P.key) {
    case CS_KEY_SPHERE_NONE_ISO: launch_fit_key<CS_KEY_SPHERE_NONE_ISO>(D, P, d_data, d_fqs, nbuf, s); break;
    case CS_KEY_SPHERE_GAUSS_FCC_GAUSS: launch_fit_key<CS_KEY_SPHERE_GAUSS_FCC_GAUSS>(D, P, d_data, d_fqs, nbuf, s); break;
    case CS_KEY_CYL_NONE_GAUSS: launch_fit_key<CS_KEY_CYL_NONE_GAUSS>(D, P, d_data, d_fqs, nbuf, s); break;
    case CS_KEY_CYL_NONE_ZDIR: launch_fit_key<CS_KEY_CYL_NONE_ZDIR>(D, P, d_data, d_fqs, nbuf, s); break;
    case CS_KEY_CYL_GAUSS_BCT_ZDIR: launch_fit_key<CS_KEY_CYL_GAUSS_BCT_ZDIR>(D, P, d_data, d_fqs, nbuf, s); break;
    case CS_KEY_CUBE_NONE_ISO: launch_fit_key<CS_KEY_CUBE_NONE_ISO>(D, P, d_data, d_fqs, nbuf, s); break;
    case CS_KEY_GENERIC: launch_fit_key<CS_KEY_GENERIC>(D, P, d_data, d_fqs, nbuf, s); break;
    default: return CS_ERR_UNSUPPORTED;
    }
    const int nb = R.nblocks;
    k_fit_reduce1<<<nb, 256, 0, s>>>(d_fqs, nbuf, R.d_psum, R.d_pcnt, R.d_pnan);
    k_fit_reduce2<<<1, 32, 0, s>>>(R.d_psum, R.d_pcnt, R.d_pnan, nb, R.d_sum, R.d_cnt, R.d_nan);
    return cudaGetLastError() == cudaSuccess ? CS_OK : CS_ERR_CUDA;
}


// ---- batch launchers -------------------------------------------------------

int launch_batch_fp64(const BatchSetDev *d_sets, const BatchGroup &g, unsigned long long *d_counter,
                      const cs_chi_node *d_chi, double *d_out, int grid, cudaStream_t s) {
    if (g.tiles <= 0) return CS_OK;
    switch (g.key) {
#define CS_CASE(K)                                                                                              \
    case K:                                                                                                     \
        cs64::k_batch_fp64<K><<<grid, CS_BATCH_TILE, 0, s>>>(d_sets, g.set_begin, g.set_end, g.tiles, d_counter, \
                                                             d_chi, d_out);                                     \
        break;
        CS_FOR_EACH_KEY_FP64(CS_CASE)
#undef CS_CASE
    default: return CS_ERR_UNSUPPORTED;
    }
    return cudaGetLastError() == cudaSuccess ? CS_OK : CS_ERR_CUDA;
}

int launch_batch_redo(const BatchSetDev *d_sets, int key, const cs_chi_node *d_chi, double *d_out, const int *d_count,
                      const int2 *d_list, long cap, cudaStream_t s) {
    const int grid = sm_count() * 4;
    switch (key) {
#define CS_CASE(K)                                                                                  \
    case K: cs64::k_batch_redo<K><<<grid, 128, 0, s>>>(d_sets, d_chi, d_out, d_count, d_list, cap); break;
        CS_FOR_EACH_KEY_FP64(CS_CASE)
#undef CS_CASE
    default: return CS_ERR_UNSUPPORTED;
    }
    return cudaGetLastError() == cudaSuccess ? CS_OK : CS_ERR_CUDA;
}

int batch_blocks_per_sm_fp64(int key) {
    int n = 0;
    switch (key) {
#define CS_CASE(K) \
    case K: cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, cs64::k_batch_fp64<K>, CS_BATCH_TILE, 0); break;
        CS_FOR_EACH_KEY_FP64(CS_CASE)
#undef CS_CASE
    default: return 0;
    }
    return n;
}


// FQS arrays and chi^2 per set of a batch whose images are in d_img.
int launch_batch_fit(const BatchSetDev *d_sets, int nsets, const double *d_img, const double *d_data, double *d_fqs,
                     long nfit, long nbuf, const BatchFitReduce &R, cudaStream_t s) {
    if (nsets <= 0) return CS_OK;
    if (cudaMemsetAsync(d_fqs, 0, sizeof(double) * (size_t)nbuf * (size_t)nsets, s) != cudaSuccess) return CS_ERR_CUDA;
    const int gx = grid_for(nfit, 256);
    k_batch_fqs<<<dim3(gx, nsets), 256, 0, s>>>(d_sets, d_img, d_data, d_fqs, nfit, nbuf);
    k_batch_fit_reduce1<<<dim3(R.nblocks, nsets), 256, 0, s>>>(d_fqs, nbuf, R.d_psum, R.d_pcnt, R.d_pnan);
    k_batch_fit_reduce2<<<(nsets + 127) / 128, 128, 0, s>>>(R.d_psum, R.d_pcnt, R.d_pnan, R.nblocks, nsets, R.d_sum,
                                                            R.d_cnt, R.d_nan);
    return cudaGetLastError() == cudaSuccess ? CS_OK : CS_ERR_CUDA;
}

}  // namespace cs
