// cs_fp64_kernels.cuh — FP64 drop-in kernel templates (internal).
//
// One thread computes one detector pixel; consecutive threads take
// consecutive ihex (the fastest image index), so the FP64 image store of a warp
// is one contiguous 256-byte segment. The reference launches one 16x16 block
// per image tile (Source/sc_calc_generic_gpu.cu:94-99); here the grid is a
// grid-stride loop sized to a multiple of the SM count so uneven per-pixel
// cost (series vs. asymptote vs. nested Romberg) does not leave SMs idle.
//
// The templates are instantiated one dispatch key per translation unit
// (cs_fp64_unit.cu, compiled once per key) so that the keys compile in
// parallel.
#ifndef CS_FP64_KERNELS_CUH
#define CS_FP64_KERNELS_CUH

#include <cuda_runtime.h>

#include "cs_batch.cuh"
#include "cs_fp64.cuh"

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
        if (!cs::batch_q_from_table(S, ihex, i, qx, qy, qz)) convert_idx2q(P, ihex, i, qx, qy, qz);
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
        if (!cs::batch_q_from_table(S, ihex, i, qx, qy, qz)) convert_idx2q(P, ihex, i, qx, qy, qz);
        out[S.out_offset + (long)(ihex - P.xmin) + (long)(P.xmax - P.xmin) * (long)(i - P.ymin)] =
            calc_pixel<KEY>(C, qx, qy, qz);
    }
}

}  // namespace cs64

#endif
