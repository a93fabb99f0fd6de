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

#include "cs_fp64.cuh"
#include "cs_launch.h"

namespace cs64 {

__device__ __forceinline__ double tail(const cs_prepared &P, double q, double core) {
    return core + P.ifluc / (1 + q * q * P.rfluc * P.rfluc);
}

// calc_partSphere_lattNone_ordisIsotropic, Source/sc_gpu_pSph_lNon_oIso.h:15-51
__device__ double calc_sphere_none_iso(const Ctx &C, double qx, double qy, double qz) {
    const cs_prepared &P = *C.P;
    const double q = sqrt(qx * qx + qy * qy + qz * qz) + CS_EPS9;
    const double pq = formpq_sphere(P, q);
    return P.base + P.izero * (pq + P.iso * pq) + P.ifluc / (1 + q * q * P.rfluc * P.rfluc);
}

// Peak sums shared by the FCC and BCT kernels
// (Source/sc_gpu_pSph_pGau_lFCC_oGau.h:53-143, sc_gpu_pCyl_pGau_lBCT_oZDi.h:133-211).
__device__ void peak_sums(const cs_prepared &P, double qx, double qy, double qz, double q, double &radintensity,
                          double &intensity) {
    double width = 1;
    if (P.debyescherrer) width = 4.0 / P.domainsize;
    if (P.para) width = (4.0 / P.domainsize) + sqr(P.reldis) * P.dist * sqr(q);
    width *= P.width_zuf;
    const double widthiso = 1.0 / P.uca;
    radintensity = 0.0;
    intensity = 0.0;
    for (int ii = 1; ii <= P.peakmax1; ii++) {
        const int mhkl = P.latpar1[ii][4];
        const int fhkl = P.latpar1[ii][5];
        if (mhkl == 0 || fhkl == 0) continue;
        const double qhkl = P.latpar3[ii][5];
        const double x2 = sqr(q - qhkl) / sqr(widthiso);
        const double sq = exp(-4 * x2 / M_PI) / (M_PI * widthiso / 2.0);
        radintensity += sq * mhkl * fhkl;
    }
    const double x2phi = 4 * q * q / (M_PI * sqr(P.phiwidth));
    for (int ii = 1; ii <= P.peakmax2; ii++) {
        const double qhkl = P.latpar3[ii][5];
        const int mhkl_fhkl = P.latpar2[ii][4] * P.latpar2[ii][5];
        if (qhkl > 0 && mhkl_fhkl != 0) {
            const double qxhkl = P.latpar3[ii][2];
            const double qyhkl = P.latpar3[ii][3];
            const double qzhkl = P.latpar3[ii][4];
            const double g3 = P.latpar3[ii][10];
            const double peaknorm1 = P.latpar3[ii][11];
            const double yphi = myacos((qx * qxhkl + qy * qyhkl + qz * qzhkl) / (q * qhkl));
            const double x2 = (q - qhkl) * (q - qhkl) / (width * width);
            const double sq = exp(-4 * x2 / M_PI) / (M_PI * width / 2.0);
            double psiord = g3 * exp(-x2phi * yphi * yphi) / peaknorm1;
            if (P.twin) {
                const double qxhklt = P.latpar3[ii][7];
                const double qyhklt = P.latpar3[ii][8];
                const double qzhklt = P.latpar3[ii][9];
                const double qhklt = P.latpar3[ii][14];
                const double g3t = P.latpar3[ii][15];
                const double peaknorm1t = P.latpar3[ii][16];
                const double yphit = myacos((qx * qxhklt + qy * qyhklt + qz * qzhklt) / (q * qhklt));
                const double phiord = g3t * exp(-x2phi * yphit * yphit) / peaknorm1t;
                psiord = P.ceff * psiord + (1 - P.ceff) * phiord;
            }
            const double savintens = intensity;
            intensity += sq * mhkl_fhkl * psiord;
            if (isinf(intensity)) {
                intensity = savintens;
                break;
            }
        }
    }
}

// calc_partSphere_peakGauss_lattFCC_ordisGauss, Source/sc_gpu_pSph_pGau_lFCC_oGau.h:15-171
__device__ double calc_sphere_fcc(const Ctx &C, double qx, double qy, double qz) {
    const cs_prepared &P = *C.P;
    const double q = sqrt(qx * qx + qy * qy + qz * qz) + CS_EPS9;
    const double pq = formpq_sphere(P, q);
    const double fq = formfq_sphere(P, q);
    const double pqiso = pq;
    double radintensity, intensity;
    peak_sums(P, qx, qy, qz, q, radintensity, intensity);
    const double sphno_cubevol = P.latpar[1] * P.latpar[2];
    const double szqiso = (1 + (1) * (8 * M_PI * M_PI * M_PI * radintensity / (4 * M_PI * sphno_cubevol) - 1) *
                                   exp(-P.ucb * q * q));
    const double szq = (1 + (fq / pq) * (2 * M_PI * intensity / sphno_cubevol - 1) * exp(-P.dwfactor * q * q));
    return P.base + P.izero * (szq * pq + P.iso * szqiso * pqiso) + P.ifluc / (1 + q * q * P.rfluc * P.rfluc);
}

// calc_partCylinder_lattNone_ordisGauss, Source/sc_gpu_pCyl_lNon_oGau.h:15-100
// (the lattice branch for F(q) is not taken: lattice is "None").
__device__ double calc_cyl_none_gauss(const Ctx &C, double qx, double qy, double qz) {
    const cs_prepared &P = *C.P;
    double pq = 0;
    const double q = sqrt(qx * qx + qy * qy + qz * qz) + CS_EPS9;
    switch (P.orcase) {
    case CS_ORC_GENERAL:
        pq = formpq_cylinder(C, qx * P.cosphic - qy * P.sinphic, qx * P.sinphic + qy * P.cosphic, q);
        break;
    case CS_ORC_XAXIS:
    case CS_ORC_YAXIS:
    case CS_ORC_ZAXIS:
        pq = formpq_cylinder(C, qx, qy, q);
        break;
    }
    return P.base + P.izero * (pq + P.iso) + P.ifluc / (1 + q * q * P.rfluc * P.rfluc);
}

// calc_partCylinder_lattNone_ordisZDir, Source/sc_gpu_pCyl_lNon_oZDi.h:17-88
__device__ double calc_cyl_none_zdir(const Ctx &C, double qx, double qy, double qz) {
    const cs_prepared &P = *C.P;
    double pq = 0;
    const double q = sqrt(qx * qx + qy * qy + qz * qz) + CS_EPS9;
    switch (P.orcase) {
    case CS_ORC_GENERAL: pq = formpq_cylinder(C, qx * P.cosphi * P.sintheta, qy * P.sinphi * P.sintheta, q); break;
    case CS_ORC_XAXIS: pq = formpq_cylinder(C, qx, 0, q); break;
    case CS_ORC_YAXIS: pq = formpq_cylinder(C, 0, qy, q); break;
    case CS_ORC_ZAXIS: pq = formpq_cylinder(C, qx, qy, q); break;
    }
    return P.base + P.izero * (pq + P.iso) + P.ifluc / (1 + q * q * P.rfluc * P.rfluc);
}

// calc_partCylinder_peakGauss_lattBCT_ordisZDir, Source/sc_gpu_pCyl_pGau_lBCT_oZDi.h:16-245
__device__ double calc_cyl_bct_zdir(const Ctx &C, double qx, double qy, double qz) {
    const cs_prepared &P = *C.P;
    double pq = 0, fq = 0;
    const double q = sqrt(qx * qx + qy * qy + qz * qz) + CS_EPS9;
    const double pqiso = 1;
    switch (P.orcase) {
    case CS_ORC_GENERAL:
        pq = formpq_cylinder(C, qx * P.cosphi * P.sintheta, qy * P.sinphi * P.sintheta, q);
        fq = formfq_cylinder(C, sqrt(P.cosphi * qx * qx + P.sinphi * qy * qy + CS_EPS9), qx * P.cosphi * P.sintheta,
                             qy * P.sinphi * P.sintheta, q);
        break;
    case CS_ORC_XAXIS:
        pq = formpq_cylinder(C, qx, 0, q);
        fq = formfq_cylinder(C, fabs(qx), qx, 0, q);
        break;
    case CS_ORC_YAXIS:
        pq = formpq_cylinder(C, 0, qy, q);
        fq = formfq_cylinder(C, fabs(qy), 0, qy, q);
        break;
    case CS_ORC_ZAXIS:
        pq = formpq_cylinder(C, qx, qy, q);
        fq = formfq_cylinder(C, q, qx, qy, q);
        break;
    }
    double radintensity, intensity;
    peak_sums(P, qx, qy, qz, q, radintensity, intensity);
    const double sphno_cubevol = P.latpar[1] * P.latpar[2];
    const double szqiso = (1 + (1) * (8 * M_PI * M_PI * M_PI * radintensity / (4 * M_PI * sphno_cubevol) - 1) *
                                   exp(-P.ucb * q * q));
    const double szq = (1 + (fq / pq) * (2 * M_PI * intensity / (sphno_cubevol)-1) * exp(-P.dwfactor * q * q));
    return P.base + P.izero * (szq * pq + P.iso * szqiso * pqiso) + P.ifluc / (1 + q * q * P.rfluc * P.rfluc);
}

template <int KEY>
__device__ __forceinline__ double calc_pixel(const Ctx &C, double qx, double qy, double qz) {
    if (KEY == CS_KEY_SPHERE_NONE_ISO) return calc_sphere_none_iso(C, qx, qy, qz);
    if (KEY == CS_KEY_SPHERE_GAUSS_FCC_GAUSS) return calc_sphere_fcc(C, qx, qy, qz);
    if (KEY == CS_KEY_CYL_NONE_GAUSS) return calc_cyl_none_gauss(C, qx, qy, qz);
    if (KEY == CS_KEY_CYL_NONE_ZDIR) return calc_cyl_none_zdir(C, qx, qy, qz);
    if (KEY == CS_KEY_CYL_GAUSS_BCT_ZDIR) return calc_cyl_bct_zdir(C, qx, qy, qz);
    return 0.0;
}

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
__global__ void k_fit_reduce1(const double *__restrict__ fqs, long n, double *__restrict__ psum,
                              unsigned long long *__restrict__ pcnt, unsigned long long *__restrict__ pnan) {
    __shared__ double ss[32];
    __shared__ unsigned long long sc[32], sn[32];
    double s = 0.0;
    unsigned long long c = 0, nn = 0;
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
        if (lane == 0) {
            psum[blockIdx.x] = s;
            pcnt[blockIdx.x] = c;
            pnan[blockIdx.x] = nn;
        }
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
    if (P.ign_switch) return false;
    switch (P.key) {
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
    default: return CS_ERR_UNSUPPORTED;
    }
    if (P.expand && P.calc_quadrants != CS_RADQ4 && P.calc_quadrants != CS_RAD1D) {
        const int q1 = P.calc_quadrants == CS_RADQ1;
        const long total = (long)P.zmax * (q1 ? P.zmax : 2 * P.zmax);
        k_mirror<<<grid_for(total, 256), 256, 0, s>>>(d_out, P.zmax, P.xmin, P.xmax, P.ymin, q1);
    }
    return cudaGetLastError() == cudaSuccess ? CS_OK : CS_ERR_CUDA;
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
    default: return CS_ERR_UNSUPPORTED;
    }
    const int nb = R.nblocks;
    k_fit_reduce1<<<nb, 256, 0, s>>>(d_fqs, nbuf, R.d_psum, R.d_pcnt, R.d_pnan);
    k_fit_reduce2<<<1, 32, 0, s>>>(R.d_psum, R.d_pcnt, R.d_pnan, nb, R.d_sum, R.d_cnt, R.d_nan);
    return cudaGetLastError() == cudaSuccess ? CS_OK : CS_ERR_CUDA;
}

}  // namespace cs
