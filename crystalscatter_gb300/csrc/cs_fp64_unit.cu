// cs_fp64_unit.cu — the FP64 drop-in kernels of one dispatch key.
//
// Compiled once per key with -DCS_UNIT_KEY=<key> (crystalscatter_gb300/build.py);
// each object holds k_image, k_redo, k_fit, k_batch_fp64 and k_batch_redo of
// that key and the host launchers of cs_fp64_unit.h.
#include <cuda_runtime.h>

#include "cs_fp64_kernels.cuh"
#include "cs_fp64_unit.h"

#ifndef CS_UNIT_KEY
#error "compile with -DCS_UNIT_KEY=<dispatch key>"
#endif

namespace cs {

template <int KEY>
void Fp64Unit<KEY>::image(const DevSet &D, const cs_prepared &P, double *d_out, int grid, cudaStream_t s) {
    const int nx = P.zzmax - P.zzmin;
    const long npix = (long)nx * (long)(P.iimax - P.iimin);
    cs64::Ctx C{D.d_prep, D.d_chi, D.d_delta};
    cs64::k_image<KEY><<<grid, 256, 0, s>>>(C, d_out, nx, npix);
}

template <int KEY>
void Fp64Unit<KEY>::redo(const DevSet &D, const cs_prepared &P, double *d_out, const MixedScratch &S, int grid,
                         cudaStream_t s) {
    const int nx = P.zzmax - P.zzmin;
    cs64::Ctx C{D.d_prep, D.d_chi, D.d_delta};
    cs64::k_redo<KEY><<<grid, 128, 0, s>>>(C, d_out, nx, S.d_count, S.d_list, S.cap);
}

template <int KEY>
void Fp64Unit<KEY>::fit(const DevSet &D, const cs_prepared &P, const double *d_data, double *d_fqs, long nbuf,
                        int grid, cudaStream_t s) {
    const long nfit = (long)P.fit_width * P.fit_height;
    cs64::Ctx C{D.d_prep, D.d_chi, D.d_delta};
    cs64::k_fit<KEY><<<grid, 256, 0, s>>>(C, d_data, d_fqs, nfit, nbuf);
}

template <int KEY>
void Fp64Unit<KEY>::batch(const BatchSetDev *d_sets, const BatchGroup &g, unsigned long long *d_counter,
                          const cs_chi_node *d_chi, double *d_out, int grid, cudaStream_t s) {
    cs64::k_batch_fp64<KEY><<<grid, CS_BATCH_TILE, 0, s>>>(d_sets, g.set_begin, g.set_end, g.tiles, d_counter, d_chi,
                                                           d_out);
}

template <int KEY>
void Fp64Unit<KEY>::batch_redo(const BatchSetDev *d_sets, const cs_chi_node *d_chi, double *d_out,
                               const int *d_count, const int2 *d_list, long cap, int grid, cudaStream_t s) {
    cs64::k_batch_redo<KEY><<<grid, 128, 0, s>>>(d_sets, d_chi, d_out, d_count, d_list, cap);
}

template <int KEY>
int Fp64Unit<KEY>::batch_blocks_per_sm() {
    int n = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, cs64::k_batch_fp64<KEY>, CS_BATCH_TILE, 0);
    return n;
}

template struct Fp64Unit<CS_UNIT_KEY>;

}  // namespace cs
