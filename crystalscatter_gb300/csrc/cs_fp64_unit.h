// cs_fp64_unit.h — per-key launchers of the FP64 drop-in kernels (internal).
//
// Fp64Unit<KEY> is defined and explicitly instantiated in cs_fp64_unit.cu,
// which the build compiles once per dispatch key (-DCS_UNIT_KEY=...): the
// keys' kernels compile in parallel instead of in one long translation unit.
// The caller (cs_kernels.cu) chooses the grids.
#ifndef CS_FP64_UNIT_H
#define CS_FP64_UNIT_H

#include <cuda_runtime.h>

#include "cs_batch.h"
#include "cs_launch.h"
#include "cs_mixed.h"

namespace cs {

template <int KEY>
struct Fp64Unit {
    // k_image over the calculated region of P
    static void image(const DevSet &D, const cs_prepared &P, double *d_out, int grid, cudaStream_t s);
    // k_redo over the redo list of the mixed path
    static void redo(const DevSet &D, const cs_prepared &P, double *d_out, const MixedScratch &S, int grid,
                     cudaStream_t s);
    // k_fit over the fit region
    static void fit(const DevSet &D, const cs_prepared &P, const double *d_data, double *d_fqs, long nbuf, int grid,
                    cudaStream_t s);
    // persistent k_batch_fp64 over one batch group
    static void batch(const BatchSetDev *d_sets, const BatchGroup &g, unsigned long long *d_counter,
                      const cs_chi_node *d_chi, double *d_out, int grid, cudaStream_t s);
    // k_batch_redo over a batch group's redo list
    static void batch_redo(const BatchSetDev *d_sets, const cs_chi_node *d_chi, double *d_out, const int *d_count,
                           const int2 *d_list, long cap, int grid, cudaStream_t s);
    // resident blocks per SM of k_batch_fp64
    static int batch_blocks_per_sm();
};

}  // namespace cs

#endif
