// cs_mixed.h — mixed-precision path: compact peak tables and redo scratch (internal).
#ifndef CS_MIXED_H
#define CS_MIXED_H

#include <cuda_runtime.h>

#include <vector>

#include "cs_launch.h"
#include "cs_prepared.h"

namespace csm {

// Reflection tables of one parameter set in the form the FP32 peak sums read:
// entries that the reference would skip are dropped, the rest sorted by q_hkl.
struct PeakTab {
    int n_aniso = 0;
    const float *aq = nullptr;   // q_hkl
    const float4 *av = nullptr;  // per reflection two entries: unit q_hkl (x, y, z), mult * g3/peaknorm1;
                                 // low parts of the unit vector, 1 - |h|/q_hkl
    const float *awl = nullptr;  // low part of av[2i].w (mult g3/peaknorm1 = av[2i].w + awl[i])
    const int *aidx = nullptr;   // row of the reflection in latpar2/latpar3
    int n_iso = 0;
    const float *iq = nullptr;
    const float *imf = nullptr;
    // per-set factors of the sums (cs::peak_constants): exp2 scales
    // 4 log2(e)/(pi w^2) and normalisations 1/(pi w/2) of the isotropic and
    // anisotropic peaks, their windows 9.4 w, and 4 log2(e)/(pi phiwidth^2);
    // the anisotropic ones only when the width does not depend on q (para 0)
    double kd_iso = 0, inv_iso = 0, kd_an = 0, inv_an = 0, kphi = 0;
    // the structure factors' 2 pi/V and 8 pi^3/(4 pi V), V the cell volume
    double c_r1 = 0, c_r2 = 0;
    float dmax_iso = 0, dmax_an = 0;
};

}  // namespace csm

namespace cs {

// Redo list of the mixed kernels (pixels recomputed in FP64).
struct MixedScratch {
    int *d_count = nullptr;  // [0] redo counter, [1] pixel queue of the mixed kernel
    int *d_list = nullptr;
    int cap = 0;
};

// Host form of the compact peak tables (built from the prepared block).
struct HostPeaks {
    std::vector<float> aq, awl, iq, imf;
    std::vector<float4> av;
    std::vector<int> aidx;
};
void build_peak_tables(const cs_prepared &P, HostPeaks &H);
// fills the per-set factors of T from the prepared block
void peak_constants(const cs_prepared &P, csm::PeakTab &T);

int launch_image_mixed(const DevSet &D, const csm::PeakTab &T, const cs_prepared &P, double *d_out, MixedScratch &S,
                       cudaStream_t s);
int launch_redo(const DevSet &D, const cs_prepared &P, double *d_out, const MixedScratch &S, cudaStream_t s);
void launch_mirror(const cs_prepared &P, double *d_out, cudaStream_t s);

}  // namespace cs

#endif
