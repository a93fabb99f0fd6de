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
    const float *amf = nullptr;  // multiplicity * structure factor (also folded into av[2i].w)
    const int *aidx = nullptr;   // row of the reflection in latpar2/latpar3
    int n_iso = 0;
    const float *iq = nullptr;
    const float *imf = nullptr;
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
    std::vector<float> aq, amf, iq, imf;
    std::vector<float4> av;
    std::vector<int> aidx;
};
void build_peak_tables(const cs_prepared &P, HostPeaks &H);

int launch_image_mixed(const DevSet &D, const csm::PeakTab &T, const cs_prepared &P, double *d_out, MixedScratch &S,
                       cudaStream_t s);
int launch_redo(const DevSet &D, const cs_prepared &P, double *d_out, const MixedScratch &S, cudaStream_t s);
void launch_mirror(const cs_prepared &P, double *d_out, cudaStream_t s);

}  // namespace cs

#endif
