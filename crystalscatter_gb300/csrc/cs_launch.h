// cs_launch.h — device-side entry points used by the C ABI (internal).
#ifndef CS_LAUNCH_H
#define CS_LAUNCH_H

#include <cuda_runtime.h>

#include "../../include/crystalscatter.h"
#include "cs_prepared.h"
#include "cs_tables.h"

namespace cs {

// Device copies of one prepared parameter set.
struct DevSet {
    const cs_prepared *d_prep = nullptr;     // prepared block in device memory
    const cs_chi_node *d_chi = nullptr;      // chi node table (shared by all sets)
    const cs_delta_node *d_delta = nullptr;  // delta node table of this set (orientation average only)
};

// Scratch of the two-pass fit reduction.
struct FitReduce {
    int nblocks = 0;
    double *d_psum = nullptr;
    unsigned long long *d_pcnt = nullptr, *d_pnan = nullptr;
    double *d_sum = nullptr;
    unsigned long long *d_cnt = nullptr, *d_nan = nullptr;
};

// The CUDA error seen by the most recent launcher in this host thread
// (cudaSuccess after a good launch). Launchers end with launch_status(),
// which reads cudaGetLastError() once, records the code here and returns
// CS_OK or CS_ERR_CUDA; callers build their message from this code (a second
// cudaGetLastError() would already read cudaSuccess).
cudaError_t last_launch_error();
int launch_status();

bool key_supported(const cs_prepared &P);
// keys with a mixed-precision kernel; the others (and twinned lattices) run
// their FP64 kernel when mixed precision is requested (exact, so within any
// mixed tolerance)
bool mixed_key(int key);
// True when the prepared set evaluates the cylinder orientation integral.
bool needs_delta_table(const cs_prepared &P);

int launch_image(const DevSet &D, const cs_prepared &P, double *d_out, cudaStream_t s);
int launch_fit(const DevSet &D, const cs_prepared &P, const double *d_data, double *d_fqs, long nbuf, FitReduce &R,
               cudaStream_t s);

// Host-side node tables (built with the host libm, node by node in the
// reference's order); see cs_tables.h.
void build_chi_table(double chi_b, cs_chi_node *tab);  // tab: CS_CHI_TABLE_LEN slots
void build_delta_table(double delta_b, double dbeta, cs_delta_node *tab);

}  // namespace cs

#endif
