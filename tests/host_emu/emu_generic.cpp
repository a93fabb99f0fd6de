// Test infrastructure: the FP64 device pixel functions (cs_fp64.cuh) compiled
// for the host, so that the generic pixel function's logic (branches, switch
// points, quadrature, operation order) is checked on the CPU against the
// reference's golden images. The handful of CUDA intrinsics the header uses
// get plain host equivalents (round-to-nearest products and sums, a one-lane
// warp); the host math library stands in for CUDA's, which is the reference's
// own. Built and loaded by tests/test_device_code_host.py only.
#include <cmath>
#include <cstring>
#define __device__
#define __host__
#define __global__
#define __forceinline__ inline
#define __noinline__ __attribute__((noinline))
#define __launch_bounds__(...)
struct EmuDim3 {
    unsigned x, y, z;
};
static EmuDim3 threadIdx{0, 0, 0};
static inline double __dmul_rn(double a, double b) { return a * b; }
static inline double __dadd_rn(double a, double b) { return a + b; }
static inline double __shfl_sync(unsigned, double v, int) { return v; }
static inline float __shfl_sync(unsigned, float v, int) { return v; }
static inline int __shfl_sync(unsigned, int v, int) { return v; }
static inline int __double2hiint(double d) {
    long long b;
    std::memcpy(&b, &d, 8);
    return (int)(b >> 32);
}
using std::isfinite;
using std::isinf;
using std::isnan;
#include "cs_fp64.cuh"
#include "cs_launch.h"

// the calculated region (rows iimin..iimax-1, columns zzmin..zzmax-1) of the
// generic pixel function, row-major
extern "C" int emu_generic_region(const cs_prepared *P, double *out) {
    static cs_chi_node chi[CS_CHI_TABLE_LEN];
    static cs_delta_node dn[CS_NODE_COUNT];
    cs::build_chi_table(P->romb_chi_b, chi);
    cs::build_delta_table(P->romb_delta_b, P->romb_dbeta, dn);
    const cs64::Ctx C{P, chi, dn};
    long k = 0;
    for (int i = P->iimin; i < P->iimax; i++)
        for (int ihex = P->zzmin; ihex < P->zzmax; ihex++) {
            double qx, qy, qz;
            cs64::convert_idx2q(*P, ihex, i, qx, qy, qz);
            out[k++] = cs64::calc_generic(C, qx, qy, qz);
        }
    return 0;
}
