// cs_batch.h — many parameter sets in one launch (internal).
//
// A batch holds N prepared parameter sets of possibly different detector
// sizes; their images lie one after another in one output buffer. Sets are
// grouped by dispatch key (one specialised kernel per key). Within a group the
// calculated pixels of all sets are cut into tiles of CS_BATCH_TILE pixels,
// numbered set after set. A persistent kernel (one resident grid) takes the
// next tile from a device counter until the group's tiles run out, so uneven
// set sizes and uneven per-pixel cost balance across the SMs without the host.
// The mixed form appends guarded pixels, as (set, pixel) pairs, to one redo
// list shared by all sets; a second persistent kernel recomputes them in FP64.
#ifndef CS_BATCH_H
#define CS_BATCH_H

#include <cuda_runtime.h>

#include "cs_launch.h"
#include "cs_mixed.h"

namespace cs {

#define CS_BATCH_TILE 256

// The keys that have batch kernels (X-macro over the specialised pixel functions).
#define CS_FOR_EACH_KEY(M)           \
    M(CS_KEY_SPHERE_NONE_ISO)        \
    M(CS_KEY_SPHERE_GAUSS_FCC_GAUSS) \
    M(CS_KEY_CYL_NONE_GAUSS)         \
    M(CS_KEY_CYL_NONE_ZDIR)          \
    M(CS_KEY_CYL_GAUSS_BCT_ZDIR)

// the keys with an FP64 kernel: the above plus the cube and the generic pixel
// function (which have no mixed-precision kernel; mixed requests run FP64)
#define CS_FOR_EACH_KEY_FP64(M) \
    CS_FOR_EACH_KEY(M)          \
    M(CS_KEY_CUBE_NONE_ISO)     \
    M(CS_KEY_GENERIC)

// One set as the batch kernels see it (array in device memory).
struct BatchSetDev {
    const cs_prepared *prep;     // the set's prepared block
    const cs_delta_node *delta;  // the set's delta node table (orientation average only) or null
    csm::PeakTab peaks;          // compact reflection tables (mixed form)
    long out_offset;             // first double of the set's image in the output buffer
    long tile_begin;             // first tile of the set within its group
    long npix;                   // calculated pixels (zzmax-zzmin)*(iimax-iimin)
    int nx;                      // zzmax - zzmin
    int key;                     // dispatch key
    // Pixel geometry table shared by the sets of one detector geometry, or
    // null: q of pixel (ihex, i) at qtab[j], qtab[j + qn], qtab[j + 2 qn]
    // (x, y, z), j = (i + qhalf) qw + (ihex + qhalf), qn = qw * qw.
    const double *qtab;
    int qhalf, qw;
};

// One pixel geometry table: the q vectors of every pixel of a square
// [-half, half]^2 detector region, computed with the drop-in's convert_idx2q
// from the prepared block of its largest set (prep). Sets whose pixel
// coordinates map to the same detector positions (mdet = ihex and ndet = i
// exactly: pixno = 2 zmax) and share pixel size, beam centre, distance and
// wavelength get bit for bit the q vectors they would compute themselves.
struct QTable {
    const cs_prepared *prep = nullptr;
    int half = 0;
    double *d = nullptr;
};
// Fills a table on stream s.
int launch_qtable(const QTable &t, cudaStream_t s);

// Sets [set_begin, set_end) of the device array share one key and own tiles
// [0, tiles) of the group.
struct BatchGroup {
    int key = 0;
    int set_begin = 0, set_end = 0;
    long tiles = 0;
};

struct BatchRedo {
    int *d_count = nullptr;   // one counter per group
    int2 *d_list = nullptr;   // per group a slice of cap entries: (set, pixel of the calculated region)
    long cap = 0;             // entries per group
};

// Persistent mixed-precision launch over one group followed by the FP64 redo
// of its guarded pixels. counter must be zero when the launch starts.
// `mid`, when given, is recorded on s between the two (kernel timing).
// chunk: the work unit (0 = block tiles of CS_BATCH_TILE pixels with
// barriers; 32..CS_BATCH_TILE = that many pixels per warp, no barrier);
// limit > 0: stop after that many units; redo = false: the main kernel only.
int launch_batch_mixed(const BatchSetDev *d_sets, const BatchGroup &g, int group_index, unsigned long long *d_counter,
                       const cs_chi_node *d_chi, double *d_out, const BatchRedo &R, int grid, cudaStream_t s,
                       cudaEvent_t mid = nullptr, int chunk = 0, long limit = 0, bool redo = true);
// Persistent FP64 launch over one group (the drop-in arithmetic).
int launch_batch_fp64(const BatchSetDev *d_sets, const BatchGroup &g, unsigned long long *d_counter,
                      const cs_chi_node *d_chi, double *d_out, int grid, cudaStream_t s);
int launch_batch_redo(const BatchSetDev *d_sets, int key, const cs_chi_node *d_chi, double *d_out,
                      const int *d_count, const int2 *d_list, long cap, cudaStream_t s);
// Two-pass chi^2 reduction of a batch: partials [set][nblocks], results [set].
struct BatchFitReduce {
    int nblocks = 256;  // the single-set reduction's block count (same partials)
    double *d_psum = nullptr;
    unsigned long long *d_pcnt = nullptr, *d_pnan = nullptr;
    double *d_sum = nullptr;
    unsigned long long *d_cnt = nullptr, *d_nan = nullptr;
};
// FQS of every set's image (d_img, batch layout) against d_data (nbuf = fit
// width x height doubles), then chi^2, count and NaN count per set.
int launch_batch_fit(const BatchSetDev *d_sets, int nsets, const double *d_img, const double *d_data, double *d_fqs,
                     long nfit, long nbuf, const BatchFitReduce &R, cudaStream_t s);

// Resident blocks per SM of the persistent kernels for a key (0 if unsupported).
int batch_blocks_per_sm_fp64(int key);
int batch_blocks_per_sm_mixed(int key);

}  // namespace cs

#endif
