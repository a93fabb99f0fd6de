// cs_batch.cpp — many parameter sets per launch (include/crystalscatter.h,
// cs_batch_*).
//
// The reference evaluates parameter sets one after another: the simplex fit
// calls doCalculation/doFitCalculation once per vertex
// (Source/sc_simplexfit2d.cpp:54-62) and each call prepares, launches and
// waits. A batch instead prepares all sets on host threads, uploads them into
// one device arena, and runs all their pixels either as one launch per set
// (the plain schedule, what a caller of the single-set interface gets) or as
// one persistent launch per dispatch key fed by a device tile counter. Either
// schedule can be captured once into a CUDA graph and replayed.
//
// Output layout: set k's image, (xmax-xmin)*(ymax-ymin) doubles in the
// reference's order (x fastest), starts at offset[k]; offsets are rounded up
// to 32 doubles so every image starts on a 256-byte boundary.

#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <atomic>
#include <chrono>
#include <cstdio>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <string>
#include <map>
#include <mutex>
#include <thread>
#include <vector>

#include "../../include/crystalscatter.h"
#include "cs_batch.h"
#include "cs_prep.h"

namespace {

double now_ms() {
    using namespace std::chrono;
    return duration_cast<duration<double, std::milli>>(steady_clock::now().time_since_epoch()).count();
}

}  // namespace

struct cs_batch {
    std::string err;
    int device = -1;
    cudaStream_t stream = nullptr;
    int sm_count = 1;

    int nsets = 0;
    int nsets_cap = 0;
    cs_prepared *hprep = nullptr;  // pinned, nsets_cap blocks (caller's order)
    cs_prepared *dprep = nullptr;  // device, same order
    std::vector<int> order;        // device set array position -> caller's index
    std::vector<cs::HostPeaks> hpeaks;
    std::vector<cs::BatchSetDev> hsets;  // in device array order
    cs::BatchSetDev *dsets = nullptr;
    size_t dsets_cap = 0;
    std::vector<cs::BatchGroup> groups;
    std::vector<size_t> offset;  // caller's order
    size_t total_doubles = 0;
    long total_pixels = 0;
    size_t upload_bytes = 0;  // host-to-device bytes of the last cs_batch_prepare
    std::vector<int> expand_sets;  // caller's indices of sets that need zeroing + mirroring
    bool any_twin = false;

    // arenas
    float *d_pk = nullptr;  // aq, awl, iq, imf of all sets
    size_t pk_cap = 0;
    float4 *d_av = nullptr;
    size_t av_cap = 0;
    int *d_ai = nullptr;  // latpar rows of the anisotropic reflections
    size_t ai_cap = 0;
    cs_delta_node *d_delta = nullptr;  // one table per set that needs one
    size_t delta_cap = 0;
    std::vector<cs::QTable> qtabs;  // pixel geometry tables, filled at every persistent run
    double *d_qtab = nullptr;
    size_t qtab_cap = 0;
    const cs_chi_node *d_chi = nullptr;
    cs_chi_node *d_chi_own = nullptr;
    double chi_b = -1;

    unsigned long long *d_counters = nullptr;  // one per group
    size_t counters_cap = 0;
    cs::BatchRedo redo;
    size_t redo_groups_cap = 0;
    long redo_cap_req = 0;  // entries per group requested by the caller (0: automatic)
    cs::MixedScratch plain_scratch;  // redo list of the plain mixed schedule (reused set after set)
    long plain_scratch_cap = 0;

    cudaGraph_t graph = nullptr;
    cudaGraphExec_t graph_exec = nullptr;
    int graph_mode = -1, graph_schedule = -1;
    double *graph_out = nullptr;

    // fit: shared target, masks, FQS arena, reduction, cached graph of one evaluation
    bool fit_set = false;
    int fit_w = 0, fit_h = 0, fit_bstop = 0, fit_border = 0;
    int nofit[4][4];
    double *d_fit = nullptr;
    size_t fit_cap = 0;
    double *d_fqs = nullptr;
    size_t fqs_cap = 0;
    double *d_fimg = nullptr;  // images of the evaluated sets
    size_t fimg_cap = 0;
    cs::BatchFitReduce fred;
    size_t fred_sets_cap = 0;
    double *h_fit_out = nullptr;  // pinned: chi2[n], cnt[n], nan[n]
    size_t h_fit_cap = 0;
    cudaGraphExec_t fit_exec = nullptr;
    std::vector<long long> fit_graph_sig;

    // schedule of the mixed persistent kernel per group: work unit (0 = block
    // tiles, 32..CS_BATCH_TILE = pixels per warp chunk) and resident blocks
    // per SM; chosen by the autotuner at the first mixed persistent run of a
    // key on a device (cached), or forced by cs_batch_set_schedule
    struct Sched {
        int chunk = -1;
        int bps = 0;
        double ns_per_px = 0;
        int tuned = 0;
    };
    std::vector<Sched> sched;
    int force_chunk = -1, force_bps = 0;

    double t_prep = 0;
    bool prepared = false;
};

namespace {

int fail(cs_batch *b, int code, const std::string &msg) {
    if (b) b->err = msg;
    return code;
}

int cuda_fail(cs_batch *b, cudaError_t e, const char *what) {
    return fail(b, CS_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

int ensure_device(cs_batch *b) {
    if (b->stream) return CS_OK;
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess || n == 0) return fail(b, CS_ERR_CUDA, "no CUDA device available (this library has no CPU path)");
    if ((e = cudaGetDevice(&b->device)) != cudaSuccess) return cuda_fail(b, e, "cudaGetDevice");
    if ((e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking)) != cudaSuccess)
        return cuda_fail(b, e, "cudaStreamCreate");
    cudaDeviceGetAttribute(&b->sm_count, cudaDevAttrMultiProcessorCount, b->device);
    if (b->sm_count <= 0) b->sm_count = 1;
    return CS_OK;
}

template <class T>
int grow(cs_batch *b, T *&ptr, size_t &cap, size_t need, const char *what) {
    if (need <= cap) return CS_OK;
    if (ptr) cudaFree(ptr);
    ptr = nullptr;
    cap = 0;
    cudaError_t e = cudaMalloc(&ptr, sizeof(T) * need);
    if (e != cudaSuccess) return cuda_fail(b, e, what);
    cap = need;
    return CS_OK;
}

void drop_graph(cs_batch *b) {
    if (b->graph_exec) cudaGraphExecDestroy(b->graph_exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    b->graph_exec = nullptr;
    b->graph = nullptr;
    b->graph_mode = b->graph_schedule = -1;
    b->graph_out = nullptr;
}

int quadrants_of(const cs_params &p, int &expand) {
    int cq = CS_RADQ4;
    if (p.radq1) cq = CS_RADQ1;
    if (p.radq2) cq = CS_RADQ2;
    if (p.radq4) cq = CS_RADQ4;
    expand = (p.expand && cq != CS_RADQ4) ? 1 : 0;
    return cq;
}

long region_pixels(const cs_prepared &P) {
    const long nx = P.zzmax - P.zzmin, ny = P.iimax - P.iimin;
    return (nx > 0 && ny > 0) ? nx * ny : 0;
}

size_t image_doubles(const cs_prepared &P) { return (size_t)(P.xmax - P.xmin) * (size_t)(P.ymax - P.ymin); }

// Redo entries per group when the caller asked for none: one per pixel of the
// largest group (8 B per pixel, as much as the image), so the list cannot
// overflow.
long auto_redo_cap(const cs_batch *b) {
    long most = 0;
    for (const auto &g : b->groups) most = std::max(most, g.tiles * (long)CS_BATCH_TILE);
    return std::max(most, 1L);
}

int ensure_redo(cs_batch *b) {
    const size_t ng = std::max<size_t>(b->groups.size(), 1);
    const long cap = b->redo_cap_req > 0 ? b->redo_cap_req : auto_redo_cap(b);
    if (ng > b->redo_groups_cap || cap != b->redo.cap) {
        cudaFree(b->redo.d_count);
        cudaFree(b->redo.d_list);
        b->redo = cs::BatchRedo{};
        b->redo_groups_cap = 0;
        cudaError_t e;
        if ((e = cudaMalloc(&b->redo.d_count, sizeof(int) * ng)) != cudaSuccess) return cuda_fail(b, e, "cudaMalloc(redo counts)");
        if ((e = cudaMalloc(&b->redo.d_list, sizeof(int2) * ng * (size_t)cap)) != cudaSuccess)
            return cuda_fail(b, e, "cudaMalloc(redo list)");
        b->redo.cap = cap;
        b->redo_groups_cap = ng;
    }
    return CS_OK;
}

// ---- autotuner of the mixed persistent kernels ----------------------------
// Candidates per dispatch key: block tiles (the barrier-synchronised form) or
// warp chunks of 32, 64, 128 or 256 pixels, at the occupancy limit of
// resident blocks per SM or half of it. Each candidate computes the same
// prefix of the group's pixels (1/32 of them, at least 8 tiles per resident
// block) with the main kernel alone, timed with CUDA events; the fastest per
// pixel wins and is cached per (device, key) for the process.
// Half-width of the square pixel region a set needs from a shared geometry
// table, or -1 when its q vectors cannot come from one: only the z-direction
// cylinder keys (whose mixed kernels take the drop-in's geometry too, so a
// batch still equals single-set calls bit for bit), in beam geometry with
// pixno = 2 zmax, where convert_idx2q's detector position of pixel (ihex, i)
// is exactly (ihex, i) whatever the detector size.
int qtable_half(const cs_prepared &P) {
    if (P.key != CS_KEY_CYL_NONE_ZDIR && P.key != CS_KEY_CYL_GAUSS_BCT_ZDIR) return -1;
    if (P.use1d || !P.usebeamstop) return -1;
    if (P.pixnox != 2.0 * P.zmax || P.pixnoy != 2.0 * P.zmax) return -1;
    const int h = std::max(std::max(std::abs(P.zzmin), std::abs(P.zzmax - 1)),
                           std::max(std::abs(P.iimin), std::abs(P.iimax - 1)));
    return h <= (1 << 14) ? h : -1;
}

// the detector geometry that decides a table's values, bit for bit
std::array<uint64_t, 6> qtable_geometry(const cs_prepared &P) {
    std::array<uint64_t, 6> g;
    const double v[6] = {P.pixx_m, P.pixy_m, P.beamx0, P.beamy0, P.det, P.wave};
    std::memcpy(g.data(), v, sizeof(v));
    return g;
}

int enqueue_qtables(cs_batch *b, cudaStream_t s) {
    for (const cs::QTable &t : b->qtabs) {
        const int rc = cs::launch_qtable(t, s);
        if (rc) return cuda_fail(b, cs::last_launch_error(), "geometry table launch");
    }
    return CS_OK;
}

std::mutex g_tune_mutex;
std::map<std::pair<int, int>, cs_batch::Sched> g_tune_cache;

int tune_group(cs_batch *b, size_t gi, double *d_out, cudaStream_t s, cs_batch::Sched &out) {
    const cs::BatchGroup &g = b->groups[gi];
    const int occ = std::max(cs::batch_blocks_per_sm_mixed(g.key), 1);
    const long gpx = g.tiles * (long)CS_BATCH_TILE;
    long sample = std::max(gpx / 32, (long)b->sm_count * occ * CS_BATCH_TILE * 8);
    sample = std::min(sample, gpx);
    std::vector<std::pair<int, int>> cand;
    for (int chunk : {0, 32, 64, 128, 256}) {
        cand.push_back({chunk, occ});
        if (occ > 1) cand.push_back({chunk, occ / 2});
    }
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaError_t e = cudaEventCreate(&e0);
    if (e == cudaSuccess) e = cudaEventCreate(&e1);
    if (e != cudaSuccess) {
        if (e0) cudaEventDestroy(e0);
        return cuda_fail(b, e, "cudaEventCreate");
    }
    int rc = enqueue_qtables(b, s);
    double best = 1e300;
    for (size_t c = 0; c <= cand.size() && rc == CS_OK; c++) {
        // entry 0 runs twice: the first pass warms up (clocks, caches) untimed
        const auto [chunk, bps] = cand[c == 0 ? 0 : c - 1];
        const long limit = sample / (chunk ? chunk : CS_BATCH_TILE);
        if ((e = cudaMemsetAsync(b->d_counters + gi, 0, sizeof(unsigned long long), s)) != cudaSuccess ||
            (e = cudaMemsetAsync(b->redo.d_count + gi, 0, sizeof(int), s)) != cudaSuccess) {
            rc = cuda_fail(b, e, "cudaMemsetAsync(tuning)");
            break;
        }
        cudaEventRecord(e0, s);
        rc = cs::launch_batch_mixed(b->dsets, g, (int)gi, b->d_counters + gi, b->d_chi, d_out, b->redo,
                                    b->sm_count * bps, s, nullptr, chunk, limit, false);
        if (rc == CS_ERR_CUDA) rc = cuda_fail(b, cs::last_launch_error(), "tuning launch");
        cudaEventRecord(e1, s);
        if (rc == CS_OK && (e = cudaEventSynchronize(e1)) != cudaSuccess) rc = cuda_fail(b, e, "tuning run");
        if (rc != CS_OK || c == 0) continue;
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        const double ns = ms * 1e6 / (double)sample;
        if (ns < best) {
            best = ns;
            out.chunk = chunk;
            out.bps = bps;
            out.ns_per_px = ns;
            out.tuned = 1;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return rc;
}

// Schedules of every group for a mixed persistent run (before any capture).
int ensure_schedule(cs_batch *b, double *d_out, cudaStream_t s) {
    if (b->sched.size() != b->groups.size()) b->sched.assign(b->groups.size(), cs_batch::Sched{});
    for (size_t gi = 0; gi < b->groups.size(); gi++) {
        cs_batch::Sched &sc = b->sched[gi];
        if (sc.chunk >= 0) continue;
        const int key = b->groups[gi].key;
        if (!cs::mixed_key(key)) continue;
        const int occ = std::max(cs::batch_blocks_per_sm_mixed(key), 1);
        if (b->force_chunk >= 0) {
            sc.chunk = b->force_chunk;
            sc.bps = b->force_bps > 0 ? std::min(b->force_bps, occ) : occ;
            sc.tuned = 0;
            continue;
        }
        const std::pair<int, int> ck{b->device, key};
        {
            std::lock_guard<std::mutex> lock(g_tune_mutex);
            auto it = g_tune_cache.find(ck);
            if (it != g_tune_cache.end()) {
                sc = it->second;
                continue;
            }
        }
        int rc = ensure_redo(b);
        if (rc) return rc;
        if ((rc = tune_group(b, gi, d_out, s, sc))) return rc;
        std::lock_guard<std::mutex> lock(g_tune_mutex);
        g_tune_cache[ck] = sc;
    }
    return CS_OK;
}

// Enqueue one evaluation of all sets on stream s. marks (persistent schedule
// only): three events per group, recorded before the group's main kernel,
// between it and its redo kernel, and after the redo.
int enqueue(cs_batch *b, double *d_out, cudaStream_t s, int mode, int schedule, cudaEvent_t *marks = nullptr) {
    cudaError_t e;
    for (int k : b->expand_sets) {
        // pixels the mirroring never writes read as 0
        if ((e = cudaMemsetAsync(d_out + b->offset[k], 0, sizeof(double) * image_doubles(b->hprep[k]), s)) != cudaSuccess)
            return cuda_fail(b, e, "cudaMemsetAsync(image)");
    }
    if (schedule == CS_SCHED_PERSISTENT) {
        if (b->groups.empty()) return CS_OK;
        if (mode == CS_MODE_MIXED && b->any_twin) return fail(b, CS_ERR_UNSUPPORTED, "no mixed-precision kernel for twinned lattices");
        if ((e = cudaMemsetAsync(b->d_counters, 0, sizeof(unsigned long long) * b->groups.size(), s)) != cudaSuccess)
            return cuda_fail(b, e, "cudaMemsetAsync(tile counters)");
        if (int rc = enqueue_qtables(b, s)) return rc;
        if (mode == CS_MODE_MIXED) {
            int rc = ensure_redo(b);
            if (rc) return rc;
            if ((e = cudaMemsetAsync(b->redo.d_count, 0, sizeof(int) * b->groups.size(), s)) != cudaSuccess)
                return cuda_fail(b, e, "cudaMemsetAsync(redo counts)");
        }
        for (size_t gi = 0; gi < b->groups.size(); gi++) {
            const cs::BatchGroup &g = b->groups[gi];
            const bool mixed = mode == CS_MODE_MIXED && cs::mixed_key(g.key);
            int per_sm = mixed ? cs::batch_blocks_per_sm_mixed(g.key) : cs::batch_blocks_per_sm_fp64(g.key);
            // the mixed kernel's schedule (autotuned, or warp chunks of 32 at
            // the occupancy limit when no run has tuned it yet)
            int chunk = 32;
            if (mixed && gi < b->sched.size() && b->sched[gi].chunk >= 0) {
                chunk = b->sched[gi].chunk;
                per_sm = b->sched[gi].bps;
            }
            long grid = (long)b->sm_count * std::max(per_sm, 1);
            grid = std::min(grid, std::max(g.tiles, 1L));
            if (marks) cudaEventRecord(marks[3 * gi], s);
            int rc = mixed
                         ? cs::launch_batch_mixed(b->dsets, g, (int)gi, b->d_counters + gi, b->d_chi, d_out, b->redo,
                                                  (int)grid, s, marks ? marks[3 * gi + 1] : nullptr, chunk)
                         : cs::launch_batch_fp64(b->dsets, g, b->d_counters + gi, b->d_chi, d_out, (int)grid, s);
            if (marks) {
                if (!mixed) cudaEventRecord(marks[3 * gi + 1], s);
                cudaEventRecord(marks[3 * gi + 2], s);
            }
            if (rc == CS_ERR_CUDA) return cuda_fail(b, cs::last_launch_error(), "batch kernel launch");
            if (rc) return fail(b, rc, "no batch kernel for this combination");
        }
    } else if (schedule == CS_SCHED_PLAIN) {
        // one launch (mixed: launch + redo) per set, as the single-set interface issues them
        for (size_t j = 0; j < b->hsets.size(); j++) {
            const cs::BatchSetDev &S = b->hsets[j];
            const cs_prepared &P = b->hprep[b->order[j]];
            cs::DevSet D;
            D.d_prep = S.prep;
            D.d_chi = b->d_chi;
            D.d_delta = S.delta;
            double *out = d_out + S.out_offset;
            int rc;
            if (mode == CS_MODE_MIXED && cs::mixed_key(P.key) && !P.twin) {
                if (S.npix > b->plain_scratch_cap) {
                    cudaFree(b->plain_scratch.d_list);
                    b->plain_scratch.d_list = nullptr;
                    if (!b->plain_scratch.d_count && (e = cudaMalloc(&b->plain_scratch.d_count, 2 * sizeof(int))) != cudaSuccess)
                        return cuda_fail(b, e, "cudaMalloc(redo count)");
                    if ((e = cudaMalloc(&b->plain_scratch.d_list, sizeof(int) * (size_t)S.npix)) != cudaSuccess)
                        return cuda_fail(b, e, "cudaMalloc(redo list)");
                    b->plain_scratch_cap = S.npix;
                    b->plain_scratch.cap = (int)S.npix;
                }
                rc = cs::launch_image_mixed(D, S.peaks, P, out, b->plain_scratch, s);
            } else {
                rc = cs::launch_image(D, P, out, s);  // mirrors expanded quadrants itself
            }
            if (rc == CS_ERR_CUDA) return cuda_fail(b, cs::last_launch_error(), "kernel launch");
            if (rc) return fail(b, rc, "no kernel for this combination");
        }
        return CS_OK;
    } else {
        return fail(b, CS_ERR_PARAM, "unknown batch schedule");
    }
    // persistent schedule: mirror the sets that expand their quadrant
    for (int k : b->expand_sets) cs::launch_mirror(b->hprep[k], d_out + b->offset[k], s);
    if ((e = cudaGetLastError()) != cudaSuccess) return cuda_fail(b, e, "mirror launch");
    return CS_OK;
}

int check_run_args(cs_batch *b, double *d_out, size_t n_doubles, int mode) {
    if (!b->prepared) return fail(b, CS_ERR_STATE, "no prepared batch");
    if (!d_out) return fail(b, CS_ERR_PARAM, "null output buffer");
    if (n_doubles < b->total_doubles) return fail(b, CS_ERR_SIZE, "output buffer too small for the batch");
    if (mode != CS_MODE_FP64 && mode != CS_MODE_MIXED) return fail(b, CS_ERR_PARAM, "unknown precision mode");
    return CS_OK;
}

}  // namespace

extern "C" {

cs_batch *cs_batch_create(void) { return new (std::nothrow) cs_batch; }

void cs_batch_destroy(cs_batch *b) {
    if (!b) return;
    if (b->stream) cudaStreamSynchronize(b->stream);
    drop_graph(b);
    cudaFree(b->dprep);
    cudaFree(b->dsets);
    cudaFree(b->d_pk);
    cudaFree(b->d_av);
    cudaFree(b->d_ai);
    cudaFree(b->d_delta);
    cudaFree(b->d_qtab);
    cudaFree(b->d_chi_own);
    cudaFree(b->d_counters);
    cudaFree(b->redo.d_count);
    cudaFree(b->redo.d_list);
    cudaFree(b->plain_scratch.d_count);
    cudaFree(b->plain_scratch.d_list);
    if (b->fit_exec) cudaGraphExecDestroy(b->fit_exec);
    cudaFree(b->d_fit);
    cudaFree(b->d_fqs);
    cudaFree(b->d_fimg);
    cudaFree(b->fred.d_psum);
    cudaFree(b->fred.d_pcnt);
    cudaFree(b->fred.d_pnan);
    cudaFree(b->fred.d_sum);
    cudaFree(b->fred.d_cnt);
    cudaFree(b->fred.d_nan);
    if (b->h_fit_out) cudaFreeHost(b->h_fit_out);
    if (b->hprep) cudaFreeHost(b->hprep);
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
}

const char *cs_batch_last_error(cs_batch *b) { return b ? b->err.c_str() : "null batch"; }

int cs_batch_prepare(cs_batch *b, const cs_params *sets, int nsets, int ign_new_switch, int ign_cbs, int host_threads) {
    if (!b) return CS_ERR_PARAM;
    if (!sets || nsets <= 0) return fail(b, CS_ERR_PARAM, "empty batch");
    b->prepared = false;
    int rc = ensure_device(b);
    if (rc) return rc;
    cudaStreamSynchronize(b->stream);  // earlier uploads/launches have left the pinned blocks
    drop_graph(b);
    const double t0 = now_ms();
    cudaError_t e;
    if (nsets > b->nsets_cap) {
        if (b->hprep) cudaFreeHost(b->hprep);
        b->hprep = nullptr;
        if (b->dprep) cudaFree(b->dprep);
        b->dprep = nullptr;
        b->nsets_cap = 0;
        if ((e = cudaMallocHost(&b->hprep, sizeof(cs_prepared) * (size_t)nsets)) != cudaSuccess)
            return cuda_fail(b, e, "cudaMallocHost(prepared blocks)");
        if ((e = cudaMalloc(&b->dprep, sizeof(cs_prepared) * (size_t)nsets)) != cudaSuccess)
            return cuda_fail(b, e, "cudaMalloc(prepared blocks)");
        b->nsets_cap = nsets;
    }
    b->nsets = nsets;
    b->hpeaks.assign(nsets, cs::HostPeaks{});

    // host preparation of all sets on host_threads threads (0: all hardware threads)
    unsigned nt = host_threads > 0 ? (unsigned)host_threads : std::max(1u, std::thread::hardware_concurrency());
    nt = std::min<unsigned>(nt, (unsigned)nsets);
    std::vector<int> status(nsets, CS_OK);
    std::vector<std::string> errs(nsets);
    std::atomic<int> next(0);
    auto worker = [&]() {
        cs::set_prep_threads(nt > 1 ? 1 : 0);  // sets in parallel, each set serial
        for (;;) {
            const int k = next.fetch_add(1);
            if (k >= nsets) break;
            int expand;
            const int cq = quadrants_of(sets[k], expand);
            cs_prepared &P = b->hprep[k];
            // a batch prepared for fitting skips checkAllParameters, as
            // doFitCalculation does (Source/sc_calc_generic_cpu.cpp:1334-1341)
            status[k] = cs::prepare(sets[k], cq, expand, ign_new_switch, ign_cbs, b->fit_set ? 0 : 1, &P, errs[k]);
            if (status[k] == CS_OK && b->fit_set) {
                P.fit_width = b->fit_w;
                P.fit_height = b->fit_h;
                P.fit_bstop = b->fit_bstop;
                P.fit_border = b->fit_border;
                for (int r = 0; r < 4; r++) {
                    P.nofit_x0[r] = b->nofit[r][0];
                    P.nofit_y0[r] = b->nofit[r][1];
                    P.nofit_x1[r] = b->nofit[r][2];
                    P.nofit_y1[r] = b->nofit[r][3];
                }
            }
            if (status[k] == CS_OK && !cs::key_supported(P)) {
                status[k] = CS_ERR_UNSUPPORTED;
                char buf[160];
                std::snprintf(buf, sizeof buf, "combination particle=%d peak=%d ltype=%d ordis=%d (key 0x%08X) has no GPU pixel function here",
                              P.particle, P.shp, P.ltype, P.ordis, (unsigned)P.key);
                errs[k] = buf;
            }
            if (status[k] == CS_OK && P.lattice) cs::build_peak_tables(P, b->hpeaks[k]);
        }
    };
    if (nt <= 1) {
        worker();
    } else {
        std::vector<std::thread> pool;
        for (unsigned i = 0; i < nt; i++) pool.emplace_back(worker);
        for (auto &t : pool) t.join();
    }
    for (int k = 0; k < nsets; k++)
        if (status[k] != CS_OK) return fail(b, status[k], "set " + std::to_string(k) + ": " + errs[k]);

    // chi node table: the same limits for every set (2*pi as float)
    if (b->chi_b != b->hprep[0].romb_chi_b) {
        for (int k = 1; k < nsets; k++)
            if (b->hprep[k].romb_chi_b != b->hprep[0].romb_chi_b) return fail(b, CS_ERR_PARAM, "chi limits differ between sets");
        std::vector<cs_chi_node> host(CS_CHI_TABLE_LEN);
        cs::build_chi_table(b->hprep[0].romb_chi_b, host.data());
        if (!b->d_chi_own && (e = cudaMalloc(&b->d_chi_own, sizeof(cs_chi_node) * CS_CHI_TABLE_LEN)) != cudaSuccess)
            return cuda_fail(b, e, "cudaMalloc(chi table)");
        if ((e = cudaMemcpy(b->d_chi_own, host.data(), sizeof(cs_chi_node) * CS_CHI_TABLE_LEN, cudaMemcpyHostToDevice)) != cudaSuccess)
            return cuda_fail(b, e, "upload chi table");
        b->chi_b = b->hprep[0].romb_chi_b;
    }
    b->d_chi = b->d_chi_own;

    // output offsets in the caller's order
    b->offset.assign(nsets, 0);
    b->expand_sets.clear();
    b->any_twin = false;
    size_t off = 0;
    long pix = 0;
    for (int k = 0; k < nsets; k++) {
        b->offset[k] = off;
        off += (image_doubles(b->hprep[k]) + 31) & ~(size_t)31;
        pix += region_pixels(b->hprep[k]);
        // twinned lattices of a key with a mixed kernel (the generic key runs FP64)
        if (b->hprep[k].twin && cs::mixed_key(b->hprep[k].key)) b->any_twin = true;
        if (b->hprep[k].expand && b->hprep[k].calc_quadrants != CS_RADQ4 && b->hprep[k].calc_quadrants != CS_RAD1D)
            b->expand_sets.push_back(k);
    }
    b->total_doubles = off;
    b->total_pixels = pix;

    // device order: grouped by key (stable), largest images first inside a group
    b->order.resize(nsets);
    for (int k = 0; k < nsets; k++) b->order[k] = k;
    std::stable_sort(b->order.begin(), b->order.end(), [&](int x, int y) {
        if (b->hprep[x].key != b->hprep[y].key) return b->hprep[x].key < b->hprep[y].key;
        return region_pixels(b->hprep[x]) > region_pixels(b->hprep[y]);
    });

    // peak arena and delta tables
    size_t nf = 0, nv = 0, nd = 0;
    for (int k = 0; k < nsets; k++) {
        const auto &H = b->hpeaks[k];
        nf += H.aq.size() + H.awl.size() + H.iq.size() + H.imf.size();
        nv += H.av.size();
        if (cs::needs_delta_table(b->hprep[k])) nd++;
    }
    if ((rc = grow(b, b->d_pk, b->pk_cap, std::max<size_t>(nf, 1), "cudaMalloc(peak arena)"))) return rc;
    if ((rc = grow(b, b->d_av, b->av_cap, std::max<size_t>(nv, 1), "cudaMalloc(peak vectors)"))) return rc;
    if ((rc = grow(b, b->d_ai, b->ai_cap, std::max<size_t>(nv, 1), "cudaMalloc(peak rows)"))) return rc;
    if ((rc = grow(b, b->d_delta, b->delta_cap, std::max<size_t>(nd, 1) * CS_NODE_COUNT, "cudaMalloc(delta tables)")))
        return rc;
    std::vector<float> pk;
    pk.reserve(nf);
    std::vector<float4> av;
    av.reserve(nv);
    std::vector<int> ai;
    ai.reserve(nv);
    std::vector<cs_delta_node> dt;
    if (nd) dt.resize(nd * CS_NODE_COUNT);
    b->hsets.assign(nsets, cs::BatchSetDev{});
    b->groups.clear();
    b->sched.clear();
    size_t di = 0;
    for (int j = 0; j < nsets; j++) {
        const int k = b->order[j];
        const cs_prepared &P = b->hprep[k];
        cs::BatchSetDev &S = b->hsets[j];
        S.prep = b->dprep + k;
        S.delta = nullptr;
        if (cs::needs_delta_table(P)) {
            cs::build_delta_table(P.romb_delta_b, P.romb_dbeta, dt.data() + di * CS_NODE_COUNT);
            S.delta = b->d_delta + di * CS_NODE_COUNT;
            di++;
        }
        const auto &H = b->hpeaks[k];
        S.peaks = csm::PeakTab{};
        if (P.lattice) {
            auto put = [&](const std::vector<float> &v) -> const float * {
                const float *p = b->d_pk + pk.size();
                pk.insert(pk.end(), v.begin(), v.end());
                return p;
            };
            S.peaks.n_aniso = (int)H.aq.size();
            S.peaks.aq = put(H.aq);
            S.peaks.awl = put(H.awl);
            S.peaks.av = b->d_av + av.size();
            S.peaks.aidx = b->d_ai + ai.size();
            av.insert(av.end(), H.av.begin(), H.av.end());
            ai.insert(ai.end(), H.aidx.begin(), H.aidx.end());
            S.peaks.n_iso = (int)H.iq.size();
            S.peaks.iq = put(H.iq);
            S.peaks.imf = put(H.imf);
            cs::peak_constants(P, S.peaks);
        }
        S.out_offset = (long)b->offset[k];
        S.npix = region_pixels(P);
        S.nx = P.zzmax - P.zzmin;
        S.key = P.key;
        if (b->groups.empty() || b->groups.back().key != P.key) {
            cs::BatchGroup g;
            g.key = P.key;
            g.set_begin = g.set_end = j;
            b->groups.push_back(g);
        }
        cs::BatchGroup &g = b->groups.back();
        S.tile_begin = g.tiles;
        g.tiles += (S.npix + CS_BATCH_TILE - 1) / CS_BATCH_TILE;
        g.set_end = j + 1;
    }
    // shared pixel geometry tables: one per detector geometry among the sets
    // that can use one, as wide as its widest set
    {
        std::map<std::array<uint64_t, 6>, size_t> by_geom;
        b->qtabs.clear();
        for (int j = 0; j < nsets; j++) {
            const cs_prepared &P = b->hprep[b->order[j]];
            const int h = qtable_half(P);
            if (h < 0) continue;
            auto it = by_geom.find(qtable_geometry(P));
            if (it == by_geom.end()) {
                it = by_geom.emplace(qtable_geometry(P), b->qtabs.size()).first;
                b->qtabs.push_back(cs::QTable{});
            }
            cs::QTable &t = b->qtabs[it->second];
            if (h > t.half || t.prep == nullptr) {
                t.half = std::max(h, t.half);
                t.prep = b->dprep + b->order[j];
            }
        }
        size_t need = 0;
        for (const cs::QTable &t : b->qtabs) need += 3 * (size_t)(2 * t.half + 1) * (size_t)(2 * t.half + 1);
        if (need && (rc = grow(b, b->d_qtab, b->qtab_cap, need, "cudaMalloc(geometry tables)"))) return rc;
        size_t off = 0;
        for (cs::QTable &t : b->qtabs) {
            t.d = b->d_qtab + off;
            off += 3 * (size_t)(2 * t.half + 1) * (size_t)(2 * t.half + 1);
        }
        for (int j = 0; j < nsets; j++) {
            cs::BatchSetDev &S = b->hsets[j];
            S.qtab = nullptr;
            S.qhalf = S.qw = 0;
            const cs_prepared &P = b->hprep[b->order[j]];
            if (qtable_half(P) < 0) continue;
            const cs::QTable &t = b->qtabs[by_geom.at(qtable_geometry(P))];
            S.qtab = t.d;
            S.qhalf = t.half;
            S.qw = 2 * t.half + 1;
        }
    }
    if ((rc = grow(b, b->dsets, b->dsets_cap, (size_t)nsets, "cudaMalloc(set table)"))) return rc;
    if ((rc = grow(b, b->d_counters, b->counters_cap, std::max<size_t>(b->groups.size(), 1), "cudaMalloc(tile counters)")))
        return rc;
    // uploads (synchronous: the host vectors go out of scope)
    if ((e = cudaMemcpyAsync(b->dprep, b->hprep, sizeof(cs_prepared) * (size_t)nsets, cudaMemcpyHostToDevice, b->stream)) != cudaSuccess)
        return cuda_fail(b, e, "upload prepared blocks");
    if (!pk.empty() && (e = cudaMemcpy(b->d_pk, pk.data(), sizeof(float) * pk.size(), cudaMemcpyHostToDevice)) != cudaSuccess)
        return cuda_fail(b, e, "upload peak arena");
    if (!av.empty() && (e = cudaMemcpy(b->d_av, av.data(), sizeof(float4) * av.size(), cudaMemcpyHostToDevice)) != cudaSuccess)
        return cuda_fail(b, e, "upload peak vectors");
    if (!ai.empty() && (e = cudaMemcpy(b->d_ai, ai.data(), sizeof(int) * ai.size(), cudaMemcpyHostToDevice)) != cudaSuccess)
        return cuda_fail(b, e, "upload peak rows");
    if (nd && (e = cudaMemcpy(b->d_delta, dt.data(), sizeof(cs_delta_node) * dt.size(), cudaMemcpyHostToDevice)) != cudaSuccess)
        return cuda_fail(b, e, "upload delta tables");
    if ((e = cudaMemcpy(b->dsets, b->hsets.data(), sizeof(cs::BatchSetDev) * (size_t)nsets, cudaMemcpyHostToDevice)) != cudaSuccess)
        return cuda_fail(b, e, "upload set table");
    if ((e = cudaStreamSynchronize(b->stream)) != cudaSuccess) return cuda_fail(b, e, "batch upload");
    b->upload_bytes = sizeof(cs_prepared) * (size_t)nsets + sizeof(float) * pk.size() + sizeof(float4) * av.size() +
                      sizeof(int) * ai.size() + sizeof(cs_delta_node) * dt.size() +
                      sizeof(cs::BatchSetDev) * (size_t)nsets;
    b->t_prep = now_ms() - t0;
    b->prepared = true;
    return CS_OK;
}

int cs_batch_info(cs_batch *b, size_t *total_doubles, long *total_pixels, int *ngroups) {
    if (!b) return CS_ERR_PARAM;
    if (!b->prepared) return fail(b, CS_ERR_STATE, "no prepared batch");
    if (total_doubles) *total_doubles = b->total_doubles;
    if (total_pixels) *total_pixels = b->total_pixels;
    if (ngroups) *ngroups = (int)b->groups.size();
    return CS_OK;
}

int cs_batch_set_schedule(cs_batch *b, int chunk, int blocks_per_sm) {
    if (!b) return CS_ERR_PARAM;
    if (chunk != -1 && chunk != 0 && (chunk < 32 || chunk > CS_BATCH_TILE || chunk % 32 || CS_BATCH_TILE % chunk))
        return fail(b, CS_ERR_PARAM, "chunk must be -1 (autotune), 0 (block tiles) or 32..256 pixels dividing 256");
    if (blocks_per_sm < 0) return fail(b, CS_ERR_PARAM, "blocks_per_sm must be >= 0");
    b->force_chunk = chunk;
    b->force_bps = blocks_per_sm;
    b->sched.clear();
    drop_graph(b);
    return CS_OK;
}

int cs_batch_schedule(cs_batch *b, int group, int *key, int *chunk, int *blocks_per_sm, double *ns_per_pixel,
                      int *tuned) {
    if (!b) return CS_ERR_PARAM;
    if (group < 0 || (size_t)group >= b->groups.size()) return fail(b, CS_ERR_PARAM, "group index out of range");
    const cs_batch::Sched sc = (size_t)group < b->sched.size() ? b->sched[group] : cs_batch::Sched{};
    if (key) *key = b->groups[group].key;
    if (chunk) *chunk = sc.chunk;
    if (blocks_per_sm) *blocks_per_sm = sc.bps;
    if (ns_per_pixel) *ns_per_pixel = sc.ns_per_px;
    if (tuned) *tuned = sc.tuned;
    return CS_OK;
}

int cs_batch_upload_bytes(cs_batch *b, size_t *bytes) {
    if (!b || !bytes) return CS_ERR_PARAM;
    if (!b->prepared) return fail(b, CS_ERR_STATE, "no prepared batch");
    *bytes = b->upload_bytes;
    return CS_OK;
}

int cs_batch_layout(cs_batch *b, int k, size_t *offset, int *xmin, int *xmax, int *ymin, int *ymax) {
    if (!b) return CS_ERR_PARAM;
    if (!b->prepared) return fail(b, CS_ERR_STATE, "no prepared batch");
    if (k < 0 || k >= b->nsets) return fail(b, CS_ERR_PARAM, "set index out of range");
    const cs_prepared &P = b->hprep[k];
    if (offset) *offset = b->offset[k];
    if (xmin) *xmin = P.xmin;
    if (xmax) *xmax = P.xmax;
    if (ymin) *ymin = P.ymin;
    if (ymax) *ymax = P.ymax;
    return CS_OK;
}

int cs_batch_set_redo_capacity(cs_batch *b, long entries_per_group) {
    if (!b || entries_per_group < 0) return CS_ERR_PARAM;
    b->redo_cap_req = entries_per_group;
    drop_graph(b);
    return CS_OK;
}

int cs_batch_launch(cs_batch *b, double *d_out, size_t n_doubles, void *stream, int mode, int schedule) {
    if (!b) return CS_ERR_PARAM;
    int rc = check_run_args(b, d_out, n_doubles, mode);
    if (rc) return rc;
    // the uploads of cs_batch_prepare have completed, so any stream may run the batch
    cudaStream_t s = stream ? (cudaStream_t)stream : b->stream;
    if (mode == CS_MODE_MIXED && schedule == CS_SCHED_PERSISTENT && (rc = ensure_schedule(b, d_out, s))) return rc;
    return enqueue(b, d_out, s, mode, schedule);
}

int cs_batch_profile(cs_batch *b, double *d_out, size_t n_doubles, void *stream, int mode, double *main_ms,
                     double *redo_ms) {
    if (!b || !main_ms || !redo_ms) return CS_ERR_PARAM;
    int rc = check_run_args(b, d_out, n_doubles, mode);
    if (rc) return rc;
    cudaStream_t s = stream ? (cudaStream_t)stream : b->stream;
    if (mode == CS_MODE_MIXED && (rc = ensure_schedule(b, d_out, s))) return rc;
    const size_t ng = b->groups.size();
    std::vector<cudaEvent_t> ev(3 * ng, nullptr);
    cudaError_t e = cudaSuccess;
    for (auto &x : ev)
        if (e == cudaSuccess) e = cudaEventCreate(&x);
    if (e == cudaSuccess) {
        rc = enqueue(b, d_out, s, mode, CS_SCHED_PERSISTENT, ev.data());
        if (rc == CS_OK && (e = cudaStreamSynchronize(s)) != cudaSuccess) rc = cuda_fail(b, e, "profiled batch run");
    } else {
        rc = cuda_fail(b, e, "cudaEventCreate");
    }
    *main_ms = *redo_ms = 0;
    for (size_t g = 0; rc == CS_OK && g < ng; g++) {
        float a = 0, c = 0;
        cudaEventElapsedTime(&a, ev[3 * g], ev[3 * g + 1]);
        cudaEventElapsedTime(&c, ev[3 * g + 1], ev[3 * g + 2]);
        *main_ms += a;
        *redo_ms += c;
    }
    for (auto &x : ev)
        if (x) cudaEventDestroy(x);
    return rc;
}

int cs_batch_capture(cs_batch *b, double *d_out, size_t n_doubles, int mode, int schedule) {
    if (!b) return CS_ERR_PARAM;
    int rc = check_run_args(b, d_out, n_doubles, mode);
    if (rc) return rc;
    drop_graph(b);
    // allocations happen before the capture (they are not capturable)
    if (schedule == CS_SCHED_PERSISTENT && mode == CS_MODE_MIXED &&
        ((rc = ensure_redo(b)) || (rc = ensure_schedule(b, d_out, b->stream))))
        return rc;
    if (schedule == CS_SCHED_PLAIN && mode == CS_MODE_MIXED) {
        // size the plain redo scratch by a dry pass over the sets
        long most = 0;
        for (const auto &S : b->hsets) most = std::max(most, S.npix);
        if (most > b->plain_scratch_cap) {
            cudaError_t e;
            cudaFree(b->plain_scratch.d_list);
            b->plain_scratch.d_list = nullptr;
            if (!b->plain_scratch.d_count && (e = cudaMalloc(&b->plain_scratch.d_count, 2 * sizeof(int))) != cudaSuccess)
                return cuda_fail(b, e, "cudaMalloc(redo count)");
            if ((e = cudaMalloc(&b->plain_scratch.d_list, sizeof(int) * (size_t)most)) != cudaSuccess)
                return cuda_fail(b, e, "cudaMalloc(redo list)");
            b->plain_scratch_cap = most;
            b->plain_scratch.cap = (int)most;
        }
    }
    cudaStreamSynchronize(b->stream);
    cudaError_t e = cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return cuda_fail(b, e, "cudaStreamBeginCapture");
    rc = enqueue(b, d_out, b->stream, mode, schedule);
    cudaGraph_t g = nullptr;
    e = cudaStreamEndCapture(b->stream, &g);
    if (rc) {
        if (g) cudaGraphDestroy(g);
        return rc;
    }
    if (e != cudaSuccess) return cuda_fail(b, e, "cudaStreamEndCapture");
    b->graph = g;
    if ((e = cudaGraphInstantiate(&b->graph_exec, g, 0)) != cudaSuccess) {
        drop_graph(b);
        return cuda_fail(b, e, "cudaGraphInstantiate");
    }
    b->graph_mode = mode;
    b->graph_schedule = schedule;
    b->graph_out = d_out;
    return CS_OK;
}

int cs_batch_replay(cs_batch *b, void *stream) {
    if (!b) return CS_ERR_PARAM;
    if (!b->graph_exec) return fail(b, CS_ERR_STATE, "no captured batch graph");
    cudaStream_t s = stream ? (cudaStream_t)stream : b->stream;
    cudaError_t e = cudaGraphLaunch(b->graph_exec, s);
    if (e != cudaSuccess) return cuda_fail(b, e, "cudaGraphLaunch");
    return CS_OK;
}

int cs_batch_graph_nodes(cs_batch *b, size_t *n) {
    if (!b || !n) return CS_ERR_PARAM;
    *n = 0;
    if (!b->graph) return fail(b, CS_ERR_STATE, "no captured batch graph");
    cudaError_t e = cudaGraphGetNodes(b->graph, nullptr, n);
    return e == cudaSuccess ? CS_OK : cuda_fail(b, e, "cudaGraphGetNodes");
}

int cs_batch_redo_pixels(cs_batch *b, void *stream, long *n, long *capacity) {
    if (!b || !n) return CS_ERR_PARAM;
    *n = 0;
    if (capacity) *capacity = b->redo.cap;
    if (!b->redo.d_count || b->groups.empty()) return CS_OK;
    cudaStream_t s = stream ? (cudaStream_t)stream : b->stream;
    cudaError_t e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cuda_fail(b, e, "batch calculation");
    std::vector<int> c(b->groups.size());
    if ((e = cudaMemcpy(c.data(), b->redo.d_count, sizeof(int) * c.size(), cudaMemcpyDeviceToHost)) != cudaSuccess)
        return cuda_fail(b, e, "read redo counts");
    long total = 0;
    bool over = false;
    for (int v : c) {
        total += v;
        if (v > b->redo.cap) over = true;
    }
    *n = total;
    if (over) return fail(b, CS_ERR_SIZE, "redo list overflow: raise the redo capacity and run again");
    return CS_OK;
}

double cs_batch_timer_ms(cs_batch *b) { return b ? b->t_prep : 0; }

int cs_batch_set_fit(cs_batch *b, int width, int height, const double *data, int bstop, int border,
                     const int *nofit) {
    if (!b) return CS_ERR_PARAM;
    if (!data || width <= 0 || height <= 0) return fail(b, CS_ERR_PARAM, "no fit data");
    int rc = ensure_device(b);
    if (rc) return rc;
    const size_t n = (size_t)width * (size_t)height;
    if ((rc = grow(b, b->d_fit, b->fit_cap, n, "cudaMalloc(fit data)"))) return rc;
    cudaError_t e = cudaMemcpy(b->d_fit, data, sizeof(double) * n, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return cuda_fail(b, e, "upload fit data");
    b->fit_w = width;
    b->fit_h = height;
    b->fit_bstop = bstop;
    b->fit_border = border;
    for (int r = 0; r < 4; r++)
        for (int c = 0; c < 4; c++) b->nofit[r][c] = nofit ? nofit[4 * r + c] : -1;
    b->fit_set = true;
    b->prepared = false;  // the fit fields go into the prepared blocks
    if (b->fit_exec) cudaGraphExecDestroy(b->fit_exec);
    b->fit_exec = nullptr;
    b->fit_graph_sig.clear();
    return CS_OK;
}

int cs_batch_fit_chi2(cs_batch *b, int mode, double *chi2, long *cnt, long *nancnt) {
    if (!b || !chi2) return CS_ERR_PARAM;
    for (int k = 0; k < b->nsets; k++) chi2[k] = 1e20;  // the reference's value of a failed evaluation
    if (!b->fit_set) return fail(b, CS_ERR_STATE, "cs_batch_set_fit has not been called");
    if (!b->prepared) return fail(b, CS_ERR_STATE, "no batch prepared after cs_batch_set_fit");
    if (mode != CS_MODE_FP64 && mode != CS_MODE_MIXED) return fail(b, CS_ERR_PARAM, "unknown precision mode");
    const long nbuf = (long)b->fit_w * b->fit_h;
    for (int k = 0; k < b->nsets; k++) {
        const cs_prepared &P = b->hprep[k];
        if (P.calc_quadrants != CS_RADQ4 || P.xmax - P.xmin != b->fit_w || P.ymax - P.ymin != b->fit_h ||
            P.zzmin != P.xmin || P.zzmax != P.xmax || P.iimin != P.ymin || P.iimax != P.ymax || P.iimin != P.xmin)
            return fail(b, CS_ERR_UNSUPPORTED,
                        "set " + std::to_string(k) +
                            ": a batch fit needs all four quadrants calculated and fit data of the image's size");
    }
    int rc;
    const size_t ns = (size_t)b->nsets;
    if ((rc = grow(b, b->d_fimg, b->fimg_cap, b->total_doubles, "cudaMalloc(fit images)"))) return rc;
    if ((rc = grow(b, b->d_fqs, b->fqs_cap, (size_t)nbuf * ns, "cudaMalloc(fqs)"))) return rc;
    if (ns > b->fred_sets_cap) {
        cudaFree(b->fred.d_psum);
        cudaFree(b->fred.d_pcnt);
        cudaFree(b->fred.d_pnan);
        cudaFree(b->fred.d_sum);
        cudaFree(b->fred.d_cnt);
        cudaFree(b->fred.d_nan);
        b->fred = cs::BatchFitReduce{};
        b->fred_sets_cap = 0;
        const size_t np = ns * (size_t)b->fred.nblocks;
        cudaError_t e;
        if ((e = cudaMalloc(&b->fred.d_psum, sizeof(double) * np)) != cudaSuccess ||
            (e = cudaMalloc(&b->fred.d_pcnt, sizeof(unsigned long long) * np)) != cudaSuccess ||
            (e = cudaMalloc(&b->fred.d_pnan, sizeof(unsigned long long) * np)) != cudaSuccess ||
            (e = cudaMalloc(&b->fred.d_sum, sizeof(double) * ns)) != cudaSuccess ||
            (e = cudaMalloc(&b->fred.d_cnt, sizeof(unsigned long long) * ns)) != cudaSuccess ||
            (e = cudaMalloc(&b->fred.d_nan, sizeof(unsigned long long) * ns)) != cudaSuccess)
            return cuda_fail(b, e, "cudaMalloc(fit reduction)");
        b->fred_sets_cap = ns;
    }
    if (3 * ns > b->h_fit_cap) {
        if (b->h_fit_out) cudaFreeHost(b->h_fit_out);
        b->h_fit_out = nullptr;
        b->h_fit_cap = 0;
        cudaError_t e = cudaMallocHost(&b->h_fit_out, sizeof(double) * 3 * ns);
        if (e != cudaSuccess) return cuda_fail(b, e, "cudaMallocHost(fit results)");
        b->h_fit_cap = 3 * ns;
    }
    if (mode == CS_MODE_MIXED && (rc = ensure_redo(b))) return rc;
    // one evaluation as a CUDA graph: images (persistent schedule), FQS, chi^2,
    // copies of the results; captured once per batch layout, replayed after
    // every re-preparation of the same layout (a fit iteration)
    std::vector<long long> sig = {(long long)mode, (long long)ns, (long long)b->total_doubles,
                                  (long long)(intptr_t)b->dsets, (long long)(intptr_t)b->d_fimg,
                                  (long long)(intptr_t)b->d_fqs, (long long)(intptr_t)b->fred.d_psum,
                                  (long long)(intptr_t)b->h_fit_out, (long long)(intptr_t)b->redo.d_list,
                                  (long long)b->redo.cap};
    for (const auto &g : b->groups) {
        sig.push_back(g.key);
        sig.push_back(g.set_begin);
        sig.push_back(g.set_end);
        sig.push_back(g.tiles);
    }
    for (int k : b->expand_sets) sig.push_back(k);
    cudaError_t e;
    if (!b->fit_exec || sig != b->fit_graph_sig) {
        if (b->fit_exec) cudaGraphExecDestroy(b->fit_exec);
        b->fit_exec = nullptr;
        cudaStreamSynchronize(b->stream);
        if ((e = cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal)) != cudaSuccess)
            return cuda_fail(b, e, "cudaStreamBeginCapture");
        rc = enqueue(b, b->d_fimg, b->stream, mode, CS_SCHED_PERSISTENT);
        if (rc == CS_OK) {
            rc = cs::launch_batch_fit(b->dsets, (int)ns, b->d_fimg, b->d_fit, b->d_fqs, nbuf, nbuf, b->fred, b->stream);
            if (rc == CS_OK) {
                cudaMemcpyAsync(b->h_fit_out, b->fred.d_sum, sizeof(double) * ns, cudaMemcpyDeviceToHost, b->stream);
                cudaMemcpyAsync(b->h_fit_out + ns, b->fred.d_cnt, sizeof(double) * ns, cudaMemcpyDeviceToHost,
                                b->stream);
                cudaMemcpyAsync(b->h_fit_out + 2 * ns, b->fred.d_nan, sizeof(double) * ns, cudaMemcpyDeviceToHost,
                                b->stream);
            } else {
                b->err = "fit kernel launch";
            }
        }
        cudaGraph_t g = nullptr;
        e = cudaStreamEndCapture(b->stream, &g);
        if (rc != CS_OK) {
            if (g) cudaGraphDestroy(g);
            return rc == CS_ERR_CUDA ? cuda_fail(b, cs::last_launch_error(), "fit evaluation") : rc;
        }
        if (e != cudaSuccess) return cuda_fail(b, e, "cudaStreamEndCapture");
        e = cudaGraphInstantiate(&b->fit_exec, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) {
            b->fit_exec = nullptr;
            return cuda_fail(b, e, "cudaGraphInstantiate");
        }
        b->fit_graph_sig = sig;
    }
    if ((e = cudaGraphLaunch(b->fit_exec, b->stream)) != cudaSuccess) return cuda_fail(b, e, "cudaGraphLaunch");
    if ((e = cudaStreamSynchronize(b->stream)) != cudaSuccess) return cuda_fail(b, e, "fit evaluation");
    if (mode == CS_MODE_MIXED) {
        long n = 0;
        if ((rc = cs_batch_redo_pixels(b, b->stream, &n, nullptr)) != CS_OK) return rc;
    }
    const unsigned long long *hc = (const unsigned long long *)(b->h_fit_out + ns);
    const unsigned long long *hn = (const unsigned long long *)(b->h_fit_out + 2 * ns);
    for (size_t k = 0; k < ns; k++) {
        chi2[k] = b->h_fit_out[k];
        if (cnt) cnt[k] = (long)hc[k];
        if (nancnt) nancnt[k] = (long)hn[k];
    }
    return CS_OK;
}

// Host out: run the prepared batch (persistent schedule) and copy all images
// into out. A redo-list overflow is handled by growing the list and running
// again.
int cs_batch_run_host(cs_batch *b, int mode, double *out, size_t n_doubles) {
    if (!b || !out) return CS_ERR_PARAM;
    if (!b->prepared) return fail(b, CS_ERR_STATE, "no prepared batch");
    if (n_doubles < b->total_doubles) return fail(b, CS_ERR_SIZE, "output buffer too small for the batch");
    if (mode != CS_MODE_FP64 && mode != CS_MODE_MIXED) return fail(b, CS_ERR_PARAM, "unknown precision mode");
    double *d_out = nullptr;
    cudaError_t e = cudaMallocAsync(&d_out, sizeof(double) * b->total_doubles, b->stream);
    if (e != cudaSuccess) return cuda_fail(b, e, "cudaMallocAsync(batch images)");
    int rc = mode == CS_MODE_MIXED ? ensure_schedule(b, d_out, b->stream) : CS_OK;
    // a redo list that overflows is grown and the batch run again (at most twice)
    for (int attempt = 0; rc == CS_OK && attempt < 3; attempt++) {
        rc = enqueue(b, d_out, b->stream, mode, CS_SCHED_PERSISTENT);
        if (rc || mode != CS_MODE_MIXED) break;
        long n = 0;
        rc = cs_batch_redo_pixels(b, b->stream, &n, nullptr);
        if (rc != CS_ERR_SIZE || attempt == 2) break;
        b->redo_cap_req = std::max<long>(n, 2 * b->redo.cap);
        rc = CS_OK;
    }
    if (rc == CS_OK && (e = cudaMemcpyAsync(out, d_out, sizeof(double) * b->total_doubles, cudaMemcpyDeviceToHost,
                                            b->stream)) != cudaSuccess)
        rc = cuda_fail(b, e, "download batch images");
    cudaFreeAsync(d_out, b->stream);
    if ((e = cudaStreamSynchronize(b->stream)) != cudaSuccess && rc == CS_OK) rc = cuda_fail(b, e, "batch calculation");
    return rc;
}

// Host in, host out: prepare, then cs_batch_run_host.
int cs_calc_batch(cs_batch *b, const cs_params *sets, int nsets, int ign_new_switch, int ign_cbs, int mode,
                  double *out, size_t n_doubles) {
    if (!b || !out) return CS_ERR_PARAM;
    int rc = cs_batch_prepare(b, sets, nsets, ign_new_switch, ign_cbs, 0);
    if (rc) return rc;
    return cs_batch_run_host(b, mode, out, n_doubles);
}

}  // extern "C"
