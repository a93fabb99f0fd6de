// cs_capi.cpp — the C ABI (include/crystalscatter.h).
//
// A handle owns: the parameter set, the quadrant state of the reference's
// stateful setters, one prepared block in pinned host memory and its device
// copy, the image in device memory and a pinned host mirror (data()), the fit
// target, and one CUDA stream. Parameter checks, preparation and timers follow
// doCalculation / doFitCalculation (Source/sc_calc_generic_cpu.cpp:1151-1443).
// There is no CPU path: a calculation without a usable GPU fails with
// CS_ERR_CUDA.

#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>

#include "../../include/crystalscatter.h"
#include "cs_launch.h"
#include "cs_mixed.h"
#include "cs_noalloc.h"
#include "cs_params_internal.h"
#include "cs_prep.h"

struct cs_handle {
    cs_params params;
    int calc_quadrants = CS_RADQ4;  // quadrant state of the reference's setRadQ* setters
    std::string err;

    cs_prepared *hprep = nullptr;  // pinned
    cs_delta_node *hdelta = nullptr;
    int device = -1;
    cudaStream_t stream = nullptr;
    cudaEvent_t upload_done = nullptr;
    cs_prepared *dprep = nullptr;
    cs_delta_node *ddelta = nullptr;

    double *dimg = nullptr;
    size_t dimg_cap = 0;
    double *himg = nullptr;
    size_t himg_cap = 0;
    int xmin = 0, xmax = 0, ymin = 0, ymax = 0;
    int new_switch = 0;
    bool prepared = false;
    double t_prep = 0, t_calc = 0;

    // mixed-precision path: compact peak tables and the FP64 redo list
    bool peaks_valid = false;
    cs::HostPeaks hpeaks;
    float *d_aq = nullptr, *d_awl = nullptr, *d_iq = nullptr, *d_imf = nullptr;
    float4 *d_av = nullptr;
    int *d_aidx = nullptr;
    size_t peak_cap = 0;
    cs::MixedScratch mscratch;
    size_t redo_cap = 0;
    // redo counter of the last launch (the handle's own scratch or the
    // allocation-free launch's static one); null after an FP64 launch
    const int *last_count = nullptr;

    // fit
    double *dfit = nullptr, *dfqs = nullptr;
    int fit_w = 0, fit_h = 0;
    int nofit[4][4];
    cs::FitReduce red;
};

namespace {

std::mutex g_chi_mutex;
cs_chi_node *g_dchi[64] = {nullptr};  // per device

double now_ms() {
    using namespace std::chrono;
    return duration_cast<duration<double, std::milli>>(steady_clock::now().time_since_epoch()).count();
}

int fail(cs_handle *h, int code, const std::string &msg) {
    if (h) h->err = msg;
    return code;
}

int cuda_fail(cs_handle *h, cudaError_t e, const char *what) {
    return fail(h, CS_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

// Device setup on first GPU use of a handle.
int ensure_device(cs_handle *h) {
    if (h->stream) return CS_OK;
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess || n == 0) return fail(h, CS_ERR_CUDA, "no CUDA device available (this library has no CPU path)");
    if ((e = cudaGetDevice(&h->device)) != cudaSuccess) return cuda_fail(h, e, "cudaGetDevice");
    if ((e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking)) != cudaSuccess)
        return cuda_fail(h, e, "cudaStreamCreate");
    if ((e = cudaEventCreateWithFlags(&h->upload_done, cudaEventDisableTiming)) != cudaSuccess)
        return cuda_fail(h, e, "cudaEventCreate");
    if ((e = cudaMalloc(&h->dprep, sizeof(cs_prepared))) != cudaSuccess) return cuda_fail(h, e, "cudaMalloc(prepared)");
    return CS_OK;
}

// The chi node table is the same for every parameter set: one copy per device.
int ensure_chi(cs_handle *h, double chi_b, const cs_chi_node **out) {
    std::lock_guard<std::mutex> lock(g_chi_mutex);
    if (h->device < 0 || h->device >= 64) return fail(h, CS_ERR_CUDA, "device index out of range");
    if (!g_dchi[h->device]) {
        cs_chi_node *host = new cs_chi_node[CS_CHI_TABLE_LEN];
        cs::build_chi_table(chi_b, host);
        cs_chi_node *dev = nullptr;
        cudaError_t e = cudaMalloc(&dev, sizeof(cs_chi_node) * CS_CHI_TABLE_LEN);
        if (e == cudaSuccess) e = cudaMemcpy(dev, host, sizeof(cs_chi_node) * CS_CHI_TABLE_LEN, cudaMemcpyHostToDevice);
        delete[] host;
        if (e != cudaSuccess) return cuda_fail(h, e, "chi node table");
        g_dchi[h->device] = dev;
    }
    *out = g_dchi[h->device];
    return CS_OK;
}

void resolve_quadrants(cs_handle *h, int &cq, int &expand) {
    // prepareData calls setRadQ1, setRadQ2, setRadQ4 (each only acts when
    // true) and then setExpandImage (sc_calc_generic.cpp:190-194,
    // sc_calc_generic_gpu.h:292-295)
    if (h->params.radq1) h->calc_quadrants = CS_RADQ1;
    if (h->params.radq2) h->calc_quadrants = CS_RADQ2;
    if (h->params.radq4) h->calc_quadrants = CS_RADQ4;
    cq = h->calc_quadrants;
    expand = (h->params.expand && cq != CS_RADQ4) ? 1 : 0;
}

// Host preparation + upload of the prepared block (and the delta table).
int prepare_and_upload(cs_handle *h, int ign_new_switch, int ign_cbs, int check, cs::DevSet &D) {
    int rc = ensure_device(h);
    if (rc) return rc;
    if (!h->hprep) {
        cudaError_t e = cudaMallocHost(&h->hprep, sizeof(cs_prepared));
        if (e != cudaSuccess) return cuda_fail(h, e, "cudaMallocHost(prepared)");
    }
    // the previous upload must have left the pinned block before it is rewritten
    cudaEventSynchronize(h->upload_done);
    int cq, expand;
    resolve_quadrants(h, cq, expand);
    std::string err;
    const double t0 = now_ms();
    rc = cs::prepare(h->params, cq, expand, ign_new_switch, ign_cbs, check, h->hprep, err);
    if (rc != CS_OK) {
        h->prepared = false;
        if (rc == CS_ERR_PARAM) h->xmin = h->xmax = h->ymin = h->ymax = 0;
        return fail(h, rc, err);
    }
    if (!cs::key_supported(*h->hprep)) {
        h->prepared = false;
        char buf[160];
        std::snprintf(buf, sizeof buf,
                      "combination particle=%d peak=%d ltype=%d ordis=%d (key 0x%08X%s) has no GPU pixel function here",
                      h->hprep->particle, h->hprep->shp, h->hprep->ltype, h->hprep->ordis, (unsigned)h->hprep->key,
                      h->hprep->ign_switch ? ", generic path requested" : "");
        return fail(h, CS_ERR_UNSUPPORTED, buf);
    }
    const cs_chi_node *dchi = nullptr;
    if ((rc = ensure_chi(h, h->hprep->romb_chi_b, &dchi))) return rc;
    cudaError_t e = cudaMemcpyAsync(h->dprep, h->hprep, sizeof(cs_prepared), cudaMemcpyHostToDevice, h->stream);
    if (e != cudaSuccess) return cuda_fail(h, e, "upload prepared block");
    D.d_prep = h->dprep;
    D.d_chi = dchi;
    D.d_delta = nullptr;
    if (cs::needs_delta_table(*h->hprep)) {
        if (!h->hdelta) {
            if ((e = cudaMallocHost(&h->hdelta, sizeof(cs_delta_node) * CS_NODE_COUNT)) != cudaSuccess)
                return cuda_fail(h, e, "cudaMallocHost(delta table)");
            if ((e = cudaMalloc(&h->ddelta, sizeof(cs_delta_node) * CS_NODE_COUNT)) != cudaSuccess)
                return cuda_fail(h, e, "cudaMalloc(delta table)");
        }
        cs::build_delta_table(h->hprep->romb_delta_b, h->hprep->romb_dbeta, h->hdelta);
        e = cudaMemcpyAsync(h->ddelta, h->hdelta, sizeof(cs_delta_node) * CS_NODE_COUNT, cudaMemcpyHostToDevice,
                            h->stream);
        if (e != cudaSuccess) return cuda_fail(h, e, "upload delta table");
        D.d_delta = h->ddelta;
    }
    cudaEventRecord(h->upload_done, h->stream);
    h->peaks_valid = false;
    h->t_prep = now_ms() - t0;
    h->xmin = h->hprep->xmin;
    h->xmax = h->hprep->xmax;
    h->ymin = h->hprep->ymin;
    h->ymax = h->hprep->ymax;
    h->prepared = true;
    return CS_OK;
}

size_t image_count(const cs_handle *h) {
    return (size_t)(h->xmax - h->xmin) * (size_t)(h->ymax - h->ymin);
}

// Peak tables and redo scratch of the mixed path for the prepared set.
int ensure_mixed(cs_handle *h) {
    cudaError_t e;
    const long npix = (long)(h->hprep->zzmax - h->hprep->zzmin) * (long)(h->hprep->iimax - h->hprep->iimin);
    if ((size_t)npix > h->redo_cap) {
        if (h->mscratch.d_list) cudaFree(h->mscratch.d_list);
        if (!h->mscratch.d_count && (e = cudaMalloc(&h->mscratch.d_count, 2 * sizeof(int))) != cudaSuccess)
            return cuda_fail(h, e, "cudaMalloc(redo count)");
        if ((e = cudaMalloc(&h->mscratch.d_list, sizeof(int) * (size_t)npix)) != cudaSuccess)
            return cuda_fail(h, e, "cudaMalloc(redo list)");
        h->redo_cap = (size_t)npix;
        h->mscratch.cap = (int)npix;
    }
    if (!h->peaks_valid && h->hprep->lattice) {
        cs::build_peak_tables(*h->hprep, h->hpeaks);
        const size_t n = std::max(h->hpeaks.aq.size(), h->hpeaks.iq.size()) + 1;
        if (n > h->peak_cap) {
            cudaFree(h->d_aq);
            cudaFree(h->d_awl);
            cudaFree(h->d_iq);
            cudaFree(h->d_imf);
            cudaFree(h->d_av);
            cudaFree(h->d_aidx);
            if ((e = cudaMalloc(&h->d_aidx, sizeof(int) * n)) != cudaSuccess ||
                (e = cudaMalloc(&h->d_aq, sizeof(float) * n)) != cudaSuccess ||
                (e = cudaMalloc(&h->d_awl, sizeof(float) * n)) != cudaSuccess ||
                (e = cudaMalloc(&h->d_iq, sizeof(float) * n)) != cudaSuccess ||
                (e = cudaMalloc(&h->d_imf, sizeof(float) * n)) != cudaSuccess ||
                (e = cudaMalloc(&h->d_av, sizeof(float4) * 2 * n)) != cudaSuccess)
                return cuda_fail(h, e, "cudaMalloc(peak tables)");
            h->peak_cap = n;
        }
        const cs::HostPeaks &H = h->hpeaks;
        // synchronous copies: the host vectors are rebuilt on the next preparation
        if (!H.aq.empty()) {
            cudaMemcpy(h->d_aq, H.aq.data(), sizeof(float) * H.aq.size(), cudaMemcpyHostToDevice);
            cudaMemcpy(h->d_awl, H.awl.data(), sizeof(float) * H.awl.size(), cudaMemcpyHostToDevice);
            cudaMemcpy(h->d_av, H.av.data(), sizeof(float4) * H.av.size(), cudaMemcpyHostToDevice);
            cudaMemcpy(h->d_aidx, H.aidx.data(), sizeof(int) * H.aidx.size(), cudaMemcpyHostToDevice);
        }
        if (!H.iq.empty()) {
            cudaMemcpy(h->d_iq, H.iq.data(), sizeof(float) * H.iq.size(), cudaMemcpyHostToDevice);
            cudaMemcpy(h->d_imf, H.imf.data(), sizeof(float) * H.imf.size(), cudaMemcpyHostToDevice);
        }
        if ((e = cudaGetLastError()) != cudaSuccess) return cuda_fail(h, e, "upload peak tables");
    }
    h->peaks_valid = true;
    return CS_OK;
}

int run_image(cs_handle *h, double *d_out, cudaStream_t s, int mode) {
    cs::DevSet D;
    D.d_prep = h->dprep;
    D.d_chi = g_dchi[h->device];
    D.d_delta = cs::needs_delta_table(*h->hprep) ? h->ddelta : nullptr;
    if (h->hprep->expand) {
        // pixels the mirroring never writes (row -zmax) read as 0
        cudaError_t e = cudaMemsetAsync(d_out, 0, sizeof(double) * image_count(h), s);
        if (e != cudaSuccess) return cuda_fail(h, e, "cudaMemsetAsync");
    }
    int rc;
    if (mode == CS_MODE_FP64) {
        h->last_count = nullptr;
        rc = cs::launch_image(D, *h->hprep, d_out, s);
    } else if (mode == CS_MODE_MIXED && (!cs::mixed_key(h->hprep->key) || h->hprep->twin)) {
        // no mixed-precision kernel for this combination: the FP64 kernel
        // serves the request (no pixel needs a redo)
        if (h->mscratch.d_count) cudaMemsetAsync(h->mscratch.d_count, 0, sizeof(int), s);
        h->last_count = h->mscratch.d_count;
        rc = cs::launch_image(D, *h->hprep, d_out, s);
    } else if (mode == CS_MODE_MIXED) {
        if ((rc = ensure_mixed(h))) return rc;
        csm::PeakTab T;
        if (h->hprep->lattice) {
            T.n_aniso = (int)h->hpeaks.aq.size();
            T.aq = h->d_aq;
            T.av = h->d_av;
            T.awl = h->d_awl;
            T.aidx = h->d_aidx;
            T.n_iso = (int)h->hpeaks.iq.size();
            T.iq = h->d_iq;
            T.imf = h->d_imf;
        }
        h->last_count = h->mscratch.d_count;
        rc = cs::launch_image_mixed(D, T, *h->hprep, d_out, h->mscratch, s);
        if (rc == CS_ERR_UNSUPPORTED) return fail(h, rc, "no mixed-precision kernel for this combination");
    } else {
        return fail(h, CS_ERR_PARAM, "unknown precision mode");
    }
    if (rc != CS_OK)
        return rc == CS_ERR_CUDA ? cuda_fail(h, cs::last_launch_error(), "kernel launch")
                                 : fail(h, rc, "no kernel for this combination");
    return CS_OK;
}

}  // namespace

extern "C" {

const char *cs_version(void) { return "crystalscatter-gb300 0.1 (sm_103a)"; }

int cs_gpu_available(void) {
    int n = 0;
    return (cudaGetDeviceCount(&n) == cudaSuccess && n > 0) ? 1 : 0;
}

cs_handle *cs_create(void) {
    cs_handle *h = new (std::nothrow) cs_handle;
    if (!h) return nullptr;
    cs::default_params(&h->params);
    for (int i = 0; i < 4; i++)
        for (int k = 0; k < 4; k++) h->nofit[i][k] = -1;
    return h;
}

void cs_destroy(cs_handle *h) {
    if (!h) return;
    if (h->stream) cudaStreamSynchronize(h->stream);
    if (h->dprep) cudaFree(h->dprep);
    if (h->ddelta) cudaFree(h->ddelta);
    if (h->dimg) cudaFree(h->dimg);
    if (h->dfit) cudaFree(h->dfit);
    if (h->dfqs) cudaFree(h->dfqs);
    if (h->red.d_psum) cudaFree(h->red.d_psum);
    if (h->red.d_pcnt) cudaFree(h->red.d_pcnt);
    if (h->red.d_pnan) cudaFree(h->red.d_pnan);
    if (h->red.d_sum) cudaFree(h->red.d_sum);
    if (h->red.d_cnt) cudaFree(h->red.d_cnt);
    if (h->red.d_nan) cudaFree(h->red.d_nan);
    if (h->hprep) cudaFreeHost(h->hprep);
    if (h->hdelta) cudaFreeHost(h->hdelta);
    cudaFree(h->d_aq);
    cudaFree(h->d_awl);
    cudaFree(h->d_iq);
    cudaFree(h->d_imf);
    cudaFree(h->d_av);
    cudaFree(h->d_aidx);
    cudaFree(h->mscratch.d_count);
    cudaFree(h->mscratch.d_list);
    if (h->himg) cudaFreeHost(h->himg);
    if (h->upload_done) cudaEventDestroy(h->upload_done);
    if (h->stream) cudaStreamDestroy(h->stream);
    delete h;
}

void cs_default_params(cs_params *p) {
    if (p) cs::default_params(p);
}

int cs_set_params(cs_handle *h, const cs_params *p) {
    if (!h || !p) return CS_ERR_PARAM;
    h->params = *p;
    return CS_OK;
}

int cs_get_params(cs_handle *h, cs_params *p) {
    if (!h || !p) return CS_ERR_PARAM;
    *p = h->params;
    return CS_OK;
}

int cs_set_param(cs_handle *h, const char *key, double value) {
    if (!h || !key) return CS_ERR_PARAM;
    if (!cs::set_param(&h->params, key, value)) return fail(h, CS_ERR_PARAM, std::string("unknown parameter key '") + key + "'");
    return CS_OK;
}

int cs_set_param_text(cs_handle *h, const char *key, const char *text) {
    if (!h || !key || !text) return CS_ERR_PARAM;
    if (!cs::set_param_text(&h->params, key, text))
        return fail(h, CS_ERR_PARAM, std::string("'") + key + "' is not a combobox parameter");
    return CS_OK;
}

int cs_set_kv(cs_handle *h, const char *kv) {
    if (!h || !kv) return CS_ERR_PARAM;
    cs::apply_kv(&h->params, kv);
    return CS_OK;
}

int cs_calc_image(cs_handle *h, int num_threads, int ign_new_switch, int ign_cbs, int mode) {
    if (!h) return CS_ERR_PARAM;
    if (num_threads != 0)
        return fail(h, CS_ERR_PARAM, "numThreads must be 0: this library computes on the GPU only");
    cs::DevSet D;
    int rc = prepare_and_upload(h, ign_new_switch, ign_cbs, 1, D);
    if (rc) return rc;
    const double t0 = now_ms();
    const size_t n = image_count(h);
    cudaError_t e;
    if (n > h->dimg_cap) {
        if (h->dimg) cudaFree(h->dimg);
        h->dimg = nullptr;
        h->dimg_cap = 0;
        if ((e = cudaMalloc(&h->dimg, sizeof(double) * n)) != cudaSuccess) return cuda_fail(h, e, "cudaMalloc(image)");
        h->dimg_cap = n;
    }
    if (n > h->himg_cap) {
        if (h->himg) cudaFreeHost(h->himg);
        h->himg = nullptr;
        h->himg_cap = 0;
        if ((e = cudaMallocHost(&h->himg, sizeof(double) * n)) != cudaSuccess) return cuda_fail(h, e, "cudaMallocHost(image)");
        h->himg_cap = n;
    }
    if ((rc = run_image(h, h->dimg, h->stream, mode))) return rc;
    if ((e = cudaMemcpyAsync(h->himg, h->dimg, sizeof(double) * n, cudaMemcpyDeviceToHost, h->stream)) != cudaSuccess)
        return cuda_fail(h, e, "image download");
    if ((e = cudaStreamSynchronize(h->stream)) != cudaSuccess) return cuda_fail(h, e, "calculation");
    h->new_switch = 1;
    h->t_calc = now_ms() - t0;
    return CS_OK;
}

int cs_calc_image_device(cs_handle *h, double *d_out, size_t n_doubles, void *stream, int ign_new_switch, int ign_cbs,
                         int mode) {
    if (!h || !d_out) return CS_ERR_PARAM;
    cs::DevSet D;
    int rc = prepare_and_upload(h, ign_new_switch, ign_cbs, 1, D);
    if (rc) return rc;
    if (image_count(h) > n_doubles) return fail(h, CS_ERR_SIZE, "output buffer too small for the image");
    cudaStream_t s = stream ? (cudaStream_t)stream : h->stream;
    if (s != h->stream) cudaStreamWaitEvent(s, h->upload_done, 0);
    return run_image(h, d_out, s, mode);
}

int cs_launch_prepared(cs_handle *h, double *d_out, size_t n_doubles, void *stream, int mode) {
    if (!h || !d_out) return CS_ERR_PARAM;
    if (!h->prepared) return fail(h, CS_ERR_STATE, "no prepared calculation");
    if (image_count(h) > n_doubles) return fail(h, CS_ERR_SIZE, "output buffer too small for the image");
    cudaStream_t s = stream ? (cudaStream_t)stream : h->stream;
    if (s != h->stream) cudaStreamWaitEvent(s, h->upload_done, 0);
    return run_image(h, d_out, s, mode);
}

int cs_launch_prepared_mixed_noalloc(cs_handle *h, double *d_out, size_t n_doubles, void *stream) {
    if (!h || !d_out) return CS_ERR_PARAM;
    if (!h->prepared) return fail(h, CS_ERR_STATE, "no prepared calculation");
    if (image_count(h) > n_doubles) return fail(h, CS_ERR_SIZE, "output buffer too small for the image");
    const cs_prepared &P = *h->hprep;
    const long npix = (long)(P.zzmax - P.zzmin) * (long)(P.iimax - P.iimin);
    if (npix > CS_NOALLOC_MAX_PIXELS) {
        char buf[200];
        std::snprintf(buf, sizeof buf,
                      "image of %ld calculated pixels exceeds the allocation-free launch's fixed scratch of %d pixels",
                      npix, CS_NOALLOC_MAX_PIXELS);
        return fail(h, CS_ERR_SIZE, buf);
    }
    const bool fp64_kernel = !cs::mixed_key(P.key) || P.twin;
    if (P.lattice && !fp64_kernel && !h->peaks_valid)
        return fail(h, CS_ERR_STATE,
                    "reflection tables of this preparation are not on the device: run one CS_MODE_MIXED calculation "
                    "on it first");
    int cur = -1;
    cudaError_t e = cudaGetDevice(&cur);
    if (e != cudaSuccess) return cuda_fail(h, e, "cudaGetDevice");
    if (cur != h->device) return fail(h, CS_ERR_STATE, "the handle's device is not the current device");
    cs::MixedScratch S;
    if ((e = cs::noalloc_scratch(h->device, S)) != cudaSuccess) return cuda_fail(h, e, "cudaGetSymbolAddress(scratch)");
    cudaStream_t s = stream ? (cudaStream_t)stream : h->stream;
    if (s != h->stream) cudaStreamWaitEvent(s, h->upload_done, 0);
    cs::DevSet D;
    D.d_prep = h->dprep;
    D.d_chi = g_dchi[h->device];
    D.d_delta = cs::needs_delta_table(P) ? h->ddelta : nullptr;
    if (P.expand) {
        // pixels the mirroring never writes read as 0
        if ((e = cudaMemsetAsync(d_out, 0, sizeof(double) * image_count(h), s)) != cudaSuccess)
            return cuda_fail(h, e, "cudaMemsetAsync");
    }
    h->last_count = S.d_count;
    int rc;
    if (fp64_kernel) {
        // no mixed-precision kernel for this combination: the FP64 kernel
        // serves the request exactly as cs_launch_prepared(..., CS_MODE_MIXED)
        // does (it needs no scratch; the static counter reads 0 redone pixels)
        if ((e = cudaMemsetAsync(S.d_count, 0, sizeof(int), s)) != cudaSuccess)
            return cuda_fail(h, e, "cudaMemsetAsync(redo counter)");
        rc = cs::launch_image(D, P, d_out, s);
    } else {
        csm::PeakTab T;
        if (P.lattice) {
            T.n_aniso = (int)h->hpeaks.aq.size();
            T.aq = h->d_aq;
            T.av = h->d_av;
            T.awl = h->d_awl;
            T.aidx = h->d_aidx;
            T.n_iso = (int)h->hpeaks.iq.size();
            T.iq = h->d_iq;
            T.imf = h->d_imf;
        }
        // clears the static counter on s, then the mixed kernel and the FP64 redo
        rc = cs::launch_image_mixed(D, T, P, d_out, S, s);
    }
    if (rc == CS_ERR_CUDA) return cuda_fail(h, cs::last_launch_error(), "kernel launch");
    if (rc != CS_OK) return fail(h, rc, "no kernel for this combination");
    return CS_OK;
}

int cs_prepared_pixels(cs_handle *h, long *npix) {
    if (!h || !npix) return CS_ERR_PARAM;
    if (!h->prepared) return fail(h, CS_ERR_STATE, "no prepared calculation");
    *npix = (long)(h->hprep->zzmax - h->hprep->zzmin) * (long)(h->hprep->iimax - h->hprep->iimin);
    return CS_OK;
}

int cs_image_dims(cs_handle *h, int *xmin, int *xmax, int *ymin, int *ymax) {
    if (!h) return CS_ERR_PARAM;
    if (xmin) *xmin = h->xmin;
    if (xmax) *xmax = h->xmax;
    if (ymin) *ymin = h->ymin;
    if (ymax) *ymax = h->ymax;
    return CS_OK;
}

const double *cs_data(cs_handle *h) { return h ? h->himg : nullptr; }

int cs_copy_image(cs_handle *h, double *out, size_t n_doubles) {
    if (!h || !out) return CS_ERR_PARAM;
    const size_t n = image_count(h);
    if (n > n_doubles) return fail(h, CS_ERR_SIZE, "output buffer too small for the image");
    if (!h->himg) return fail(h, CS_ERR_STATE, "no image calculated");
    std::memcpy(out, h->himg, sizeof(double) * n);
    return CS_OK;
}

double cs_timer_ms(cs_handle *h, int which) {
    if (!h) return 0;
    return which == 0 ? h->t_prep : h->t_calc;
}

int cs_new_switch_used(cs_handle *h) { return h ? h->new_switch : 0; }

int cs_set_fit_data(cs_handle *h, int width, int height, const double *data) {
    if (!h) return CS_ERR_PARAM;
    if (h->dfit) cudaFree(h->dfit);
    if (h->dfqs) cudaFree(h->dfqs);
    h->dfit = h->dfqs = nullptr;
    h->fit_w = h->fit_h = 0;
    if (!data || width <= 0 || height <= 0) return fail(h, CS_ERR_PARAM, "no fit data");
    int rc = ensure_device(h);
    if (rc) return rc;
    const size_t n = (size_t)width * (size_t)height;
    cudaError_t e;
    if ((e = cudaMalloc(&h->dfit, sizeof(double) * n)) != cudaSuccess) return cuda_fail(h, e, "cudaMalloc(fit data)");
    if ((e = cudaMalloc(&h->dfqs, sizeof(double) * n)) != cudaSuccess) return cuda_fail(h, e, "cudaMalloc(fit fqs)");
    if ((e = cudaMemcpy(h->dfit, data, sizeof(double) * n, cudaMemcpyHostToDevice)) != cudaSuccess)
        return cuda_fail(h, e, "upload fit data");
    if (!h->red.d_psum) {
        h->red.nblocks = 256;
        if ((e = cudaMalloc(&h->red.d_psum, sizeof(double) * h->red.nblocks)) != cudaSuccess ||
            (e = cudaMalloc(&h->red.d_pcnt, sizeof(unsigned long long) * h->red.nblocks)) != cudaSuccess ||
            (e = cudaMalloc(&h->red.d_pnan, sizeof(unsigned long long) * h->red.nblocks)) != cudaSuccess ||
            (e = cudaMalloc(&h->red.d_sum, sizeof(double))) != cudaSuccess ||
            (e = cudaMalloc(&h->red.d_cnt, sizeof(unsigned long long))) != cudaSuccess ||
            (e = cudaMalloc(&h->red.d_nan, sizeof(unsigned long long))) != cudaSuccess)
            return cuda_fail(h, e, "cudaMalloc(fit reduction)");
    }
    h->fit_w = width;
    h->fit_h = height;
    return CS_OK;
}

int cs_set_nofit_rect(cs_handle *h, int id, int x0, int y0, int x1, int y1) {
    if (!h) return CS_ERR_PARAM;
    if (id < 0 || id >= 4) return CS_ERR_PARAM;
    h->nofit[id][0] = x0;
    h->nofit[id][1] = y0;
    h->nofit[id][2] = x1;
    h->nofit[id][3] = y1;
    return CS_OK;
}

int cs_fit_chi2(cs_handle *h, int num_threads, int bstop, int border, int mode, double *chi2, long *cnt,
                long *nancnt) {
    if (!h || !chi2) return CS_ERR_PARAM;
    *chi2 = 1e20;  // the reference's value for a failed fit evaluation
    if (num_threads != 0) return fail(h, CS_ERR_PARAM, "numThreads must be 0: this library computes on the GPU only");
    if (!h->dfit) return fail(h, CS_ERR_STATE, "setFitData has not been called");
    if (mode != CS_MODE_FP64) return fail(h, CS_ERR_UNSUPPORTED, "mixed precision mode not available in this build");
    cs::DevSet D;
    // doFitCalculation runs prepareCalculation without checkAllParameters
    int rc = prepare_and_upload(h, 0, 0, 0, D);
    if (rc) return rc;
    cudaEventSynchronize(h->upload_done);
    cs_prepared &P = *h->hprep;
    P.fit_width = h->fit_w;
    P.fit_height = h->fit_h;
    P.fit_bstop = bstop;
    P.fit_border = border;
    for (int i = 0; i < 4; i++) {
        P.nofit_x0[i] = h->nofit[i][0];
        P.nofit_y0[i] = h->nofit[i][1];
        P.nofit_x1[i] = h->nofit[i][2];
        P.nofit_y1[i] = h->nofit[i][3];
    }
    const double t0 = now_ms();
    cudaError_t e = cudaMemcpyAsync(h->dprep, h->hprep, sizeof(cs_prepared), cudaMemcpyHostToDevice, h->stream);
    if (e != cudaSuccess) return cuda_fail(h, e, "upload prepared block");
    cudaEventRecord(h->upload_done, h->stream);
    const long nbuf = (long)h->fit_w * h->fit_h;
    // pixels the kernel does not reach keep 0 like a freshly allocated buffer
    if ((e = cudaMemsetAsync(h->dfqs, 0, sizeof(double) * nbuf, h->stream)) != cudaSuccess)
        return cuda_fail(h, e, "cudaMemsetAsync(fqs)");
    D.d_prep = h->dprep;
    rc = cs::launch_fit(D, P, h->dfit, h->dfqs, nbuf, h->red, h->stream);
    if (rc == CS_ERR_CUDA) return cuda_fail(h, cs::last_launch_error(), "fit kernel launch");
    if (rc != CS_OK) return fail(h, rc, "no fit kernel for this combination");
    double s = 0;
    unsigned long long c = 0, nn = 0;
    cudaMemcpyAsync(&s, h->red.d_sum, sizeof(double), cudaMemcpyDeviceToHost, h->stream);
    cudaMemcpyAsync(&c, h->red.d_cnt, sizeof(c), cudaMemcpyDeviceToHost, h->stream);
    cudaMemcpyAsync(&nn, h->red.d_nan, sizeof(nn), cudaMemcpyDeviceToHost, h->stream);
    if ((e = cudaStreamSynchronize(h->stream)) != cudaSuccess) return cuda_fail(h, e, "fit calculation");
    h->t_calc = now_ms() - t0;
    *chi2 = s;
    if (cnt) *cnt = (long)c;
    if (nancnt) *nancnt = (long)nn;
    return CS_OK;
}

const char *cs_last_error(cs_handle *h) { return h ? h->err.c_str() : "null handle"; }

int cs_mixed_redo_pixels(cs_handle *h, long *n) {
    if (!h || !n) return CS_ERR_PARAM;
    *n = 0;
    if (!h->last_count) return CS_OK;
    int v = 0;
    cudaStreamSynchronize(h->stream);
    cudaError_t e = cudaMemcpy(&v, h->last_count, sizeof(int), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_fail(h, e, "read redo count");
    *n = v;
    return CS_OK;
}

// Host preparation alone (prepareCalculation, Source/sc_calc_generic_cpu.cpp:319),
// without any CUDA call: used by tests and by the CPU oracle to obtain the
// prepared block of a parameter set.
size_t cs_prepared_size(void) { return sizeof(cs_prepared); }

int cs_prepare_params(const cs_params *p, int ign_new_switch, int ign_cbs, void *out, size_t out_size, char *err,
                      size_t errlen) {
    if (!p || !out || out_size < sizeof(cs_prepared)) return CS_ERR_PARAM;
    int cq = CS_RADQ4;
    if (p->radq1) cq = CS_RADQ1;
    if (p->radq2) cq = CS_RADQ2;
    if (p->radq4) cq = CS_RADQ4;
    const int expand = (p->expand && cq != CS_RADQ4) ? 1 : 0;
    std::string e;
    const int rc = cs::prepare(*p, cq, expand, ign_new_switch, ign_cbs, 1, (cs_prepared *)out, e);
    if (err && errlen) {
        std::strncpy(err, e.c_str(), errlen - 1);
        err[errlen - 1] = 0;
    }
    return rc;
}

}  // extern "C"
