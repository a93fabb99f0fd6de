/*
 * crystalscatter.h — C ABI of the GB300 implementation of CrystalScatter's
 * per-pixel 2D small-angle scattering pattern calculation.
 *
 * The ABI replaces the public surface of the reference class
 * SasCalc_GENERIC_calculation (Source/sc_calc_generic_gpu.h:77-598) and the
 * console key/value entry (Source/sc_mainCons.cpp:858-913). Every function
 * takes plain pointers and sizes; no C++ or CUDA types cross the boundary.
 * A handle holds one parameter set, its prepared constants, its device
 * buffers and one CUDA stream. A handle is not thread safe; use one handle per
 * host thread (the reference itself allows one calculation per process).
 *
 * Status codes: every int-returning call returns CS_OK or an error code and
 * leaves a message in cs_last_error(). Parameter rejections carry exactly the
 * reference's message text (SasCalc_GENERIC_calculation::checkAllParameters,
 * Source/sc_calc_generic_cpu.cpp:198-308).
 */
#ifndef CRYSTALSCATTER_H
#define CRYSTALSCATTER_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CS_OK 0
#define CS_ERR_PARAM 1       /* parameters rejected (reference checkAllParameters / isCbsValid) */
#define CS_ERR_CUDA 2        /* CUDA runtime error, no usable GPU or extension not loaded */
#define CS_ERR_TIMEOUT 3     /* a bounded device-side wait gave up */
#define CS_ERR_UNSUPPORTED 4 /* the reference computes no coefficients for this combination */
#define CS_ERR_ALLOC 5       /* host or device allocation failed */
#define CS_ERR_STATE 6       /* call order error (e.g. fit without fit data) */
#define CS_ERR_SIZE 7        /* caller buffer too small / size limit exceeded */

/* Precision of a calculation. */
#define CS_MODE_FP64 0  /* plain FP64 GPU drop-in: same operation order as the reference */
#define CS_MODE_MIXED 1 /* FP32 bulk with FP64 guard bands; <= 1e-5 relative to FP64 */

/* Quadrant selection (reference _radQX, Source/sc_math.h:26-31). */
#define CS_RAD_Q1 0
#define CS_RAD_Q2 1
#define CS_RAD_Q4 2

/*
 * All parameters of one calculation. Field meaning, units and defaults follow
 * the reference setters (Source/sc_calc_generic_gpu.h:108-353) and the
 * console defaults (SC_CalcCons, Source/sc_calcCons.cpp:24-100, 649-668):
 *   lengths in nm, pixel sizes in mm, distance in m, angles in degrees.
 * Combobox fields hold the reference's 0-based combobox index
 * (ComboBoxPeak: 0 = Lorentzian ... 7 = Anisotropic Gaussian; the engine
 * adds 1 exactly like setComboBoxPeak).
 */
typedef struct cs_params {
    /* Lattice group: setLatticeParams, sc_calc_generic_gpu.h:123-144 */
    int ltype;
    double uca, ucb, ucc, ucalpha, ucbeta, ucgamma;
    double ceff;
    int twinned;
    double ceffcyl, reff, acpl, bcpl, ifluc, rfluc;
    /* Particle group: setParticleParams, sc_calc_generic_gpu.h:192-209 */
    int particle, ordis, interior;
    double radius, radiusi, sigma, dbeta, length, sigmal, alphash, rho, alpha;
    /* Peak shape group: setPeakShapeParams, sc_calc_generic_gpu.h:235-263 */
    int peak;
    double peakpar, debyewaller, azi, domainsize;
    int debyescherrer, para;
    double ax1[3], ax2[3], ax3[3], sigxyz[3];
    /* Orientation group: setOrientationParams, sc_calc_generic_gpu.h:274-285 */
    double ucpsi, ucn1, ucn2, ucn3, theta, phi, rottheta, rotphi;
    /* Calculation group: setCalculationParams, sc_calc_generic_gpu.h:296-307 */
    int gridpoints, hklmax;
    double qmax, qmin;
    int radq1, radq2, radq4, expand, use1d;
    /* Experiment group: setExperimentParams, sc_calc_generic_gpu.h:318-330 */
    double pixnox, pixnoy, pixx_mm, pixy_mm, det, wavelength, beamx, beamy;
    int usebeamstop; /* "CenterBeam": 1 = beam-centre geometry, 0 = midpoint/qmax */
    /* Controls group: setControlParams, sc_calc_generic_gpu.h:337-342 */
    double bfactor;
    int waxs;
    double p1;
    /* Pixel manipulation group: setPixelManipulationParams, sc_calc_generic_gpu.h:348-353 */
    double iso, izero, base;
    /* Training-data randomisation (tpvPerformRandom, Source/sc_calc_generic_cpu.cpp:1028-1143) of two
       values that are not setter parameters: the domain-size width factor is 1 + tpv_domain_dev and
       the Debye-Waller factor d^2/3 is multiplied by 1 + tpv_dw_dev. 0 = not randomised. */
    double tpv_domain_dev, tpv_dw_dev;
} cs_params;

typedef struct cs_handle cs_handle;

/* Library / device */
const char *cs_version(void);
int cs_gpu_available(void); /* 1 when a CUDA device is usable (reference gpuAvailable, sc_calc_generic_gpu.h:441) */

/* Measured arithmetic peaks of the current device (no counterpart in the
   reference; the denominators of the pixel kernels' compute roofline), each
   from a few milliseconds of independent dependent chains on every SM, timed
   with CUDA events on `stream` (cudaStream_t as void*, NULL = the default
   stream). out[0] FP32 FMA, out[1] packed FP32 pair FMA (f32x2), out[2] FP64
   FMA, all in TFLOP/s (2 flops per FMA); out[3] the special-function unit's
   ex2.approx.f32 in Tops/s. n >= 4. */
int cs_measure_pipe_peaks(void *stream, double *out, int n);

/* Handle lifetime: constructor / cleanup() (sc_calc_generic_cpu.cpp:102, 994) */
cs_handle *cs_create(void);
void cs_destroy(cs_handle *h);

/* Parameters */
void cs_default_params(cs_params *p);                   /* SC_CalcCons defaults */
int cs_set_params(cs_handle *h, const cs_params *p);    /* grouped set*Params */
int cs_get_params(cs_handle *h, cs_params *p);
/* One parameter by the reference's own key (SC_Calc_GENERIC::prepareData keys,
   Source/sc_calc_generic.cpp:142-238, plus RadioButtonQ1/Q2/Q4, ExpandImage,
   CenterBeam, EditAxis1x..3z and Editdom1..3 as in SC_CalcCons). Combobox
   keys take the numeric index. Mirrors SC_CalcCons::updateParamValue
   (Source/sc_calcCons.cpp:573). */
int cs_set_param(cs_handle *h, const char *key, double value);
/* Combobox by text, e.g. ("ComboBoxParticle", "cylinder"); mirrors
   SC_CalcCons::updateParamValue(QString,QString) (sc_calcCons.cpp:610). */
int cs_set_param_text(cs_handle *h, const char *key, const char *text);
/* The console --mcpval string "key=value;key=value" with the lower-case JSON
   keys of generateJsonKeyList (Source/sc_mainCons.cpp:76-119) and the value
   rules of calculateFromChatbotKeyValList (sc_mainCons.cpp:858-900). */
int cs_set_kv(cs_handle *h, const char *kv);

/* Calculation: doCalculation(numThreads, bIgnoreNewSwitch, bIgnoreCbs)
   (Source/sc_calc_generic_cpu.cpp:1151). num_threads must be 0 (GPU); any
   other value is rejected: this library has no CPU fallback. The image is
   kept in the handle's host buffer (data()) and device buffer. */
int cs_calc_image(cs_handle *h, int num_threads, int ign_new_switch, int ign_cbs, int mode);
/* Image extents (minX/maxX/minY/maxY, sc_calc_generic_gpu.h:579-582). The
   image holds (xmax-xmin)*(ymax-ymin) doubles, row-major in y. */
int cs_image_dims(cs_handle *h, int *xmin, int *xmax, int *ymin, int *ymax);
const double *cs_data(cs_handle *h); /* data(), valid until the next calculation */
int cs_copy_image(cs_handle *h, double *out, size_t n_doubles);
double cs_timer_ms(cs_handle *h, int which); /* 0 = prep (higResTimerElapsedPrep), 1 = calc */
int cs_new_switch_used(cs_handle *h);        /* newSwitchUsed() */

/* Device-resident variant: prepares on the host, then writes the image into
   the caller's device buffer d_out (n_doubles capacity) on the caller's CUDA
   stream (cudaStream_t passed as void*, NULL = the handle's stream). No
   host<->device copy of the image. Returns after enqueueing (asynchronous). */
int cs_calc_image_device(cs_handle *h, double *d_out, size_t n_doubles, void *stream, int ign_new_switch,
                         int ign_cbs, int mode);
/* Re-launch the last prepared calculation into d_out without host work. */
int cs_launch_prepared(cs_handle *h, double *d_out, size_t n_doubles, void *stream, int mode);

/* Allocation-free mixed-precision launch. No counterpart in the reference:
   it exists for callers that must not allocate while they calculate, such as
   a fit or monitoring loop that keeps its device memory fixed after set-up, or
   one that runs work on other streams and cannot accept the device-wide
   synchronisation of cudaFree. cs_launch_prepared(..., CS_MODE_MIXED) may
   allocate the handle's redo list (the pixels recomputed in FP64) on first use
   or when a larger image comes along; this variant keeps that list in a fixed
   static device array of CS_NOALLOC_MAX_PIXELS entries instead.
   - It calls no cudaMalloc/cudaFree and no allocating library routine (no
     PyTorch): it enqueues memsets and kernels on `stream` (NULL = the
     handle's stream) and returns.
   - Requirements: a prepared handle (cs_calc_image, cs_calc_image_device or
     cs_launch_prepared ran for the current parameters); for parameter sets
     with a lattice, one earlier CS_MODE_MIXED call on that preparation, which
     uploads the reflection tables (otherwise CS_ERR_STATE); the handle's
     device is the current device (otherwise CS_ERR_STATE).
   - Images of more than CS_NOALLOC_MAX_PIXELS calculated pixels are rejected
     with CS_ERR_SIZE and a message naming the limit.
   - The first call on a device does the set-up: it looks up the address of
     the static array (cudaGetSymbolAddress), which may load the library's
     device module. Make that first call before any stream capture.
   - The static list is cleared (a memset on `stream`) at the start of every
     call; the result is the same as cs_launch_prepared(..., CS_MODE_MIXED),
     also for combinations without a mixed-precision kernel (twinned
     lattices, the generic pixel function, cubes), which run their FP64
     kernel there as here. cs_mixed_redo_pixels then reports this launch's
     redo count (read from the static counter).
   - There is one static list per device: calls whose work overlaps on the GPU
     (other streams, other handles, other threads) race on it. Order them on
     one stream or synchronise between them. */
#define CS_NOALLOC_MAX_PIXELS 1048576
int cs_launch_prepared_mixed_noalloc(cs_handle *h, double *d_out, size_t n_doubles, void *stream);
int cs_prepared_pixels(cs_handle *h, long *npix);

/* 2D fit support: setFitData (sc_calc_generic_cpu.cpp:8220), setNoFitRect
   (sc_calc_generic_gpu.h:365), doFitCalculation (sc_calc_generic_cpu.cpp:1334).
   chi2 = sum of FQSVERGL over unmasked pixels, reduced on the device. */
int cs_set_fit_data(cs_handle *h, int width, int height, const double *data);
int cs_set_nofit_rect(cs_handle *h, int id, int x0, int y0, int x1, int y1);
int cs_fit_chi2(cs_handle *h, int num_threads, int bstop, int border, int mode, double *chi2, long *cnt,
                long *nancnt);

const char *cs_last_error(cs_handle *h);

/* Pixels of the last mixed-precision calculation whose FP32 result sat inside
   a decision guard band and were recomputed in FP64 (no counterpart in the
   reference; reported alongside accuracy figures). It covers the handle's
   last launch of either mixed entry point; after an FP64 launch it is 0. */
int cs_mixed_redo_pixels(cs_handle *h, long *n);

/* Host preparation alone, without any CUDA call (the reference's private
   prepareCalculation, Source/sc_calc_generic_cpu.cpp:319-988): fills the
   prepared constant block (layout: crystalscatter_gb300/csrc/cs_prepared.h,
   cs_prepared_size() bytes) for a parameter set, with the quadrant flags of
   the parameter set applied to the default quadrant state. Used by the test
   oracle and by tests of the preparation. */
size_t cs_prepared_size(void);
int cs_prepare_params(const cs_params *p, int ign_new_switch, int ign_cbs, void *out, size_t out_size, char *err,
                      size_t errlen);

/* ---- Batches: many parameter sets per launch --------------------------------
   The reference evaluates parameter sets one at a time (a sweep, or the
   simplex fit's vertices, Source/sc_simplexfit2d.cpp:54-62, each through
   doCalculation). A batch prepares N sets at once (host threads), keeps them
   resident on the device, and computes all their images either with one
   launch per set (CS_SCHED_PLAIN, what N calls of the single-set interface
   issue) or with one persistent launch per dispatch key fed by a device tile
   queue (CS_SCHED_PERSISTENT). Each set is checked as doCalculation checks it
   (checkAllParameters(bIgnoreCbs)); the first rejected set fails the batch
   with its index in the message. Quadrant flags of each set apply to the
   default quadrant state (as cs_prepare_params). Images lie one after another
   in one buffer, each starting at a multiple of 32 doubles; cs_batch_layout
   gives offset and extents per set. cs_calc_batch is the host-buffer form.
   Results are the same as the single-set calls give for each set. */
typedef struct cs_batch cs_batch;
#define CS_SCHED_PLAIN 0
#define CS_SCHED_PERSISTENT 1
cs_batch *cs_batch_create(void);
void cs_batch_destroy(cs_batch *b);
const char *cs_batch_last_error(cs_batch *b);
/* host_threads: threads for the host preparation (0 = all hardware threads). */
int cs_batch_prepare(cs_batch *b, const cs_params *sets, int nsets, int ign_new_switch, int ign_cbs, int host_threads);
int cs_batch_info(cs_batch *b, size_t *total_doubles, long *total_pixels, int *ngroups);
/* Host-to-device bytes that the last cs_batch_prepare uploaded (prepared
   blocks, reflection and node tables, set table). */
int cs_batch_upload_bytes(cs_batch *b, size_t *bytes);

/* Schedule of the mixed-precision persistent kernel (no counterpart in the
   reference). Work comes from a device counter either as block tiles of 256
   pixels (chunk 0; the block's threads synchronise per tile) or as warp
   chunks of 32, 64, 128 or 256 pixels (no barrier), with blocks_per_sm
   resident blocks (0 = the occupancy limit). By default (chunk -1) an
   autotuner chooses both per dispatch key at the first mixed persistent run
   (cs_batch_launch/capture/profile/run_host) on a device: every candidate
   computes the same 1/32 of the group's pixels, timed with CUDA events, and
   the fastest per pixel is kept for the process. cs_batch_set_schedule
   forces a schedule (chunk -1 returns to the autotuner);
   cs_batch_schedule reports the one in use for a key group (tuned = 1 when
   the autotuner chose it, ns_per_pixel its timed sample). */
int cs_batch_set_schedule(cs_batch *b, int chunk, int blocks_per_sm);
int cs_batch_schedule(cs_batch *b, int group, int *key, int *chunk, int *blocks_per_sm, double *ns_per_pixel,
                      int *tuned);
int cs_batch_layout(cs_batch *b, int k, size_t *offset, int *xmin, int *xmax, int *ymin, int *ymax);
/* Enqueue all images of the prepared batch into d_out (device memory,
   n_doubles capacity) on stream (NULL = the batch's stream); asynchronous. */
int cs_batch_launch(cs_batch *b, double *d_out, size_t n_doubles, void *stream, int mode, int schedule);
/* One persistent run of the batch (as cs_batch_launch with
   CS_SCHED_PERSISTENT) with CUDA events on `stream` around each key group's
   main kernel and its FP64 redo kernel; waits for it and returns the summed
   durations in milliseconds (redo_ms is 0 for CS_MODE_FP64). Kernel timing
   for benchmarks; no counterpart in the reference. */
int cs_batch_profile(cs_batch *b, double *d_out, size_t n_doubles, void *stream, int mode, double *main_ms,
                     double *redo_ms);
/* Capture the same work as a CUDA graph (once) and replay it. The graph
   writes into the d_out given at capture; preparing the batch again drops it. */
int cs_batch_capture(cs_batch *b, double *d_out, size_t n_doubles, int mode, int schedule);
int cs_batch_replay(cs_batch *b, void *stream);
int cs_batch_graph_nodes(cs_batch *b, size_t *n);
/* Mixed persistent form: guarded pixels of the last run (waits for stream).
   CS_ERR_SIZE when the redo list overflowed (some pixels then keep their
   FP32 value): raise the capacity (entries per key group, 0 = automatic: one
   per pixel of the largest group, which cannot overflow) and run again. */
int cs_batch_redo_pixels(cs_batch *b, void *stream, long *n, long *capacity);
int cs_batch_set_redo_capacity(cs_batch *b, long entries_per_group);
double cs_batch_timer_ms(cs_batch *b); /* host preparation time of the last cs_batch_prepare */
/* Batch fit: doFitCalculation (Source/sc_calc_generic_cpu.cpp:1334-1443) for
   every set of a batch against one target, e.g. the vertices of a simplex.
   cs_batch_set_fit stores the target (width x height doubles, the image's
   size) and the masks of doFitCalculation/setNoFitRect (bstop, border, nofit
   = 4 rectangles x {x0,y0,x1,y1}, -1 = unused, NULL = none); batches prepared
   afterwards skip checkAllParameters as doFitCalculation does.
   cs_batch_fit_chi2 computes every set's image (persistent schedule), the
   per-pixel FQSVERGL and its sum, count of non-zero and count of NaN terms
   per set (chi2/cnt/nancnt arrays of nsets entries, chi2 = 1e20 on failure).
   One evaluation is captured as a CUDA graph and replayed while the batch
   keeps its layout (same set count, image sizes and dispatch keys), so a fit
   iteration costs the host preparation plus one graph launch. Needs all four
   quadrants calculated (RadioButtonQ4) and fit data of the image's size. */
int cs_batch_set_fit(cs_batch *b, int width, int height, const double *data, int bstop, int border,
                     const int *nofit);
int cs_batch_fit_chi2(cs_batch *b, int mode, double *chi2, long *cnt, long *nancnt);

/* 2D simplex fit: SasCalc_SimplexFit2D::doSimplexFit2D
   (Source/sc_simplexfit2d.cpp:250-611) over the parameters listed in
   `params` (reference keys as for cs_set_param; `used` = fitted, else held at
   fitstart), starting from `base`, judged by the chi^2 of doFitCalculation
   against `data` (width x height doubles) with the masks bstoppix, borderpix
   and nofit (4 rectangles x {x0,y0,x1,y1}, -1 unused, NULL none). stp, maxit,
   ftol: the reference's step factor, iteration limit and relative tolerance.
   The reference's trajectory is reproduced, including its initialisation of
   the first parameter of every initial vertex to 0 + step and its centroid
   factor over all listed parameters. Results: fitres of every parameter (the
   best vertex), and the report. schedule CS_FIT_SEQUENTIAL evaluates one
   vertex at a time through the drop-in fit call; CS_FIT_BATCHED evaluates the
   independent vertices and, per iteration, the reference's next candidate
   vertices speculatively as one batch (same decisions and result, fewer
   host round trips, more images). mode CS_MODE_MIXED judges vertices by the
   mixed-precision images. chi2_stop > 0 (no counterpart in the reference; 0
   keeps the reference's behaviour) also ends the fit once the best vertex's
   chi^2 is at or below it. */
#define CS_FIT_SEQUENTIAL 0
#define CS_FIT_BATCHED 1
typedef struct cs_fit_param {
    char key[48];     /* reference parameter key, e.g. "EditRadius" */
    double min, max;  /* limits; min 0 and max 360 (an angle) are not checked */
    double fitstart;  /* start value */
    double fitres;    /* result (out) */
    int used;         /* 1 = fitted, 0 = held fixed */
    int fitvalid;     /* 1 after a fit (out) */
} cs_fit_param;
typedef struct cs_fit_report {
    int repetitions; /* simplex iterations run */
    int aborted;     /* 1 when the reference's NaN / zero abort ended the fit */
    long images;     /* fit evaluations calculated on the GPU */
    double chi2;     /* chi^2 of the best vertex */
    double ms;       /* wall time of the fit (higResTimerElapsed) */
    char info[256];  /* message on error */
} cs_fit_report;
int cs_simplex_fit(const cs_params *base, const double *data, int width, int height, const int *nofit,
                   cs_fit_param *params, int nparams, double stp, int maxit, double ftol, int borderpix, int bstoppix,
                   int mode, int schedule, double chi2_stop, cs_fit_report *report);
/* The same simplex over a caller's objective instead of the image chi^2
   (no GPU involved): fn receives npoints parameter vectors of nparams values
   each (the table order of the simplex: fitted keys sorted, then fixed keys
   sorted) and writes one value per point; points outside the limits get 1e20
   without a call. CS_FIT_SEQUENTIAL passes one point per call. */
typedef void (*cs_objective_fn)(const double *points, int npoints, int nparams, double *values, void *ctx);
int cs_simplex_minimize(cs_objective_fn fn, void *ctx, cs_fit_param *params, int nparams, double stp, int maxit,
                        double ftol, int schedule, double chi2_stop, cs_fit_report *report);

/* ---- Surrogate network (no counterpart in the reference) -------------------
   A multilayer perceptron n_in -> hidden -> hidden -> hidden -> n_out (GELU
   after the hidden layers) that maps parameter vectors to log intensities on a
   coarse detector grid; it proposes start points for the simplex fit. BF16
   weights and activations into tensor-core GEMMs with FP32 accumulation; FP32
   master weights updated by Adam on the device. hidden and n_out must be
   multiples of 128, n_in <= 256. All data pointers are device pointers
   (FP32, row-major, n rows); stream NULL = the network's own stream, which is
   ordered with the legacy default stream (work queued there before the call
   is seen, work queued there after it waits). */
typedef struct cs_mlp cs_mlp;
cs_mlp *cs_mlp_create(int n_in, int hidden, int n_out, unsigned long long seed);
void cs_mlp_destroy(cs_mlp *m);
const char *cs_mlp_last_error(cs_mlp *m);
int cs_mlp_forward(cs_mlp *m, const float *d_x, int n, float *d_y, void *stream);
/* gradients of the mean squared error over the n x n_out outputs (kept in the
   network, read with cs_mlp_get_layer); loss (host) may be NULL */
int cs_mlp_gradients(cs_mlp *m, const float *d_x, const float *d_t, int n, float *loss, void *stream);
/* gradients, then one Adam step (beta 0.9 / 0.999, eps 1e-8) with rate lr */
int cs_mlp_train_step(cs_mlp *m, const float *d_x, const float *d_t, int n, float lr, float *loss, void *stream);
/* layer l = 0..3: rows x cols of its weight matrix (cols of layer 0 padded to
   a multiple of 32); FP32 weights, bias and last gradients to/from host */
int cs_mlp_layer_dims(cs_mlp *m, int l, int *rows, int *cols);
int cs_mlp_get_layer(cs_mlp *m, int l, float *w, float *b, float *gw, float *gb);
int cs_mlp_set_layer(cs_mlp *m, int l, const float *w, const float *b);
/* bilinear upsampling of n square s x s FP32 images by an integer factor
   (pixel-centre aligned, clamped at the border), device pointers */
int cs_upsample_bilinear(const float *d_in, int n, int s, int factor, float *d_out, void *stream);

/* ---- r-phi transform of the training-data generator ------------------------
   Replaces SasCalc_PostProc::generateRphi (Source/sc_postproc.cpp:53-334)
   with the scaling options of scaleAndClipData (:764-823): the s x s polar
   image (row = angle, column = radius) of a device image d_img (rows y0..y1-1,
   columns x0..x1-1, FP64, row-major) around the beam centre (xcenter,
   ycenter) in the same coordinates, into device d_out (s*s doubles; entries
   no radius step writes are 0). Minimum coordinates must be at most 0
   (CS_ERR_PARAM otherwise, and for s < 2 or an image without radius steps).
   Returns after the stream has finished the transform. */
#define CS_RPHI_SCALE 1  /* divide by the maximum (running maximum from 0) */
#define CS_RPHI_CLIP 2   /* (log10(|v| / 1e-20) + 6) / 6, clamped at 0 */
#define CS_RPHI_CLIP40 4 /* 1 - (1 - v) / 0.6, clamped at 0 */
int cs_rphi_device(const double *d_img, int x0, int x1, int y0, int y1, int xcenter, int ycenter, int s, int flags,
                   double *d_out, void *stream);

/* Host-buffer forms: run the prepared batch (persistent schedule, a redo
   overflow handled internally) and copy all images into out; cs_calc_batch
   prepares first. */
int cs_batch_run_host(cs_batch *b, int mode, double *out, size_t n_doubles);
int cs_calc_batch(cs_batch *b, const cs_params *sets, int nsets, int ign_new_switch, int ign_cbs, int mode,
                  double *out, size_t n_doubles);

#ifdef __cplusplus
}
#endif
#endif /* CRYSTALSCATTER_H */
