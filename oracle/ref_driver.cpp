// Test-oracle driver around the reference's own FP64 CPU calculation class.
//
// This file is TEST INFRASTRUCTURE. It is compiled together with the
// reference sources (Source/sc_calc_generic_cpu.cpp and
// Source/sc_calc_generic_gpu.cu, the latter as plain C++ so that only the CPU
// path exists) by oracle/build_ref.sh into oracle/_ref/libscref.so. Nothing in
// the product links it; tests use it to pin the oracle restatement and to
// generate golden fixtures.
//
// Parameters are set by the reference's own parameter keys (the names used by
// SC_Calc_GENERIC::prepareData, Source/sc_calc_generic.cpp:142-238) and are
// applied through the reference's setters in the same order as prepareData.

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <list>
#include <map>
#include <string>
#include <pthread.h>
#include <vector>

// The driver reads a few private members (known-answer tests of the host
// preparation); the reference class is not modified.
#define private public
#include "sc_calc_generic_gpu.h"
#undef private

// layout of the prepared block that the CPU oracle (oracle/cs_oracle.c) reads
#include "../crystalscatter_gb300/csrc/cs_prepared.h"

namespace {

struct RefHandle {
    SasCalc_GENERIC_calculation *calc = nullptr;
    std::map<std::string, double> kv;
    std::string err;
    std::vector<double> fitdata;
};

double getv(RefHandle *h, const char *k, double dflt) {
    auto it = h->kv.find(k);
    return it == h->kv.end() ? dflt : it->second;
}

// Same setter order as SC_Calc_GENERIC::prepareData (sc_calc_generic.cpp:142-238).
// Defaults are those of SC_CalcCons (guiLayoutNeu defaults, sc_calcCons.cpp:24-100
// and the inpValues defaults of SC_CalcCons::dataGetter, sc_calcCons.cpp:649-668).
void apply(RefHandle *h) {
    SasCalc_GENERIC_calculation *c = h->calc;
    c->setLType((int)getv(h, "LType", 12));
    c->setUCA(getv(h, "uca", 30));
    c->setUCB(getv(h, "ucb", 30));
    c->setUCC(getv(h, "ucc", 30));
    c->setUCalpha(getv(h, "ucalpha", 90));
    c->setUCbeta(getv(h, "ucbeta", 90));
    c->setUCgamma(getv(h, "ucgamma", 90));
    c->setCeffF(getv(h, "EditCeff", 1));
    c->setCheckBoxTwinned(getv(h, "CheckBoxTwinned", 0) != 0);
    c->setCeffCyl(getv(h, "EditCeffcyl", 0));
    c->setReff(getv(h, "reff", 0));
    c->setAcpl(getv(h, "acpl", 0));
    c->setBcpl(getv(h, "bcpl", 0));
    c->setIFluc(getv(h, "ifluc", 0));
    c->setRFluc(getv(h, "rfluc", 0));

    c->setComboBoxParticle((int)getv(h, "ComboBoxParticle", -1));
    c->setOrdis((int)getv(h, "Ordis", 7));
    c->setComboBoxInterior((int)getv(h, "ComboBoxInterior", 0));
    c->setRadiusF(getv(h, "EditRadius", 1.0));
    c->setRadiusI(getv(h, "EditRadiusi", 0.5));
    c->setSigmaF(getv(h, "EditSigma", 0.07));
    c->setDBetaF(getv(h, "EditDbeta", 0.4));
    c->setLength(getv(h, "Length", 1));
    c->setSigmaL(getv(h, "SigmaL", 0.06));
    c->setAlpha(getv(h, "Alpha", 0));
    c->setRho(getv(h, "EditRho", 0));
    c->setRotAlpha(getv(h, "RotAlpha", 0));

    c->setComboBoxPeak((int)getv(h, "ComboBoxPeak", 1));
    c->setPeakPar(getv(h, "EditPeakPar", 0));
    c->setDisplacement(getv(h, "EditDebyeWaller", 2));
    c->setAzi(getv(h, "EditAzi", 180));
    c->setDomainsize(getv(h, "EditDomainSize", 400));
    c->setRadioButtonDebyeScherrer(getv(h, "RadButDebyeScherrer", 0) != 0);
    c->setRadioButtonPara(getv(h, "RadioButtonPara", 0) != 0);
    c->setAx1(Double3(getv(h, "EditAxis1x", 1), getv(h, "EditAxis1y", 0), getv(h, "EditAxis1z", 0)));
    c->setAx2(Double3(getv(h, "EditAxis2x", 0), getv(h, "EditAxis2y", 1), getv(h, "EditAxis2z", 0)));
    c->setAx3(Double3(getv(h, "EditAxis3x", 0), getv(h, "EditAxis3y", 0), getv(h, "EditAxis3z", 1)));
    c->setSigXYZ(Double3(getv(h, "Editdom1", 40), getv(h, "Editdom2", 40), getv(h, "Editdom3", 40)));

    c->setUCpsi(getv(h, "ucpsi", 0));
    c->setUCn1(getv(h, "ucn1", 1));
    c->setUCn2(getv(h, "ucn2", 1));
    c->setUCn3(getv(h, "ucn3", 1));
    c->setPolTheta(getv(h, "theta", 90));
    c->setPolPhi(getv(h, "phi", 0));
    c->setRotTheta(getv(h, "rotTheta", 90));
    c->setRotPhi(getv(h, "rotPhi", 90));

    c->setHKLmax((int)getv(h, "HKLmax", 5));
    c->setQMax(getv(h, "EditQmax", 1));
    c->setGridPoints((int)getv(h, "GridPoints", 64), false);
    c->setRadQ1(getv(h, "RadioButtonQ1", 0) > 0);
    c->setRadQ2(getv(h, "RadioButtonQ2", 0) > 0);
    c->setRadQ4(getv(h, "RadioButtonQ4", 1) > 0);
    c->setExpandImage(getv(h, "ExpandImage", 0) > 0);

    c->setpixnox(getv(h, "EditPixelNoX", 2048));
    c->setpixnoy(getv(h, "EditPixelNoY", 2048));
    c->setpixx(getv(h, "EditPixelX", 1));
    c->setpixy(getv(h, "EditPixelY", 1));
    c->setdet(getv(h, "EditDet", 1));
    c->setwave(getv(h, "EditWavelength", 0.09499));
    c->setBeamStop(getv(h, "BeamPosX", 0), getv(h, "BeamPosY", 0));
    c->setUseBeamStop(getv(h, "CenterBeam", 0) != 0);

    c->setBFactorF(getv(h, "EditBFactor", 1));
    c->setCheckBoxWAXS(getv(h, "CheckBoxWAXS", 0) != 0);
    c->setP1(getv(h, "P1", 0));

    c->setIso(getv(h, "iso", 0));
    c->setIZero(getv(h, "I0", 10000));
    c->setBase(getv(h, "Base", 0));
}

}  // namespace

extern "C" {

// The reference keeps static state (the instance pointer and the pthread
// array, sc_calc_generic_cpu.cpp:98-99) and frees the thread bookkeeping of
// the previous run through the current instance, so a second instance in the
// same process crashes in a multi-threaded run. All handles therefore share
// one calculation object, as the console program does.
static SasCalc_GENERIC_calculation *g_calc = nullptr;

void *ref_create(void) {
    RefHandle *h = new RefHandle;
    if (!g_calc) g_calc = new SasCalc_GENERIC_calculation();
    h->calc = g_calc;
    for (int i = 0; i < 4; i++) h->calc->setNoFitRect(i, -1, -1, -1, -1);
    return h;
}

void ref_destroy(void *p) {
    RefHandle *h = static_cast<RefHandle *>(p);
    delete h;
}

void ref_set(void *p, const char *key, double value) {
    static_cast<RefHandle *>(p)->kv[key] = value;
}

void ref_clear(void *p) { static_cast<RefHandle *>(p)->kv.clear(); }

// doCalculation(numThreads, bIgnoreNewSwitch, bIgnoreCbs), sc_calc_generic_cpu.cpp:1151.
int ref_run(void *p, int nthreads, int ign_new_switch, int ign_cbs) {
    RefHandle *h = static_cast<RefHandle *>(p);
    apply(h);
    if (nthreads < 1) nthreads = 1;  // 0 would mean "GPU"; this build has none
    h->calc->doCalculation(nthreads, ign_new_switch != 0, ign_cbs != 0);
    h->err = h->calc->getLastErrorMessage();
    return h->err.empty() ? 0 : 1;
}

const char *ref_error(void *p) { return static_cast<RefHandle *>(p)->err.c_str(); }

void ref_dims(void *p, int *xmin, int *xmax, int *ymin, int *ymax) {
    SasCalc_GENERIC_calculation *c = static_cast<RefHandle *>(p)->calc;
    *xmin = c->minX();
    *xmax = c->maxX();
    *ymin = c->minY();
    *ymax = c->maxY();
}

// Copies the image: (maxX-minX)*(maxY-minY) doubles, row-major in y as data().
long ref_image(void *p, double *out, long cap) {
    SasCalc_GENERIC_calculation *c = static_cast<RefHandle *>(p)->calc;
    long n = (long)(c->maxX() - c->minX()) * (long)(c->maxY() - c->minY());
    if (n > cap) return -n;
    if (n > 0) std::memcpy(out, c->data(), sizeof(double) * n);
    return n;
}

double ref_timer(void *p, int which) {
    SasCalc_GENERIC_calculation *c = static_cast<RefHandle *>(p)->calc;
    return which == 0 ? c->higResTimerElapsedPrep : c->higResTimerElapsedCalc;
}

// Known-answer access to the prepared constants.
int ref_get_array(void *p, const char *name, double *out) {
    SasCalc_GENERIC_calculation *c = static_cast<RefHandle *>(p)->calc;
    auto *CR = c->params.CR;
    if (!CR) return -1;
    struct { const char *n; double *a; } tab[] = {
        {"carr1p", CR->carr1p}, {"carr2p", CR->carr2p}, {"carr3p", CR->carr3p},
        {"carr4p", CR->carr4p}, {"carr5p", CR->carr5p}, {"carr6p", CR->carr6p},
        {"carr7p", CR->carr7p}, {"carr8p", CR->carr8p}, {"carr9p", CR->carr9p},
        {"carr1f", CR->carr1f}, {"carr2f", CR->carr2f}, {"carr3f", CR->carr3f},
        {"carr4f", CR->carr4f}, {"carr5f", CR->carr5f}, {"carr6f", CR->carr6f},
        {"carr7f", CR->carr7f}, {"carr8f", CR->carr8f}, {"carr9f", CR->carr9f},
    };
    for (auto &t : tab)
        if (!std::strcmp(name, t.n)) {
            std::memcpy(out, t.a, sizeof(double) * coeffarray_len);
            return coeffarray_len;
        }
    if (!std::strcmp(name, "carr11pm")) {
        std::memcpy(out, CR->carr11pm, sizeof(double) * imax2d_len * imax2d_len);
        return imax2d_len * imax2d_len;
    }
    if (!std::strcmp(name, "carr22pm")) {
        std::memcpy(out, CR->carr22pm, sizeof(double) * imax2d_len * imax2d_len);
        return imax2d_len * imax2d_len;
    }
    return -1;
}

double ref_get_scalar(void *p, const char *name) {
    SasCalc_GENERIC_calculation *c = static_cast<RefHandle *>(p)->calc;
    auto &P = c->params;
    struct { const char *n; double v; } tab[] = {
        {"limq1", P.limq1}, {"limq2", P.limq2}, {"limq3", P.limq3}, {"limq4", P.limq4},
        {"limq5", P.limq5}, {"limq6", P.limq6}, {"limq7", P.limq7}, {"limq8", P.limq8},
        {"limq9", P.limq9}, {"limq1f", P.limq1f}, {"limq2f", P.limq2f}, {"limq3f", P.limq3f},
        {"limq4f", P.limq4f}, {"limq5f", P.limq5f}, {"limq6f", P.limq6f}, {"limq7f", P.limq7f},
        {"limq8f", P.limq8f}, {"limq9f", P.limq9f}, {"norm", P.norm}, {"por", P.por},
        {"orcase", (double)P.orcase}, {"order", c->order}, {"p1", P.p1},
        {"peakmax1", (double)c->peakmax1}, {"peakmax2", (double)c->peakmax2},
        {"latpar1", c->latpar[1]}, {"latpar2", c->latpar[2]}, {"latpar3", c->latpar[3]},
        {"ucvol", c->ucvol}, {"phiwidth", c->phiwidth}, {"dwfactor", c->dwfactor},
        {"reldis", c->reldis}, {"dist", c->dist}, {"cdim", (double)c->cdim},
        {"zzmin", (double)c->zzmin}, {"zzmax", (double)c->zzmax},
        {"iimin", (double)c->iimin}, {"iimax", (double)c->iimax},
        {"cosphic", c->cosphic}, {"sinphic", c->sinphic},
        {"ri11", c->ri11}, {"ri12", c->ri12}, {"ri13", c->ri13},
        {"ri21", c->ri21}, {"ri22", c->ri22}, {"ri23", c->ri23},
        {"ri31", c->ri31}, {"ri32", c->ri32}, {"ri33", c->ri33},
        {"newswitch", (double)c->newSwitchUsed()},
    };
    for (auto &t : tab)
        if (!std::strcmp(name, t.n)) return t.v;
    return NAN;
}

// latpar1/latpar2: int[2500][6]; latpar3: float[2500][17].
int ref_get_latpar(void *p, int which, void *out) {
    SasCalc_GENERIC_calculation *c = static_cast<RefHandle *>(p)->calc;
    const int L = SasCalc_GENERIC_calculation::latparlen;
    if (which == 1 && c->latpar1ptr) { std::memcpy(out, c->latpar1ptr, sizeof(int) * L * 6); return L * 6; }
    if (which == 2 && c->latpar2ptr) { std::memcpy(out, c->latpar2ptr, sizeof(int) * L * 6); return L * 6; }
    if (which == 3 && c->latpar3ptr) { std::memcpy(out, c->latpar3ptr, sizeof(float) * L * 17); return L * 17; }
    return -1;
}

// Fit support: setFitData (sc_calc_generic_cpu.cpp:8220), setNoFitRect
// (sc_calc_generic_gpu.h:365) and doFitCalculation (sc_calc_generic_cpu.cpp:1334).
int ref_set_fit_data(void *p, int w, int h_, const double *data) {
    RefHandle *h = static_cast<RefHandle *>(p);
    return h->calc->setFitData(w, h_, data) ? 0 : 1;
}

void ref_set_nofit_rect(void *p, int id, int x0, int y0, int x1, int y1) {
    static_cast<RefHandle *>(p)->calc->setNoFitRect(id, x0, y0, x1, y1);
}

double ref_fit(void *p, int nthreads, int bstop, int border, long *cnt, long *nancnt) {
    RefHandle *h = static_cast<RefHandle *>(p);
    apply(h);
    if (nthreads < 1) nthreads = 1;
    return h->calc->doFitCalculation(nthreads, bstop, border, *cnt, *nancnt);
}

// The reference's own host preparation without the image: the checks and
// prepareCalculation() of doCalculation (sc_calc_generic_cpu.cpp:1151-1166).
// Returns 0, or 1 with the error message (ref_error) when the parameters are
// rejected or the preparation fails.
int ref_prepare(void *p, int ign_new_switch, int ign_cbs) {
    RefHandle *h = static_cast<RefHandle *>(p);
    apply(h);
    SasCalc_GENERIC_calculation *c = h->calc;
    c->numberOfThreads = 1;
    c->bIgnoreNewSwitch = ign_new_switch != 0;
    h->err = c->checkAllParameters(ign_cbs != 0);
    if (!h->err.empty()) return 1;
    if (!c->prepareCalculation()) {
        h->err = c->getLastErrorMessage();
        if (h->err.empty()) h->err = "prepareCalculation failed";
        return 1;
    }
    return 0;
}

// The prepared constants of the last ref_prepare / ref_run, written into the
// prepared-block layout that the CPU oracle evaluates (cs_prepared.h): every
// field the oracle reads, taken from the reference object's own members after
// its prepareCalculation. The dispatch key is formed as calcCPU_selection
// forms it (sc_calc_generic_gpu.cu:190-218). Fields the oracle does not read
// stay zero. Returns the block size, or -1 when out_size is too small.
long ref_export_prepared(void *p, void *out, size_t out_size) {
    if (out_size < sizeof(cs_prepared)) return -1;
    SasCalc_GENERIC_calculation *c = static_cast<RefHandle *>(p)->calc;
    auto &R = c->params;
    cs_prepared *P = static_cast<cs_prepared *>(out);
    std::memset(P, 0, sizeof(cs_prepared));
    const int lt = (int)c->ltype;
    P->particle = (int)c->ComboBoxParticle;
    P->shp = (int)c->shp;
    P->ltype = lt;
    P->ordis = (int)R.ordis;
    P->ign_switch = c->bIgnoreNewSwitch ? 1 : 0;
    const int key = (P->particle << 24) | (lt == 12 ? 0 : (P->shp << 16)) | (lt << 8) | P->ordis;
    const bool special = !c->bIgnoreNewSwitch &&
                         (key == CS_KEY_SPHERE_NONE_ISO || key == CS_KEY_SPHERE_GAUSS_FCC_GAUSS ||
                          key == CS_KEY_CYL_NONE_GAUSS || key == CS_KEY_CYL_NONE_ZDIR ||
                          key == CS_KEY_CYL_GAUSS_BCT_ZDIR || key == CS_KEY_CUBE_NONE_ISO);
    P->key = special ? key : CS_KEY_GENERIC;
    P->cs = R.cs;
    P->part = R.part;
    P->cdim = c->cdim;
    P->partdim = c->partdim;
    P->orcase = (int)R.orcase;
    P->lattice = c->lattice ? 1 : 0;
    P->twin = c->twin ? 1 : 0;
    P->debyescherrer = c->RadioButtonDebyeScherrer ? 1 : 0;
    P->para = c->RadioButtonPara ? 1 : 0;
    // geometry
    P->use1d = c->use1d ? 1 : 0;
    P->usebeamstop = c->useBeamStop ? 1 : 0;
    P->zmax = c->zmax;
    P->zzmin = c->zzmin;
    P->zzmax = c->zzmax;
    P->iimin = c->iimin;
    P->iimax = c->iimax;
    P->xmin = c->_xmin;
    P->xmax = c->_xmax;
    P->ymin = c->_ymin;
    P->ymax = c->_ymax;
    P->calc_quadrants = (int)c->calcQuadrants;
    P->expand = c->bExpandImage ? 1 : 0;
    P->qmax = c->qmax;
    P->qmin = c->qmin;
    P->pixnox = c->pixnox;
    P->pixnoy = c->pixnoy;
    P->pixx_m = c->pixx_m;
    P->pixy_m = c->pixy_m;
    P->beamx0 = c->beamX0;
    P->beamy0 = c->beamY0;
    P->det = c->det;
    P->wave = c->wave;
    // pixel manipulation
    P->base = c->base;
    P->izero = c->izero;
    P->iso = c->iso;
    P->ifluc = c->ifluc;
    P->rfluc = c->rfluc;
    // particle
    P->radius = R.radius;
    P->radiusi = R.radiusi;
    P->sigma = R.sigma;
    P->sigmal = R.sigmal;
    P->length = R.length;
    P->p1 = R.p1;
    P->rho = R.rho;
    P->alphash1 = R.alphash1;
    P->alpha = R.alpha;
    P->poltheta = R.polTheta;
    P->polphi = R.polPhi;
    P->dbeta = R.dbeta;
    P->norm = R.norm;
    P->por = R.por;
    P->order = c->order;
    const double lq[10] = {0, R.limq1, R.limq2, R.limq3, R.limq4, R.limq5, R.limq6, R.limq7, R.limq8, R.limq9};
    const double lf[10] = {0, R.limq1f, R.limq2f, R.limq3f, R.limq4f, R.limq5f, R.limq6f, R.limq7f, R.limq8f, R.limq9f};
    for (int i = 0; i < 10; i++) {
        P->limq[i] = lq[i];
        P->limqf[i] = lf[i];
    }
    P->cosphic = c->cosphic;
    P->sinphic = c->sinphic;
    P->cosphi = c->cosphi;
    P->sinphi = c->sinphi;
    P->costheta = c->costheta;
    P->sintheta = c->sintheta;
    // lattice
    P->peakmax1 = c->peakmax1;
    P->peakmax2 = c->peakmax2;
    for (int i = 0; i < 4; i++) P->latpar[i] = c->latpar[i];
    P->dwfactor = c->dwfactor;
    P->uca = R.uca;
    P->ucb = R.ucb;
    P->domainsize = R.domainsize;
    P->width_zuf = R.width_zuf;
    P->reldis = c->reldis;
    P->dist = c->dist;
    P->phiwidth = c->phiwidth;
    P->ceff = R.ceff;
    // coefficient arrays
    if (R.CR) {
        const double *cp[9] = {R.CR->carr1p, R.CR->carr2p, R.CR->carr3p, R.CR->carr4p, R.CR->carr5p,
                               R.CR->carr6p, R.CR->carr7p, R.CR->carr8p, R.CR->carr9p};
        const double *cf[9] = {R.CR->carr1f, R.CR->carr2f, R.CR->carr3f, R.CR->carr4f, R.CR->carr5f,
                               R.CR->carr6f, R.CR->carr7f, R.CR->carr8f, R.CR->carr9f};
        for (int k = 0; k < 9; k++) {
            std::memcpy(P->carrp[k], cp[k], sizeof(double) * CS_COEFF_LEN);
            std::memcpy(P->carrf[k], cf[k], sizeof(double) * CS_COEFF_LEN);
        }
        std::memcpy(P->carr11pm, R.CR->carr11pm, sizeof(double) * CS_IMAX2D * CS_IMAX2D);
    }
    // reflection tables (same [2500][6] / [2500][17] layout as the reference's)
    const int L = SasCalc_GENERIC_calculation::latparlen;
    if (c->latpar1ptr) std::memcpy(P->latpar1, c->latpar1ptr, sizeof(int) * L * 6);
    if (c->latpar2ptr) std::memcpy(P->latpar2, c->latpar2ptr, sizeof(int) * L * 6);
    if (c->latpar3ptr) std::memcpy(P->latpar3, c->latpar3ptr, sizeof(float) * L * 17);
    for (int i = 0; i < 4; i++) P->nofit_x0[i] = P->nofit_x1[i] = P->nofit_y0[i] = P->nofit_y1[i] = -1;
    return (long)sizeof(cs_prepared);
}

// Per-pixel FQS values left by the last fit call (arrFitFqs, fitWidth*fitHeight).
long ref_fit_fqs(void *p, double *out, long cap) {
    SasCalc_GENERIC_calculation *c = static_cast<RefHandle *>(p)->calc;
    long n = (long)c->_arrFitSize;
    if (n > cap) return -n;
    if (n > 0 && c->arrFitFqs) std::memcpy(out, c->arrFitFqs, sizeof(double) * n);
    return n;
}

// Training-data randomisation then calculation, as the generator does per
// image (Source/sc_mainCons.cpp:1170, :1236-1246): the handle's values are
// applied, the saved TPV state is cleared, the C library's generator is
// seeded, tpvPerformRandom (sc_calc_generic_cpu.cpp:1028) randomises the
// entries of ids ('\n'-separated "key=value"), and doCalculation runs. Its
// log text goes to log.
int ref_tpv_run(void *p, const char *ids, unsigned seed, int nthreads, int ign_cbs, char *log, size_t cap) {
    RefHandle *h = static_cast<RefHandle *>(p);
    apply(h);
    h->calc->tpvPerformRandom(std::list<std::string>());
    std::list<std::string> lst;
    std::string cur;
    for (const char *c = ids; *c; c++) {
        if (*c == '\n') {
            if (!cur.empty()) lst.push_back(cur);
            cur.clear();
        } else {
            cur += *c;
        }
    }
    if (!cur.empty()) lst.push_back(cur);
    srand(seed);
    const std::string rv = h->calc->tpvPerformRandom(lst);
    if (log && cap) {
        std::strncpy(log, rv.c_str(), cap - 1);
        log[cap - 1] = 0;
    }
    if (nthreads < 1) nthreads = 1;
    h->calc->doCalculation(nthreads, false, ign_cbs != 0);
    h->err = h->calc->getLastErrorMessage();
    return h->err.empty() ? 0 : 1;
}

}  // extern "C"
