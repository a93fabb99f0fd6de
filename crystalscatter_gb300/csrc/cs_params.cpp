// cs_params.cpp — parameter defaults, reference parameter keys and the
// console key/value string.
//
// Defaults are those the console front end gives every parameter
// (SC_CalcCons constructor over SC_Calc_GENERIC::guiLayoutNeu,
// Source/sc_calcCons.cpp:24-100 and Source/sc_calc_generic.cpp:36-138, plus the
// inpValues defaults of SC_CalcCons::dataGetter, sc_calcCons.cpp:649-668). The
// key -> field mapping follows SC_Calc_GENERIC::prepareData
// (sc_calc_generic.cpp:142-238). The --mcpval parser follows
// generateJsonKeyList and calculateFromChatbotKeyValList
// (Source/sc_mainCons.cpp:76-119, 858-900).

#include <cctype>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "cs_params_internal.h"

namespace cs {

// Combobox texts of guiLayoutNeu (sc_calc_generic.cpp:39-131); the position is
// the value. These strings are part of the key/value interface.
static const std::vector<std::string> kLType = {
    "Lamellae", "Hexagonally packed cylinders (P6/mm)", "Square packed cylinders (P4/mm)",
    "Rectangular centered cylinders (cmm)", "BCC (lm3m)", "FCC (Fm3m)", "HCP (P6/mmc)", "SC (Pm3m)", "BCT (l4/mm)",
    "Gyroid (Ia3d)", "OBDD (Pn3m)", "Plumbers Nightmare (Im3m)", "None", "CP-Layers", "2DHex (GISAXS)",
    "2DSquare (GISAXS)", "1DLam (GISAXS)", "Fd3m", "Orthorombic", "LDQ12"};
static const std::vector<std::string> kParticle = {
    "sphere", "cylinder", "disk", "vesicle", "cube", "ellipsoid", "triaxial ellipsoid", "super ellipsoid, barrel",
    "superball", "excluded volume chain", "Kratky Porod chain"};
static const std::vector<std::string> kOrdis = {
    "Gaussian", "Exponential", "Onsager", "Maier-Saupe", "Cut-off", "Laguerre", "z-dir", "isotropic",
    "mirrored Gaussian", "mirrored Exponential", "mirrored Onsager", "mirrored Maier-Saupe", "mirrored Cut-off",
    "fiber pattern"};
static const std::vector<std::string> kInterior = {"homogeneous", "core + homogeneous sh", "core + inhomogeneous sh",
                                                   "multi-shell", "myelin"};
static const std::vector<std::string> kPeak = {"Lorentzian", "Gaussian", "mod. 1 Lorentzian", "mod. 2 Lorentzian",
                                               "Pseudo-Voigt", "Pearson VII", "Gamma", "Anisotropic Gaussian"};

static int index_of(const std::vector<std::string> &v, const std::string &s) {
    for (size_t i = 0; i < v.size(); i++)
        if (v[i] == s) return (int)i;
    return -1;
}

void default_params(cs_params *p) {
    std::memset(p, 0, sizeof(*p));
    p->ltype = 12;  // "None"
    p->uca = p->ucb = p->ucc = 30;
    p->ucalpha = p->ucbeta = p->ucgamma = 90;
    p->ceff = 1;
    p->twinned = 0;
    p->ceffcyl = 0;
    p->reff = 0;
    p->acpl = p->bcpl = 0;
    p->ifluc = p->rfluc = 0;
    // The particle default "Sphere" is not in the (lower-case) combobox list,
    // so the console starts with index -1 and rejects a calculation until a
    // particle is set (QStringList::indexOf is case sensitive).
    p->particle = -1;
    p->ordis = 7;     // "isotropic"
    p->interior = 0;  // "homogeneous"
    p->radius = 1.0;
    p->radiusi = 0.5;
    p->sigma = 0.07;
    p->dbeta = 0.4;
    p->length = 1;
    p->sigmal = 0.06;
    p->alphash = 0;
    p->rho = 0;
    p->alpha = 0;
    p->peak = 1;  // "Gaussian"
    p->peakpar = 0;
    p->debyewaller = 2;
    p->azi = 180;
    p->domainsize = 400;
    p->debyescherrer = 0;
    p->para = 0;
    p->ax1[0] = 1; p->ax1[1] = 0; p->ax1[2] = 0;
    p->ax2[0] = 0; p->ax2[1] = 1; p->ax2[2] = 0;
    p->ax3[0] = 0; p->ax3[1] = 0; p->ax3[2] = 1;
    p->sigxyz[0] = p->sigxyz[1] = p->sigxyz[2] = 40;
    p->ucpsi = 0;
    p->ucn1 = p->ucn2 = p->ucn3 = 1;
    p->theta = 90;
    p->phi = 0;
    p->rottheta = 90;
    p->rotphi = 90;
    p->gridpoints = 64;
    p->hklmax = 5;
    p->qmax = 1;
    p->qmin = 0;
    p->radq1 = 0;
    p->radq2 = 0;
    p->radq4 = 1;
    p->expand = 0;
    p->use1d = 0;
    p->pixnox = p->pixnoy = 2048;
    p->pixx_mm = p->pixy_mm = 1;
    p->det = 1;
    p->wavelength = 0.09499;
    p->beamx = p->beamy = 0;
    p->usebeamstop = 0;
    p->bfactor = 1;
    p->waxs = 0;
    p->p1 = 0;
    p->iso = 0;
    p->izero = 10000;
    p->base = 0;
}

// Numeric assignment by reference key. Returns 1 when the key is known.
int set_param(cs_params *p, const char *key, double v) {
    const std::string k(key);
    // value.number of a select is converted to int by prepareData (v.select)
    auto sel = [&](int *f) { *f = (int)v; };
    auto flag = [&](int *f) { *f = (v != 0) ? 1 : 0; };
    auto pos = [&](int *f) { *f = (v > 0) ? 1 : 0; };
    if (k == "LType") sel(&p->ltype);
    else if (k == "uca") p->uca = v;
    else if (k == "ucb") p->ucb = v;
    else if (k == "ucc") p->ucc = v;
    else if (k == "ucalpha") p->ucalpha = v;
    else if (k == "ucbeta") p->ucbeta = v;
    else if (k == "ucgamma") p->ucgamma = v;
    else if (k == "EditCeff") p->ceff = v;
    else if (k == "CheckBoxTwinned") flag(&p->twinned);
    else if (k == "EditCeffcyl") p->ceffcyl = v;
    else if (k == "reff") p->reff = v;
    else if (k == "acpl") p->acpl = v;
    else if (k == "bcpl") p->bcpl = v;
    else if (k == "ifluc") p->ifluc = v;
    else if (k == "rfluc") p->rfluc = v;
    else if (k == "ComboBoxParticle") sel(&p->particle);
    else if (k == "Ordis") sel(&p->ordis);
    else if (k == "ComboBoxInterior") sel(&p->interior);
    else if (k == "EditRadius") p->radius = v;
    else if (k == "EditRadiusi") p->radiusi = v;
    else if (k == "EditSigma") p->sigma = v;
    else if (k == "EditDbeta") p->dbeta = v;
    else if (k == "Length") p->length = v;
    else if (k == "SigmaL") p->sigmal = v;
    else if (k == "Alpha") p->alphash = v;
    else if (k == "EditRho") p->rho = v;
    else if (k == "RotAlpha") p->alpha = v;
    else if (k == "ComboBoxPeak") sel(&p->peak);
    else if (k == "EditPeakPar") p->peakpar = v;
    else if (k == "EditDebyeWaller") p->debyewaller = v;
    else if (k == "EditAzi") p->azi = v;
    else if (k == "EditDomainSize") p->domainsize = v;
    else if (k == "RadButDebyeScherrer") flag(&p->debyescherrer);
    else if (k == "RadioButtonPara") flag(&p->para);
    else if (k == "EditAxis1x") p->ax1[0] = v;
    else if (k == "EditAxis1y") p->ax1[1] = v;
    else if (k == "EditAxis1z") p->ax1[2] = v;
    else if (k == "EditAxis2x") p->ax2[0] = v;
    else if (k == "EditAxis2y") p->ax2[1] = v;
    else if (k == "EditAxis2z") p->ax2[2] = v;
    else if (k == "EditAxis3x") p->ax3[0] = v;
    else if (k == "EditAxis3y") p->ax3[1] = v;
    else if (k == "EditAxis3z") p->ax3[2] = v;
    else if (k == "Editdom1") p->sigxyz[0] = v;
    else if (k == "Editdom2") p->sigxyz[1] = v;
    else if (k == "Editdom3") p->sigxyz[2] = v;
    else if (k == "ucpsi") p->ucpsi = v;
    else if (k == "ucn1") p->ucn1 = v;
    else if (k == "ucn2") p->ucn2 = v;
    else if (k == "ucn3") p->ucn3 = v;
    else if (k == "theta") p->theta = v;
    else if (k == "phi") p->phi = v;
    else if (k == "rotTheta") p->rottheta = v;
    else if (k == "rotPhi") p->rotphi = v;
    else if (k == "GridPoints") p->gridpoints = (int)v;
    else if (k == "HKLmax") p->hklmax = (int)v;
    else if (k == "EditQmax") p->qmax = v;
    else if (k == "EditQmin") p->qmin = v;
    else if (k == "RadioButtonQ1") pos(&p->radq1);
    else if (k == "RadioButtonQ2") pos(&p->radq2);
    else if (k == "RadioButtonQ4") pos(&p->radq4);
    else if (k == "ExpandImage") pos(&p->expand);
    else if (k == "EditPixelNoX") p->pixnox = v;
    else if (k == "EditPixelNoY") p->pixnoy = v;
    else if (k == "EditPixelX") p->pixx_mm = v;
    else if (k == "EditPixelY") p->pixy_mm = v;
    else if (k == "EditDet") p->det = v;
    else if (k == "EditWavelength") p->wavelength = v;
    else if (k == "BeamPosX") p->beamx = v;
    else if (k == "BeamPosY") p->beamy = v;
    else if (k == "CenterBeam") flag(&p->usebeamstop);
    else if (k == "EditBFactor") p->bfactor = v;
    else if (k == "CheckBoxWAXS") flag(&p->waxs);
    else if (k == "P1") p->p1 = v;
    else if (k == "iso") p->iso = v;
    else if (k == "I0") p->izero = v;
    else if (k == "Base") p->base = v;
    else return 0;
    return 1;
}

// Combobox assignment by text (SC_CalcCons::updateParamValue(QString,QString)).
// Returns 1 when key is a combobox (the value may be -1 for an unknown text).
int set_param_text(cs_params *p, const char *key, const char *text) {
    const std::string k(key), t(text);
    if (k == "LType") p->ltype = index_of(kLType, t);
    else if (k == "ComboBoxParticle") p->particle = index_of(kParticle, t);
    else if (k == "Ordis") p->ordis = index_of(kOrdis, t);
    else if (k == "ComboBoxInterior") p->interior = index_of(kInterior, t);
    else if (k == "ComboBoxPeak") p->peak = index_of(kPeak, t);
    else return 0;
    return 1;
}

// JSON key -> reference key of generateJsonKeyList (sc_mainCons.cpp:76-119):
// the reference key without its "Edit"/"CheckBox"/"RadBut" prefix, "ComboBox"
// -> "CB", "RadioButton" -> "RB", "VAx" -> "Ax", lower-cased. Keys that the
// console deliberately hides from the key/value interface are absent.
static const char *const kJsonKeys[][2] = {
    {"ltype", "LType"}, {"uca", "uca"}, {"ucb", "ucb"}, {"ucc", "ucc"}, {"ucalpha", "ucalpha"}, {"ucbeta", "ucbeta"},
    {"ucgamma", "ucgamma"}, {"ceff", "EditCeff"}, {"twinned", "CheckBoxTwinned"}, {"ceffcyl", "EditCeffcyl"},
    {"reff", "reff"}, {"acpl", "acpl"}, {"bcpl", "bcpl"}, {"ifluc", "ifluc"}, {"rfluc", "rfluc"},
    {"cbparticle", "ComboBoxParticle"}, {"ordis", "Ordis"}, {"cbinterior", "ComboBoxInterior"},
    {"radius", "EditRadius"}, {"radiusi", "EditRadiusi"}, {"sigma", "EditSigma"}, {"dbeta", "EditDbeta"},
    {"length", "Length"}, {"sigmal", "SigmaL"}, {"alpha", "Alpha"}, {"rho", "EditRho"}, {"rotalpha", "RotAlpha"},
    {"cbpeak", "ComboBoxPeak"}, {"peakpar", "EditPeakPar"}, {"debyewaller", "EditDebyeWaller"}, {"azi", "EditAzi"},
    {"domainsize", "EditDomainSize"}, {"debyescherrer", "RadButDebyeScherrer"}, {"rbpara", "RadioButtonPara"},
    {"ax1", "VAx1"}, {"ax2", "VAx2"}, {"ax3", "VAx3"}, {"ay1", "Ay1"}, {"ay2", "Ay2"}, {"ay3", "Ay3"},
    {"az1", "Az1"}, {"az2", "Az2"}, {"az3", "Az3"}, {"sigx", "SigX"}, {"sigy", "SigY"}, {"sigz", "SigZ"},
    {"ucpsi", "ucpsi"}, {"ucn1", "ucn1"}, {"ucn2", "ucn2"}, {"ucn3", "ucn3"}, {"theta", "theta"}, {"phi", "phi"},
    {"rottheta", "rotTheta"}, {"rotphi", "rotPhi"}, {"gridpoints", "GridPoints"}, {"hklmax", "HKLmax"},
    {"qmax", "EditQmax"}, {"pixelnox", "EditPixelNoX"}, {"pixelnoy", "EditPixelNoY"}, {"pixelx", "EditPixelX"},
    {"pixely", "EditPixelY"}, {"det", "EditDet"}, {"wavelength", "EditWavelength"}, {"beamposx", "BeamPosX"},
    {"beamposy", "BeamPosY"}, {"iso", "iso"}, {"i0", "I0"}, {"base", "Base"},
};

const char *json_to_ref_key(const char *json) {
    for (auto &e : kJsonKeys)
        if (!std::strcmp(e[0], json)) return e[1];
    return nullptr;
}

static std::string trim(const std::string &s) {
    size_t a = 0, b = s.size();
    while (a < b && std::isspace((unsigned char)s[a])) a++;
    while (b > a && std::isspace((unsigned char)s[b - 1])) b--;
    return s.substr(a, b - a);
}

// QString::toDouble: the whole (trimmed) string must be a number, else 0.
static double qt_to_double(const std::string &s) {
    const std::string t = trim(s);
    if (t.empty()) return 0.0;
    char *end = nullptr;
    double v = std::strtod(t.c_str(), &end);
    if (end == t.c_str() || *end != '\0') return 0.0;
    return v;
}

// calculateFromChatbotKeyValList (sc_mainCons.cpp:858-900). Returns the number
// of entries applied; unknown keys are skipped like the console does.
int apply_kv(cs_params *p, const char *kv) {
    int applied = 0;
    std::string s(kv ? kv : "");
    size_t start = 0;
    while (start <= s.size()) {
        size_t semi = s.find(';', start);
        std::string item = s.substr(start, semi == std::string::npos ? std::string::npos : semi - start);
        start = (semi == std::string::npos) ? s.size() + 1 : semi + 1;
        if (item.empty()) continue;
        size_t eq = item.find('=');
        if (eq == std::string::npos) continue;
        const std::string key = item.substr(0, eq);
        const std::string val = trim(item.substr(eq + 1));
        const char *ref = json_to_ref_key(key.c_str());
        if (!ref || val.empty()) continue;  // unknown key ("?") or empty value: no change
        const unsigned char c0 = (unsigned char)val[0];
        if (std::isdigit(c0) || c0 == '-' || c0 == '+') {
            applied += set_param(p, ref, qt_to_double(val));
        } else if (c0 == 'F' || c0 == 'T') {
            // booleans; note that a combobox text starting with 'F' or 'T'
            // (e.g. "FCC (Fm3m)") lands here too, exactly like the console
            applied += set_param(p, ref, c0 == 'T' ? 1.0 : 0.0);
        } else if (val == "NULL") {
            continue;
        } else {
            applied += set_param_text(p, ref, val.c_str());
        }
    }
    return applied;
}

}  // namespace cs
