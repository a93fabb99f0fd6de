// cs_prep.h — host preparation entry points (internal to the library).
#ifndef CS_PREP_H
#define CS_PREP_H

#include <string>

#include "../../include/crystalscatter.h"
#include "cs_prepared.h"

namespace cs {

// checkAllParameters(ignCbs), Source/sc_calc_generic_cpu.cpp:198-308; shp is
// the peak code (combobox index + 1). Empty string = accepted.
std::string check_all_parameters(const cs_params &in, int shp, int ign_cbs);

// prepareCalculation, Source/sc_calc_generic_cpu.cpp:319-988. calc_quadrants
// (CS_RADQ1/2/4) and expand carry the reference's stateful quadrant setters.
// Returns CS_OK, CS_ERR_PARAM (message = reference text) or CS_ERR_UNSUPPORTED.
// check = 0 skips checkAllParameters like doFitCalculation does.
int prepare(const cs_params &in, int calc_quadrants, int expand, int ign_new_switch, int ign_cbs, int check,
            cs_prepared *out, std::string &err);

// Threads the calling thread uses for the per-n loops of the coefficient
// preparation (0: up to 8 hardware threads; 1: serial, e.g. inside a thread
// that prepares one of many sets).
void set_prep_threads(int n);

// The reference's own Gamma function (Source/sc_calc_generic_gpu.cu:613-673),
// evaluated on the host where pixel kernels need pixel-independent ratios.
double ref_gamma(double z);

}  // namespace cs

#endif
