// cs_params_internal.h — parameter defaults and key mapping (internal).
#ifndef CS_PARAMS_INTERNAL_H
#define CS_PARAMS_INTERNAL_H

#include "../../include/crystalscatter.h"

namespace cs {

void default_params(cs_params *p);
int set_param(cs_params *p, const char *key, double v);
int set_param_text(cs_params *p, const char *key, const char *text);
const char *json_to_ref_key(const char *json);
int apply_kv(cs_params *p, const char *kv);

}  // namespace cs

#endif
