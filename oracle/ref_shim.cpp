// C-linkage entry points into the reference's own HWE and incomplete-gamma code, compiled
// from the reference checkout into oracle/_ref/.  Oracle build only.
#include <cstdint>
#include "snphwe.h"
#include "gamma_inc.h"

extern "C" double ref_SNPHWE2(int32_t hets, int32_t hom1, int32_t hom2, uint32_t midp)
{
  return SNPHWE2(hets, hom1, hom2, midp);
}

extern "C" double ref_kf_gammaq(double s, double z) { return (double)kf_gammaq(s, z); }
