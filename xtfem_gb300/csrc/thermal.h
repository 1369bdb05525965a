// thermal.h -- what the mechanical slab loop needs of a thermal slab loop
// when the two are coupled.
#pragma once

#include "../../include/xtfem_gb300_host.h"

namespace xt {

// One thermal slab (as xt_thermal_step).
int thermal_advance(xt_thermal_s& t, double* stats);
// The last slab's nodal temperatures on the device, interleaved (nn x 3),
// on the thermal loop's stream, complete when thermal_advance returns.
const double* thermal_temperature(const xt_thermal_s& t);
int thermal_nodes(const xt_thermal_s& t);

}  // namespace xt
