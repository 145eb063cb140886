// The adjoint engine's entry for other parts of the library.
#pragma once

#include <cstddef>

#include "../../include/scafes_gb300.h"

namespace scafes {

// scafes_adj_backward with the initial iterate already on the device
// (u0_dev: FP64 in the padded layout of make_layout for the handle's grid).
int adj_backward_device_u0(scafes_adj* a, const double* u0_dev, const double* dJ_duT, int n_steps, double* grad_k,
                           double* grad_u0, size_t n);

}  // namespace scafes
