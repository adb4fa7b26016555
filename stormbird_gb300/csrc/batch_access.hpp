// Internal access to the cases of a batch (batch_host.cu), for the CompleteSailModel sweeps
// (csm_host.cu), which run one steady-state condition per case of a batch. Not part of the
// C ABI. Errors are raised as SbFail, like the rest of the host code.
#pragma once

#include <cstddef>

#include "sim_core.hpp"

struct sb_batch;

namespace sbhost {

size_t batch_case_count(const sb_batch* b);
sb_sim* batch_case(sb_batch* b, size_t i);
long long batch_line_offset(const sb_batch* b, size_t i);
// Controller flow measurements of every case for (time, ship velocity of each case): case i's
// lines at 3 * line offset: |u| [N], angle of attack [N], apparent wind direction [N].
const double* batch_controller_inputs(sb_batch* b, double time, const double* ship_velocities);
// Per case: its integrated forces [S][6][3] then its integrated moments [S][6][3] (component
// 5 = total) after the last step, case after case.
const double* batch_wing_totals(sb_batch* b);

}  // namespace sbhost
