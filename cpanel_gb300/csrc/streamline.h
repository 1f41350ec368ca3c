// Lockstep Runge-Kutta-Fehlberg 4(5) streamlines (streamline::streamline / rkf,
// CPanel/streamline.cpp:20-78); the arguments are those of cpg_streamlines_field.
#pragma once
#include <cstdint>

#include "../../include/cpanel_gpu.h"

namespace cpg {
int streamlines_rkf45(cpg_velocity_fn fn, void* user, double speed, const double* starts, int n_lines, double x_max,
                      double tol, int max_points, double* pts, double* vel, int32_t* counts, int32_t* ended);
}
