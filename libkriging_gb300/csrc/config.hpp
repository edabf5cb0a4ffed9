// config.hpp -- process-global numerical and optimiser settings, same names, defaults and environment variables
// as libKriging's statics:
//   LinearAlgebra::{num_nugget, chol_rcond_check, min_rcond, max_inc_choldiag, warn_chol}
//       (src/lib/LinearAlgebra.cpp:33-63, :100)
//   Optim::{reparametrize, theta_lower_factor, theta_upper_factor, variogram_bounds_heuristic, log_level,
//           max_restart, max_iteration, gradient_tolerance, objective_rel_tolerance}  (src/lib/Optim.cpp:39-139)
#pragma once

namespace lkg {

struct Config {
  // LinearAlgebra
  double num_nugget = 1e-10;
  bool chol_rcond_check = true;
  double min_rcond = 1e-18;
  int max_inc_choldiag = 10;
  bool warn_chol = false;
  // Optim
  bool reparametrize = true;
  double theta_lower_factor = 0.02;
  double theta_upper_factor = 10.0;
  bool variogram_bounds_heuristic = true;
  int log_level = 0;
  int max_restart = 10;
  int max_iteration = 20;
  double gradient_tolerance = 0.001;
  double objective_rel_tolerance = 0.001;
};

// The single process-wide instance; initialised from the LK_* environment variables on first use.
Config& config();

}  // namespace lkg
