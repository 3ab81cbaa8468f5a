// Shared helpers for the mgcfd_gb300 library: status/error reporting and the
// physical constants of the reference (const.h:27-51).
#pragma once

#include <string>

#include "mgcfd_gb300.h"

namespace mgcfd {

constexpr double kGamma = 1.4;   // const.h:27
constexpr int kRK = 3;           // const.h:31
constexpr int kNVar = 5;         // const.h:38-41: [rho, rho*u, rho*v, rho*w, rho*E]

// Records `msg` as the calling thread's last error and returns `status`.
int set_error(int status, const std::string& msg);
void clear_error();

// Skips counted by mgcfd_op_restrict_noalloc (restrict_noalloc.cu), which
// mgcfd_op_map_errors adds to the other entry points' count.
int restrict_noalloc_map_errors(unsigned long long* count, bool reset);

}  // namespace mgcfd
