// gm_internal.h -- shared host-side helpers of the library (not part of the ABI).
#pragma once

#include <string>

#include "glemur.h"

namespace gm {

// Record a message for gm_last_error() and return the code.
int fail(int code, const std::string& msg);

}  // namespace gm
