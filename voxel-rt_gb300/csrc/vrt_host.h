// Internal declarations of the host-only sources (host.cpp, terrain.cpp), which build
// without CUDA headers.
#pragma once

#include "../../include/vrt.h"

namespace vrt {
// Record a message for vrt_last_error() and return status.
int set_error(int status, const char* fmt, ...);
}  // namespace vrt
