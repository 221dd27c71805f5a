// host_errors.h -- the library's error channel for host-only translation units: records the
// message that sayram_last_error() returns and passes the status code through.
#pragma once

#include <string>

namespace sg {
int host_fail(int code, const std::string& msg);
}
