// pimc_internal.h -- shared by the library's translation units, not part of
// the C ABI.
#pragma once
#include <string>

// records msg as the calling thread's pimc_last_error() text; returns code
int pimc_fail(int code, const std::string &msg);
