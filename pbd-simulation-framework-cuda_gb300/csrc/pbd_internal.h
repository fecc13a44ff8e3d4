// pbd_internal.h -- helpers shared by the translation units of libpbd (not installed).
#pragma once
#include <string>

namespace pbd {
// Thread-local text returned by pbd_last_error().
void set_error(const std::string& msg);
void clear_error();
}  // namespace pbd
