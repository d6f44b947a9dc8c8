// Thread-local last-error message behind ma_last_error().
#pragma once
#include <string>

#include "../../../include/miniaero_gpu.h"

namespace miniaero {
ma_status set_error(ma_status s, const std::string& msg);
const char* last_error();
}  // namespace miniaero
