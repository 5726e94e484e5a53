// spk_error.h - per-thread message for spk_last_error().
#pragma once

namespace spk {
void set_error(const char* fmt, ...);
}  // namespace spk
