// Internal helpers shared by the engine's translation units.
#pragma once

namespace fpgm {
// Records a printf-style message as the calling thread's last error and returns code.
int set_error(int code, const char *fmt, ...);
}  // namespace fpgm
