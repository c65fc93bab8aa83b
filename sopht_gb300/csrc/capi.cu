// Error reporting and version of the C ABI.
#include <cstdarg>
#include <cstdio>

#include "common.cuh"

namespace sg {

static thread_local char g_last_error[1024] = "";

void set_last_error(const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_last_error, sizeof(g_last_error), fmt, ap);
    va_end(ap);
}

}  // namespace sg

extern "C" const char* sg_last_error(void) { return sg::g_last_error; }

extern "C" int sg_version(void) { return 100; }
