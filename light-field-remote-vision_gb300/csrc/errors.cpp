// errors.cpp -- thread-local error messages behind lfrv_last_error().
#include "lfrv_internal.h"

#include <cstring>

namespace {
thread_local char g_last_error[1024] = "";
}

namespace lfrv {

int fail(int status, const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    std::vsnprintf(g_last_error, sizeof(g_last_error), fmt, ap);
    va_end(ap);
    return status;
}

void raise(int status, const char *fmt, ...) {
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    std::vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    throw Error{status, std::string(buf)};
}

}  // namespace lfrv

extern "C" const char *lfrv_last_error(void) { return g_last_error; }

extern "C" const char *lfrv_version(void) { return "lfrv-gb300 0.1 (sm_103a)"; }
