// errors.cpp -- thread-local error message behind cnncrf_last_error().
// The reference printed and called exit(-1) (stereo/error_util.h:29-52);
// here every failure returns a status and leaves its message here.
#include <cstdio>

#include "common.h"

namespace cnncrf {

static thread_local std::string g_last_error;

int fail(int status, const char *fmt, ...)
{
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_last_error = buf;
    return status;
}

void clear_error() { g_last_error.clear(); }

} // namespace cnncrf

extern "C" const char *cnncrf_last_error(void) { return cnncrf::g_last_error.c_str(); }
extern "C" int cnncrf_abi_version(void) { return CNNCRF_ABI_VERSION; }
