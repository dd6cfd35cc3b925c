// Error reporting and version of the C ABI.
#include "common.cuh"
#include <string>

namespace ngb {

static thread_local std::string t_last_error;

void set_error(const char* fmt, ...)
{
    char    buf[1024];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    t_last_error = buf;
}

void clear_error() { t_last_error.clear(); }

}  // namespace ngb

extern "C" {

const char* ngb_last_error(void) { return ngb::t_last_error.c_str(); }

int ngb_version(void) { return 1; }

}  // extern "C"
