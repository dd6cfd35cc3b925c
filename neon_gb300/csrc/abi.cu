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

size_t ngb_abi_struct_size(int32_t which)
{
    switch (which) {
        case 0: return sizeof(ngb_lbm_dense_desc);
        case 1: return sizeof(ngb_bgrid_desc);
        case 2: return sizeof(ngb_poisson_desc);
        case 3: return sizeof(ngb_cg_params);
        case 4: return sizeof(ngb_cg_result);
        case 5: return sizeof(ngb_learned_params);
        case 6: return sizeof(ngb_learned_result);
        default: return 0;
    }
}

}  // extern "C"
