// Status plumbing and library-level queries for the C ABI.
#include "dpl_common.cuh"

namespace dpl {

static thread_local std::string g_last_error;

void set_error(const std::string& msg) { g_last_error = msg; }

dpl_status fail(dpl_status st, const std::string& msg) {
    g_last_error = msg;
    return st;
}

dpl_status check_launch(const char* what) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(DPL_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
    return DPL_OK;
}

}  // namespace dpl

extern "C" const char* dpl_last_error_message(void) { return dpl::g_last_error.c_str(); }

extern "C" int dpl_version(void) { return 1000; }

extern "C" int dpl_max_nslc(void) { return dpl::kMaxNslc; }
