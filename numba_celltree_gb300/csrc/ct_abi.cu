// ct_abi.cu -- error reporting and version entry points of the C ABI.
#include <cstdio>
#include <cstring>

#include "ct_internal.h"

static thread_local char g_msg[512] = "";

int ct_fail(int status, const char* msg) {
    snprintf(g_msg, sizeof(g_msg), "%s", msg ? msg : "");
    return status;
}

extern "C" {

int ct_abi_version(void) { return CT_ABI_VERSION; }

const char* ct_last_error_message(void) { return g_msg; }

int ct_host_register(void* ptr, size_t bytes, int32_t read_only) {
    if (!ptr || bytes == 0) return ct_fail(CT_ERR_ARG, "nothing to register");
    unsigned flags = read_only ? cudaHostRegisterReadOnly : cudaHostRegisterDefault;
    cudaError_t e = cudaHostRegister(ptr, bytes, flags);
    if (e != cudaSuccess) {
        (void)cudaGetLastError();  // not sticky: clear it so that later launch checks do not see it
        return ct_fail(CT_ERR_CUDA, cudaGetErrorString(e));
    }
    return CT_OK;
}

int ct_host_unregister(void* ptr) {
    cudaError_t e = cudaHostUnregister(ptr);
    if (e != cudaSuccess) {
        (void)cudaGetLastError();
        return ct_fail(CT_ERR_CUDA, cudaGetErrorString(e));
    }
    return CT_OK;
}

}  // extern "C"
