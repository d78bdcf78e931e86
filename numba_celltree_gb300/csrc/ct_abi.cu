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

}  // extern "C"
