// Error reporting and per-device launch attributes shared by the C-ABI entry points.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include "abi_util.h"

namespace bats {

static thread_local char g_last_error[512] = "";

void set_last_error(int status, const char* where, const char* what) {
    std::snprintf(g_last_error, sizeof(g_last_error), "%s: %s (status %d)", where, what, status);
}

// cudaFuncSetAttribute(MaxDynamicSharedMemorySize) once per (kernel, device), for any dynamic size: a kernel's
// static shared memory counts toward the 48 KB that needs no opt-in. Returns a cudaError_t.
int max_dynamic_smem_set(const void* func, int bytes) {
    if (bytes <= 0) return (int)cudaSuccess;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return (int)e;
    struct Entry {
        const void* f;
        int dev;
        int bytes;
    };
    static thread_local Entry cache[64];
    static thread_local int used = 0;
    for (int q = 0; q < used; ++q)
        if (cache[q].f == func && cache[q].dev == dev && cache[q].bytes >= bytes) return (int)cudaSuccess;
    e = cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    if (e != cudaSuccess) return (int)e;
    if (used < 64) cache[used++] = Entry{func, dev, bytes};
    return (int)cudaSuccess;
}

bool pdl_enabled() {
    static const bool on = [] {
        const char* v = std::getenv("BATS_GB300_PDL");
        return v && v[0] == '1' && v[1] == '\0';
    }();
    return on;
}

int pdl_attribute(cudaLaunchAttribute* attr) {
    if (!pdl_enabled()) return 0;
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    return 1;
}

// Status word of bounded device-side waits: a kernel that gives up waiting ORs BATS_STATUS_TIMEOUT
// (1) into it and returns; bats_read_device_status reports and clears it.
static __device__ int g_device_status;

int device_status(int** out) {
    static std::mutex mu;
    static int* cache[128] = {nullptr};
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return (int)e;
    if (dev < 0 || dev >= 128) return (int)cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(mu);
    if (!cache[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_device_status);
        if (e != cudaSuccess) return (int)e;
        cache[dev] = reinterpret_cast<int*>(p);
    }
    *out = cache[dev];
    return (int)cudaSuccess;
}

}  // namespace bats

extern "C" int bats_read_device_status(int* out, int clear) {
    BATS_REQUIRE(out, BATS_ERR_NULL, "read_device_status: null pointer");
    BATS_CUDA(cudaMemcpyFromSymbol(out, bats::g_device_status, sizeof(int)));
    if (clear) {
        const int zero = 0;
        BATS_CUDA(cudaMemcpyToSymbol(bats::g_device_status, &zero, sizeof(int)));
    }
    if (*out != 0) {
        bats::set_last_error(BATS_ERR_TIMEOUT, "read_device_status", "a device-side wait gave up (timeout)");
        return BATS_ERR_TIMEOUT;
    }
    return BATS_OK;
}

extern "C" const char* bats_last_error(void) { return bats::g_last_error; }

extern "C" const char* bats_status_string(int status) {
    switch (status) {
        case BATS_OK: return "ok";
        case BATS_ERR_BAD_SHAPE: return "bad shape or argument";
        case BATS_ERR_NULL: return "null pointer";
        case BATS_ERR_CAPACITY: return "capacity exceeded";
        case BATS_ERR_WORKSPACE: return "workspace too small";
        case BATS_ERR_CUDA: return "CUDA error";
        case BATS_ERR_TIMEOUT: return "device wait timed out";
        default: return "unknown status";
    }
}

extern "C" int bats_abi_version(void) { return BATS_ABI_VERSION; }
