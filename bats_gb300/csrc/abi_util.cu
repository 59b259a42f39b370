// Error reporting and per-device launch attributes shared by the C-ABI entry points.
#include <cstdio>
#include <cstring>
#include "abi_util.h"

namespace bats {

static thread_local char g_last_error[512] = "";

void set_last_error(int status, const char* where, const char* what) {
    std::snprintf(g_last_error, sizeof(g_last_error), "%s: %s (status %d)", where, what, status);
}

// cudaFuncSetAttribute(MaxDynamicSharedMemorySize) once per (kernel, device). Returns a cudaError_t.
int max_dynamic_smem_set(const void* func, int bytes) {
    if (bytes <= 48 * 1024) return (int)cudaSuccess;
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

}  // namespace bats

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
