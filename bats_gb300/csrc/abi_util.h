// Status handling shared by the C-ABI entry points.
#pragma once
#include <cuda_runtime.h>
#include "../../include/bats_gb300.h"

namespace bats {
void set_last_error(int status, const char* where, const char* what);
int max_dynamic_smem_set(const void* func, int bytes);
// Device address of this device's status word (bounded waits that gave up OR their flag into it).
int device_status(int** out);
struct SolveConst;
SolveConst make_solve_const(float c, float dtt, float tau, float max_sim);
}  // namespace bats

#define BATS_REQUIRE(cond, status, msg)                        \
    do {                                                       \
        if (!(cond)) {                                         \
            bats::set_last_error((status), __func__, (msg));   \
            return (status);                                   \
        }                                                      \
    } while (0)

#define BATS_CUDA(expr)                                                           \
    do {                                                                          \
        cudaError_t _e = (expr);                                                  \
        if (_e != cudaSuccess) {                                                  \
            bats::set_last_error(BATS_ERR_CUDA, __func__, cudaGetErrorString(_e)); \
            return BATS_ERR_CUDA;                                                 \
        }                                                                         \
    } while (0)
