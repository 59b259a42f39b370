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

// Every kernel of the library is launched through bats::launch and starts with pdl_prologue (device side):
// it allows its dependents to launch, then waits for the grids it depends on. With BATS_GB300_PDL=1 in the
// environment, launches carry programmatic stream serialization, so the next kernel's CTAs become resident
// while the current kernel's last CTAs finish, and wait there (they read nothing before the wait returns,
// when the prerequisite grids have completed and their memory is visible). Off by default: measured on a
// GB300 it gained 1.3 % on the literal train step (26 kernels then) but cost the serving loop 30 % of its median
// latency (the waiting CTAs hold SM slots that concurrent lanes' kernels need) and the conv step 5 %.
// Without the attribute the prologue's two instructions are no-ops.
bool pdl_enabled();
// Launch attribute list for cudaLaunchKernelEx: the programmatic-serialization attribute when enabled.
int pdl_attribute(cudaLaunchAttribute* attr);

template <typename... KArgs, typename... Args>
cudaError_t launch(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t stream,
                   Args&&... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = stream;
    cudaLaunchAttribute attr[1];
    cfg.attrs = attr;
    cfg.numAttrs = (unsigned)pdl_attribute(attr);
    return cudaLaunchKernelEx(&cfg, kernel, static_cast<KArgs>(args)...);
}
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
