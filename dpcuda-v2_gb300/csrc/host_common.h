// host_common.h -- error reporting and launch helpers shared by the host-side
// translation units of the library.
#pragma once
#include <cuda_runtime.h>

#include "../../include/dpg.h"

namespace dpg {
// Records a message for dpg_last_error() (thread-local) and returns `code`.
int set_error(int code, const char *fmt, ...);
}  // namespace dpg

#define DPG_CK(x)                                                                          \
    do {                                                                                   \
        cudaError_t e_ = (x);                                                              \
        if (e_ != cudaSuccess)                                                             \
            return ::dpg::set_error(DPG_ERR_CUDA, "%s:%d %s: %s", __FILE__, __LINE__, #x,  \
                                    cudaGetErrorString(e_));                               \
    } while (0)

#define DPG_TRY(x)                   \
    do {                             \
        int r_ = (x);                \
        if (r_ != DPG_OK) return r_; \
    } while (0)
