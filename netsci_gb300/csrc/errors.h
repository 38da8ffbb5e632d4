// Host-side error plumbing shared by every translation unit of the library.
#pragma once

#include <cuda_runtime.h>

#include <stdexcept>
#include <string>

#include "netsci_gb300.h"

namespace nsg {

// Thrown inside the library; the C ABI maps it to a status code plus a
// thread-local message (nsg_last_error()).
struct Error : std::runtime_error {
    int status;
    Error(int s, const std::string& m) : std::runtime_error(m), status(s) {}
};

[[noreturn]] inline void fail(int status, const std::string& msg) { throw Error(status, msg); }
[[noreturn]] inline void invalid(const std::string& msg) { throw Error(NSG_ERR_INVALID, msg); }
[[noreturn]] inline void io_fail(const std::string& msg) { throw Error(NSG_ERR_IO, msg); }

inline void cuda_check(cudaError_t e, const char* what) {
    if (e != cudaSuccess) {
        fail(NSG_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
    }
}

#define NSG_CUDA(call) ::nsg::cuda_check((call), #call)

// Device error flags written by kernels (bounded waits that ran out).
enum DeviceFault : int {
    FAULT_NONE = 0,
    FAULT_WAIT_TIMEOUT = 1,
    FAULT_BAD_INDEX = 2,
};

}  // namespace nsg
