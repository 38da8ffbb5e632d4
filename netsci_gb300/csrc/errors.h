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
        cudaGetLastError();  // a failed call also leaves its error pending; clear it
        fail(NSG_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
    }
}

#define NSG_CUDA(call) ::nsg::cuda_check((call), #call)

// Device error flags written by kernels (bounded waits that ran out).
enum DeviceFault : int {
    FAULT_NONE = 0,
    FAULT_WAIT_TIMEOUT = 1,
    FAULT_BAD_INDEX = 2,
    FAULT_TIE_OVERFLOW = 4,     // more tied samples than the tie list holds (lists are
                                // sized for every sample: a broken invariant)
    FAULT_TIE_UNRESOLVED = 8,   // the sort-order replay met a broken invariant
};

// Throws NSG_ERR_DEVICE_FAULT describing a non-zero device fault word.
inline void raise_fault(int f) {
    if (!f) return;
    std::string m = "device fault:";
    if (f & FAULT_WAIT_TIMEOUT) m += " a bounded wait ran out;";
    if (f & FAULT_BAD_INDEX) m += " a frame map entry is outside [0, ld);";
    if (f & FAULT_TIE_OVERFLOW) m += " more tied samples than the tie list holds;";
    if (f & FAULT_TIE_UNRESOLVED) m += " a tied sample's sort replay met a broken invariant;";
    fail(NSG_ERR_DEVICE_FAULT, m);
}

}  // namespace nsg
