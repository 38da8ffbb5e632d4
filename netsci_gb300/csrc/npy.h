// Minimal .npy (format 1.0/2.0) reader and writer for little-endian
// C-order arrays of float32, float64 and int32: what CuArray load/save and
// the checkpoint files need (the reference uses the vendored cnpy library
// for this, cnpy/include/cnpy.h:73-221).
#pragma once

#include <cstddef>
#include <string>
#include <vector>

namespace nsg {

struct NpyArray {
    std::string descr;                // e.g. "<f4"
    std::vector<size_t> shape;
    std::vector<unsigned char> data;  // raw little-endian payload
    size_t word_size() const;
    size_t count() const;
};

// Throws nsg::Error(NSG_ERR_IO, ...) on failure.
NpyArray npy_read(const std::string& path);
void npy_write(const std::string& path, const void* data, const std::string& descr,
               size_t word_size, const std::vector<size_t>& shape);

template <typename T>
const char* npy_descr();

}  // namespace nsg
