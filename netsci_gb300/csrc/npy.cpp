#include "npy.h"

#include <cstdint>
#include <cstdio>
#include <cstring>
#include <memory>

#include "netsci_gb300.h"
#include "errors.h"

namespace nsg {

size_t NpyArray::word_size() const {
    if (descr.size() < 3) return 0;
    return static_cast<size_t>(std::stoul(descr.substr(2)));
}

size_t NpyArray::count() const {
    size_t c = 1;
    for (size_t s : shape) c *= s;
    return c;
}

template <>
const char* npy_descr<float>() { return "<f4"; }
template <>
const char* npy_descr<double>() { return "<f8"; }
template <>
const char* npy_descr<int>() { return "<i4"; }

namespace {

struct FileCloser {
    void operator()(FILE* f) const { if (f) std::fclose(f); }
};
using FilePtr = std::unique_ptr<FILE, FileCloser>;

std::string dict_value(const std::string& header, const std::string& key) {
    size_t p = header.find("'" + key + "'");
    if (p == std::string::npos) io_fail("npy header lacks " + key);
    p = header.find(':', p);
    if (p == std::string::npos) io_fail("malformed npy header");
    ++p;
    while (p < header.size() && header[p] == ' ') ++p;
    if (p >= header.size()) io_fail("malformed npy header");
    size_t e;
    if (header[p] == '\'') {
        e = header.find('\'', p + 1);
        return header.substr(p + 1, e - p - 1);
    }
    if (header[p] == '(') {
        e = header.find(')', p);
        return header.substr(p, e - p + 1);
    }
    e = header.find_first_of(",}", p);
    return header.substr(p, e - p);
}

}  // namespace

NpyArray npy_read(const std::string& path) {
    FilePtr f(std::fopen(path.c_str(), "rb"));
    if (!f) io_fail("cannot open " + path);
    unsigned char magic[8];
    if (std::fread(magic, 1, 8, f.get()) != 8 || std::memcmp(magic, "\x93NUMPY", 6) != 0) {
        io_fail(path + " is not a .npy file");
    }
    size_t hlen = 0;
    if (magic[6] == 1) {
        unsigned char b[2];
        if (std::fread(b, 1, 2, f.get()) != 2) io_fail("truncated npy header");
        hlen = b[0] | (b[1] << 8);
    } else {
        unsigned char b[4];
        if (std::fread(b, 1, 4, f.get()) != 4) io_fail("truncated npy header");
        hlen = b[0] | (b[1] << 8) | (b[2] << 16) | (static_cast<size_t>(b[3]) << 24);
    }
    std::string header(hlen, '\0');
    if (std::fread(&header[0], 1, hlen, f.get()) != hlen) io_fail("truncated npy header");
    NpyArray a;
    a.descr = dict_value(header, "descr");
    if (dict_value(header, "fortran_order").find("True") != std::string::npos) {
        io_fail("Fortran-order .npy files are not supported");
    }
    std::string shp = dict_value(header, "shape");
    for (size_t i = 0; i < shp.size();) {
        if (shp[i] >= '0' && shp[i] <= '9') {
            size_t e = i;
            while (e < shp.size() && shp[e] >= '0' && shp[e] <= '9') ++e;
            a.shape.push_back(static_cast<size_t>(std::stoull(shp.substr(i, e - i))));
            i = e;
        } else {
            ++i;
        }
    }
    if (a.descr.size() < 3 || (a.descr[0] != '<' && a.descr[0] != '|')) {
        io_fail("unsupported npy dtype " + a.descr);
    }
    const size_t bytes = a.count() * a.word_size();
    a.data.resize(bytes);
    if (bytes && std::fread(a.data.data(), 1, bytes, f.get()) != bytes) {
        io_fail("truncated npy payload in " + path);
    }
    return a;
}

void npy_write(const std::string& path, const void* data, const std::string& descr,
               size_t word_size, const std::vector<size_t>& shape) {
    std::string dict = "{'descr': '" + descr + "', 'fortran_order': False, 'shape': (";
    size_t count = 1;
    for (size_t i = 0; i < shape.size(); ++i) {
        dict += std::to_string(shape[i]);
        if (shape.size() == 1 || i + 1 < shape.size()) dict += ",";
        if (i + 1 < shape.size()) dict += " ";
        count *= shape[i];
    }
    dict += "), }";
    // pad so that magic(6) + version(2) + len(2) + dict + '\n' is a multiple
    // of 16: the header length the reference's files carry (cnpy), so that
    // checkpoint files are byte-identical to the reference's
    size_t total = 10 + dict.size() + 1;
    dict.append((16 - total % 16) % 16, ' ');
    dict += '\n';
    FilePtr f(std::fopen(path.c_str(), "wb"));
    if (!f) io_fail("cannot write " + path);
    const unsigned char pre[8] = {0x93, 'N', 'U', 'M', 'P', 'Y', 1, 0};
    const uint16_t hl = static_cast<uint16_t>(dict.size());
    const unsigned char hlb[2] = {static_cast<unsigned char>(hl & 0xff),
                                  static_cast<unsigned char>(hl >> 8)};
    bool ok = std::fwrite(pre, 1, 8, f.get()) == 8 && std::fwrite(hlb, 1, 2, f.get()) == 2 &&
              std::fwrite(dict.data(), 1, dict.size(), f.get()) == dict.size();
    const size_t bytes = count * word_size;
    if (ok && bytes) ok = std::fwrite(data, 1, bytes, f.get()) == bytes;
    if (!ok) io_fail("short write to " + path);
}

}  // namespace nsg
