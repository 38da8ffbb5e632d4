// DCD reader: header parsing, frame geometry, raw frame reads with pread.
#include "dcd.h"

#include <fcntl.h>
#include <sys/stat.h>
#include <unistd.h>

#include <cerrno>
#include <cstring>
#include <vector>

#include "errors.h"

namespace nsg {
namespace {

uint32_t bswap32(uint32_t v) {
    return (v >> 24) | ((v >> 8) & 0xff00u) | ((v << 8) & 0xff0000u) | (v << 24);
}

uint64_t bswap64(uint64_t v) {
    return (static_cast<uint64_t>(bswap32(static_cast<uint32_t>(v))) << 32) |
           bswap32(static_cast<uint32_t>(v >> 32));
}

uint32_t load32(const unsigned char* p, bool swap) {
    uint32_t v;
    std::memcpy(&v, p, 4);
    return swap ? bswap32(v) : v;
}

// A record marker at p (4 or 8 bytes) as a byte count.
int64_t load_marker(const unsigned char* p, int width, bool swap) {
    if (width == 4) return static_cast<int32_t>(load32(p, swap));
    uint64_t v;
    std::memcpy(&v, p, 8);
    if (swap) v = bswap64(v);
    return static_cast<int64_t>(v);
}

const uint32_t kCord = static_cast<uint32_t>('C') | (static_cast<uint32_t>('O') << 8) |
                       (static_cast<uint32_t>('R') << 16) | (static_cast<uint32_t>('D') << 24);

}  // namespace

DcdFile::DcdFile(const std::string& path) : path_(path) {
    fd_ = ::open(path.c_str(), O_RDONLY);
    if (fd_ < 0) io_fail("cannot open DCD file '" + path + "': " + std::strerror(errno));
    struct stat st;
    if (::fstat(fd_, &st) != 0) {
        ::close(fd_);
        io_fail("cannot stat DCD file '" + path + "'");
    }
    const int64_t fsize = st.st_size;
    // The header is at most a few KB (titles are capped at 1000 x 80).
    std::vector<unsigned char> h(static_cast<size_t>(std::min<int64_t>(fsize, 1 << 17)));
    const ssize_t got = ::pread(fd_, h.data(), h.size(), 0);
    auto bad = [&](const std::string& why) {
        ::close(fd_);
        fd_ = -1;
        io_fail("DCD file '" + path + "': " + why);
    };
    if (got < 0 || static_cast<size_t>(got) != h.size()) bad("read error");
    if (h.size() < 8 + 84) bad("too short for a DCD header");

    // first record: 84 bytes starting with "CORD"; marker width and byte order
    DcdInfo& I = info_;
    const uint32_t w0 = load32(&h[0], false), w1 = load32(&h[4], false);
    if (w0 == 84 && w1 == kCord) {
        I.marker = 4;
    } else if (w0 == 84 && w1 == 0 && load32(&h[8], false) == kCord) {
        I.marker = 8;
    } else if (bswap32(w0) == 84 && w1 == kCord) {
        I.marker = 4;
        I.swap = true;
    } else if (w0 == 0 && bswap32(w1) == 84 && load32(&h[8], false) == kCord) {
        I.marker = 8;
        I.swap = true;
    } else {
        bad("unrecognised header (not a DCD file)");
    }
    const int M = I.marker;
    size_t pos = M + 4;  // past the marker and "CORD"
    if (h.size() < pos + 80 + M) bad("truncated header");
    const unsigned char* w = &h[pos];   // the 20 header words
    auto word = [&](int i) { return static_cast<int32_t>(load32(w + 4 * i, I.swap)); };
    I.nsets_header = word(0);
    I.istart = word(1);
    I.nsavc = word(2);
    const int nfixed = word(8);
    I.charmm = word(19) != 0;
    if (I.charmm) {
        I.unit_cell = word(10) != 0;
        I.four_dims = word(11) == 1;
        uint32_t dbits = load32(w + 36, I.swap);
        float df;
        std::memcpy(&df, &dbits, 4);
        I.delta = df;
    } else {
        uint64_t dbits;
        std::memcpy(&dbits, w + 36, 8);
        if (I.swap) dbits = bswap64(dbits);
        std::memcpy(&I.delta, &dbits, 8);
    }
    pos += 80;
    if (load_marker(&h[pos], M, I.swap) != 84) bad("first record does not end with 84");
    pos += M;

    // title record
    if (h.size() < pos + M + 4) bad("truncated title record");
    const int64_t tlen = load_marker(&h[pos], M, I.swap);
    if (tlen < 4 || (tlen - 4) % 80 != 0) bad("malformed title record");
    pos += M;
    const int32_t ntitle = static_cast<int32_t>(load32(&h[pos], I.swap));
    if (ntitle < 0 || ntitle > 1000 || tlen != 4 + 80LL * ntitle) bad("malformed title record");
    pos += static_cast<size_t>(tlen);
    if (h.size() < pos + 2 * M + 4) bad("truncated title record");
    if (load_marker(&h[pos], M, I.swap) != tlen) bad("title record markers disagree");
    pos += M;

    // atom count record
    if (load_marker(&h[pos], M, I.swap) != 4) bad("malformed atom-count record");
    pos += M;
    I.natoms = static_cast<int32_t>(load32(&h[pos], I.swap));
    pos += 4;
    if (h.size() < pos + M || load_marker(&h[pos], M, I.swap) != 4) bad("malformed atom-count record");
    pos += M;
    if (I.natoms <= 0) bad("no atoms");
    if (nfixed != 0) {
        ::close(fd_);
        fd_ = -1;
        fail(NSG_ERR_UNSUPPORTED, "DCD file '" + path + "': fixed atoms are not supported");
    }
    I.header_bytes = static_cast<int64_t>(pos);

    // frame geometry
    const int64_t rec = 2LL * M + 4LL * I.natoms;
    const int64_t cell = I.unit_cell ? 2LL * M + 48 : 0;
    const int ndims = I.four_dims ? 4 : 3;
    I.frame_bytes = cell + ndims * rec;
    I.x_off = cell + M;
    I.y_off = cell + rec + M;
    I.z_off = cell + 2 * rec + M;
    const int64_t body = fsize - I.header_bytes;
    if (body < I.frame_bytes) bad("contains no frames");
    const int64_t n = body / I.frame_bytes;
    if (n > 0x7fffffff) bad("too many frames");
    I.nsets = static_cast<int>(n);
}

DcdFile::~DcdFile() {
    if (fd_ >= 0) ::close(fd_);
}

void DcdFile::read_frames(int f0, int count, void* dst) const {
    if (f0 < 0 || count < 0 || static_cast<int64_t>(f0) + count > info_.nsets) {
        invalid("DCD frames [" + std::to_string(f0) + ", " + std::to_string(f0 + count) +
                ") outside the file's " + std::to_string(info_.nsets) + " frames");
    }
    unsigned char* out = static_cast<unsigned char*>(dst);
    int64_t left = static_cast<int64_t>(count) * info_.frame_bytes;
    int64_t off = info_.header_bytes + static_cast<int64_t>(f0) * info_.frame_bytes;
    while (left > 0) {
        const size_t chunk = static_cast<size_t>(std::min<int64_t>(left, 1LL << 30));
        const ssize_t got = ::pread(fd_, out, chunk, off);
        if (got <= 0) {
            if (got < 0 && errno == EINTR) continue;
            io_fail("DCD file '" + path_ + "': read error");
        }
        out += got;
        off += got;
        left -= got;
    }
}

void DcdFile::check_frame(const void* frame, int f) const {
    const unsigned char* p = static_cast<const unsigned char*>(frame);
    const int M = info_.marker;
    const int64_t rec = 4LL * info_.natoms;
    auto expect = [&](int64_t at, int64_t len) {
        if (load_marker(p + at, M, info_.swap) != len ||
            load_marker(p + at + M + len, M, info_.swap) != len) {
            io_fail("DCD file '" + path_ + "': malformed record in frame " + std::to_string(f));
        }
    };
    if (info_.unit_cell) expect(0, 48);
    expect(info_.x_off - M, rec);
    expect(info_.y_off - M, rec);
    expect(info_.z_off - M, rec);
}

void DcdFile::coordinates(const void* frame, float* x, float* y, float* z) const {
    const unsigned char* p = static_cast<const unsigned char*>(frame);
    float* dst[3] = {x, y, z};
    const int64_t off[3] = {info_.x_off, info_.y_off, info_.z_off};
    for (int c = 0; c < 3; ++c) {
        for (int a = 0; a < info_.natoms; ++a) {
            const uint32_t v = load32(p + off[c] + 4LL * a, info_.swap);
            std::memcpy(&dst[c][a], &v, 4);
        }
    }
}

}  // namespace nsg
