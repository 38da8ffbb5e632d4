// DCD trajectory reader (CHARMM / NAMD / X-PLOR binary trajectories), the
// format netchem reads through its DCD plugin (netchem/src/dcd/dcd.cpp:111-
// 440, 775-950).
//
// Layout: Fortran unformatted records, each payload framed by its byte
// length before and after (4-byte markers, or 8-byte ones from "-i8"
// builds), in either byte order:
//   header  84 bytes: "CORD", 20 ints (NSET, ISTART, NSAVC, ..., NAMNF at
//           word 8, DELTA at word 9, CHARMM flags at words 10-11, CHARMM
//           version at word 19; non-zero version = CHARMM format)
//   titles  NTITLE, NTITLE x 80 characters
//   atoms   NATOM
//   frames  [unit cell: 6 doubles, when CHARMM word 10 is set]
//           x[NATOM], y[NATOM], z[NATOM] floats, [w[NATOM] when word 11 == 1]
// With no fixed atoms every frame has the same size, so frame f starts at
// header_bytes + f * frame_bytes and any frame can be read directly. The
// frame count is taken from the file size, as the plugin does.
#pragma once

#include <cstddef>
#include <cstdint>
#include <string>

namespace nsg {

struct DcdInfo {
    int natoms = 0;
    int nsets = 0;           // frames in the file (from its size)
    int nsets_header = 0;    // NSET as written in the header
    int istart = 0, nsavc = 0;
    double delta = 0;
    bool charmm = false, unit_cell = false, four_dims = false;
    bool swap = false;       // byte order opposite to this machine's
    int marker = 4;          // record marker bytes (4 or 8)
    int64_t header_bytes = 0;
    int64_t frame_bytes = 0;
    // byte offsets of the x, y, z payloads inside a frame
    int64_t x_off = 0, y_off = 0, z_off = 0;
};

class DcdFile {
public:
    explicit DcdFile(const std::string& path);   // reads and checks the header
    ~DcdFile();
    DcdFile(const DcdFile&) = delete;
    DcdFile& operator=(const DcdFile&) = delete;
    const DcdInfo& info() const { return info_; }
    // Raw bytes of frames [f0, f0 + count) into dst (count * frame_bytes).
    void read_frames(int f0, int count, void* dst) const;
    // Raw bytes of one frame; dst holds frame_bytes.
    void read_frame(int f, void* dst) const { read_frames(f, 1, dst); }
    // Checks the record markers of a frame held in memory.
    void check_frame(const void* frame, int f) const;
    // x, y, z of one frame (host order) from its raw bytes.
    void coordinates(const void* frame, float* x, float* y, float* z) const;

private:
    int fd_ = -1;
    std::string path_;
    DcdInfo info_;
};

}  // namespace nsg
