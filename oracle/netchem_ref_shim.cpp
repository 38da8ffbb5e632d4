// ORACLE — TEST INFRASTRUCTURE ONLY.
//
// C entry points over the reference's own netchem pieces that build without
// external libraries: its DCD plugin (netchem/src/dcd/dcd.cpp) and its Atom
// class (netchem/src/atom.cpp, utils.cpp). Tests use them to pin the oracle's
// DCD reader and PDB parsing. Compiled by oracle/Makefile (target `ref`) from
// the reference sources where they lie; the result goes to oracle/_ref/.

#include <cstring>
#include <fstream>
#include <string>

#include "atom.h"
#include "dcd/dcd.h"
#include "utils.h"

extern "C" {

// Frames of a DCD file through the plugin: counts only when out is null,
// else out[f][c][a] for every frame. Returns 0, or the plugin's error code.
int ref_dcd_frames(const char* path, int* natoms, int* nsets, float* out) {
    int na = 0, ns = 0;
    dcdhandle* h = open_dcd_read(path, &na, &ns);
    if (!h) return -1;
    *natoms = na;
    *nsets = ns;
    int rc = 0;
    if (out) {
        molfile_timestep_t ts;
        std::memset(&ts, 0, sizeof(ts));
        for (int f = 0; f < ns && rc == 0; ++f) {
            rc = read_next_timestep(h, na, &ts);
            float* o = out + static_cast<size_t>(f) * 3 * na;
            std::memcpy(o, h->x, sizeof(float) * na);
            std::memcpy(o + na, h->y, sizeof(float) * na);
            std::memcpy(o + 2 * na, h->z, sizeof(float) * na);
        }
    }
    close_file_read(h);
    return rc;
}

// ATOM records of a PDB file through the reference's Atom(line, index):
// mass, residue id, hash, tag (40 chars each), element (4), name (8).
// Returns the number of atoms (at most cap are written).
int ref_pdb_atoms(const char* path, int cap, float* mass, int* resid, unsigned* hash,
                  char* tags, char* elements, char* names) {
    std::ifstream in(path);
    std::string line;
    int n = 0;
    while (std::getline(in, line)) {
        if (!utils::isRecordAtom(line)) continue;
        if (n < cap) {
            Atom a(line, n);
            mass[n] = a.mass();
            resid[n] = a.residueId();
            hash[n] = a.hash();
            std::strncpy(tags + 40 * n, a.tag().c_str(), 39);
            std::strncpy(elements + 4 * n, a.element().c_str(), 3);
            std::strncpy(names + 8 * n, a.name().c_str(), 7);
        }
        ++n;
    }
    return n;
}

}  // extern "C"
