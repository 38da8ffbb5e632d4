// netchem: PDB topology, DCD frames -> node centres of mass on the device
// (netchem/src/{atom,atoms,node,network,utils}.cpp).
#include <cuda_runtime.h>

#include <algorithm>
#include <cctype>
#include <cstring>
#include <fstream>
#include <map>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "cuarray.h"
#include "dcd.h"
#include "engine.h"
#include "errors.h"
#include "netchem/network.h"
#include "node_com.h"

namespace {

// Standard atomic weights in kg/mol, the values netchem's element table
// holds (netchem/include/chemical_properties.h:49-168); an element missing
// from it (vanadium among them) weighs 0, as a std::map lookup there gives.
struct Weight {
    const char* symbol;
    double kg_per_mol;
};
const Weight kWeights[] = {
    {"H", 1.00794e-3},    {"He", 4.002602e-3},  {"Li", 6.941e-3},      {"Be", 9.01218e-3},
    {"B", 10.811e-3},     {"C", 12.011e-3},     {"N", 14.00674e-3},    {"O", 15.9994e-3},
    {"F", 18.998403e-3},  {"Ne", 20.1797e-3},   {"Na", 22.989768e-3},  {"Mg", 24.305e-3},
    {"Al", 26.981539e-3}, {"Si", 28.0855e-3},   {"P", 30.973762e-3},   {"S", 32.066e-3},
    {"Cl", 35.4527e-3},   {"Ar", 39.948e-3},    {"K", 39.0983e-3},     {"Ca", 40.078e-3},
    {"Sc", 44.95591e-3},  {"Ti", 47.88e-3},     {"Cr", 51.9961e-3},    {"Mn", 54.93805e-3},
    {"Fe", 55.847e-3},    {"Co", 58.9332e-3},   {"Ni", 58.6934e-3},    {"Cu", 63.546e-3},
    {"Zn", 65.39e-3},     {"Ga", 69.723e-3},    {"Ge", 72.61e-3},      {"As", 74.92159e-3},
    {"Se", 78.96e-3},     {"Br", 79.904e-3},    {"Kr", 83.8e-3},       {"Rb", 85.4678e-3},
    {"Sr", 87.62e-3},     {"Y", 88.90585e-3},   {"Zr", 91.224e-3},     {"Nb", 92.90638e-3},
    {"Mo", 95.94e-3},     {"Tc", 97.9072e-3},   {"Ru", 101.07e-3},     {"Rh", 102.9055e-3},
    {"Pd", 106.42e-3},    {"Ag", 107.8682e-3},  {"Cd", 112.411e-3},    {"In", 114.818e-3},
    {"Sn", 118.71e-3},    {"Sb", 121.76e-3},    {"Te", 127.6e-3},      {"I", 126.90447e-3},
    {"Xe", 131.29e-3},    {"Cs", 132.90543e-3}, {"Ba", 137.327e-3},    {"La", 138.9055e-3},
    {"Ce", 140.115e-3},   {"Pr", 140.90765e-3}, {"Nd", 144.24e-3},     {"Pm", 144.9127e-3},
    {"Sm", 150.36e-3},    {"Eu", 151.965e-3},   {"Gd", 157.25e-3},     {"Tb", 158.92534e-3},
    {"Dy", 162.5e-3},     {"Ho", 164.93032e-3}, {"Er", 167.26e-3},     {"Tm", 168.93421e-3},
    {"Yb", 173.04e-3},    {"Lu", 174.967e-3},   {"Hf", 178.49e-3},     {"Ta", 180.9479e-3},
    {"W", 183.84e-3},     {"Re", 186.207e-3},   {"Os", 190.23e-3},     {"Ir", 192.22e-3},
    {"Pt", 195.08e-3},    {"Au", 196.96654e-3}, {"Hg", 200.59e-3},     {"Tl", 204.3833e-3},
    {"Pb", 207.2e-3},     {"Bi", 208.98037e-3}, {"Po", 208.9824e-3},   {"At", 209.9871e-3},
    {"Rn", 222.0176e-3},  {"Fr", 223.0197e-3},  {"Ra", 226.0254e-3},   {"Ac", 227.0278e-3},
    {"Th", 232.0381e-3},  {"Pa", 231.03588e-3}, {"U", 238.0289e-3},    {"Np", 237.048e-3},
    {"Pu", 244.0642e-3},  {"Am", 243.0614e-3},  {"Cm", 247.0703e-3},   {"Bk", 247.0703e-3},
    {"Cf", 251.0796e-3},  {"Es", 252.083e-3},   {"Fm", 257.0951e-3},   {"Md", 258.1e-3},
    {"No", 259.1009e-3},  {"Lr", 262.11e-3},    {"Rf", 261e-3},        {"Db", 262e-3},
    {"Sg", 266e-3},       {"Bh", 264e-3},       {"Hs", 269e-3},        {"Mt", 268e-3},
    {"Ds", 269e-3},       {"Rg", 272e-3},       {"Cn", 277e-3},        {"Nh", 0.0},
    {"Fl", 289e-3},       {"Mc", 0.0},          {"Lv", 0.0},           {"Ts", 0.0},
    {"Og", 0.0},
};

double atomic_weight(const std::string& symbol) {
    for (const Weight& w : kWeights) {
        if (symbol == w.symbol) return w.kg_per_mol;
    }
    return 0.0;
}

std::string strip(const std::string& s) {
    std::string out;
    for (char c : s) {
        if (!std::isspace(static_cast<unsigned char>(c))) out.push_back(c);
    }
    return out;
}

// PDB fixed columns [pos, pos + len), clipped at the end of the line; a
// line that ends before pos is an error (std::string::substr's rule).
std::string field(const std::string& line, size_t pos, size_t len, int atom) {
    if (pos > line.size()) {
        nsg::invalid("PDB ATOM record " + std::to_string(atom) + " is too short (" +
                     std::to_string(line.size()) + " columns)");
    }
    return line.substr(pos, len);
}

// Multiplicative string hash of netchem/src/utils.cpp:94-110 (h = 37,
// h = h * 54059 ^ c * 76963 per character, characters taken as signed).
unsigned int hash_string(const std::string& s) {
    unsigned int h = 37u;
    for (char c : s) {
        const int ci = static_cast<int>(static_cast<signed char>(c));
        h = (h * 54059u) ^ static_cast<unsigned int>(ci * 76963);
    }
    return h;
}

}  // namespace

// ---- Atom / Atoms / Node --------------------------------------------------------
Atom::Atom(const std::string& line, int atomIndex) {
    // netchem/src/atom.cpp:177-291
    serial_ = atomIndex + 1;
    index_ = atomIndex;
    const int a = atomIndex;
    name_ = strip(field(line, 12, 3, a));
    residueName_ = strip(field(line, 17, 3, a));
    chainId_ = strip(field(line, 21, 1, a));
    const std::string resid = strip(field(line, 22, 4, a));
    const std::string occ = strip(field(line, 54, 6, a));
    segmentId_ = strip(field(line, 72, 4, a));
    element_ = strip(field(line, 76, 2, a));
    try {
        residueId_ = std::stoi(resid);
        occupancy_ = static_cast<float>(std::stod(occ));
    } catch (const std::exception&) {
        nsg::invalid("PDB ATOM record " + std::to_string(a) + ": residue id or occupancy is not a number");
    }
    // the reference reads the temperature factor from the occupancy columns
    temperatureFactor_ = occupancy_;
    for (char& c : element_) c = static_cast<char>(std::tolower(static_cast<unsigned char>(c)));
    if (!element_.empty()) {
        element_[0] = static_cast<char>(std::toupper(static_cast<unsigned char>(element_[0])));
    }
    tag_ = residueName_ + "_" + resid + "_" + chainId_ + "_" + segmentId_;
    mass_ = static_cast<float>(1000.0 * atomic_weight(element_));
    hash_ = hash_string(std::to_string(index_) + "_" + tag_);
}

void Atoms::addAtom(Atom* atom) {
    tags_.insert(atom->tag());
    atoms_.push_back(atom);
}

Atom* Atoms::at(int atomIndex) {
    if (atomIndex < 0 || atomIndex >= numAtoms()) throw std::out_of_range("atom index out of range");
    return atoms_[atomIndex];
}

Atoms::~Atoms() {
    for (Atom* a : atoms_) delete a;
}

Node::Node(unsigned int numFrames, unsigned int index) : index_(index), numFrames_(numFrames) {}

// ---- Network --------------------------------------------------------------------
struct Network::DeviceState {
    nsg::DeviceBuffer coords;   // numNodes x 3 x ld
};

Network::Network() : nodeCoordinates_(new CuArray<float>()), atoms_(new Atoms()) {}

Network::~Network() {
    for (Node* n : nodes_) delete n;
    delete nodeCoordinates_;
    delete atoms_;
}

Node* Network::nodeFromAtomIndex(int atomIndex) {
    if (atomIndex < 0 || atomIndex >= static_cast<int>(nodeAtomIndexVector_.size())) {
        throw std::out_of_range("atom index out of range");
    }
    return nodeAtomIndexVector_[atomIndex];
}

const float* Network::deviceCoordinates() const {
    return dev_ ? dev_->coords.as<float>() : nullptr;
}

void Network::parsePdb(const std::string& fname) {
    // netchem/src/network.cpp:258-278: every line containing "ATOM" is an
    // atom record, indexed in file order.
    std::ifstream in(fname);
    if (!in) nsg::io_fail("cannot open PDB file '" + fname + "'");
    std::string line;
    int idx = atoms_->numAtoms();
    while (std::getline(in, line)) {
        if (line.find("ATOM") != std::string::npos) {
            atoms_->addAtom(new Atom(line, idx));
            ++idx;
        }
    }
}

void Network::init(const std::string& trajectoryFile, const std::string& topologyFile,
                   int firstFrame, int lastFrame, int stride) {
    // netchem/src/network.cpp:29-75
    if (stride < 1) nsg::invalid("stride must be >= 1");
    if (firstFrame < 0) nsg::invalid("firstFrame must be >= 0");
    for (Node* n : nodes_) delete n;
    nodes_.clear();
    nodeAtomIndexVector_.clear();
    delete atoms_;
    atoms_ = new Atoms();
    dev_.reset();
    numNodes_ = numFrames_ = deviceLd_ = 0;

    parsePdb(topologyFile);
    std::map<std::string, Node*> byTag;
    nodeAtomIndexVector_.assign(atoms_->numAtoms(), nullptr);
    for (Atom* atom : atoms_->atoms()) {
        auto it = byTag.find(atom->tag());
        if (it == byTag.end()) {
            Node* n = new Node(0, static_cast<unsigned int>(nodes_.size()));
            n->tag_ = atom->tag();
            nodes_.push_back(n);
            it = byTag.emplace(atom->tag(), n).first;
        }
        Node* n = it->second;
        n->atoms_.push_back(atom);
        n->totalMass_ += atom->mass();
        nodeAtomIndexVector_[atom->index()] = n;
    }
    numNodes_ = static_cast<int>(nodes_.size());
    parseDcd(trajectoryFile, firstFrame, lastFrame, stride);
    for (Node* n : nodes_) n->numFrames_ = static_cast<unsigned int>(numFrames_);
}

void Network::parseDcd(const std::string& fname, int firstFrame, int lastFrame, int stride) {
    // netchem/src/network.cpp:101-255, on the device: frames are read raw
    // into pinned memory, copied in batches and reduced by launch_node_com.
    nsg::DcdFile dcd(fname);
    const nsg::DcdInfo& I = dcd.info();
    if (lastFrame == -1) lastFrame = I.nsets - 1;
    if (stride < 1) nsg::invalid("stride must be >= 1");
    if (firstFrame < 0 || lastFrame < firstFrame) nsg::invalid("need 0 <= firstFrame <= lastFrame");
    if (lastFrame >= I.nsets) {
        nsg::invalid("lastFrame " + std::to_string(lastFrame) + " is past the trajectory's " +
                     std::to_string(I.nsets) + " frames");
    }
    if (I.natoms != atoms_->numAtoms()) {
        nsg::invalid("the trajectory has " + std::to_string(I.natoms) + " atoms, the topology " +
                     std::to_string(atoms_->numAtoms()));
    }
    const int m = (lastFrame - firstFrame) / stride + 1;
    const int N = numNodes_;
    numFrames_ = m;
    const int ld = (m + 63) / 64 * 64;
    deviceLd_ = ld;

    // node tables (CSR over atoms in index order)
    std::vector<int> start(N + 1, 0), members;
    members.reserve(atoms_->numAtoms());
    std::vector<float> amass(atoms_->numAtoms()), nmass(N);
    for (int i = 0; i < N; ++i) {
        start[i] = static_cast<int>(members.size());
        for (Atom* a : nodes_[i]->atoms_) members.push_back(a->index());
        nmass[i] = nodes_[i]->totalMass_;
    }
    start[N] = static_cast<int>(members.size());
    for (Atom* a : atoms_->atoms()) amass[a->index()] = a->mass();

    auto state = std::make_unique<DeviceState>();
    state->coords.reset(sizeof(float) * static_cast<size_t>(N) * 3 * ld);
    nsg::DeviceBuffer d_start(sizeof(int) * (N + 1)), d_members(sizeof(int) * std::max<size_t>(1, members.size())),
        d_amass(sizeof(float) * std::max<size_t>(1, amass.size())), d_nmass(sizeof(float) * std::max(1, N));
    cudaStream_t st = nullptr;
    NSG_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    struct StreamGuard {
        cudaStream_t s;
        ~StreamGuard() { cudaStreamDestroy(s); }
    } sg{st};
    NSG_CUDA(cudaMemcpyAsync(d_start.get(), start.data(), sizeof(int) * (N + 1), cudaMemcpyHostToDevice, st));
    if (!members.empty()) {
        NSG_CUDA(cudaMemcpyAsync(d_members.get(), members.data(), sizeof(int) * members.size(),
                                 cudaMemcpyHostToDevice, st));
        NSG_CUDA(cudaMemcpyAsync(d_amass.get(), amass.data(), sizeof(float) * amass.size(),
                                 cudaMemcpyHostToDevice, st));
    }
    if (N) NSG_CUDA(cudaMemcpyAsync(d_nmass.get(), nmass.data(), sizeof(float) * N, cudaMemcpyHostToDevice, st));

    // frame batches: two pinned staging buffers of up to 64 MB, so the read
    // of batch b + 1 overlaps the copy and kernel of batch b
    const long long fb = I.frame_bytes;
    const int batch = static_cast<int>(std::max<long long>(1, std::min<long long>(m, (64LL << 20) / fb)));
    const size_t stage_bytes = static_cast<size_t>(batch) * fb;
    void* pinned[2] = {nullptr, nullptr};
    cudaEvent_t copied[2] = {nullptr, nullptr};
    struct PinnedGuard {
        void** p;
        cudaEvent_t* e;
        ~PinnedGuard() {
            for (int i = 0; i < 2; ++i) {
                if (e[i]) cudaEventDestroy(e[i]);
                if (p[i]) cudaFreeHost(p[i]);
            }
        }
    } pg{pinned, copied};
    nsg::DeviceBuffer raw[2];
    for (int i = 0; i < 2; ++i) {
        NSG_CUDA(cudaHostAlloc(&pinned[i], stage_bytes, cudaHostAllocDefault));
        NSG_CUDA(cudaEventCreateWithFlags(&copied[i], cudaEventDisableTiming));
        raw[i].reset(stage_bytes);
    }
    nsg::NodeComArgs a{};
    a.frame_bytes = fb;
    a.x_off = I.x_off;
    a.y_off = I.y_off;
    a.z_off = I.z_off;
    a.swap = I.swap ? 1 : 0;
    a.nnodes = N;
    a.node_start = d_start.as<int>();
    a.node_atoms = d_members.as<int>();
    a.atom_mass = d_amass.as<float>();
    a.node_mass = d_nmass.as<float>();
    a.out = state->coords.as<float>();
    a.row_stride = 3LL * ld;
    a.plane_stride = ld;
    int b = 0;
    for (int i0 = 0; i0 < m; i0 += batch, b ^= 1) {
        const int cnt = std::min(batch, m - i0);
        NSG_CUDA(cudaEventSynchronize(copied[b]));   // staging buffer b is free again
        unsigned char* dst = static_cast<unsigned char*>(pinned[b]);
        if (stride == 1) {
            dcd.read_frames(firstFrame + i0, cnt, dst);
        } else {
            for (int j = 0; j < cnt; ++j) dcd.read_frame(firstFrame + (i0 + j) * stride, dst + j * fb);
        }
        for (int j = 0; j < cnt; ++j) dcd.check_frame(dst + j * fb, firstFrame + (i0 + j) * stride);
        NSG_CUDA(cudaMemcpyAsync(raw[b].get(), dst, static_cast<size_t>(cnt) * fb, cudaMemcpyHostToDevice, st));
        NSG_CUDA(cudaEventRecord(copied[b], st));
        a.frames = raw[b].as<unsigned char>();
        a.nframes = cnt;
        a.frame0 = i0;
        nsg::launch_node_com(a, st);
    }
    nsg::launch_pad_inf(state->coords.as<float>(), 3LL * N, m, ld, st);

    nodeCoordinates_->init(N, 3 * m);
    if (N > 0) {
        NSG_CUDA(cudaMemcpy2DAsync(nodeCoordinates_->host(), sizeof(float) * m, state->coords.get(),
                                   sizeof(float) * ld, sizeof(float) * m, static_cast<size_t>(3) * N,
                                   cudaMemcpyDeviceToHost, st));
    }
    NSG_CUDA(cudaStreamSynchronize(st));
    dev_ = std::move(state);
}

void Network::nodeCoordinates(const std::string& nodeCoordinatesFile) {
    // netchem/src/network.cpp:302-312
    CuArray<float>* c = new CuArray<float>();
    if (c->load(nodeCoordinatesFile) != 0) {
        delete c;
        nsg::io_fail("cannot load node coordinates from '" + nodeCoordinatesFile + "'");
    }
    delete nodeCoordinates_;
    nodeCoordinates_ = c;
    dev_.reset();
    deviceLd_ = 0;
}
