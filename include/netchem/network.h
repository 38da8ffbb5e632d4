// Trajectory -> node coordinates: the netchem classes Atom, Atoms, Node and
// Network (netchem/include/{atom,atoms,node,network}.h), same method names
// and meanings.
//
// Network::init(trajectoryFile, topologyFile, firstFrame, lastFrame, stride)
// reads the ATOM records of a PDB topology, groups atoms into nodes by their
// tag "<residue name>_<residue id>_<chain id>_<segment id>" (node index = order
// of first appearance), reads frames firstFrame, firstFrame + stride, ...,
// <= lastFrame of a DCD trajectory and computes each node's mass-weighted
// centre per frame: X[node][f], X[node][m + f], X[node][2m + f] (x, y, z
// planes of m frames). The frames go straight from the file into pinned
// memory, to the device and through one kernel; the result stays resident on
// the device in the layout the KSG entry points take (rows of 3 planes of ld
// floats, ld a multiple of 64, +inf padding) and is copied to the host
// CuArray nodeCoordinates().
//
// Differences from the reference, all where it has no defined result:
// lastFrame == -1 selects up to the last frame of the file (the reference
// computes its frame count from -1 before resolving it); a lastFrame past the
// end of the file, a DCD with fixed atoms, a malformed record or a PDB ATOM line
// too short for its fields raise std::runtime_error / std::invalid_argument
// instead of looping, misreading or crashing.
#ifndef NETSCI_GB300_NETCHEM_NETWORK_H
#define NETSCI_GB300_NETCHEM_NETWORK_H

#include <memory>
#include <set>
#include <string>
#include <vector>

#include "cuarray.h"

class Atom {
public:
    Atom() = default;
    // One PDB ATOM line; atomIndex is the running index of ATOM records
    // (netchem/src/atom.cpp:177-291).
    Atom(const std::string& pdbLine, int atomIndex);
    int index() const { return index_; }
    std::string name() { return name_; }
    std::string element() { return element_; }
    std::string residueName() { return residueName_; }
    int residueId() const { return residueId_; }
    std::string chainId() { return chainId_; }
    std::string segmentId() { return segmentId_; }
    float temperatureFactor() const { return temperatureFactor_; }
    float occupancy() const { return occupancy_; }
    int serial() const { return serial_; }
    std::string tag() { return tag_; }
    float mass() const { return mass_; }
    unsigned int hash() const { return hash_; }

private:
    int index_ = 0, residueId_ = 0, serial_ = 0;
    std::string name_, element_, residueName_, chainId_, segmentId_, tag_;
    float temperatureFactor_ = 0.f, occupancy_ = 0.f, mass_ = 0.f;
    unsigned int hash_ = 0;
};

class Atoms {
public:
    void addAtom(Atom* atom);          // takes ownership
    int numAtoms() const { return static_cast<int>(atoms_.size()); }
    Atom* at(int atomIndex);           // std::out_of_range past the end
    int numUniqueTags() const { return static_cast<int>(tags_.size()); }
    std::vector<Atom*>& atoms() { return atoms_; }
    ~Atoms();

private:
    std::vector<Atom*> atoms_;
    std::set<std::string> tags_;
};

class Node {
public:
    Node() = default;
    Node(unsigned int numFrames, unsigned int index);
    std::string tag() { return tag_; }
    unsigned int numAtoms() const { return static_cast<unsigned int>(atoms_.size()); }
    unsigned int index() const { return index_; }
    float totalMass() const { return totalMass_; }
    // 0 for nodes made by Network::init, as in the reference (which sets the
    // node hash only in Node::addAtom, a path init does not take).
    unsigned int hash() const { return hash_; }
    std::vector<Atom*> atoms() const { return atoms_; }

private:
    friend class Network;
    unsigned int index_ = 0, numFrames_ = 0, hash_ = 0;
    float totalMass_ = 0.f;
    std::string tag_;
    std::vector<Atom*> atoms_;
};

class Network {
public:
    Network();
    ~Network();
    Network(const Network&) = delete;
    Network& operator=(const Network&) = delete;

    void init(const std::string& trajectoryFile, const std::string& topologyFile, int firstFrame,
              int lastFrame, int stride = 1);
    int numNodes() const { return numNodes_; }
    CuArray<float>* nodeCoordinates() { return nodeCoordinates_; }
    std::vector<Node*>& nodes() { return nodes_; }
    int numFrames() const { return numFrames_; }
    Node* nodeFromAtomIndex(int atomIndex);
    Atoms* atoms() const { return atoms_; }
    void parsePdb(const std::string& fname);
    void parseDcd(const std::string& fname, int firstFrame, int lastFrame, int stride);
    // Replace the node coordinates by a .npy file (netchem/src/network.cpp:302-312).
    void nodeCoordinates(const std::string& nodeCoordinatesFile);

    // Device copy of the node coordinates: row n at deviceCoordinates() +
    // n * 3 * deviceLd(), planes x, y, z of deviceLd() floats, frames past
    // numFrames() are +inf. Null before init() / after nodeCoordinates(file).
    const float* deviceCoordinates() const;
    int deviceLd() const { return deviceLd_; }

private:
    struct DeviceState;
    int numNodes_ = 0, numFrames_ = 0, deviceLd_ = 0;
    CuArray<float>* nodeCoordinates_ = nullptr;
    std::vector<Node*> nodes_;
    std::vector<Node*> nodeAtomIndexVector_;
    Atoms* atoms_ = nullptr;
    std::unique_ptr<DeviceState> dev_;
};

#endif
