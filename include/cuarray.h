// CuArray<T>: row-major 2-D host buffer with an optional device mirror.
//
// Same public interface and semantics as the reference container
// (cuarray/include/cuarray.h:23-489): zero-initialised init(m, n), shallow
// and deep row-range copies, set() bounds check returning 1,
// toDevice()/toHost() returning 1 when either side is unallocated, sort()
// and argsort() in descending order, .npy load/save. Element types int,
// float and double are instantiated.
#ifndef NETSCI_GB300_CUARRAY_H
#define NETSCI_GB300_CUARRAY_H

#include <cstddef>
#include <string>

typedef int CuArrayError;

template <typename T>
class CuArray {
public:
    CuArray();
    ~CuArray();
    CuArray(const CuArray&) = delete;
    CuArray& operator=(const CuArray&) = delete;

    // Fresh zero-filled m x n host buffer; releases what was held.
    CuArrayError init(int m, int n);
    // m x n host buffer holding a copy of `host`.
    CuArrayError init(T* host, int m, int n);
    // View of rows start..end (inclusive) of `cuArray` without copying;
    // requires (end-start+1) * cuArray->n() == m * n.
    CuArrayError fromCuArrayShallowCopy(CuArray<T>* cuArray, int start, int end, int m, int n);
    // Owned copy of rows start..end (inclusive); same size rule.
    CuArrayError fromCuArrayDeepCopy(CuArray<T>* cuArray, int start, int end, int m, int n);

    int n() const;
    int m() const;
    int size() const;
    size_t bytes() const;
    T*& host();
    T*& device();

    CuArrayError allocateHost();
    CuArrayError allocateDevice();
    CuArrayError allocatedHost() const;
    CuArrayError allocatedDevice() const;
    CuArrayError toDevice();
    CuArrayError toHost();
    CuArrayError deallocateHost();
    CuArrayError deallocateDevice();

    // Copies of external buffers: 1 x dim1, or dim1 x dim2.
    CuArrayError fromNumpy(T* NUMPY_ARRAY, int NUMPY_ARRAY_DIM1);
    CuArrayError fromNumpy(T* NUMPY_ARRAY, int NUMPY_ARRAY_DIM1, int NUMPY_ARRAY_DIM2);
    // New[]-allocated copies of the host buffer plus shape cells.
    void toNumpy(T** NUMPY_ARRAY, int** NUMPY_ARRAY_DIM1, int** NUMPY_ARRAY_DIM2);
    void toNumpy(T** NUMPY_ARRAY, int** NUMPY_ARRAY_DIM1);

    T get(int i, int j) const;
    CuArrayError set(T value, int i, int j);

    CuArrayError load(const std::string& fname);
    void save(const std::string& fname);

    // Row i copied and sorted descending / row i's indices by descending value.
    CuArray<T>* sort(int i);
    T& operator[](int i) const;
    int owner() const;
    CuArray<int>* argsort(int i);

private:
    void release();
    // Host storage of `count` elements: page-locked (cudaHostAlloc) from
    // kPinnedMinBytes up when a CUDA device is present, so host<->device
    // copies of large arrays run at the link's speed; else new[].
    T* alloc_host(size_t count);
    void free_host();
    T* host_;
    T* device_;
    T* pinned_ = nullptr;  // host_ came from cudaHostAlloc (freed with cudaFreeHost)
    int n_{};
    int m_{};
    int size_{};
    size_t bytes_{};
    int allocatedDevice_{};
    int allocatedHost_{};
    int owner_{};
};

// Non-owning view of one row.
template <typename T>
class CuArrayRow {
public:
    CuArrayRow(CuArray<T>* cuArray, int i);
    T& operator[](int i) const;
    int n() const;
    T* data() const;

private:
    T* data_;
    int n_{};
};

#endif  // NETSCI_GB300_CUARRAY_H
