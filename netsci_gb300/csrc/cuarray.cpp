// CuArray<T> implementation. Interface and observable semantics follow the
// reference container (cuarray/src/cuarray.cu:8-454); storage management is
// this library's own: re-initialising a CuArray releases only what it owns
// (the reference's fromNumpy marks a view as owner before freeing it), and
// CUDA failures are reported through the CuArrayError return value.
#include "cuarray.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <numeric>
#include <vector>

#include "errors.h"
#include "npy.h"

template <typename T>
CuArray<T>::CuArray() : host_(nullptr), device_(nullptr) {}

template <typename T>
CuArray<T>::~CuArray() {
    release();
}

namespace {
// Arrays at least this large get page-locked host storage.
constexpr size_t kPinnedMinBytes = size_t(16) << 20;
}  // namespace

template <typename T>
T* CuArray<T>::alloc_host(size_t count) {
    if (count == 0) count = 1;
    const size_t bytes = count * sizeof(T);
    if (bytes >= kPinnedMinBytes) {
        void* p = nullptr;
        if (cudaHostAlloc(&p, bytes, cudaHostAllocPortable) == cudaSuccess) {
            pinned_ = static_cast<T*>(p);
            return pinned_;
        }
        cudaGetLastError();  // no device: ordinary memory
    }
    pinned_ = nullptr;
    return new T[count];
}

template <typename T>
void CuArray<T>::free_host() {
    if (pinned_) {
        cudaFreeHost(pinned_);
        pinned_ = nullptr;
    } else if (host_) {
        delete[] host_;
    }
    host_ = nullptr;
}

template <typename T>
void CuArray<T>::release() {
    if (allocatedHost_ && owner_ && host_) free_host();
    pinned_ = nullptr;
    if (allocatedDevice_ && device_) cudaFree(device_);
    host_ = nullptr;
    device_ = nullptr;
    allocatedHost_ = 0;
    allocatedDevice_ = 0;
}

template <typename T>
CuArrayError CuArray<T>::init(int m, int n) {
    if (m < 0 || n < 0) return 1;
    release();
    m_ = m;
    n_ = n;
    size_ = m * n;
    bytes_ = static_cast<size_t>(size_) * sizeof(T);
    owner_ = 1;
    host_ = alloc_host(static_cast<size_t>(size_));
    std::fill(host_, host_ + size_, T(0));
    allocatedHost_ = 1;
    return 0;
}

template <typename T>
CuArrayError CuArray<T>::init(T* host, int m, int n) {
    if (m < 0 || n < 0 || (!host && m * n > 0)) return 1;
    release();
    m_ = m;
    n_ = n;
    size_ = m * n;
    bytes_ = static_cast<size_t>(size_) * sizeof(T);
    owner_ = 1;
    host_ = alloc_host(static_cast<size_t>(size_));
    if (size_) std::copy(host, host + size_, host_);
    allocatedHost_ = 1;
    return 0;
}

template <typename T>
CuArrayError CuArray<T>::fromCuArrayShallowCopy(CuArray<T>* src, int start, int end, int m,
                                                int n) {
    if (!src || start < 0 || end < start || end >= src->m_) return 1;
    if ((end - start + 1) * src->n_ != m * n) return 1;
    release();
    owner_ = 0;
    m_ = m;
    n_ = n;
    size_ = m * n;
    bytes_ = static_cast<size_t>(size_) * sizeof(T);
    host_ = src->host_ + static_cast<size_t>(start) * src->n_;
    allocatedHost_ = 1;
    return 0;
}

template <typename T>
CuArrayError CuArray<T>::fromCuArrayDeepCopy(CuArray<T>* src, int start, int end, int m, int n) {
    if (!src || start < 0 || end < start || end >= src->m_) return 1;
    if ((end - start + 1) * src->n_ != m * n) return 1;
    // the new storage is filled before this array's own is released (src may
    // be this array)
    T* const old_pinned = pinned_;
    pinned_ = nullptr;
    T* copy = alloc_host(static_cast<size_t>(m) * n);
    T* const copy_pinned = pinned_;
    std::copy(src->host_ + static_cast<size_t>(start) * src->n_,
              src->host_ + static_cast<size_t>(end + 1) * src->n_, copy);
    pinned_ = old_pinned;
    release();
    pinned_ = copy_pinned;
    owner_ = 1;
    m_ = m;
    n_ = n;
    size_ = m * n;
    bytes_ = static_cast<size_t>(size_) * sizeof(T);
    host_ = copy;
    allocatedHost_ = 1;
    return 0;
}

template <typename T>
int CuArray<T>::n() const { return n_; }
template <typename T>
int CuArray<T>::m() const { return m_; }
template <typename T>
int CuArray<T>::size() const { return size_; }
template <typename T>
size_t CuArray<T>::bytes() const { return bytes_; }
template <typename T>
T*& CuArray<T>::host() { return host_; }
template <typename T>
T*& CuArray<T>::device() { return device_; }
template <typename T>
int CuArray<T>::owner() const { return owner_; }
template <typename T>
CuArrayError CuArray<T>::allocatedHost() const { return allocatedHost_; }
template <typename T>
CuArrayError CuArray<T>::allocatedDevice() const { return allocatedDevice_; }

template <typename T>
CuArrayError CuArray<T>::allocateHost() {
    if (!allocatedHost_ && owner_) {
        host_ = alloc_host(static_cast<size_t>(size_));
        allocatedHost_ = 1;
    }
    return allocatedHost_ ? 0 : 1;
}

template <typename T>
CuArrayError CuArray<T>::allocateDevice() {
    if (!allocatedDevice_) {
        void* p = nullptr;
        if (cudaMalloc(&p, bytes_ > 0 ? bytes_ : 1) != cudaSuccess) {
            cudaGetLastError();
            return 1;
        }
        device_ = static_cast<T*>(p);
        allocatedDevice_ = 1;
    }
    return 0;
}

template <typename T>
CuArrayError CuArray<T>::toDevice() {
    if (allocatedDevice_ && allocatedHost_) {
        if (bytes_ && cudaMemcpy(device_, host_, bytes_, cudaMemcpyHostToDevice) != cudaSuccess) {
            cudaGetLastError();
            return 1;
        }
        return 0;
    }
    return 1;
}

template <typename T>
CuArrayError CuArray<T>::toHost() {
    if (allocatedDevice_ && allocatedHost_) {
        if (bytes_ && cudaMemcpy(host_, device_, bytes_, cudaMemcpyDeviceToHost) != cudaSuccess) {
            cudaGetLastError();
            return 1;
        }
        return 0;
    }
    return 1;
}

template <typename T>
CuArrayError CuArray<T>::deallocateHost() {
    if (allocatedHost_ && owner_) {
        free_host();
        allocatedHost_ = 0;
    }
    return allocatedHost_ ? 1 : 0;
}

template <typename T>
CuArrayError CuArray<T>::deallocateDevice() {
    if (allocatedDevice_) {
        cudaFree(device_);
        device_ = nullptr;
        allocatedDevice_ = 0;
    }
    return allocatedDevice_ ? 1 : 0;
}

template <typename T>
T& CuArray<T>::operator[](int i) const { return host_[i]; }

template <typename T>
CuArrayError CuArray<T>::fromNumpy(T* data, int dim1) {
    return init(data, 1, dim1);
}

template <typename T>
CuArrayError CuArray<T>::fromNumpy(T* data, int dim1, int dim2) {
    return init(data, dim1, dim2);
}

template <typename T>
void CuArray<T>::toNumpy(T** out, int** dim1, int** dim2) {
    *dim1 = new int(m_);
    *dim2 = new int(n_);
    *out = new T[size_ > 0 ? size_ : 1];
    if (size_) std::copy(host_, host_ + size_, *out);
}

template <typename T>
void CuArray<T>::toNumpy(T** out, int** dim1) {
    *dim1 = new int(size_);
    *out = new T[size_ > 0 ? size_ : 1];
    if (size_) std::copy(host_, host_ + size_, *out);
}

template <typename T>
T CuArray<T>::get(int i, int j) const {
    return host_[static_cast<size_t>(i) * n_ + j];
}

template <typename T>
CuArrayError CuArray<T>::set(T value, int i, int j) {
    if (i >= 0 && j >= 0 && i < m_ && j < n_ && host_) {
        host_[static_cast<size_t>(i) * n_ + j] = value;
        return 0;
    }
    return 1;
}

namespace {
template <typename S, typename T>
void convert(const unsigned char* raw, size_t count, std::vector<T>& out) {
    out.resize(count);
    for (size_t i = 0; i < count; ++i) {
        S v;
        std::memcpy(&v, raw + i * sizeof(S), sizeof(S));
        out[i] = static_cast<T>(v);
    }
}
}  // namespace

template <typename T>
CuArrayError CuArray<T>::load(const std::string& fname) {
    nsg::NpyArray a = nsg::npy_read(fname);
    std::vector<T> vals;
    const size_t cnt = a.count();
    if (a.descr == "<f4") convert<float>(a.data.data(), cnt, vals);
    else if (a.descr == "<f8") convert<double>(a.data.data(), cnt, vals);
    else if (a.descr == "<i4") convert<int32_t>(a.data.data(), cnt, vals);
    else if (a.descr == "<i8") convert<int64_t>(a.data.data(), cnt, vals);
    else nsg::io_fail("unsupported .npy dtype " + a.descr);
    int m = 1, n = 0;
    if (a.shape.size() == 0) {
        n = 1;
    } else if (a.shape.size() == 1) {
        n = static_cast<int>(a.shape[0]);
    } else if (a.shape.size() == 2) {
        m = static_cast<int>(a.shape[0]);
        n = static_cast<int>(a.shape[1]);
        if (m == 0 || n == 0) {
            n = std::max(m, n);
            m = 1;
        }
    } else {
        nsg::io_fail("only 1-D and 2-D .npy arrays can be loaded into a CuArray");
    }
    return init(vals.data(), m, n);
}

template <typename T>
void CuArray<T>::save(const std::string& fname) {
    nsg::npy_write(fname, host_, nsg::npy_descr<T>(), sizeof(T),
                   {static_cast<size_t>(m_), static_cast<size_t>(n_)});
}

template <typename T>
CuArray<T>* CuArray<T>::sort(int i) {
    auto* out = new CuArray<T>();
    out->fromCuArrayDeepCopy(this, i, i, 1, n_);
    std::sort(out->host_, out->host_ + out->n(), [](T a, T b) { return a > b; });
    return out;
}

template <typename T>
CuArray<int>* CuArray<T>::argsort(int i) {
    auto* out = new CuArray<int>();
    out->init(1, n_);
    std::iota(out->host(), out->host() + n_, 0);
    const T* row = host_ + static_cast<size_t>(i) * n_;
    std::stable_sort(out->host(), out->host() + n_, [row](int a, int b) { return row[a] > row[b]; });
    return out;
}

template <typename T>
CuArrayRow<T>::CuArrayRow(CuArray<T>* a, int i)
    : data_(a->host() + static_cast<size_t>(i) * a->n()), n_(a->n()) {}
template <typename T>
T& CuArrayRow<T>::operator[](int i) const { return data_[i]; }
template <typename T>
int CuArrayRow<T>::n() const { return n_; }
template <typename T>
T* CuArrayRow<T>::data() const { return data_; }

template class CuArray<int>;
template class CuArray<float>;
template class CuArray<double>;
template class CuArrayRow<int>;
template class CuArrayRow<float>;
template class CuArrayRow<double>;
