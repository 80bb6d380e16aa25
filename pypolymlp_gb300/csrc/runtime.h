// Host runtime shared by the C ABI translation units: error reporting,
// device buffers, the uploaded model and batch staging.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "device_model.cuh"
#include "host/flat_tables.h"
#include "host/model_tables.h"
#include "polymlp_gb300.h"

namespace pg {

void set_last_error(const std::string& msg);

// The stream every entry point issues its work on: the calling thread's
// stream set by pg_set_stream (default: the legacy default stream).
cudaStream_t current_stream();

#define PG_CUDA(call)                                                                                     \
    do {                                                                                                  \
        cudaError_t e_ = (call);                                                                          \
        if (e_ != cudaSuccess)                                                                            \
            throw std::runtime_error(std::string("CUDA error: ") + cudaGetErrorString(e_) + " at " #call); \
    } while (0)

template <class F>
int guarded(F&& f) {
    try {
        f();
        return 0;
    } catch (const std::exception& e) {
        set_last_error(e.what());
    } catch (...) {
        set_last_error("unknown error");
    }
    return 1;
}

// Owning device buffer (cudaMalloc/cudaFree).
class DevBuf {
  public:
    DevBuf() = default;
    explicit DevBuf(size_t bytes) { alloc(bytes); }
    ~DevBuf() { release(); }
    DevBuf(const DevBuf&) = delete;
    DevBuf& operator=(const DevBuf&) = delete;
    DevBuf(DevBuf&& o) noexcept : p_(o.p_), n_(o.n_) {
        o.p_ = nullptr;
        o.n_ = 0;
    }
    DevBuf& operator=(DevBuf&& o) noexcept {
        if (this != &o) {
            release();
            p_ = o.p_;
            n_ = o.n_;
            o.p_ = nullptr;
            o.n_ = 0;
        }
        return *this;
    }
    void alloc(size_t bytes) {
        release();
        if (bytes == 0) bytes = 16;
        PG_CUDA(cudaMalloc(&p_, bytes));
        n_ = bytes;
    }
    // grow-only reservation
    void reserve(size_t bytes) {
        if (bytes > n_) alloc(bytes);
    }
    void release() {
        if (p_) cudaFree(p_);
        p_ = nullptr;
        n_ = 0;
    }
    template <class T>
    T* as() const {
        return reinterpret_cast<T*>(p_);
    }
    size_t bytes() const { return n_; }

  private:
    void* p_ = nullptr;
    size_t n_ = 0;
};

// Copies on the current stream that return when the data have arrived (the
// host side may be freed or read right after).
inline void copy_h2d(void* dst, const void* src, size_t bytes) {
    if (!bytes) return;
    const cudaStream_t st = current_stream();
    PG_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, st));
    PG_CUDA(cudaStreamSynchronize(st));
}
inline void copy_d2h(void* dst, const void* src, size_t bytes) {
    if (!bytes) return;
    const cudaStream_t st = current_stream();
    PG_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, st));
    PG_CUDA(cudaStreamSynchronize(st));
}
// Zero device memory, ordered on the current stream.
inline void zero_async(void* dst, size_t bytes) {
    if (bytes) PG_CUDA(cudaMemsetAsync(dst, 0, bytes, current_stream()));
}

template <class V>
void upload(DevBuf& b, const std::vector<V>& v) {
    b.alloc(v.size() * sizeof(V));
    copy_h2d(b.as<void>(), v.data(), v.size() * sizeof(V));
}

// Model uploaded to the device for one precision.
struct DeviceModel {
    DevModel dm{};
    std::vector<DevBuf> bufs;
    void build(const FlatModel& fm, bool fp64);
};

// Batch of structures staged on the device with neighbour lists and per-atom data.
struct DeviceBatch {
    int n_st = 0, n_atoms = 0;
    long long n_pairs = 0;
    std::vector<int> st_atom_off, st_trans_off, types, atom_st;
    std::vector<double> trans, pos;
    double coord_max = 0.0;  // largest |coordinate| or |translation component| of the batch
    DevBuf d_st_atom_off, d_st_trans_off, d_trans, d_pos, d_types, d_atom_st, d_posf, d_transf;
    int n_cl = 0;             // structures searched with a cell list
    DevBuf d_st_cl, d_cl_grid, d_cl_geom, d_cl_bin_start, d_cl_atoms, d_frac, d_tn, d_keys, d_maxcnt;
    DevBuf d_counts, d_nb_off, d_nb_j, d_nb_d, d_nb_df, d_total;
    std::vector<long long> nb_off;  // host copy, only after host_offsets()
    // Host: translations and wrapped positions (NeighborCell), uploaded to the device.
    void upload_structures(const pg_structures* st, int s_begin, int s_end, double cutoff);
    // Device: full neighbour lists (count, scan, fill).
    void build_neighbors(double cutoff, cudaStream_t stream);
    void stage(const pg_structures* st, int s_begin, int s_end, double cutoff, cudaStream_t stream);
    void host_offsets();
    struct DevBatch view(double cutoff) const;
};

// Per-kernel timing with CUDA events on the launching stream (enabled by
// pg_profile_enable or PG_PROFILE=1); read back with pg_profile_read.
class ProfScope {
  public:
    ProfScope(const char* name, cudaStream_t st);
    ~ProfScope();

  private:
    const char* name_;
    cudaStream_t st_;
    cudaEvent_t a_ = nullptr, b_ = nullptr;
};

}  // namespace pg
