// Uploaded model (tables + device views) and the per-batch X-row pipeline.
#pragma once

#include <memory>
#include <utility>
#include <vector>

#include "kernels.h"
#include "runtime.h"

namespace pg {

// Per-batch offsets of per-atom data.
struct RowPlan {
    long long a_tot = 0, d_tot = 0, g_tot = 0, s_tot = 0;
    DevBuf d_a_off, d_d_off, d_g_off, d_s_off;
};

struct AtomOffsets {
    std::vector<long long> a_off, d_off, g_off, s_off;
    long long a_tot = 0, d_tot = 0, g_tot = 0, s_tot = 0;
};

struct Model {
    ModelTables tables;
    FlatModel flat;
    DeviceModel dev64, dev32;   // device tables and pg_rows block shapes for FP64 and FP32
    int max_k = 1, max_k0 = 1;
    // per-batch scratch (grow-only)
    DevBuf s_A, s_D, s_G, s_DS, s_Dp, s_mirror, s_gslot, s_order, s_missing;

    explicit Model(const pg_feature_params* p);

    void atom_offsets(const DeviceBatch& b, AtomOffsets& o) const;
    size_t bytes_per_atom(bool fp64, double mean_pairs) const;
    std::vector<std::pair<int, int>> plan_batches(const pg_structures* st, bool fp64, size_t limit) const;

    void plan_rows(const DeviceBatch& b, RowPlan& plan) const;
    template <typename T>
    void run_rows(DeviceBatch& b, const RowPlan& plan, const long long* d_e_row, const long long* d_f_row,
                  const long long* d_s_row, T* Xd, long long ld, cudaStream_t stream);
    void check_mirrors();
    template <typename T>
    void batch_rows(DeviceBatch& b, const long long* d_e_row, const long long* d_f_row, const long long* d_s_row,
                    T* Xd, long long ld, cudaStream_t stream);
};

size_t device_batch_bytes();

}  // namespace pg

// Opaque C handle of a model (include/polymlp_gb300.h).
struct pg_model {
    std::unique_ptr<pg::Model> m;
};
