// Device-side batch view and host launchers of the CUDA kernels.
#pragma once

#include <cuda_runtime.h>

#include "device_model.cuh"
#include "runtime.h"

namespace pg {

// --------------------------------------------------------------- batch view
struct DevBatch {
    int n_st;
    int n_atoms;
    const int* st_atom_off;    // n_st + 1
    const int* st_trans_off;   // n_st + 1
    const double* trans;       // 3 per translation
    const double* pos;         // 3 per atom (wrapped as NeighborCell does)
    const int* types;          // per atom
    const int* atom_st;        // per atom: structure index
    const float4* posf;        // FP32 copies of pos (w unused), for the candidate pre-filter
    const float4* transf;      // FP32 copies of trans
    double cutoff;
    float prefilter_r2;        // FP32 squared distance above which a candidate is surely beyond the cutoff
    float inner_r2;            // FP32 squared distance below which a candidate is surely inside it
    // cell lists of the large structures (st_cl[s] >= 0): per such structure a
    // grid of bins over its atoms' fractional coordinates
    const int* st_cl;          // per structure: cell-list index or -1
    const int4* cl_grid;       // per cell list: bins along the three axes, first bin
    const double* cl_geom;     // per cell list: fmin[3], bins per fractional unit[3], query radius[3]
    const int* cl_bin_start;   // per bin (all cell lists) + 1: start in cl_atoms
    const int* cl_atoms;       // batch atom indices, by bin then index
    const double* frac;        // per atom: fractional coordinates on the reduced axis (cell-list structures)
    const int4* tn;            // per translation: its integer coefficients
    // per neighbour-list entry: FP32 displacement and squared distance (after
    // the lists are built), for the FP32 kernels
    const float4* nb_df;
};

// Displacement and distance of neighbour-list entry k in T, and whether the
// pair counts: sqrt(dx^2 + dy^2 + dz^2) < cutoff in FP64 (local.cpp's test).
// The FP32 form decides from the FP32 squared distance when it is clearly
// inside and falls back to the FP64 test near the cutoff.  Warp-uniform.
template <typename T>
__device__ __forceinline__ bool pair_geometry(const DevModel& M, const DevBatch& B, const double* nb_d, long long k,
                                              T& dx, T& dy, T& dz, T& dis);
template <>
__device__ __forceinline__ bool pair_geometry<double>(const DevModel& M, const DevBatch& B, const double* nb_d,
                                                      long long k, double& dx, double& dy, double& dz, double& dis) {
    dx = nb_d[3 * k];
    dy = nb_d[3 * k + 1];
    dz = nb_d[3 * k + 2];
    dis = sqrt(__dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz)));
    return dis < M.cutoff;
}
template <>
__device__ __forceinline__ bool pair_geometry<float>(const DevModel& M, const DevBatch& B, const double* nb_d,
                                                     long long k, float& dx, float& dy, float& dz, float& dis) {
    const float4 g = B.nb_df[k];
    dx = g.x;
    dy = g.y;
    dz = g.z;
    dis = sqrtf(g.w);
    if (g.w < M.rc2_safe_f) return true;
    const double ex = nb_d[3 * k], ey = nb_d[3 * k + 1], ez = nb_d[3 * k + 2];
    return sqrt(__dadd_rn(__dadd_rn(__dmul_rn(ex, ex), __dmul_rn(ey, ey)), __dmul_rn(ez, ez))) < M.cutoff;
}

constexpr int kCellListMinAtoms = 1024;  // structures this large use a cell list
constexpr int kCellListMaxPairs = 4096;  // per atom, for the in-block ordering

constexpr int kRowsThreads = 256;  // threads of pg_rows / pg_rows_pairs blocks
constexpr int kMaxTypePairs = 64;
constexpr int kMaxSuperChunk = 32;  // pairs per stage-A super-chunk (at most)

void launch_nb_count(const DevBatch& B, int* counts, int* max_cl, cudaStream_t st);
void launch_nb_fill(const DevBatch& B, const long long* off, int* nb_j, double* nb_d, float4* nb_df, long long* keys,
                    bool any_cl, cudaStream_t st);
// Displacements of the existing list entries (keys[q] = entry q's neighbour and
// translation) from the batch's current positions.
void launch_nb_refresh(const DevBatch& B, const long long* off, const long long* keys, int* nb_j, double* nb_d,
                       float4* nb_df, cudaStream_t st);
template <typename T>
void launch_anlm(const DevModel& M, const DevBatch& B, const long long* nb_off, const int* nb_j, const double* nb_d,
                 const long long* a_off, void* A, int max_k0, cudaStream_t st);
template <typename T>
void launch_features_adjoint(const DevModel& M, const DevBatch& B, const long long* a_off, const void* A,
                             const long long* d_off, T* D, const long long* g_off, void* G, int max_k,
                             cudaStream_t st);
void launch_exclusive_scan(const int* counts, int n, long long* offsets, long long* total, cudaStream_t st);
size_t rows_pairs_smem_bytes(const DevModel& M, bool fp64, int ps);
int rows_pairs_chunk(const DevModel& M, bool fp64);
void launch_nb_mirror(int n_atoms, const long long* nb_off, const int* nb_j, const double* nb_d, long long* mirror,
                      long long* gslot, int* missing, cudaStream_t st);
template <typename T>
void launch_rows_pairs(const DevModel& M, const DevBatch& B, const long long* nb_off, const int* nb_j,
                       const double* nb_d, const long long* gslot, const long long* s_off, const long long* g_off,
                       const void* G, const long long* f_row, int* order, T* Dp, T* DS, cudaStream_t st);
template <typename T>
void launch_rows(const DevModel& M, const DevBatch& B, const long long* nb_off, const int* nb_j,
                 const long long* d_off, const T* D, const T* Dp, const long long* s_off, const T* DS,
                 const long long* f_row, T* X, long long ld, cudaStream_t st);
template <typename T>
void launch_rows_es(const DevModel& M, const DevBatch& B, const long long* d_off, const T* D, const long long* s_off,
                    const T* DS, const long long* e_row, const long long* f_row, const long long* s_row, T* X,
                    long long ld, cudaStream_t st);

// Tensor-core Gram (gram_tc.cu): scratch (the four BF16 fixed-point slices
// of X and their exponents per segment and column, work units, float-float
// partial tiles of the row splits, error flag) and entry points.
struct GramTcScratch {
    DevBuf H, E, units, P, err;
    int n_units = 0, n_splits = 0, F = 0;
    long long rows = -1;
};
void gram_tc_accumulate(const float* X, long long ld, long long rows, int F, double* G, GramTcScratch& S,
                        cudaStream_t st);
void gram_tc_check(GramTcScratch& S);

}  // namespace pg
