// Ridge solve on the device in FP64, replacing solver_ridge
// (src/pypolymlp/mlp_dev/standard/solvers.py:48-84), which calls LAPACK posv
// (Cholesky of X^T X + alpha I, two triangular solves) for each alpha and
// fills the coefficients with 1e30 when the factorisation fails (:40-44).
//
// All alphas are factored together: the shifted matrices A + alpha_a I sit
// side by side in HBM and every launch covers all of them (blockIdx.y = the
// alpha), so the sweep costs the launches of one factorisation and no host
// round trip per alpha or per step.  Blocked right-looking Cholesky
// A = L L^T (lower, column-major, block 64):
//   pg_chol_diag    factor the diagonal block in shared memory,
//   pg_chol_panel   panel rows below it: L21 = A21 L11^-T (one thread per row),
//   pg_chol_update  trailing update A22 -= L21 L21^T (128 x 128 lower tiles,
//                   8 x 8 outputs a thread; the tile of a block decoded from
//                   its index).
// The triangular solves L z = b and L^T x = z run in one block per alpha up to
// F = 4,096, above that blocked (64 columns at a time, the updates over many
// blocks).
// A non-positive or non-finite pivot sets info = column + 1 and stops that
// alpha's factorisation; its solution is filled with 1e30.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "runtime.h"

namespace pg {

constexpr int kCB = 64;

// A[m] = A0 + alphas[m] I for the n matrices (F x F each, column-major).
__global__ void pg_add_diag(double* A, const double* A0, int F, const double* alphas, int n) {
    const size_t ff = (size_t)F * F;
    const size_t tot = ff * n;
    for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < tot; q += (size_t)gridDim.x * blockDim.x) {
        const size_t m = q / ff, r = q % ff;
        const size_t i = r % F, j = r / F;
        A[q] = A0[r] + (i == j ? alphas[m] : 0.0);
    }
}

// Factor A_m[k:k+b, k:k+b] in place (lower), m = blockIdx.x.  info[m] != 0
// stops all later work on that matrix.
__global__ void pg_chol_diag(double* A, int F, int k, int* info) {
    __shared__ double S[kCB][kCB + 1];
    __shared__ int bad;
    const int mi = blockIdx.x;
    A += (size_t)mi * F * F;
    const int b = min(kCB, F - k);
    if (threadIdx.x == 0) bad = 0;
    if (info[mi] != 0) return;
    for (int q = threadIdx.x; q < b * b; q += blockDim.x) {
        const int i = q % b, j = q / b;
        S[i][j] = A[(size_t)(k + j) * F + k + i];
    }
    __syncthreads();
    for (int j = 0; j < b; ++j) {
        if (threadIdx.x == 0) {
            const double d = S[j][j];
            if (!(d > 0.0) || !isfinite(d)) {
                bad = k + j + 1;
            } else {
                S[j][j] = sqrt(d);
            }
        }
        __syncthreads();
        if (bad) break;
        const double djj = S[j][j];
        for (int i = j + 1 + threadIdx.x; i < b; i += blockDim.x) S[i][j] /= djj;
        __syncthreads();
        for (int q = threadIdx.x; q < (b - j - 1) * (b - j - 1); q += blockDim.x) {
            const int i = j + 1 + q % (b - j - 1), c = j + 1 + q / (b - j - 1);
            if (c <= i) S[i][c] -= S[i][j] * S[c][j];
        }
        __syncthreads();
    }
    if (bad) {
        if (threadIdx.x == 0) info[mi] = bad;
        return;
    }
    for (int q = threadIdx.x; q < b * b; q += blockDim.x) {
        const int i = q % b, j = q / b;
        if (j <= i) A[(size_t)(k + j) * F + k + i] = S[i][j];
    }
}

// Rows i >= k+b of matrix blockIdx.y: solve x L11^T = a (forward substitution along the row).
__global__ void pg_chol_panel(double* A, int F, int k, const int* info) {
    __shared__ double L[kCB][kCB + 1];
    const int mi = blockIdx.y;
    if (info[mi] != 0) return;
    A += (size_t)mi * F * F;
    const int b = min(kCB, F - k);
    for (int q = threadIdx.x; q < b * b; q += blockDim.x) {
        const int i = q % b, j = q / b;
        L[i][j] = A[(size_t)(k + j) * F + k + i];
    }
    __syncthreads();
    const int row = k + b + blockIdx.x * blockDim.x + threadIdx.x;
    if (row >= F) return;
    double x[kCB];
    for (int j = 0; j < b; ++j) {
        // four interleaved partial sums: a quarter of the dependent chain
        double v0 = A[(size_t)(k + j) * F + row], v1 = 0.0, v2 = 0.0, v3 = 0.0;
        int p = 0;
        for (; p + 4 <= j; p += 4) {
            v0 -= x[p] * L[j][p];
            v1 -= x[p + 1] * L[j][p + 1];
            v2 -= x[p + 2] * L[j][p + 2];
            v3 -= x[p + 3] * L[j][p + 3];
        }
        for (; p < j; ++p) v0 -= x[p] * L[j][p];
        x[j] = ((v0 + v1) + (v2 + v3)) / L[j][j];
    }
    for (int j = 0; j < b; ++j) A[(size_t)(k + j) * F + row] = x[j];
}

// Lower tile (ti, tj), ti >= tj, of lower-triangle index t (row-major order).
__device__ __forceinline__ void lower_tile(int t, int& ti, int& tj) {
    int i = (int)((sqrt(8.0 * t + 1.0) - 1.0) * 0.5);
    while ((i + 1) * (i + 2) / 2 <= t) ++i;
    while (i * (i + 1) / 2 > t) --i;
    ti = i;
    tj = t - i * (i + 1) / 2;
}

// A22 -= L21 L21^T over the lower triangle of matrix blockIdx.y; block x =
// index of a lower 128 x 128 tile.  The two 128-row panels of L21 (width <=
// kCB) sit in shared memory k-major; thread (ty, tx) of 16 x 16 accumulates
// the 8 x 8 outputs rows ty + 16u, columns tx + 16v (strided, so that a warp's
// loads of a k row are consecutive).
constexpr int kUT = 128;  // update tile
constexpr size_t kUpdSmem = 2 * (size_t)kCB * kUT * sizeof(double);
__global__ void __launch_bounds__(256, 1) pg_chol_update(double* A, int F, int k, const int* info) {
    extern __shared__ double upd[];  // Pi[kCB][kUT], Pj[kCB][kUT]
    double* Pi = upd;
    double* Pj = upd + kCB * kUT;
    const int mi = blockIdx.y;
    if (info[mi] != 0) return;
    A += (size_t)mi * F * F;
    const int b = min(kCB, F - k);
    const int s0 = k + b;
    int ti, tj;
    lower_tile(blockIdx.x, ti, tj);
    const int i0 = s0 + ti * kUT, j0 = s0 + tj * kUT;
    for (int q = threadIdx.x; q < kCB * kUT; q += 256) {
        const int r = q % kUT, p = q / kUT;
        Pi[p * kUT + r] = (i0 + r < F && p < b) ? A[(size_t)(k + p) * F + i0 + r] : 0.0;
        Pj[p * kUT + r] = (j0 + r < F && p < b) ? A[(size_t)(k + p) * F + j0 + r] : 0.0;
    }
    __syncthreads();
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    double acc[8][8];
#pragma unroll
    for (int u = 0; u < 8; ++u)
#pragma unroll
        for (int v = 0; v < 8; ++v) acc[u][v] = 0.0;
    for (int p = 0; p < b; ++p) {
        double a[8], c[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            a[u] = Pi[p * kUT + ty + 16 * u];
            c[u] = Pj[p * kUT + tx + 16 * u];
        }
#pragma unroll
        for (int u = 0; u < 8; ++u)
#pragma unroll
            for (int v = 0; v < 8; ++v) acc[u][v] = fma(a[u], c[v], acc[u][v]);
    }
#pragma unroll
    for (int u = 0; u < 8; ++u)
#pragma unroll
        for (int v = 0; v < 8; ++v) {
            const int i = i0 + ty + 16 * u, j = j0 + tx + 16 * v;
            if (i < F && j < F && j <= i) A[(size_t)j * F + i] -= acc[u][v];
        }
}

// L z = b, then L^T x = z for matrix m = blockIdx.x with right-hand side
// b + m b_stride (b_stride 0: one right-hand side for every matrix); 1024 threads.
__global__ void pg_chol_solve(const double* L, int F, const double* b, long long b_stride, double* x,
                              const int* info) {
    extern __shared__ double v[];  // F entries
    __shared__ double red[32];
    const int mi = blockIdx.x;
    L += (size_t)mi * F * F;
    b += (size_t)mi * b_stride;
    x += (size_t)mi * F;
    if (info[mi] != 0) {
        for (int i = threadIdx.x; i < F; i += blockDim.x) x[i] = 1e30;
        return;
    }
    for (int i = threadIdx.x; i < F; i += blockDim.x) v[i] = b[i];
    __syncthreads();
    for (int j = 0; j < F; ++j) {
        const double zj = v[j] / L[(size_t)j * F + j];
        __syncthreads();
        if (threadIdx.x == 0) v[j] = zj;
        for (int i = j + 1 + threadIdx.x; i < F; i += blockDim.x) v[i] -= L[(size_t)j * F + i] * zj;
        __syncthreads();
    }
    // backward: x_j = (z_j - sum_{i>j} L[i,j] x_i) / L[j,j]
    for (int j = F - 1; j >= 0; --j) {
        double s = 0.0;
        for (int i = j + 1 + threadIdx.x; i < F; i += blockDim.x) s += L[(size_t)j * F + i] * v[i];
        for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
        if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
        __syncthreads();
        if (threadIdx.x < 32) {
            double t = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.0;
            for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
            if (threadIdx.x == 0) v[j] = (v[j] - t) / L[(size_t)j * F + j];
        }
        __syncthreads();
    }
    for (int i = threadIdx.x; i < F; i += blockDim.x) x[i] = v[i];
}

// Factor the n matrices A (F x F each, column-major, lower used) in place;
// d_info (n ints, zeroed by the caller) receives each status.  No host
// synchronisation: the launches are queued on st.
void cholesky_device(double* A, int F, int n, int* d_info, cudaStream_t st) {
    static std::once_flag attr;
    std::call_once(attr, [] {
        PG_CUDA(cudaFuncSetAttribute(pg_chol_update, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kUpdSmem));
    });
    for (int k = 0; k < F; k += kCB) {
        pg_chol_diag<<<n, 256, 0, st>>>(A, F, k, d_info);
        const int b = std::min(kCB, F - k);
        const int rest = F - k - b;
        if (rest <= 0) break;
        pg_chol_panel<<<dim3((unsigned)((rest + 127) / 128), (unsigned)n), 128, 0, st>>>(A, F, k, d_info);
        const int nt = (rest + kUT - 1) / kUT;
        pg_chol_update<<<dim3((unsigned)(nt * (nt + 1) / 2), (unsigned)n), 256, kUpdSmem, st>>>(A, F, k, d_info);
    }
    PG_CUDA(cudaGetLastError());
}

// Blocked triangular solves for large F (many blocks, x in global memory):
// per diagonal block of kTB columns, one block per matrix solves the block
// with the 64 x 64 triangle in shared memory, then a matrix-vector update of
// the rest of x spreads over many blocks.  Forward L z = b, then backward
// L^T x = z, in place in x (blockIdx.y or blockIdx.x = the matrix).
constexpr int kTB = 64;
__global__ void pg_trsv_diag(const double* L, int F, int k0, double* x, const int* info, int backward) {
    __shared__ double S[kTB][kTB + 1];
    __shared__ double xs[kTB];
    const int mi = blockIdx.x;
    if (info[mi] != 0) return;
    L += (size_t)mi * F * F;
    x += (size_t)mi * F;
    const int tb = min(kTB, F - k0), t = threadIdx.x;
    for (int q = t; q < tb * tb; q += blockDim.x) {
        const int r = q % tb, c = q / tb;
        S[r][c] = L[(size_t)(k0 + c) * F + k0 + r];
    }
    double v = t < tb ? x[k0 + t] : 0.0;
    __syncthreads();
    if (!backward) {
        for (int j = 0; j < tb; ++j) {
            if (t == j) xs[j] = v / S[j][j];
            __syncthreads();
            if (t > j && t < tb) v -= S[t][j] * xs[j];
        }
    } else {
        for (int j = tb - 1; j >= 0; --j) {
            if (t == j) xs[j] = v / S[j][j];
            __syncthreads();
            if (t < j) v -= S[j][t] * xs[j];
        }
    }
    if (t < tb) x[k0 + t] = xs[t];
}
// forward: x[r] -= sum_c L[r, k0 + c] x[k0 + c] for r >= k0 + tb;
// backward: x[r] -= sum_c L[k0 + c, r] x[k0 + c] for r < k0.
__global__ void pg_trsv_update(const double* L, int F, int k0, double* x, const int* info, int backward) {
    __shared__ double xs[kTB];
    const int mi = blockIdx.y;
    if (info[mi] != 0) return;
    L += (size_t)mi * F * F;
    x += (size_t)mi * F;
    const int tb = min(kTB, F - k0);
    if (threadIdx.x < tb) xs[threadIdx.x] = x[k0 + threadIdx.x];
    __syncthreads();
    const int r = (backward ? 0 : k0 + tb) + blockIdx.x * blockDim.x + threadIdx.x;
    if (backward ? r >= k0 : r >= F) return;
    double s0 = 0.0, s1 = 0.0;
    if (!backward) {
        int c = 0;
        for (; c + 2 <= tb; c += 2) {
            s0 += L[(size_t)(k0 + c) * F + r] * xs[c];
            s1 += L[(size_t)(k0 + c + 1) * F + r] * xs[c + 1];
        }
        if (c < tb) s0 += L[(size_t)(k0 + c) * F + r] * xs[c];
    } else {
        const double* row = L + (size_t)r * F + k0;
        int c = 0;
        for (; c + 2 <= tb; c += 2) {
            s0 += row[c] * xs[c];
            s1 += row[c + 1] * xs[c + 1];
        }
        if (c < tb) s0 += row[c] * xs[c];
    }
    x[r] -= s0 + s1;
}
__global__ void pg_trsv_init(int F, const double* b, long long b_stride, double* x, const int* info) {
    const int mi = blockIdx.y;
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= F) return;
    x[(size_t)mi * F + r] = info[mi] != 0 ? 1e30 : b[(size_t)mi * b_stride + r];
}

// Up to kSolveOneBlockF one block per matrix (F-vector in shared memory, no
// launch per block column); above it the blocked solves.
constexpr int kSolveOneBlockF = 4096;
void chol_solve_device(const double* L, int F, int n, const double* b, long long b_stride, double* x,
                       const int* d_info, cudaStream_t st) {
    if (F <= kSolveOneBlockF) {
        const size_t smem = (size_t)F * sizeof(double);
        PG_CUDA(cudaFuncSetAttribute(pg_chol_solve, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        pg_chol_solve<<<n, 1024, smem, st>>>(L, F, b, b_stride, x, d_info);
        PG_CUDA(cudaGetLastError());
        return;
    }
    const unsigned rows = (unsigned)((F + 255) / 256);
    pg_trsv_init<<<dim3(rows, (unsigned)n), 256, 0, st>>>(F, b, b_stride, x, d_info);
    for (int k0 = 0; k0 < F; k0 += kTB) {
        pg_trsv_diag<<<n, kTB, 0, st>>>(L, F, k0, x, d_info, 0);
        const int rest = F - k0 - std::min(kTB, F - k0);
        if (rest > 0)
            pg_trsv_update<<<dim3((unsigned)((rest + 255) / 256), (unsigned)n), 256, 0, st>>>(L, F, k0, x, d_info, 0);
    }
    for (int k0 = (F - 1) / kTB * kTB; k0 >= 0; k0 -= kTB) {
        pg_trsv_diag<<<n, kTB, 0, st>>>(L, F, k0, x, d_info, 1);
        if (k0 > 0)
            pg_trsv_update<<<dim3((unsigned)((k0 + 255) / 256), (unsigned)n), 256, 0, st>>>(L, F, k0, x, d_info, 1);
    }
    PG_CUDA(cudaGetLastError());
}


// (A + alpha_a I) x_a = rhs_a for every alpha: rhs is F x n_alpha with
// rhs_stride F (one right-hand side per alpha) or 0 (the same for all).
void ridge_batched(int F, const double* xtx, const double* rhs, long long rhs_stride, const double* alphas,
                   int n_alpha, double* coefs, int* info) {
    if (F <= 0 || !xtx || !rhs || !alphas || !coefs || !info || n_alpha < 0) throw std::runtime_error("bad arguments");
    if (n_alpha == 0) return;
    cudaStream_t st = current_stream();
    const size_t ff = (size_t)F * F * sizeof(double);
    // as many alphas per group as half the free memory holds
    size_t free_b = 0, total_b = 0;
    PG_CUDA(cudaMemGetInfo(&free_b, &total_b));
    const int group = (int)std::max<size_t>(1, std::min<size_t>((size_t)n_alpha, free_b / 2 / ff));
    DevBuf A0(ff), A(ff * group), b((size_t)F * n_alpha * 8), x((size_t)F * group * 8), al(n_alpha * 8),
        d_info(sizeof(int) * group);
    PG_CUDA(cudaMemcpyAsync(A0.as<void>(), xtx, ff, cudaMemcpyHostToDevice, st));
    const size_t nb = rhs_stride ? (size_t)F * n_alpha : (size_t)F;
    PG_CUDA(cudaMemcpyAsync(b.as<void>(), rhs, nb * 8, cudaMemcpyHostToDevice, st));
    PG_CUDA(cudaMemcpyAsync(al.as<void>(), alphas, (size_t)n_alpha * 8, cudaMemcpyHostToDevice, st));
    for (int a0 = 0; a0 < n_alpha; a0 += group) {
        const int n = std::min(group, n_alpha - a0);
        pg_add_diag<<<2048, 256, 0, st>>>(A.as<double>(), A0.as<double>(), F, al.as<double>() + a0, n);
        PG_CUDA(cudaMemsetAsync(d_info.as<void>(), 0, sizeof(int) * n, st));
        cholesky_device(A.as<double>(), F, n, d_info.as<int>(), st);
        chol_solve_device(A.as<double>(), F, n, b.as<double>() + (rhs_stride ? (size_t)a0 * F : 0),
                          rhs_stride ? F : 0, x.as<double>(), d_info.as<int>(), st);
        PG_CUDA(cudaMemcpyAsync(coefs + (size_t)a0 * F, x.as<double>(), (size_t)F * n * 8, cudaMemcpyDeviceToHost, st));
        PG_CUDA(cudaMemcpyAsync(info + a0, d_info.as<int>(), sizeof(int) * n, cudaMemcpyDeviceToHost, st));
        PG_CUDA(cudaStreamSynchronize(st));
    }
}

}  // namespace pg

using namespace pg;

extern "C" int pg_solve_ridge(int F, const double* xtx, const double* xty, const double* alphas, int n_alpha,
                              double* coefs, int* info) {
    return guarded([&] { ridge_batched(F, xtx, xty, 0, alphas, n_alpha, coefs, info); });
}

extern "C" int pg_solve_ridge_rhs(int F, const double* xtx, const double* rhs, const double* alphas, int n_alpha,
                                  double* coefs, int* info) {
    return guarded([&] { ridge_batched(F, xtx, rhs, F, alphas, n_alpha, coefs, info); });
}

// ---------------------------------------------------------------------------
// Ridge solve that allocates no memory.
//
// Some callers cannot allocate device memory when they solve: code that runs
// inside an inference server or a host framework whose allocator owns every
// byte of the GPU (a cudaMalloc of ours would fail or would fragment its
// pool), or a real-time loop that must never enter the allocator.  They hand
// over device buffers they already own.  This variant of the blocked
// Cholesky solve keeps its workspace (the factor of xtx + alpha I and the
// status word) in one file-scope device array instead of cudaMalloc'ed
// buffers.
//
// Limits and sharing: n_features <= kNoAllocMaxF (1024); every GPU that loads
// this library holds the array (8 MiB + 256 bytes) until the process exits.
// All calls on a device share the one array and it keeps the last call's
// contents (the status word is cleared at the start of each call), so calls
// whose GPU work overlaps - from several host threads or streams - race on it.
constexpr int kNoAllocMaxF = 1024;
constexpr size_t kNoAllocBytes = (size_t)kNoAllocMaxF * kNoAllocMaxF * sizeof(double) + 256;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

namespace {
std::mutex g_noalloc_mu;
void* g_noalloc_ptr[64] = {};  // device address of the array, per device (set up once)
}  // namespace

// Device address of g_noalloc_scratch on the current device.  The first call on
// a device looks it up with cudaGetSymbolAddress (no allocation).
static unsigned char* noalloc_scratch() {
    int dev = 0;
    PG_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) throw std::runtime_error("device index out of range");
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (!g_noalloc_ptr[dev]) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess)
            throw std::runtime_error(std::string("cudaGetSymbolAddress failed: ") + cudaGetErrorString(e));
        g_noalloc_ptr[dev] = p;
    }
    return static_cast<unsigned char*>(g_noalloc_ptr[dev]);
}

// A = A0 + alpha I (one matrix, alpha by value).
__global__ void pg_add_diag1(double* A, const double* A0, int F, double alpha) {
    const size_t n = (size_t)F * F;
    for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < n; q += (size_t)gridDim.x * blockDim.x) {
        const size_t i = q % F, j = q / F;
        A[q] = A0[q] + (i == j ? alpha : 0.0);
    }
}

extern "C" int pg_solve_ridge_noalloc(int F, const double* d_xtx, const double* d_xty, double alpha,
                                      double* d_coefs, int* info) {
    return guarded([&] {
        if (!d_xtx || !d_xty || !d_coefs || !info) throw std::runtime_error("null argument");
        if (F <= 0) throw std::runtime_error("n_features must be positive");
        if (F > kNoAllocMaxF)
            throw std::runtime_error("pg_solve_ridge_noalloc: n_features " + std::to_string(F) +
                                     " exceeds the maximum of " + std::to_string(kNoAllocMaxF) +
                                     " (use pg_solve_ridge)");
        cudaStream_t st = 0;
        unsigned char* base = noalloc_scratch();
        double* A = reinterpret_cast<double*>(base);
        int* d_info = reinterpret_cast<int*>(base + (size_t)kNoAllocMaxF * kNoAllocMaxF * sizeof(double));
        PG_CUDA(cudaMemsetAsync(d_info, 0, sizeof(int), st));
        pg_add_diag1<<<1024, 256, 0, st>>>(A, d_xtx, F, alpha);
        cholesky_device(A, F, 1, d_info, st);
        chol_solve_device(A, F, 1, d_xty, 0, d_coefs, d_info, st);
        PG_CUDA(cudaMemcpyAsync(info, d_info, sizeof(int), cudaMemcpyDeviceToHost, st));
        PG_CUDA(cudaStreamSynchronize(st));
    });
}
