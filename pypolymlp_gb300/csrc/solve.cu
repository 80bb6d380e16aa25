// Ridge solve on the device in FP64, replacing solver_ridge
// (src/pypolymlp/mlp_dev/standard/solvers.py:48-84), which calls LAPACK posv
// (Cholesky of X^T X + alpha I, two triangular solves) for each alpha and
// fills the coefficients with 1e30 when the factorisation fails (:40-44).
//
// Blocked right-looking Cholesky A = L L^T (lower, column-major, block 64):
//   pg_chol_diag    factor the diagonal block in shared memory (one block),
//   pg_chol_panel   panel rows below it: L21 = A21 L11^-T (one thread per row),
//   pg_chol_update  trailing update A22 -= L21 L21^T (64x64 tiles, lower only).
// Triangular solves L z = b and L^T x = z run in one block each.
// A non-positive or non-finite pivot sets info = column + 1 and stops.
#include <cuda_runtime.h>

#include <cmath>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "runtime.h"

namespace pg {

constexpr int kCB = 64;

__global__ void pg_add_diag(double* A, const double* A0, int F, double alpha) {
    const size_t n = (size_t)F * F;
    for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < n; q += (size_t)gridDim.x * blockDim.x) {
        const size_t i = q % F, j = q / F;
        A[q] = A0[q] + (i == j ? alpha : 0.0);
    }
}

// Factor A[k:k+b, k:k+b] in place (lower).  info[0] != 0 stops all later work.
__global__ void pg_chol_diag(double* A, int F, int k, int* info) {
    __shared__ double S[kCB][kCB + 1];
    __shared__ int bad;
    const int b = min(kCB, F - k);
    if (threadIdx.x == 0) bad = 0;
    if (*info != 0) return;
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
        if (threadIdx.x == 0) *info = bad;
        return;
    }
    for (int q = threadIdx.x; q < b * b; q += blockDim.x) {
        const int i = q % b, j = q / b;
        if (j <= i) A[(size_t)(k + j) * F + k + i] = S[i][j];
    }
}

// Rows i >= k+b: solve x L11^T = a (forward substitution along the row).
__global__ void pg_chol_panel(double* A, int F, int k, const int* info) {
    __shared__ double L[kCB][kCB + 1];
    if (*info != 0) return;
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
        double v = A[(size_t)(k + j) * F + row];
        for (int p = 0; p < j; ++p) v -= x[p] * L[j][p];
        x[j] = v / L[j][j];
    }
    for (int j = 0; j < b; ++j) A[(size_t)(k + j) * F + row] = x[j];
}

// A22 -= L21 L21^T over the lower triangle; tiles listed by (ti, tj), ti >= tj.
__global__ void __launch_bounds__(256) pg_chol_update(double* A, int F, int k, const int2* tiles, const int* info) {
    __shared__ double Pi[kCB][kCB + 1];
    __shared__ double Pj[kCB][kCB + 1];
    if (*info != 0) return;
    const int b = min(kCB, F - k);
    const int s0 = k + b;
    const int2 t = tiles[blockIdx.x];
    const int i0 = s0 + t.x * kCB, j0 = s0 + t.y * kCB;
    for (int q = threadIdx.x; q < kCB * kCB; q += 256) {
        const int r = q % kCB, p = q / kCB;
        Pi[r][p] = (i0 + r < F && p < b) ? A[(size_t)(k + p) * F + i0 + r] : 0.0;
        Pj[r][p] = (j0 + r < F && p < b) ? A[(size_t)(k + p) * F + j0 + r] : 0.0;
    }
    __syncthreads();
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    double acc[4][4] = {};
    for (int p = 0; p < b; ++p) {
        double a[4], c[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            a[u] = Pi[ty * 4 + u][p];
            c[u] = Pj[tx * 4 + u][p];
        }
#pragma unroll
        for (int u = 0; u < 4; ++u)
#pragma unroll
            for (int v = 0; v < 4; ++v) acc[u][v] = fma(a[u], c[v], acc[u][v]);
    }
#pragma unroll
    for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int v = 0; v < 4; ++v) {
            const int i = i0 + ty * 4 + u, j = j0 + tx * 4 + v;
            if (i < F && j < F && j <= i) A[(size_t)j * F + i] -= acc[u][v];
        }
}

// L z = b, then L^T x = z; one block of 1024 threads.
__global__ void pg_chol_solve(const double* L, int F, const double* b, double* x, const int* info) {
    extern __shared__ double v[];  // F entries
    __shared__ double red[32];
    if (*info != 0) {
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

// Factor A (F x F, column-major, lower used) in place; returns info.
int cholesky_device(double* A, int F, int* d_info, cudaStream_t st) {
    std::vector<int2> tiles;
    DevBuf d_tiles;
    for (int k = 0; k < F; k += kCB) {
        pg_chol_diag<<<1, 256, 0, st>>>(A, F, k, d_info);
        const int b = std::min(kCB, F - k);
        const int rest = F - k - b;
        if (rest <= 0) break;
        pg_chol_panel<<<(rest + 127) / 128, 128, 0, st>>>(A, F, k, d_info);
        const int nt = (rest + kCB - 1) / kCB;
        tiles.clear();
        for (int i = 0; i < nt; ++i)
            for (int j = 0; j <= i; ++j) tiles.push_back(make_int2(i, j));
        upload(d_tiles, tiles);
        pg_chol_update<<<(int)tiles.size(), 256, 0, st>>>(A, F, k, d_tiles.as<int2>(), d_info);
    }
    PG_CUDA(cudaGetLastError());
    int info = 0;
    PG_CUDA(cudaMemcpyAsync(&info, d_info, sizeof(int), cudaMemcpyDeviceToHost, st));
    PG_CUDA(cudaStreamSynchronize(st));
    return info;
}

}  // namespace pg

using namespace pg;

extern "C" int pg_solve_ridge(int F, const double* xtx, const double* xty, const double* alphas, int n_alpha,
                              double* coefs, int* info) {
    return guarded([&] {
        if (F <= 0 || !xtx || !xty || !alphas || !coefs || !info) throw std::runtime_error("bad arguments");
        if ((size_t)F * sizeof(double) > 200 * 1024) throw std::runtime_error("n_features too large for the solver");
        cudaStream_t st = 0;
        DevBuf A0((size_t)F * F * 8), A((size_t)F * F * 8), b(F * 8), x(F * 8), d_info(sizeof(int));
        PG_CUDA(cudaMemcpy(A0.as<void>(), xtx, (size_t)F * F * 8, cudaMemcpyHostToDevice));
        PG_CUDA(cudaMemcpy(b.as<void>(), xty, (size_t)F * 8, cudaMemcpyHostToDevice));
        const size_t smem = (size_t)F * sizeof(double);
        PG_CUDA(cudaFuncSetAttribute(pg_chol_solve, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        for (int a = 0; a < n_alpha; ++a) {
            pg_add_diag<<<1024, 256, 0, st>>>(A.as<double>(), A0.as<double>(), F, alphas[a]);
            PG_CUDA(cudaMemsetAsync(d_info.as<void>(), 0, sizeof(int), st));
            info[a] = cholesky_device(A.as<double>(), F, d_info.as<int>(), st);
            pg_chol_solve<<<1, 1024, smem, st>>>(A.as<double>(), F, b.as<double>(), x.as<double>(), d_info.as<int>());
            PG_CUDA(cudaGetLastError());
            PG_CUDA(cudaMemcpy(coefs + (size_t)a * F, x.as<double>(), (size_t)F * 8, cudaMemcpyDeviceToHost));
        }
    });
}

// ---------------------------------------------------------------------------
// Factor once, solve many: the Cholesky factor of xtx + alpha I kept on the
// device, for preconditioned iterations that apply its inverse repeatedly.
struct pg_ridge_factor {
    int F = 0;
    DevBuf L, b, x, info;
};

extern "C" int pg_ridge_factor_create(int F, const double* xtx, double alpha, pg_ridge_factor** out, int* info) {
    return guarded([&] {
        if (F <= 0 || !xtx || !out || !info) throw std::runtime_error("bad arguments");
        if ((size_t)F * sizeof(double) > 200 * 1024) throw std::runtime_error("n_features too large for the solver");
        auto f = std::make_unique<pg_ridge_factor>();
        f->F = F;
        DevBuf A0((size_t)F * F * 8);
        f->L.alloc((size_t)F * F * 8);
        f->b.alloc((size_t)F * 8);
        f->x.alloc((size_t)F * 8);
        f->info.alloc(sizeof(int));
        PG_CUDA(cudaMemcpy(A0.as<void>(), xtx, (size_t)F * F * 8, cudaMemcpyHostToDevice));
        pg_add_diag<<<1024, 256, 0, 0>>>(f->L.as<double>(), A0.as<double>(), F, alpha);
        PG_CUDA(cudaMemset(f->info.as<void>(), 0, sizeof(int)));
        *info = cholesky_device(f->L.as<double>(), F, f->info.as<int>(), 0);
        *out = f.release();
    });
}

extern "C" int pg_ridge_factor_solve(pg_ridge_factor* f, const double* rhs, int n_rhs, double* x) {
    return guarded([&] {
        if (!f || !rhs || !x || n_rhs < 0) throw std::runtime_error("bad arguments");
        const int F = f->F;
        const size_t smem = (size_t)F * sizeof(double);
        PG_CUDA(cudaFuncSetAttribute(pg_chol_solve, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        for (int q = 0; q < n_rhs; ++q) {
            PG_CUDA(cudaMemcpy(f->b.as<void>(), rhs + (size_t)q * F, (size_t)F * 8, cudaMemcpyHostToDevice));
            pg_chol_solve<<<1, 1024, smem, 0>>>(f->L.as<double>(), F, f->b.as<double>(), f->x.as<double>(),
                                               f->info.as<int>());
            PG_CUDA(cudaGetLastError());
            PG_CUDA(cudaMemcpy(x + (size_t)q * F, f->x.as<double>(), (size_t)F * 8, cudaMemcpyDeviceToHost));
        }
    });
}

extern "C" int pg_ridge_factor_destroy(pg_ridge_factor* f) {
    return guarded([&] { delete f; });
}

// ---------------------------------------------------------------------------
// Ridge solve that allocates no memory.
//
// Some callers cannot allocate device memory when they solve: code that runs
// inside an inference server or a host framework whose allocator owns every
// byte of the GPU, code that runs while a CUDA stream is being captured (where
// cudaMalloc is not allowed), or a real-time loop that must not touch the
// allocator.  They hand over device buffers they already own.  This variant of
// the blocked Cholesky solve keeps its workspace (the factor of
// xtx + alpha I, the list of update tiles and the status word) in one
// file-scope device array instead of cudaMalloc'ed buffers.
//
// Limits and sharing: n_features <= kNoAllocMaxF (1024); every GPU that loads
// this library holds the array (8 MiB + a few KiB) until the process exits.
// All calls on a device share the one array and it keeps the last call's
// contents (the status word is cleared at the start of each call), so calls
// whose GPU work overlaps - from several host threads or streams - race on it.
constexpr int kNoAllocMaxF = 1024;
constexpr int kNoAllocMaxTiles = (kNoAllocMaxF / kCB) * (kNoAllocMaxF / kCB + 1) / 2;
constexpr size_t kNoAllocBytes = (size_t)kNoAllocMaxF * kNoAllocMaxF * sizeof(double) +
                                 (size_t)kNoAllocMaxTiles * sizeof(int2) + 256;

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
        int2* tiles = reinterpret_cast<int2*>(base + (size_t)kNoAllocMaxF * kNoAllocMaxF * sizeof(double));
        int* d_info = reinterpret_cast<int*>(reinterpret_cast<unsigned char*>(tiles) +
                                             (size_t)kNoAllocMaxTiles * sizeof(int2));
        PG_CUDA(cudaMemsetAsync(d_info, 0, sizeof(int), st));
        pg_add_diag<<<1024, 256, 0, st>>>(A, d_xtx, F, alpha);
        std::vector<int2> tl;
        for (int k = 0; k < F; k += kCB) {
            pg_chol_diag<<<1, 256, 0, st>>>(A, F, k, d_info);
            const int b = std::min(kCB, F - k);
            const int rest = F - k - b;
            if (rest <= 0) break;
            pg_chol_panel<<<(rest + 127) / 128, 128, 0, st>>>(A, F, k, d_info);
            const int nt = (rest + kCB - 1) / kCB;
            tl.clear();
            for (int i = 0; i < nt; ++i)
                for (int j = 0; j <= i; ++j) tl.push_back(make_int2(i, j));
            // the tile list of this step is consumed by the next kernel on the same stream
            PG_CUDA(cudaMemcpyAsync(tiles, tl.data(), tl.size() * sizeof(int2), cudaMemcpyHostToDevice, st));
            pg_chol_update<<<(int)tl.size(), 256, 0, st>>>(A, F, k, tiles, d_info);
            PG_CUDA(cudaStreamSynchronize(st));  // the host tile list is reused next step
        }
        const size_t smem = (size_t)F * sizeof(double);
        PG_CUDA(cudaFuncSetAttribute(pg_chol_solve, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        pg_chol_solve<<<1, 1024, smem, st>>>(A, F, d_xty, d_coefs, d_info);
        PG_CUDA(cudaGetLastError());
        PG_CUDA(cudaMemcpyAsync(info, d_info, sizeof(int), cudaMemcpyDeviceToHost, st));
        PG_CUDA(cudaStreamSynchronize(st));
    });
}
