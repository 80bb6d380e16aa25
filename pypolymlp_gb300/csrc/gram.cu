// Regression assembly on the device: X^T X, X^T y, y^T y and the energy-row
// column statistics, replacing the numpy loop of calc_xtx_xty
// (src/pypolymlp/mlp_dev/core/data_sequential.py:97-153) with X generated in
// HBM by pg_rows.
//
//   pg_syrk_f64        FP64 path: upper-triangle tiles of X^T X on the
//                      CUDA cores (64x64 tile per block, 4x4 per thread).
//   gram_tc (file gram_tc.cu) mixed path: X (FP32) split into four BF16
//                      fixed-point slices per 1,024-row segment, 13 slice
//                      products on the tcgen05 tensor cores with exact FP32
//                      partial sums, float-float segment sums: the Gram of
//                      the FP32 rows to ~1e-12.
//   helpers            energy-row sums, row weighting, X^T y.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstring>
#include <memory>

#include "kernels.h"
#include "model.h"

namespace pg {


// ------------------------------------------------------------ statistics
// xe_sum[c] += sum_r X[e_rows[r], c], xe_sq_sum[c] += sum X^2 (unweighted energy rows).
template <typename T>
__global__ void pg_energy_stats(const T* X, long long ld, int F, const long long* e_rows, int n_e, double* xe_sum,
                                double* xe_sq) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= F) return;
    double s = 0, q = 0;
    for (int r = 0; r < n_e; ++r) {
        const double v = (double)X[(size_t)c * ld + e_rows[r]];
        s += v;
        q += v * v;
    }
    xe_sum[c] += s;
    xe_sq[c] += q;
}

// X[r, c] *= w[r]
template <typename T>
__global__ void pg_scale_rows(T* X, long long ld, long long n_rows, int F, const double* w) {
    const long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (r >= n_rows) return;
    const T wr = (T)w[r];
    for (int c = blockIdx.y; c < F; c += gridDim.y) X[(size_t)c * ld + r] *= wr;
}

// xty[c] += sum_r X[r, c] * y[r]  (one block per column, FP64 accumulation)
template <typename T>
__global__ void pg_xty(const T* X, long long ld, long long n_rows, const double* y, double* xty) {
    const int c = blockIdx.x;
    double s = 0;
    for (long long r = threadIdx.x; r < n_rows; r += blockDim.x) s += (double)X[(size_t)c * ld + r] * y[r];
    __shared__ double red[256];
    red[threadIdx.x] = s;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) xty[c] += red[0];
}

// ------------------------------------------------------------ FP64 SYRK
// G (F x F, column-major, upper triangle used) += X^T X over rows [0, n_rows).
constexpr int kS64 = 64, kK64 = 16;

__global__ void __launch_bounds__(256) pg_syrk_f64(const double* X, long long ld, long long n_rows, int F,
                                                   const int2* tiles, double* G) {
    const int2 tl = tiles[blockIdx.x];
    const int i0 = tl.x * kS64, j0 = tl.y * kS64;
    __shared__ double As[kK64][kS64 + 1];
    __shared__ double Bs[kK64][kS64 + 1];
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    double acc[4][4] = {};
    for (long long k0 = 0; k0 < n_rows; k0 += kK64) {
        // load: 16 rows x 64 columns each (row index fastest -> coalesced)
        for (int q = threadIdx.x; q < kK64 * kS64; q += 256) {
            const int kk = q % kK64, cc = q / kK64;
            const long long r = k0 + kk;
            const int ci = i0 + cc, cj = j0 + cc;
            As[kk][cc] = (r < n_rows && ci < F) ? X[(size_t)ci * ld + r] : 0.0;
            Bs[kk][cc] = (r < n_rows && cj < F) ? X[(size_t)cj * ld + r] : 0.0;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < kK64; ++kk) {
            double a[4], b[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                a[u] = As[kk][ty * 4 + u];
                b[u] = Bs[kk][tx * 4 + u];
            }
#pragma unroll
            for (int u = 0; u < 4; ++u)
#pragma unroll
                for (int v = 0; v < 4; ++v) acc[u][v] = fma(a[u], b[v], acc[u][v]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int v = 0; v < 4; ++v) {
            const int i = i0 + ty * 4 + u, j = j0 + tx * 4 + v;
            if (i < F && j < F && i <= j) G[(size_t)j * F + i] += acc[u][v];
        }
}

// Mirror the upper triangle into the lower one.
__global__ void pg_symmetrize(double* G, int F) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = blockIdx.y;
    if (j < F && i < j) G[(size_t)i * F + j] = G[(size_t)j * F + i];
}

void launch_syrk_f64(const double* X, long long ld, long long n_rows, int F, const int2* tiles, int n_tiles,
                     double* G, cudaStream_t st) {
    pg_syrk_f64<<<n_tiles, 256, 0, st>>>(X, ld, n_rows, F, tiles, G);
}



// ------------------------------------------------------------ residuals
constexpr int kMaxCoef = 16;

// R[row, k] = y[row] - sum_c X[row, c] C[c, k]  (FP64 accumulation, one thread per row)
template <typename T>
__global__ void pg_residual(const T* X, long long ld, long long rows, int F, const double* C, int nc,
                            const double* y, double* R) {
    const long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (r >= rows) return;
    double acc[kMaxCoef];
    for (int k = 0; k < nc; ++k) acc[k] = 0.0;
    for (int c = 0; c < F; ++c) {
        const double x = (double)X[(size_t)c * ld + r];
        for (int k = 0; k < nc; ++k) acc[k] += x * C[(size_t)k * F + c];
    }
    const double yr = y ? y[r] : 0.0;  // no targets: R = -X C
    for (int k = 0; k < nc; ++k) R[(size_t)k * rows + r] = yr - acc[k];
}

// XtR[c, k] += sum_r X[r, c] R[r, k]  (one block per column)
template <typename T>
__global__ void pg_xtr(const T* X, long long ld, long long rows, int F, const double* R, int nc, double* XtR) {
    const int c = blockIdx.x;
    __shared__ double red[kMaxCoef][256];
    double acc[kMaxCoef];
    for (int k = 0; k < nc; ++k) acc[k] = 0.0;
    for (long long r = threadIdx.x; r < rows; r += blockDim.x) {
        const double x = (double)X[(size_t)c * ld + r];
        for (int k = 0; k < nc; ++k) acc[k] += x * R[(size_t)k * rows + r];
    }
    for (int k = 0; k < nc; ++k) red[k][threadIdx.x] = acc[k];
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o)
            for (int k = 0; k < nc; ++k) red[k][threadIdx.x] += red[k][threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0)
        for (int k = 0; k < nc; ++k) XtR[(size_t)k * F + c] += red[k][0];
}

// sq[kind * nc + k] += sum of R^2 over the rows of kind (0 energy, 1 force, 2 stress)
__global__ void pg_residual_sq(const double* R, long long rows, int nc, long long n_e, long long s_end,
                               double* sq) {
    const int k = blockIdx.y;
    double e = 0, f = 0, s = 0;
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < rows;
         r += (long long)gridDim.x * blockDim.x) {
        const double v = R[(size_t)k * rows + r];
        if (r < n_e) e += v * v;
        else if (r < s_end) s += v * v;
        else f += v * v;
    }
    __shared__ double red[3][256];
    red[0][threadIdx.x] = e;
    red[1][threadIdx.x] = f;
    red[2][threadIdx.x] = s;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o)
            for (int q = 0; q < 3; ++q) red[q][threadIdx.x] += red[q][threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0)
        for (int q = 0; q < 3; ++q) atomicAdd(&sq[q * nc + k], red[q][0]);
}

// ------------------------------------------------------------ batches
// A batch of structures staged on the device with its row layout, weights and
// weighted targets: everything the regression assembly reads from HBM.
struct Prepared {
    DeviceBatch b;
    RowPlan plan;
    long long rows = 0;
    int n_e = 0;
    long long s_end = 0;  // first force row (energies, then stresses, then forces)
    double yty = 0.0;
    DevBuf d_e, d_f, d_s, d_w, d_y;
};

// Split a caller's batch into device-sized sub-batches with batch-local rows.
std::vector<std::unique_ptr<Prepared>> prepare_batches(Model& m, const pg_structures* st, const int64_t* e_row,
                                                       const int64_t* f_row, const int64_t* s_row, int64_t n_rows,
                                                       const double* w, const double* y, bool fp64) {
    for (int s = 0; s < st->n_st; ++s) {
        if (e_row[s] < 0 || e_row[s] >= n_rows) throw std::runtime_error("energy row out of range");
        if (f_row[s] >= 0 && (f_row[s] + 3LL * st->n_atoms[s] > n_rows || s_row[s] < 0 || s_row[s] + 6 > n_rows))
            throw std::runtime_error("force/stress rows out of range");
    }
    std::vector<std::unique_ptr<Prepared>> out;
    for (const auto& bt : m.plan_batches(st, fp64, device_batch_bytes())) {
        const int s0 = bt.first, s1 = bt.second, nb = s1 - s0;
        auto P = std::make_unique<Prepared>();
        std::vector<long long> le(nb), lf(nb, -1), ls(nb, -1);
        std::vector<double> wl(nb), yl(nb);
        long long r = nb;
        for (int q = 0; q < nb; ++q) {
            le[q] = q;
            wl[q] = w[e_row[s0 + q]];
            yl[q] = y[e_row[s0 + q]];
        }
        for (int q = 0; q < nb; ++q)
            if (f_row[s0 + q] >= 0) {
                ls[q] = r;
                for (int c = 0; c < 6; ++c) {
                    wl.push_back(w[s_row[s0 + q] + c]);
                    yl.push_back(y[s_row[s0 + q] + c]);
                }
                r += 6;
            }
        for (int q = 0; q < nb; ++q)
            if (f_row[s0 + q] >= 0) {
                lf[q] = r;
                const long long nr = 3LL * st->n_atoms[s0 + q];
                for (long long c = 0; c < nr; ++c) {
                    wl.push_back(w[f_row[s0 + q] + c]);
                    yl.push_back(y[f_row[s0 + q] + c]);
                }
                r += nr;
            }
        P->rows = r;
        P->n_e = nb;
        P->s_end = nb;
        for (int q = 0; q < nb; ++q)
            if (f_row[s0 + q] >= 0) P->s_end += 6;
        for (double v : yl) P->yty += v * v;
        P->b.upload_structures(st, s0, s1, m.flat.cutoff);
        m.plan_rows(P->b, P->plan);
        upload(P->d_e, le);
        upload(P->d_f, lf);
        upload(P->d_s, ls);
        upload(P->d_w, wl);
        upload(P->d_y, yl);
        out.push_back(std::move(P));
    }
    return out;
}

// ------------------------------------------------------------ pg_gram object
struct Gram {
    Model* m;
    int precision;
    int F;
    DevBuf G, xty, xe_sum, xe_sq, tiles64, Xd;
    GramTcScratch tc;
    int n_tiles64 = 0;
    double yty = 0;
    long long n_rows_total = 0;
    cudaStream_t stream = current_stream();

    Gram(Model* mm, int prec) : m(mm), precision(prec), F(mm->flat.n_features) {
        G.alloc((size_t)F * F * sizeof(double));
        xty.alloc(F * sizeof(double));
        xe_sum.alloc(F * sizeof(double));
        xe_sq.alloc(F * sizeof(double));
        reset();
        auto tile_list = [&](int tsz, DevBuf& buf, int& n) {
            const int nt = (F + tsz - 1) / tsz;
            std::vector<int2> t;
            for (int j = 0; j < nt; ++j)
                for (int i = 0; i <= j; ++i) t.push_back(make_int2(i, j));
            upload(buf, t);
            n = (int)t.size();
        };
        tile_list(kS64, tiles64, n_tiles64);
    }

    void reset() {
        PG_CUDA(cudaMemsetAsync(G.as<void>(), 0, G.bytes(), stream));
        PG_CUDA(cudaMemsetAsync(xty.as<void>(), 0, xty.bytes(), stream));
        PG_CUDA(cudaMemsetAsync(xe_sum.as<void>(), 0, xe_sum.bytes(), stream));
        PG_CUDA(cudaMemsetAsync(xe_sq.as<void>(), 0, xe_sq.bytes(), stream));
        yty = 0;
        n_rows_total = 0;
    }

    // Device work for one prepared batch: neighbours, rows, statistics, weights, X^T y, X^T X.
    void accumulate(Prepared& P) {
        const bool fp64 = precision == PG_FP64;
        const long long rows = P.rows;
        Xd.reserve((size_t)rows * F * (fp64 ? 8 : 4));
        dim3 sg((unsigned)((rows + 255) / 256), (unsigned)std::min(F, 64));
        if (fp64) {
            double* X = Xd.as<double>();
            m->run_rows<double>(P.b, P.plan, P.d_e.as<long long>(), P.d_f.as<long long>(), P.d_s.as<long long>(), X,
                                rows, stream);
            pg_energy_stats<double><<<(F + 127) / 128, 128, 0, stream>>>(X, rows, F, P.d_e.as<long long>(), P.n_e,
                                                                        xe_sum.as<double>(), xe_sq.as<double>());
            pg_scale_rows<double><<<sg, 256, 0, stream>>>(X, rows, rows, F, P.d_w.as<double>());
            pg_xty<double><<<F, 256, 0, stream>>>(X, rows, rows, P.d_y.as<double>(), xty.as<double>());
            ProfScope ps("pg_syrk_f64", stream);
            launch_syrk_f64(X, rows, rows, F, tiles64.as<int2>(), n_tiles64, G.as<double>(), stream);
        } else {
            float* X = Xd.as<float>();
            m->run_rows<float>(P.b, P.plan, P.d_e.as<long long>(), P.d_f.as<long long>(), P.d_s.as<long long>(), X,
                               rows, stream);
            pg_energy_stats<float><<<(F + 127) / 128, 128, 0, stream>>>(X, rows, F, P.d_e.as<long long>(), P.n_e,
                                                                       xe_sum.as<double>(), xe_sq.as<double>());
            pg_scale_rows<float><<<sg, 256, 0, stream>>>(X, rows, rows, F, P.d_w.as<double>());
            pg_xty<float><<<F, 256, 0, stream>>>(X, rows, rows, P.d_y.as<double>(), xty.as<double>());
            ProfScope ps("pg_gram_tc", stream);
            gram_tc_accumulate(X, rows, rows, F, G.as<double>(), tc, stream);
        }
        PG_CUDA(cudaGetLastError());
        yty += P.yty;
        n_rows_total += rows;
    }

    // Weighted residuals of coefficient columns C (F x nc, device) on one batch:
    // XtR += X^T R and sq += per-kind sums of R^2 (rows regenerated on the device).
    // Without targets (use_y false) R = -X C, so XtR accumulates -X^T X C.
    void residual(Prepared& P, const double* C, int nc, double* XtR, double* sq, DevBuf& R, bool use_y = true) {
        const bool fp64 = precision == PG_FP64;
        const long long rows = P.rows;
        Xd.reserve((size_t)rows * F * (fp64 ? 8 : 4));
        R.reserve((size_t)rows * nc * sizeof(double));
        dim3 sg((unsigned)((rows + 255) / 256), (unsigned)std::min(F, 64));
        const unsigned nblk = (unsigned)((rows + 255) / 256);
        if (fp64) {
            double* X = Xd.as<double>();
            m->run_rows<double>(P.b, P.plan, P.d_e.as<long long>(), P.d_f.as<long long>(), P.d_s.as<long long>(), X,
                                rows, stream);
            pg_scale_rows<double><<<sg, 256, 0, stream>>>(X, rows, rows, F, P.d_w.as<double>());
            pg_residual<double><<<nblk, 256, 0, stream>>>(X, rows, rows, F, C, nc,
                                                          use_y ? P.d_y.as<double>() : nullptr, R.as<double>());
            pg_xtr<double><<<F, 256, 0, stream>>>(X, rows, rows, F, R.as<double>(), nc, XtR);
        } else {
            float* X = Xd.as<float>();
            m->run_rows<float>(P.b, P.plan, P.d_e.as<long long>(), P.d_f.as<long long>(), P.d_s.as<long long>(), X,
                               rows, stream);
            pg_scale_rows<float><<<sg, 256, 0, stream>>>(X, rows, rows, F, P.d_w.as<double>());
            pg_residual<float><<<nblk, 256, 0, stream>>>(X, rows, rows, F, C, nc,
                                                         use_y ? P.d_y.as<double>() : nullptr, R.as<double>());
            pg_xtr<float><<<F, 256, 0, stream>>>(X, rows, rows, F, R.as<double>(), nc, XtR);
        }
        if (sq) {
            dim3 g2(std::min(1024u, nblk), nc);
            pg_residual_sq<<<g2, 256, 0, stream>>>(R.as<double>(), rows, nc, P.n_e, P.s_end, sq);
        }
        PG_CUDA(cudaGetLastError());
    }
};

}  // namespace pg

using namespace pg;

struct pg_gram {
    std::unique_ptr<Gram> g;
};
struct pg_batch {
    std::vector<std::unique_ptr<Prepared>> parts;
    int precision;
};

extern "C" {

__global__ void pg_f64_to_f32(const double* src, float* dst, size_t n) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        dst[i] = (float)src[i];
}

int pg_gram_xtx(const double* x, int64_t n_rows, int n_features, int64_t ld, int precision, double* xtx) {
    return guarded([&] {
        if (!x || !xtx || n_rows < 0 || n_features <= 0 || ld < n_rows) throw std::runtime_error("bad arguments");
        if (precision != PG_FP64 && precision != PG_MIXED) throw std::runtime_error("unknown precision");
        const int F = n_features;
        cudaStream_t st = current_stream();
        DevBuf X64((size_t)std::max<int64_t>(1, n_rows) * F * 8), G((size_t)F * F * 8);
        zero_async(G.as<void>(), G.bytes());
        if (n_rows > 0) {
            PG_CUDA(cudaMemcpy2DAsync(X64.as<void>(), (size_t)n_rows * 8, x, (size_t)ld * 8, (size_t)n_rows * 8, F,
                                      cudaMemcpyHostToDevice, st));
            PG_CUDA(cudaStreamSynchronize(st));
        }
        if (n_rows > 0 && precision == PG_FP64) {
            const int nt = (F + kS64 - 1) / kS64;
            std::vector<int2> t;
            for (int j = 0; j < nt; ++j)
                for (int i = 0; i <= j; ++i) t.push_back(make_int2(i, j));
            DevBuf tiles;
            upload(tiles, t);
            launch_syrk_f64(X64.as<double>(), n_rows, n_rows, F, tiles.as<int2>(), (int)t.size(), G.as<double>(), st);
        } else if (n_rows > 0) {
            DevBuf X32((size_t)n_rows * F * 4);
            pg_f64_to_f32<<<1024, 256, 0, st>>>(X64.as<double>(), X32.as<float>(), (size_t)n_rows * F);
            GramTcScratch tc;
            gram_tc_accumulate(X32.as<float>(), n_rows, n_rows, F, G.as<double>(), tc, st);
            PG_CUDA(cudaStreamSynchronize(st));
            gram_tc_check(tc);
        }
        dim3 grid((F + 255) / 256, F);
        pg_symmetrize<<<grid, 256, 0, st>>>(G.as<double>(), F);
        PG_CUDA(cudaGetLastError());
        copy_d2h(xtx, G.as<double>(), (size_t)F * F * 8);
    });
}

int pg_gram_create(pg_model* m, int precision, pg_gram** out) {
    return guarded([&] {
        if (!m || !out) throw std::runtime_error("null argument");
        if (precision != PG_FP64 && precision != PG_MIXED) throw std::runtime_error("unknown precision");
        auto h = new pg_gram;
        try {
            h->g = std::make_unique<Gram>(m->m.get(), precision);
        } catch (...) {
            delete h;
            throw;
        }
        *out = h;
    });
}

int pg_gram_destroy(pg_gram* g) {
    return guarded([&] { delete g; });
}

int pg_gram_reset(pg_gram* g) {
    return guarded([&] {
        if (!g) throw std::runtime_error("null gram");
        g->g->stream = current_stream();
        g->g->reset();
    });
}

int pg_gram_accumulate(pg_gram* gh, const pg_structures* st, const int64_t* e_row, const int64_t* f_row,
                       const int64_t* s_row, int64_t n_rows, const double* w, const double* y) {
    return guarded([&] {
        if (!gh || !st || !e_row || !f_row || !s_row || !w || !y) throw std::runtime_error("null argument");
        Gram& g = *gh->g;
        g.stream = current_stream();
        auto parts = prepare_batches(*g.m, st, e_row, f_row, s_row, n_rows, w, y, g.precision == PG_FP64);
        for (auto& P : parts) g.accumulate(*P);
        PG_CUDA(cudaStreamSynchronize(g.stream));
        g.m->check_mirrors();
        gram_tc_check(g.tc);
    });
}

int pg_batch_create(pg_model* mh, const pg_structures* st, const int64_t* e_row, const int64_t* f_row,
                    const int64_t* s_row, int64_t n_rows, const double* w, const double* y, int precision,
                    pg_batch** out) {
    return guarded([&] {
        if (!mh || !st || !e_row || !f_row || !s_row || !w || !y || !out) throw std::runtime_error("null argument");
        auto h = new pg_batch;
        try {
            h->parts = prepare_batches(*mh->m, st, e_row, f_row, s_row, n_rows, w, y, precision == PG_FP64);
            h->precision = precision;
        } catch (...) {
            delete h;
            throw;
        }
        PG_CUDA(cudaStreamSynchronize(current_stream()));
        *out = h;
    });
}

int pg_batch_destroy(pg_batch* b) {
    return guarded([&] { delete b; });
}

int pg_batch_pair_counts(pg_batch* b, int n_type, int64_t* counts) {
    return guarded([&] {
        if (!b || !counts || n_type <= 0) throw std::runtime_error("bad arguments");
        std::fill(counts, counts + (size_t)n_type * n_type, (int64_t)0);
        for (auto& P : b->parts) {
            const DeviceBatch& B = P->b;
            if (B.n_pairs <= 0 || B.n_atoms <= 0) continue;
            std::vector<long long> off(B.n_atoms + 1), f(B.n_st);
            std::vector<int> nb((size_t)B.n_pairs);
            copy_d2h(off.data(), B.d_nb_off.as<long long>(), off.size() * sizeof(long long));
            copy_d2h(nb.data(), B.d_nb_j.as<int>(), nb.size() * sizeof(int));
            copy_d2h(f.data(), P->d_f.as<long long>(), f.size() * sizeof(long long));
            for (int i = 0; i < B.n_atoms; ++i) {
                if (f[B.atom_st[i]] < 0) continue;
                const int a = B.types[i];
                if (a < 0 || a >= n_type) throw std::runtime_error("atom type out of range");
                for (long long q = off[i]; q < off[i + 1]; ++q) counts[a * n_type + B.types[nb[q]]]++;
            }
        }
    });
}

int pg_gram_accumulate_batch(pg_gram* gh, pg_batch* b) {
    return guarded([&] {
        if (!gh || !b) throw std::runtime_error("null argument");
        gh->g->stream = current_stream();
        for (auto& P : b->parts) gh->g->accumulate(*P);
    });
}

int pg_batch_residual(pg_gram* gh, pg_batch* b, const double* coefs, int n_coef, double* xtr, double* sq,
                      int64_t* n_rows) {
    return guarded([&] {
        if (!gh || !b || !coefs || n_coef < 1) throw std::runtime_error("bad arguments");
        if (n_coef > kMaxCoef) throw std::runtime_error("at most 16 coefficient vectors per residual pass");
        Gram& g = *gh->g;
        g.stream = current_stream();
        const int F = g.F;
        DevBuf C((size_t)F * n_coef * 8), XtR((size_t)F * n_coef * 8), SQ((size_t)3 * n_coef * 8), R;
        copy_h2d(C.as<void>(), coefs, (size_t)F * n_coef * 8);
        zero_async(XtR.as<void>(), XtR.bytes());
        zero_async(SQ.as<void>(), SQ.bytes());
        long long rows = 0;
        for (auto& P : b->parts) {
            g.residual(*P, C.as<double>(), n_coef, XtR.as<double>(), SQ.as<double>(), R);
            rows += P->rows;
        }
        PG_CUDA(cudaStreamSynchronize(g.stream));
        g.m->check_mirrors();
        if (xtr) copy_d2h(xtr, XtR.as<double>(), (size_t)F * n_coef * 8);
        if (sq) copy_d2h(sq, SQ.as<double>(), (size_t)3 * n_coef * 8);
        if (n_rows) *n_rows = rows;
    });
}

int pg_gram_result(pg_gram* gh, double* xtx, double* xty, double* yty, double* xe_sum, double* xe_sq_sum,
                   int64_t* n_rows_total) {
    return guarded([&] {
        if (!gh) throw std::runtime_error("null gram");
        Gram& g = *gh->g;
        g.stream = current_stream();
        const int F = g.F;
        dim3 grid((F + 255) / 256, F);
        pg_symmetrize<<<grid, 256, 0, g.stream>>>(g.G.as<double>(), F);
        PG_CUDA(cudaGetLastError());
        PG_CUDA(cudaStreamSynchronize(g.stream));
        g.m->check_mirrors();
        gram_tc_check(g.tc);
        if (xtx) copy_d2h(xtx, g.G.as<double>(), (size_t)F * F * sizeof(double));
        if (xty) copy_d2h(xty, g.xty.as<double>(), F * sizeof(double));
        if (xe_sum) copy_d2h(xe_sum, g.xe_sum.as<double>(), F * sizeof(double));
        if (xe_sq_sum) copy_d2h(xe_sq_sum, g.xe_sq.as<double>(), F * sizeof(double));
        if (yty) *yty = g.yty;
        if (n_rows_total) *n_rows_total = g.n_rows_total;
    });
}

}  // extern "C"
