// Energy / force / stress evaluation on the GPU (PotentialPropertiesFast,
// src/pypolymlp/cxx/src/compute/py_properties_fast.cpp:19-77, PolymlpEval,
// src/pypolymlp/cxx/src/compute/polymlp_eval.cpp:24-403).
//
// The reference already evaluates by an adjoint: per atom it forms
// prod_sum = dE_i/da_nlm (polymlp_potential.cpp:235-295) and contracts it with
// da/dr per half-list pair.  Here, per atom i (full neighbour list):
//   pg_anlm            a_nlm (m <= 0), long neighbour sums (FP64, or float-float
//                      in the FP32 kernel)                             (xrows.cu)
//   pg_eval_adjoint    features d, beta_k = dE_i/dd_k from the polynomial with
//                      the coefficients, E_i, and the folded adjoint
//                      A_i[h] = sum_e beta_k(e) G_e (no G stored)
//   pg_eval_pairs      per pair image p = (i -> j, d): g_p = Re(A_i . dphi(d)/dd),
//                      32 pairs at a time with their bases built together
//   pg_nb_mirror       index of the mirror image (j -> i, -d) of every pair
//                      (exact: -d is bit-identical; xrows.cu)
//   pg_eval_gather     F_b = sum_{q in list(b)} (g_q - g_mirror(q))   (no atomics)
//   pg_eval_gather     also the per-centre virial -sum_{p in list(i)} d_p (x) g_p
//   pg_eval_reduce     E = sum_i E_i and stress = sum_i virial_i per structure
// Energies match the reference's Euler-split pair sums, and forces/stress its
// half-list collection, up to summation order.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <memory>

#include "kernels.h"
#include "model.h"

namespace pg {

// Extra per-type device tables of the evaluator.
struct EvalType {
    const int *tp_head_off, *tp_heads;
    const int* tp_head_nk;  // per tp_heads entry: radial index | Y_lm index << 8
    const int *kcol_off, *kcol_col, *kcol_o1, *kcol_o2;
    // adjoint terms by head: head h owns terms head_toff[h] .. head_toff[h + 1]
    // (its entries in head_ent order, their terms in order); per term the
    // packed a ids (as tcode), the feature of its entry and its coefficient
    // (the sign of a conjugate head folded into conjugate terms)
    const int* head_toff;
    const int4* htcode;
    const int* htk;
    const double* htcoef64;
    const float* htcoef32;
};

template <typename T>
__device__ __forceinline__ const T* head_term_coef(const EvalType& e);
template <>
__device__ __forceinline__ const double* head_term_coef<double>(const EvalType& e) { return e.htcoef64; }
template <>
__device__ __forceinline__ const float* head_term_coef<float>(const EvalType& e) { return e.htcoef32; }

struct EvalTables {
    EvalType types[kMaxTypes];
};

// One block per atom.
template <typename T>
__global__ void pg_eval_adjoint(DevModel M, EvalTables ET, const int* types, const long long* a_off,
                                const cplx<T>* Anoconj, const T* coef, cplx<T>* Aout, double* Eatom) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int i = blockIdx.x;
    const int t1 = types[i];
    const DevType& ty = M.types[t1];
    const EvalType& et = ET.types[t1];
    cplx<T>* a = reinterpret_cast<cplx<T>*>(smem_raw);
    T* d = reinterpret_cast<T*>(a + ty.K);
    T* beta = d + ty.n_lin;
    __shared__ double red[32];
    load_full_a<T>(ty, Anoconj + a_off[i], a);
    __syncthreads();
    constexpr int NW = 8;  // 256 threads
    __shared__ cplx<T> s_v[NW][kTermWin];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    warp_feature_values<T>(ty, a, d, s_v[warp], warp, NW, lane);
    __syncthreads();
    // beta_k = sum over polynomial columns containing k of coef * product of the others
    for (int k = threadIdx.x; k < ty.n_lin; k += blockDim.x) {
        T b = 0;
        for (int q = et.kcol_off[k]; q < et.kcol_off[k + 1]; ++q) {
            T w = coef[et.kcol_col[q]];
            const int o1 = et.kcol_o1[q], o2 = et.kcol_o2[q];
            if (o1 >= 0) w *= d[o1];
            if (o2 >= 0) w *= d[o2];
            b += w;
        }
        beta[k] = b;
    }
    // E_i = sum over columns of coef * polynomial value (long sums per thread, FP64 block sum)
    LongSum<T> ls;
    for (int col = threadIdx.x; col < M.F; col += blockDim.x) {
        const int nc = ty.col_ncomp[col];
        if (nc == 0) continue;
        T p = (T)1;
        for (int c = 0; c < nc; ++c) p *= d[ty.comp_k[col * 3 + c]];
        ls.add(coef[col] * p);
    }
    double e = (double)ls.value();
    for (int o = 16; o > 0; o >>= 1) e += __shfl_down_sync(0xffffffffu, e, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = e;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += red[w];
        Eatom[i] = s;
    }
    // A[h] = sum over entries with head h of beta_k(e) G_e: windowed warp sums
    // over the head-ordered terms, 32 heads per warp (beta is complete: the
    // block synchronised after it)
    cplx<T>* Ao = Aout + a_off[i];
    const T* hcoef = head_term_coef<T>(et);
    for (int h0 = 32 * warp; h0 < ty.K0; h0 += 32 * NW) {
        const int h = h0 + lane;
        const int tb = et.head_toff[h0], te = et.head_toff[min(h0 + 32, ty.K0)];
        const int ms = h < ty.K0 ? et.head_toff[h] : te, me = h < ty.K0 ? et.head_toff[h + 1] : te;
        T re = 0, im = 0;
        for (int w0 = tb; w0 < te; w0 += kTermWin) {
            // the window's codes, features and coefficients are requested together
            constexpr int kU = kTermWin / 32;
            int4 c4[kU];
            int tk[kU];
            T cf[kU];
#pragma unroll
            for (int u = 0; u < kU; ++u) {
                const int t = min(w0 + 32 * u + lane, te - 1);
                c4[u] = et.htcode[t];
                tk[u] = et.htk[t];
                cf[u] = hcoef[t];
            }
#pragma unroll
            for (int u = 0; u < kU; ++u)
                if (w0 + 32 * u + lane < te) {
                    const T c = beta[tk[u]] * cf[u];
                    const cplx<T> p = packed_term_product<T>(c4[u], a);
                    cplx<T> v = {c * p.re, c * p.im};
                    if (c4[u].w >> 8) v.im = -v.im;
                    s_v[warp][32 * u + lane] = v;
                }
            __syncwarp();
            const int lo = max(ms, w0), hi = min(me, w0 + kTermWin);
            for (int t = lo; t < hi; ++t) {
                re += s_v[warp][t - w0].re;
                im += s_v[warp][t - w0].im;
            }
            __syncwarp();
        }
        if (h < ty.K0) Ao[h] = {re, im};
    }
}

// One block per centre atom; its pair images taken 32 at a time.  With
// phi_h = f_n(r) Y_lm and the adjoint regrouped by Y_lm key,
//   g_p = sum_key Re(B_key . dY_key/dd) + (d/r) sum_key Re(C_key . Y_key),
//   B_key = sum_n A[tp, n, key] f_n(r),  C_key = sum_n A[tp, n, key] f_n'(r),
// so a pair costs about 4 K0(tp) + 16 n_ylm multiply-adds.  The block builds
// the chunk's bases at once (thread = pair and two Legendre columns,
// ylm_column, or pair and radial functions) into shared memory; then the 8
// threads of a pair take every 8th key and sum over the radial functions, and
// their partial sums are added by shuffles (16 threads a pair in FP64).
// pairs per chunk: 32 (FP32), 16 (FP64, so that two blocks fit an SM)
template <typename T>
constexpr int eval_chunk() { return sizeof(T) == 4 ? 32 : 16; }
template <typename T>
__global__ void __launch_bounds__(256) pg_eval_pairs(DevModel M, EvalTables ET, DevBatch B, const long long* nb_off,
                                                     const int* nb_j, const double* nb_d, const long long* a_off,
                                                     const cplx<T>* Aadj, double* g_out) {
    constexpr int PS = eval_chunk<T>(), TPP = 256 / PS;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int i = blockIdx.x;
    const int t1 = B.types[i];
    const EvalType& et = ET.types[t1];
    const int NY = M.n_ylm, NF = M.n_fn_max, L = M.maxl;
    cplx<T>* Akn = reinterpret_cast<cplx<T>*>(smem_raw);        // [n_tp][NY][NF]: the adjoint by (key, n)
    T* tab = reinterpret_cast<T*>(Akn + (size_t)M.n_tp * NY * NF);  // [PS][NY][8]: Y, dY/dx, dY/dy, dY/dz
    T* rad = tab + (size_t)PS * NY * 8;                             // [PS][NF][2]: f, f'
    T* s_tab = rad + (size_t)PS * NF * 2;
    const cplx<T>* Ai = Aadj + a_off[i];
    for (int q = threadIdx.x; q < M.n_tp * NY * NF; q += blockDim.x) Akn[q] = {(T)0, (T)0};
    load_ylm_tab<T>(M.ylm_tab, s_tab, M.n_ylm, M.maxl);
    __syncthreads();
    for (int tp = 0; tp < M.n_tp; ++tp)
        for (int q = et.tp_head_off[tp] + threadIdx.x; q < et.tp_head_off[tp + 1]; q += blockDim.x) {
            const int nk = et.tp_head_nk[q];
            Akn[((size_t)tp * NY + (nk >> 8)) * NF + (nk & 0xff)] = Ai[et.tp_heads[q]];
        }
    const YlmTab<T> ytab = ylm_tab_view<T>(s_tab, M.n_ylm, M.maxl);
    const int p = threadIdx.x / TPP, t = threadIdx.x - (threadIdx.x / TPP) * TPP;
    const int ny = M.gtinv ? min(TPP, L / 2 + 1) : 1;
    const int nfree = TPP - ny;
    const long long pe = nb_off[i + 1];
    for (long long k0 = nb_off[i]; k0 < pe; k0 += PS) {
        const int n = (int)min((long long)PS, pe - k0);
        T dx = 0, dy = 0, dz = 0, dis = 1;
        bool ok = false;
        int tp = 0;
        if (p < n) {
            ok = pair_geometry<T>(M, B, nb_d, k0 + p, dx, dy, dz, dis);
            tp = M.type_pairs[t1 * M.n_type + B.types[nb_j[k0 + p]]];
        }
        const int nfn = M.tp_nfn[tp];
        __syncthreads();  // the previous chunk's tables are read
        // ---- bases (threads 0 .. ny-1 of a pair: Legendre columns; the others: radial functions)
        if (ok) {
            T* rows = tab + (size_t)p * NY * 8;
            if (!M.gtinv) {
                if (t == 0)
                    for (int v = 0; v < 8; ++v) rows[v] = v == 0 ? (T)1 : (T)0;
            } else if (t < ny) {
                const YlmDir<T> dir = ylm_dir<T>(dx, dy, dz, dis);
                for (int a = t; 2 * a <= L; a += ny)
                    for (int side = 0; side < 2; ++side) {
                        const int mp = side ? L - a : a;
                        if (side && mp == a) break;
                        ylm_column<T>(mp, L, ytab, dir, rows, 8);
                    }
            }
            const int r0t = nfree > 0 ? t - ny : t, rstep = nfree > 0 ? nfree : TPP;
            if (r0t >= 0)
                for (int q = r0t; q < nfn; q += rstep) {
                    T f, fd;
                    radial_one<T>(M, tp, q, dis, f, fd);
                    rad[((size_t)p * NF + q) * 2] = f;
                    rad[((size_t)p * NF + q) * 2 + 1] = fd;
                }
        }
        __syncthreads();
        // ---- g_p: thread t of pair p takes keys t, t + TPP, ..
        T s0 = 0, sx = 0, sy = 0, sz = 0;
        if (ok) {
            const T* rp = rad + (size_t)p * NF * 2;
            for (int key = t; key < NY; key += TPP) {
                const cplx<T>* ak = Akn + ((size_t)tp * NY + key) * NF;
                T bre = 0, bim = 0, cre = 0, cim = 0;
                for (int q = 0; q < nfn; ++q) {
                    const cplx<T> av = ak[q];
                    const T f = rp[2 * q], fd = rp[2 * q + 1];
                    bre += av.re * f;
                    bim += av.im * f;
                    cre += av.re * fd;
                    cim += av.im * fd;
                }
                const T* row = tab + ((size_t)p * NY + key) * 8;
                s0 += cre * row[0] - cim * row[1];
                sx += bre * row[2] - bim * row[3];
                sy += bre * row[4] - bim * row[5];
                sz += bre * row[6] - bim * row[7];
            }
        }
#pragma unroll
        for (int o = 1; o < TPP; o <<= 1) {
            s0 += __shfl_xor_sync(0xffffffffu, s0, o);
            sx += __shfl_xor_sync(0xffffffffu, sx, o);
            sy += __shfl_xor_sync(0xffffffffu, sy, o);
            sz += __shfl_xor_sync(0xffffffffu, sz, o);
        }
        if (t == 0 && p < n) {
            double gx = 0.0, gy = 0.0, gz = 0.0;
            if (ok) {
                const T sc = s0 / dis;
                gx = (double)(sc * dx + sx);
                gy = (double)(sc * dy + sy);
                gz = (double)(sc * dz + sz);
            }
            g_out[3 * (k0 + p)] = gx;
            g_out[3 * (k0 + p) + 1] = gy;
            g_out[3 * (k0 + p) + 2] = gz;
        }
    }
}

// F_b = sum_{q in list(b)} (g_q - g_mirror(q)); one thread per atom, FP64.
__global__ void pg_eval_gather(int n_atoms, const long long* nb_off, const long long* mirror, const double* g,
                               const double* nb_d, double* forces, double* vir) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= n_atoms) return;
    double f[3] = {0, 0, 0}, v[6] = {0, 0, 0, 0, 0, 0};
    for (long long q = nb_off[b]; q < nb_off[b + 1]; ++q) {
        const long long m = mirror[q];
        const double gx = g[3 * q], gy = g[3 * q + 1], gz = g[3 * q + 2];
        f[0] += gx - (m >= 0 ? g[3 * m] : 0.0);
        f[1] += gy - (m >= 0 ? g[3 * m + 1] : 0.0);
        f[2] += gz - (m >= 0 ? g[3 * m + 2] : 0.0);
        const double dx = nb_d[3 * q], dy = nb_d[3 * q + 1], dz = nb_d[3 * q + 2];
        v[0] -= dx * gx;
        v[1] -= dy * gy;
        v[2] -= dz * gz;
        v[3] -= dx * gy;
        v[4] -= dy * gz;
        v[5] -= dz * gx;
    }
    for (int c = 0; c < 3; ++c) forces[3 * (size_t)b + c] = f[c];
    for (int c = 0; c < 6; ++c) vir[6 * (size_t)b + c] = v[c];
}

// Per structure: E = sum_i E_i and stress = sum_i vir_i, with vir_i =
// -sum_{p in list(i)} d_p (x) g_p (xx yy zz xy yz zx, xy = -d_x g_y): the
// half-list sum of polymlp_eval.cpp:293-336, whose pair force is
// -(g_ij - g_ji), written per directed pair and summed per centre first.
__global__ void pg_eval_reduce(const int* st_atom_off, const double* Eatom, const double* vir, double* energy,
                               double* stress) {
    const int s = blockIdx.x;
    const int a0 = st_atom_off[s], a1 = st_atom_off[s + 1];
    double acc[7] = {0, 0, 0, 0, 0, 0, 0};
    for (int a = a0 + threadIdx.x; a < a1; a += blockDim.x) {
        acc[0] += Eatom[a];
        for (int q = 0; q < 6; ++q) acc[1 + q] += vir[6 * (size_t)a + q];
    }
    __shared__ double red[7][256];
    for (int q = 0; q < 7; ++q) red[q][threadIdx.x] = acc[q];
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o)
            for (int q = 0; q < 7; ++q) red[q][threadIdx.x] += red[q][threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        energy[s] = red[0][0];
        for (int q = 0; q < 6; ++q) stress[6 * s + q] = red[q + 1][0];
    }
}

struct Evaluator {
    std::unique_ptr<Model> m;
    int precision;
    DevBuf coef, coef32;  // the coefficients in FP64 and FP32
    std::vector<DevBuf> bufs;
    EvalTables et{};
    DevBuf d_aoff, s_Anc, s_Aadj, s_E, s_vir, s_g, s_mirror, s_missing, d_E, d_S, d_F;
    cudaStream_t stream = current_stream();
    // Structures bound for repeated evaluation (molecular dynamics): one
    // batch whose neighbour lists are built with cutoff + skin and kept; new
    // positions only refresh the displacements of the kept entries (the
    // kernels drop entries beyond the cutoff), until some atom has moved more
    // than skin / 2 since the lists were built.
    std::unique_ptr<DeviceBatch> bound;
    double skin = 0.0;
    std::vector<int> bound_n_atoms, bound_types;
    std::vector<double> bound_axis, bound_ref, bound_shift, bound_pos;

    Evaluator(const pg_feature_params* fp, const double* coeffs, int n, int prec) : precision(prec) {
        m = std::make_unique<Model>(fp);
        if (n != m->flat.n_features) throw std::runtime_error("coefficient count does not match the model");
        upload(coef, std::vector<double>(coeffs, coeffs + n));
        upload(coef32, std::vector<float>(coeffs, coeffs + n));
        bufs.reserve(32 * kMaxTypes);
        auto up = [&](const std::vector<int>& v) -> const int* {
            bufs.emplace_back();
            upload(bufs.back(), v);
            return bufs.back().as<int>();
        };
        for (int t = 0; t < m->flat.n_type; ++t) {
            const FlatType& ft = m->flat.types[t];
            EvalType& e = et.types[t];
            e.tp_head_off = up(ft.tp_head_off);
            e.tp_heads = up(ft.tp_heads);
            if ((int)ft.tp_heads.size() != ft.K0) throw std::runtime_error("internal: heads without a type pair");
            std::vector<int> nk(ft.tp_heads.size());
            for (size_t q = 0; q < nk.size(); ++q) {
                const int h = ft.tp_heads[q];
                if (ft.head_nid[h] > 255 || ft.head_key[h] > (1 << 22))
                    throw std::runtime_error("model too large for the packed head indices");
                nk[q] = ft.head_nid[h] | (ft.head_key[h] << 8);
            }
            e.tp_head_nk = up(nk);
            e.kcol_off = up(ft.kcol_off);
            e.kcol_col = up(ft.kcol_col);
            e.kcol_o1 = up(ft.kcol_o1);
            e.kcol_o2 = up(ft.kcol_o2);
            if (ft.K >= 65536) throw std::runtime_error("too many a_nlm entries for the packed term ids");
            std::vector<int> toff(1, 0), tk;
            std::vector<int4> tcode;
            std::vector<double> tcoef;
            for (int h = 0; h < ft.K0; ++h) {
                const double cc = (ft.head_m[h] & 1) ? -1.0 : 1.0;
                for (int q = ft.head_ent_off[h]; q < ft.head_ent_off[h + 1]; ++q) {
                    const int ent = ft.head_ent[q];
                    for (int u = ft.term_off[ent]; u < ft.term_off[ent + 1]; ++u) {
                        const FlatTerm& t = ft.g_terms[u];
                        int id[6] = {0, 0, 0, 0, 0, 0};
                        for (int r = 0; r < t.n; ++r) id[r] = t.ids[r];
                        tcode.push_back(make_int4(id[0] | (id[1] << 16), id[2] | (id[3] << 16),
                                                  id[4] | (id[5] << 16), t.n | (t.conj << 8)));
                        tcoef.push_back(t.conj ? cc * t.coeff : t.coeff);
                        tk.push_back(ft.ent_k[ent]);
                    }
                }
                toff.push_back((int)tcode.size());
            }
            e.head_toff = up(toff);
            e.htk = up(tk);
            bufs.emplace_back();
            upload(bufs.back(), tcode);
            e.htcode = bufs.back().as<int4>();
            bufs.emplace_back();
            upload(bufs.back(), tcoef);
            e.htcoef64 = bufs.back().as<double>();
            bufs.emplace_back();
            upload(bufs.back(), std::vector<float>(tcoef.begin(), tcoef.end()));
            e.htcoef32 = bufs.back().as<float>();
        }
    }

    // energy_only: E per structure without the pair gradients (forces and
    // stress are not written); lists_ready: the batch's neighbour lists are
    // current (a bound batch).
    template <typename T>
    void run_batch(DeviceBatch& b, double* energy, double* forces, double* stress, bool energy_only = false,
                   bool lists_ready = false) {
        const DeviceModel& dmod = sizeof(T) == 8 ? m->dev64 : m->dev32;
        const DevModel& M = dmod.dm;
        if (!lists_ready) b.build_neighbors(m->flat.cutoff, stream);
        const DevBatch B = b.view(m->flat.cutoff);
        AtomOffsets off;
        m->atom_offsets(b, off);
        const long long a_tot = off.a_tot;
        upload(d_aoff, off.a_off);
        s_Anc.reserve(2 * sizeof(T) * std::max<long long>(1, a_tot));
        s_Aadj.reserve(2 * sizeof(T) * std::max<long long>(1, a_tot));
        s_E.reserve(sizeof(double) * std::max(1, b.n_atoms));
        s_vir.reserve(sizeof(double) * 6 * std::max(1, b.n_atoms));
        s_g.reserve(sizeof(double) * 3 * std::max<long long>(1, b.n_pairs));
        s_mirror.reserve(sizeof(long long) * std::max<long long>(1, b.n_pairs));
        s_missing.reserve(sizeof(int));
        d_E.reserve(sizeof(double) * std::max(1, b.n_st));
        d_S.reserve(sizeof(double) * 6 * std::max(1, b.n_st));
        d_F.reserve(sizeof(double) * 3 * std::max(1, b.n_atoms));
        PG_CUDA(cudaMemsetAsync(s_missing.as<void>(), 0, sizeof(int), stream));
        if (b.n_atoms > 0) {
            {
                ProfScope ps("pg_anlm", stream);
                launch_anlm<T>(M, B, b.d_nb_off.as<long long>(), b.d_nb_j.as<int>(), b.d_nb_d.as<double>(),
                               d_aoff.as<long long>(), s_Anc.as<void>(), m->max_k0, stream);
            }
            int max_lin = 1;
            for (const auto& ft : m->flat.types) max_lin = std::max(max_lin, ft.n_lin);
            const size_t sm1 = (size_t)m->max_k * 2 * sizeof(T) + 2 * (size_t)max_lin * sizeof(T) + 16;
            PG_CUDA(cudaFuncSetAttribute(pg_eval_adjoint<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm1));
            {
                ProfScope ps("pg_eval_adjoint", stream);
                pg_eval_adjoint<T><<<b.n_atoms, 256, sm1, stream>>>(M, et, d_types(b), d_aoff.as<long long>(),
                                                                   s_Anc.as<cplx<T>>(),
                                                                   (sizeof(T) == 8 ? coef : coef32).template as<T>(),
                                                                   reinterpret_cast<cplx<T>*>(s_Aadj.as<void>()),
                                                                   s_E.as<double>());
            }
            if (energy_only) {
                PG_CUDA(cudaMemsetAsync(s_vir.as<void>(), 0, sizeof(double) * 6 * b.n_atoms, stream));
                ProfScope ps("pg_eval_reduce", stream);
                pg_eval_reduce<<<b.n_st, 256, 0, stream>>>(b.d_st_atom_off.as<int>(), s_E.as<double>(),
                                                           s_vir.as<double>(), d_E.as<double>(), d_S.as<double>());
                PG_CUDA(cudaGetLastError());
                PG_CUDA(cudaMemcpyAsync(energy, d_E.as<double>(), sizeof(double) * b.n_st, cudaMemcpyDeviceToHost,
                                        stream));
                PG_CUDA(cudaStreamSynchronize(stream));
                return;
            }
            const int threads = 256;
            const size_t sm2 = (size_t)M.n_tp * M.n_ylm * M.n_fn_max * sizeof(cplx<T>) +
                               (size_t)eval_chunk<T>() * M.n_ylm * 8 * sizeof(T) +
                               (size_t)eval_chunk<T>() * M.n_fn_max * 2 * sizeof(T) +
                               (size_t)ylm_table_size(M.n_ylm, M.maxl) * sizeof(T);
            PG_CUDA(cudaFuncSetAttribute(pg_eval_pairs<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm2));
            {
                ProfScope ps("pg_eval_pairs", stream);
                pg_eval_pairs<T><<<b.n_atoms, threads, sm2, stream>>>(
                    M, et, B, b.d_nb_off.as<long long>(), b.d_nb_j.as<int>(), b.d_nb_d.as<double>(),
                    d_aoff.as<long long>(), reinterpret_cast<const cplx<T>*>(s_Aadj.as<void>()), s_g.as<double>());
            }
            {
                ProfScope ps("pg_nb_mirror", stream);
                launch_nb_mirror(b.n_atoms, b.d_nb_off.as<long long>(), b.d_nb_j.as<int>(), b.d_nb_d.as<double>(),
                                 s_mirror.as<long long>(), nullptr, s_missing.as<int>(), stream);
            }
            {
                ProfScope ps("pg_eval_gather", stream);
                pg_eval_gather<<<(b.n_atoms + 127) / 128, 128, 0, stream>>>(
                    b.n_atoms, b.d_nb_off.as<long long>(), s_mirror.as<long long>(), s_g.as<double>(),
                    b.d_nb_d.as<double>(), d_F.as<double>(), s_vir.as<double>());
            }
            ProfScope ps("pg_eval_reduce", stream);
            pg_eval_reduce<<<b.n_st, 256, 0, stream>>>(b.d_st_atom_off.as<int>(), s_E.as<double>(),
                                                       s_vir.as<double>(), d_E.as<double>(), d_S.as<double>());
        } else {
            PG_CUDA(cudaMemsetAsync(d_E.as<void>(), 0, sizeof(double) * b.n_st, stream));
            PG_CUDA(cudaMemsetAsync(d_S.as<void>(), 0, sizeof(double) * 6 * b.n_st, stream));
        }
        PG_CUDA(cudaGetLastError());
        if (energy_only) {  // no atoms
            PG_CUDA(cudaMemcpyAsync(energy, d_E.as<double>(), sizeof(double) * b.n_st, cudaMemcpyDeviceToHost,
                                    stream));
            PG_CUDA(cudaStreamSynchronize(stream));
            return;
        }
        int missing = 0;
        PG_CUDA(cudaMemcpyAsync(&missing, s_missing.as<int>(), sizeof(int), cudaMemcpyDeviceToHost, stream));
        PG_CUDA(cudaMemcpyAsync(energy, d_E.as<double>(), sizeof(double) * b.n_st, cudaMemcpyDeviceToHost, stream));
        PG_CUDA(cudaMemcpyAsync(stress, d_S.as<double>(), sizeof(double) * 6 * b.n_st, cudaMemcpyDeviceToHost, stream));
        if (b.n_atoms > 0)
            PG_CUDA(cudaMemcpyAsync(forces, d_F.as<double>(), sizeof(double) * 3 * b.n_atoms, cudaMemcpyDeviceToHost,
                                    stream));
        PG_CUDA(cudaStreamSynchronize(stream));
        if (missing) throw std::runtime_error("internal: neighbour list is not symmetric");
    }

    static const int* d_types(const DeviceBatch& b) { return b.d_types.as<int>(); }

    // Bind structures: stage them and build lists with cutoff + skin.
    void bind(const pg_structures* st, double skin_) {
        if (!(skin_ >= 0.0) || !std::isfinite(skin_)) throw std::runtime_error("skin must be finite and >= 0");
        const bool fp64 = precision == PG_FP64;
        if (m->plan_batches(st, fp64, device_batch_bytes()).size() != 1)
            throw std::runtime_error("bound structures must fit one device batch");
        long long n_tot = 0;
        for (int s = 0; s < st->n_st; ++s) n_tot += st->n_atoms[s];
        auto b = std::make_unique<DeviceBatch>();
        b->upload_structures(st, 0, st->n_st, m->flat.cutoff + skin_);
        b->build_neighbors(m->flat.cutoff + skin_, stream);
        bound_n_atoms.assign(st->n_atoms, st->n_atoms + st->n_st);
        bound_types.assign(st->types, st->types + n_tot);
        bound_axis.assign(st->axis, st->axis + 9 * (size_t)st->n_st);
        bound_ref.assign(st->positions, st->positions + 3 * n_tot);
        bound_shift.resize(3 * n_tot);
        for (size_t q = 0; q < bound_shift.size(); ++q) bound_shift[q] = b->pos[q] - bound_ref[q];
        bound_pos = b->pos;
        skin = skin_;
        bound = std::move(b);
    }

    // New Cartesian positions of the bound atoms (same order); returns whether
    // the lists were rebuilt.
    bool update(const double* positions) {
        if (!bound) throw std::runtime_error("no structures are bound (pg_eval_bind)");
        const size_t n3 = bound_ref.size();
        double d2max = 0.0;
        for (size_t a = 0; a < n3; a += 3) {
            double d2 = 0.0;
            for (int c = 0; c < 3; ++c) {
                const double d = positions[a + c] - bound_ref[a + c];
                d2 += d * d;
            }
            if (!std::isfinite(d2)) throw std::runtime_error("non-finite position");
            d2max = std::max(d2max, d2);
        }
        if (d2max > 0.25 * skin * skin) {
            pg_structures st{(int)bound_n_atoms.size(), bound_n_atoms.data(), bound_axis.data(), positions,
                             bound_types.data()};
            bind(&st, skin);
            return true;
        }
        for (size_t q = 0; q < n3; ++q) bound_pos[q] = positions[q] + bound_shift[q];
        copy_h2d(bound->d_pos.as<void>(), bound_pos.data(), n3 * sizeof(double));
        const DevBatch B = bound->view(m->flat.cutoff + skin);
        launch_nb_refresh(B, bound->d_nb_off.as<long long>(), bound->d_keys.as<long long>(), bound->d_nb_j.as<int>(),
                          bound->d_nb_d.as<double>(), bound->d_nb_df.as<float4>(), stream);
        PG_CUDA(cudaGetLastError());
        return false;
    }

    void run_bound(double* energy, double* forces, double* stress, bool energy_only) {
        if (!bound) throw std::runtime_error("no structures are bound (pg_eval_bind)");
        if (precision == PG_FP64) run_batch<double>(*bound, energy, forces, stress, energy_only, true);
        else run_batch<float>(*bound, energy, forces, stress, energy_only, true);
    }

    size_t workspace_bytes() const {
        size_t n = d_aoff.bytes() + s_Anc.bytes() + s_Aadj.bytes() + s_E.bytes() + s_vir.bytes() + s_g.bytes() +
                   s_mirror.bytes() + s_missing.bytes() + d_E.bytes() + d_S.bytes() + d_F.bytes();
        if (bound)
            n += bound->d_nb_j.bytes() + bound->d_nb_d.bytes() + bound->d_nb_df.bytes() + bound->d_keys.bytes() +
                 bound->d_nb_off.bytes() + bound->d_pos.bytes();
        return n;
    }
};

}  // namespace pg

using namespace pg;

struct pg_eval {
    std::unique_ptr<Evaluator> e;
};

extern "C" {

int pg_eval_create(const pg_feature_params* fp, const double* coeffs, int n_coeffs, int precision, pg_eval** out) {
    return guarded([&] {
        if (!fp || !coeffs || !out) throw std::runtime_error("null argument");
        if (precision != PG_FP64 && precision != PG_MIXED) throw std::runtime_error("unknown precision");
        auto h = new pg_eval;
        try {
            h->e = std::make_unique<Evaluator>(fp, coeffs, n_coeffs, precision);
        } catch (...) {
            delete h;
            throw;
        }
        *out = h;
    });
}

int pg_eval_destroy(pg_eval* e) {
    return guarded([&] { delete e; });
}

int pg_eval_bind(pg_eval* eh, const pg_structures* st, double skin) {
    return guarded([&] {
        if (!eh || !st) throw std::runtime_error("null argument");
        eh->e->stream = current_stream();
        eh->e->bind(st, skin);
    });
}

int pg_eval_update(pg_eval* eh, const double* positions, int* rebuilt) {
    return guarded([&] {
        if (!eh || !positions) throw std::runtime_error("null argument");
        eh->e->stream = current_stream();
        const bool r = eh->e->update(positions);
        if (rebuilt) *rebuilt = r ? 1 : 0;
    });
}

int pg_eval_bound_energy(pg_eval* eh, double* energy) {
    return guarded([&] {
        if (!eh || !energy) throw std::runtime_error("null argument");
        eh->e->stream = current_stream();
        eh->e->run_bound(energy, nullptr, nullptr, true);
    });
}

int pg_eval_bound_run(pg_eval* eh, double* energy, double* forces, double* stress) {
    return guarded([&] {
        if (!eh || !energy || !forces || !stress) throw std::runtime_error("null argument");
        eh->e->stream = current_stream();
        eh->e->run_bound(energy, forces, stress, false);
    });
}

int pg_eval_workspace_bytes(const pg_eval* eh, int64_t* bytes) {
    return guarded([&] {
        if (!eh || !bytes) throw std::runtime_error("null argument");
        *bytes = (int64_t)eh->e->workspace_bytes();
    });
}

int pg_eval_run(pg_eval* eh, const pg_structures* st, double* energy, double* forces, double* stress) {
    return guarded([&] {
        if (!eh || !st || !energy || !forces || !stress) throw std::runtime_error("null argument");
        Evaluator& ev = *eh->e;
        ev.stream = current_stream();
        const bool fp64 = ev.precision == PG_FP64;
        DeviceBatch b;
        long long a = 0;
        for (const auto& bt : ev.m->plan_batches(st, fp64, device_batch_bytes())) {
            b.upload_structures(st, bt.first, bt.second, ev.m->flat.cutoff);
            if (fp64) ev.run_batch<double>(b, energy + bt.first, forces + 3 * a, stress + 6 * bt.first);
            else ev.run_batch<float>(b, energy + bt.first, forces + 3 * a, stress + 6 * bt.first);
            a += b.n_atoms;
        }
    });
}

}  // extern "C"
