// Training rows of X on the GPU.
//
//   pg_nb_count / pg_nb_fill   full neighbour list of every atom of a batch
//                              (NeighborFull, compute/neighbor_full.cpp:10-76):
//                              same (j, translation) order and bit-identical
//                              displacements (IEEE double, no contraction).
//   pg_anlm                    a_nlm for m <= 0 of every atom (local.cpp:62-114),
//                              sums over neighbours accumulated in FP64.
//   pg_features_adjoint        invariant features d_k of every atom and the
//                              sparse adjoint G_k[h] = d d_k / d a_h with the
//                              conjugate half folded in (features.cpp:155-248).
//   pg_rows                    energy, force and stress rows of X for a block
//                              of target atoms and a chunk of columns:
//                              X_force[3j+c, col] = sum over pairs of
//                              +-Re(G_col(i) . d a(i)/d r_j,c), with G_col the
//                              polynomial-weighted adjoint (model.cpp:159-267).
//                              Each thread owns one column, so the sums are
//                              race free and deterministic.
//   pg_rows_reduce             per-structure sum of the energy/stress partials.
#include <cuda_runtime.h>

#include "kernels.h"

namespace pg {

// ------------------------------------------------------------ K1 neighbours
// One warp per centre atom; candidates (j, t) in j-major order.  Only
// __dadd_rn/__dmul_rn are used so nothing is contracted into an FMA.
__device__ __forceinline__ bool pair_keep(const DevBatch& B, int i, int j, int t, double rc2, double tol2,
                                          double& dx, double& dy, double& dz) {
    const double* pi = B.pos + 3 * (size_t)i;
    const double* pj = B.pos + 3 * (size_t)j;
    const double* tr = B.trans + 3 * (size_t)t;
    dx = __dadd_rn(__dadd_rn(pj[0], -pi[0]), tr[0]);
    dy = __dadd_rn(__dadd_rn(pj[1], -pi[1]), tr[1]);
    dz = __dadd_rn(__dadd_rn(pj[2], -pi[2]), tr[2]);
    const double r2 = __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
    return r2 < rc2 && r2 > tol2;
}

__global__ void pg_nb_count(DevBatch B, int* counts) {
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (warp >= B.n_atoms) return;
    const int i = warp;
    const int s = B.atom_st[i];
    const int a0 = B.st_atom_off[s], n = B.st_atom_off[s + 1] - a0;
    const int t0 = B.st_trans_off[s], nt = B.st_trans_off[s + 1] - t0;
    const double rc2 = __dmul_rn(B.cutoff, B.cutoff), tol2 = __dmul_rn(1e-10, 1e-10);
    const long long total = (long long)n * nt;
    int cnt = 0;
    for (long long q = lane; q < total; q += 32) {
        const int j = (int)(q / nt), t = (int)(q % nt);
        double dx, dy, dz;
        cnt += pair_keep(B, i, a0 + j, t0 + t, rc2, tol2, dx, dy, dz) ? 1 : 0;
    }
    for (int o = 16; o > 0; o >>= 1) cnt += __shfl_down_sync(0xffffffffu, cnt, o);
    if (lane == 0) counts[i] = cnt;
}

__global__ void pg_nb_fill(DevBatch B, const long long* offsets, int* nb_j, double* nb_d) {
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (warp >= B.n_atoms) return;
    const int i = warp;
    const int s = B.atom_st[i];
    const int a0 = B.st_atom_off[s], n = B.st_atom_off[s + 1] - a0;
    const int t0 = B.st_trans_off[s], nt = B.st_trans_off[s + 1] - t0;
    const double rc2 = __dmul_rn(B.cutoff, B.cutoff), tol2 = __dmul_rn(1e-10, 1e-10);
    const long long total = (long long)n * nt;
    long long w = offsets[i];
    const long long wend = offsets[i + 1];
    for (long long base = 0; base < total; base += 32) {
        const long long q = base + lane;
        double dx = 0, dy = 0, dz = 0;
        int j = 0;
        bool keep = false;
        if (q < total) {
            j = (int)(q / nt);
            keep = pair_keep(B, i, a0 + j, t0 + (int)(q % nt), rc2, tol2, dx, dy, dz);
        }
        const unsigned m = __ballot_sync(0xffffffffu, keep);
        if (keep) {
            const long long k = w + __popc(m & ((1u << lane) - 1u));
            if (k < wend) {
                nb_j[k] = a0 + j;
                nb_d[3 * k] = dx;
                nb_d[3 * k + 1] = dy;
                nb_d[3 * k + 2] = dz;
            }
        }
        w += __popc(m);
    }
}

// ---------------------------------------------------------------- K2 a_nlm
// Block per centre atom.  Warps compute the basis of one neighbour each;
// every thread then adds fn * Y into the heads it owns (FP64 sums).
template <typename T>
__global__ void pg_anlm(DevModel M, DevBatch B, const long long* nb_off, const int* nb_j, const double* nb_d,
                        const long long* a_off, double2* A) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int i = blockIdx.x;
    const int t1 = B.types[i];
    const DevType& ty = M.types[t1];
    const int nw = blockDim.x >> 5, warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const size_t slot = basis_slot_elems<T>(M.n_fn_max, M.n_ylm, M.maxl);
    T* sb = reinterpret_cast<T*>(smem_raw);
    double2* acc = reinterpret_cast<double2*>(
        (reinterpret_cast<uintptr_t>(sb + slot * nw) + 15) & ~uintptr_t(15));
    int* s_tp = reinterpret_cast<int*>(acc + ty.K0);
    int* s_ok = s_tp + nw;
    T* s_tab = reinterpret_cast<T*>(s_ok + nw + 4);
    s_tab = reinterpret_cast<T*>((reinterpret_cast<uintptr_t>(s_tab) + 15) & ~uintptr_t(15));
    load_ylm_tab<T>(M.ylm_tab, s_tab, M.n_ylm, M.maxl);
    const YlmTab<T> tab = ylm_tab_view<T>(s_tab, M.n_ylm, M.maxl);
    for (int h = threadIdx.x; h < ty.K0; h += blockDim.x) acc[h] = make_double2(0.0, 0.0);
    __syncthreads();
    const long long b = nb_off[i], e = nb_off[i + 1];
    for (long long base = b; base < e; base += nw) {
        const long long k = base + warp;
        BasisView<T> bv = basis_view<T>(sb + slot * warp, M.n_fn_max, M.n_ylm, M.maxl);
        if (k < e) {
            const double dx = nb_d[3 * k], dy = nb_d[3 * k + 1], dz = nb_d[3 * k + 2];
            double dis = 0.0;
            if (lane == 0) dis = sqrt(__dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz)));
            dis = __shfl_sync(0xffffffffu, dis, 0);
            const bool ok = dis < M.cutoff;
            const int tp = M.type_pairs[t1 * M.n_type + B.types[nb_j[k]]];
            if (lane == 0) {
                s_tp[warp] = tp;
                s_ok[warp] = ok;
            }
            if (ok) {
                warp_radial<T, false>(M, tp, dis, bv, lane);
                if (M.gtinv) {
                    warp_ylm<T, false>(M.maxl, M.n_ylm, tab, dx, dy, dz, dis, bv, lane);
                } else if (lane == 0) {
                    bv.Y[0] = {(T)1, (T)0};
                }
            }
        } else if (lane == 0) {
            s_ok[warp] = 0;
        }
        __syncthreads();
        for (int h = threadIdx.x; h < ty.K0; h += blockDim.x) {
            const int htp = ty.head_tp[h], nid = ty.head_nid[h], key = ty.head_key[h];
            // partial sum over this batch of pairs in T, added to the FP64 total
            T px = 0, py = 0;
            for (int w = 0; w < nw; ++w) {
                if (!s_ok[w] || s_tp[w] != htp) continue;
                BasisView<T> v = basis_view<T>(sb + slot * w, M.n_fn_max, M.n_ylm, M.maxl);
                const T f = v.fn[nid];
                if (!(f >= (T)1e-20)) continue;
                const cplx<T> y = v.Y[key];
                px += f * y.re;
                py += f * y.im;
            }
            double2 a = acc[h];
            a.x += (double)px;
            a.y += (double)py;
            acc[h] = a;
        }
        __syncthreads();
    }
    double2* out = A + a_off[i];
    for (int h = threadIdx.x; h < ty.K0; h += blockDim.x) out[h] = acc[h];
}

// ----------------------------------------------- K4 features and adjoint G
template <typename T>
__global__ void pg_features_adjoint(DevModel M, DevBatch B, const long long* a_off, const double2* A,
                                    const long long* d_off, T* D, const long long* g_off, cplx<T>* G) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int i = blockIdx.x;
    const int t1 = B.types[i];
    const DevType& ty = M.types[t1];
    cplx<T>* a = reinterpret_cast<cplx<T>*>(smem_raw);
    const double2* Ai = A + a_off[i];
    for (int f = threadIdx.x; f < ty.K; f += blockDim.x) {
        const double2 s = Ai[ty.full_src[f]];
        if (ty.full_is_conj[f]) {
            const double cc = ty.full_cc[f];
            a[f] = {(T)(cc * s.x), (T)(-cc * s.y)};
        } else {
            a[f] = {(T)s.x, (T)s.y};
        }
    }
    __syncthreads();
    T* Di = D + d_off[i];
    for (int k = threadIdx.x; k < ty.n_lin; k += blockDim.x) {
        T v = 0;
        for (int q = ty.val_off[k]; q < ty.val_off[k + 1]; ++q) {
            const FlatTerm& t = ty.val_terms[q];
            v += (T)t.coeff * term_product_real<T>(t, a);
        }
        Di[k] = v;
    }
    cplx<T>* Gi = G + g_off[i];
    for (int e = threadIdx.x; e < ty.n_ent; e += blockDim.x) {
        const int h = ty.ent_head[e];
        const T cc = (ty.head_m[h] & 1) ? (T)-1 : (T)1;
        cplx<T> g = {(T)0, (T)0};
        for (int q = ty.term_off[e]; q < ty.term_off[e + 1]; ++q) {
            const FlatTerm& t = ty.g_terms[q];
            const cplx<T> p = term_product<T>(t, a);
            const T c = (T)t.coeff;
            if (t.conj) {
                g.re += cc * c * p.re;
                g.im -= cc * c * p.im;
            } else {
                g.re += c * p.re;
                g.im += c * p.im;
            }
        }
        Gi[e] = g;
    }
}

// --------------------------------------------------------------- K5 rows
template <typename T, int TR>
__global__ void __launch_bounds__(sizeof(T) == 4 ? 512 : 256, 1) pg_rows(DevModel M, DevBatch B, const long long* nb_off, const int* nb_j, const double* nb_d,
                        const long long* d_off, const T* D, const long long* g_off, const cplx<T>* G,
                        const RowItem* items, const long long* f_row, int chunk_cap_ent, T* X, long long ld,
                        double* partial /* [item][7][F] */) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    // grid: x = column chunk (fastest, so the chunks of one structure run together), y = work item
    const RowItem it = items[blockIdx.y];
    const int CH = blockDim.x;
    const int c0 = blockIdx.x * CH;            // first column of this chunk
    const int cq = c0 + threadIdx.x;
    const bool col_ok = cq < M.F;              // position threadIdx.x of the chunk exists
    const int nw = CH >> 5, warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int s = it.st;
    const int sa0 = B.st_atom_off[s], n = B.st_atom_off[s + 1] - sa0;
    const int blk0 = it.a0;  // local index of the first target atom
    const bool force = f_row[s] >= 0;
    const int ntp = M.n_tp;

    // shared layout: out[TR*3][CH] | gval[cap] | gmeta[cap] | tpo[CH][ntp+1] | table | basis slots | slot info
    T* out = reinterpret_cast<T*>(smem_raw);
    cplx<T>* gval = reinterpret_cast<cplx<T>*>(out + (size_t)TR * 3 * CH);
    int* gmeta = reinterpret_cast<int*>(gval + chunk_cap_ent);
    int* tpo = gmeta + chunk_cap_ent;
    T* s_tab = reinterpret_cast<T*>(
        (reinterpret_cast<uintptr_t>(tpo + (size_t)CH * (ntp + 1)) + 15) & ~uintptr_t(15));
    const size_t slot = basis_slot_elems<T>(M.n_fn_max, M.n_ylm, M.maxl);
    T* sb = reinterpret_cast<T*>(
        (reinterpret_cast<uintptr_t>(s_tab + ylm_table_size(M.n_ylm, M.maxl)) + 15) & ~uintptr_t(15));
    T* sdx = reinterpret_cast<T*>((reinterpret_cast<uintptr_t>(sb + slot * nw) + 15) & ~uintptr_t(15));
    T* sdy = sdx + nw;
    T* sdz = sdy + nw;
    T* sdis = sdz + nw;
    int* stp = reinterpret_cast<int*>(sdis + nw);
    int* sj = stp + nw;
    int* sok = sj + nw;
    // per-column energy and stress sums (FP64), indexed by column position in the chunk
    double* cacc = reinterpret_cast<double*>((reinterpret_cast<uintptr_t>(sok + nw) + 15) & ~uintptr_t(15));
    for (int q = threadIdx.x; q < 7 * CH; q += CH) cacc[q] = 0.0;

    load_ylm_tab<T>(M.ylm_tab, s_tab, M.n_ylm, M.maxl);
    const YlmTab<T> tab = ylm_tab_view<T>(s_tab, M.n_ylm, M.maxl);
    for (int q = threadIdx.x; q < TR * 3 * CH; q += CH) out[q] = (T)0;
    int* my_tpo = tpo + (size_t)threadIdx.x * (ntp + 1);
    __syncthreads();

    for (int i = 0; i < n; ++i) {
        const int gi = sa0 + i;
        const int t1 = B.types[gi];
        const DevType& ty = M.types[t1];
        const bool centre_in = (i >= blk0 && i < blk0 + TR);
        const T* Di = D + d_off[gi];
        // --- the column this thread takes for centres of type t1, and its adjoint, grouped by type pair
        const int col = col_ok ? ty.col_perm[cq] : 0;
        const int cpos = col - c0;
        const int nc = col_ok ? ty.col_ncomp[col] : 0;
        const int my_off = col_ok ? ty.col_ent_off[col] : 0;
        if (nc > 0 && centre_in) {
            T pe = (T)1;
            for (int c = 0; c < nc; ++c) pe *= Di[ty.comp_k[col * 3 + c]];
            cacc[cpos] += (double)pe;
        }
        if (!force) {
            __syncthreads();  // the next centre may map this column to another thread
            continue;
        }
        {
            const cplx<T>* Gi = G + g_off[gi];
            T wt[3];
            int kk[3];
            for (int c = 0; c < nc; ++c) {
                kk[c] = ty.comp_k[col * 3 + c];
                T w = (T)1;
                for (int q = 0; q < 2; ++q) {
                    const int o = ty.comp_w[(col * 3 + c) * 2 + q];
                    if (o >= 0) w *= Di[o];
                }
                wt[c] = w;
            }
            int w = my_off;
            for (int t = 0; t < ntp; ++t) {
                my_tpo[t] = w;
                for (int c = 0; c < nc; ++c) {
                    const int* eo = ty.ent_tp_off + (size_t)kk[c] * (ntp + 1);
                    for (int e = eo[t]; e < eo[t + 1]; ++e) {
                        const cplx<T> g = Gi[e];
                        gval[w] = {wt[c] * g.re, wt[c] * g.im};
                        gmeta[w] = ty.ent_meta[e] >> 8;  // nid | key << 8
                        ++w;
                    }
                }
            }
            my_tpo[ntp] = w;
        }
        // --- pair images of centre i that touch this block
        long long pb = nb_off[gi], pe_ = nb_off[gi + 1];
        if (!centre_in) {
            // entries are sorted by neighbour index: find [lo, hi) with j in block
            long long lo = pb, hi = pe_;
            while (lo < hi) {
                const long long mid = (lo + hi) >> 1;
                if (nb_j[mid] - sa0 < blk0) lo = mid + 1;
                else hi = mid;
            }
            long long lo2 = lo, hi2 = pe_;
            while (lo2 < hi2) {
                const long long mid = (lo2 + hi2) >> 1;
                if (nb_j[mid] - sa0 < blk0 + TR) lo2 = mid + 1;
                else hi2 = mid;
            }
            pb = lo;
            pe_ = lo2;
        }
        // sums over the pairs of this centre in T; added to the FP64 totals per centre
        T self[3] = {0, 0, 0};
        T cst[6] = {0, 0, 0, 0, 0, 0};
        __syncthreads();  // gval/gmeta/tpo of centre i are complete
        for (long long base = pb; base < pe_; base += nw) {
            const long long k = base + warp;
            BasisView<T> bv = basis_view<T>(sb + slot * warp, M.n_fn_max, M.n_ylm, M.maxl);
            if (k < pe_) {
                const double dx = nb_d[3 * k], dy = nb_d[3 * k + 1], dz = nb_d[3 * k + 2];
                double dis = 0.0;
                if (lane == 0)
                    dis = sqrt(__dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz)));
                dis = __shfl_sync(0xffffffffu, dis, 0);
                const bool ok = dis < M.cutoff;
                const int j = nb_j[k];
                const int tp = M.type_pairs[t1 * M.n_type + B.types[j]];
                if (lane == 0) {
                    sdx[warp] = (T)dx;
                    sdy[warp] = (T)dy;
                    sdz[warp] = (T)dz;
                    sdis[warp] = (T)dis;
                    stp[warp] = tp;
                    sj[warp] = j - sa0;
                    sok[warp] = ok;
                }
                if (ok) {
                    warp_radial<T, true>(M, tp, dis, bv, lane);
                    if (M.gtinv) {
                        warp_ylm<T, true>(M.maxl, M.n_ylm, tab, dx, dy, dz, dis, bv, lane);
                    } else if (lane == 0) {
                        bv.Y[0] = {(T)1, (T)0};
                        bv.dY[0] = bv.dY[1] = bv.dY[2] = {(T)0, (T)0};
                    }
                }
            } else if (lane == 0) {
                sok[warp] = 0;
            }
            __syncthreads();
            if (col_ok && nc > 0) {
                const int nb = (int)min((long long)nw, pe_ - base);
                for (int w = 0; w < nb; ++w) {
                    if (!sok[w]) continue;
                    const int tp = stp[w];
                    const int e0 = my_tpo[tp], e1 = my_tpo[tp + 1];
                    if (e0 == e1) continue;
                    BasisView<T> v = basis_view<T>(sb + slot * w, M.n_fn_max, M.n_ylm, M.maxl);
                    T s0 = 0, sx = 0, sy = 0, sz = 0;
                    for (int q = e0; q < e1; ++q) {
                        const int meta = gmeta[q];
                        const int nid = meta & 0xff, key = meta >> 8;
                        const T f = v.fn[nid];
                        const cplx<T> g = gval[q];
                        s0 += v.fnd[nid] * creal_mul(g, v.Y[key]);
                        sx += f * creal_mul(g, v.dY[key]);
                        sy += f * creal_mul(g, v.dY[M.n_ylm + key]);
                        sz += f * creal_mul(g, v.dY[2 * M.n_ylm + key]);
                    }
                    const T dx = sdx[w], dy = sdy[w], dz = sdz[w];
                    const T sc = s0 / sdis[w];
                    const T vx = sc * dx + sx, vy = sc * dy + sy, vz = sc * dz + sz;
                    const int jl = sj[w];
                    if (centre_in) {
                        if (jl != i) {
                            self[0] += vx;
                            self[1] += vy;
                            self[2] += vz;
                        }
                        cst[0] -= vx * dx;
                        cst[1] -= vy * dy;
                        cst[2] -= vz * dz;
                        cst[3] -= vx * dy;
                        cst[4] -= vy * dz;
                        cst[5] -= vz * dx;
                    }
                    if (jl != i && jl >= blk0 && jl < blk0 + TR) {
                        T* o = out + (size_t)(jl - blk0) * 3 * CH + cpos;
                        o[0] -= vx;
                        o[CH] -= vy;
                        o[2 * CH] -= vz;
                    }
                }
            }
            __syncthreads();
        }
        if (centre_in && col_ok) {
            T* o = out + (size_t)(i - blk0) * 3 * CH + cpos;
            o[0] += self[0];
            o[CH] += self[1];
            o[2 * CH] += self[2];
            for (int q = 0; q < 6; ++q) cacc[(size_t)(q + 1) * CH + cpos] += (double)cst[q];
        }
        __syncthreads();  // before gval is rebuilt for the next centre
    }
    if (!col_ok) return;
    // column positions are in natural order: thread q writes column c0 + q
    if (force) {
        const long long r0 = f_row[s];
        const int na = min(TR, n - blk0);
        for (int a = 0; a < na; ++a)
            for (int c = 0; c < 3; ++c)
                X[(size_t)cq * ld + r0 + 3 * (blk0 + a) + c] = out[(size_t)a * 3 * CH + c * CH + threadIdx.x];
    }
    double* p = partial + (size_t)blockIdx.y * 7 * M.F;
    for (int q = 0; q < 7; ++q) p[(size_t)q * M.F + cq] = cacc[(size_t)q * CH + threadIdx.x];
}

// Sum the per-block energy/stress partials of each structure into X.
template <typename T>
__global__ void pg_rows_reduce(int F, const int* item_off /* n_st+1 */, const double* partial,
                               const long long* e_row, const long long* s_row, T* X, long long ld) {
    const int s = blockIdx.x;
    for (int col = threadIdx.x + blockIdx.y * blockDim.x; col < F; col += blockDim.x * gridDim.y) {
        double acc[7] = {0, 0, 0, 0, 0, 0, 0};
        for (int b = item_off[s]; b < item_off[s + 1]; ++b)
            for (int q = 0; q < 7; ++q) acc[q] += partial[((size_t)b * 7 + q) * F + col];
        X[(size_t)col * ld + e_row[s]] = (T)acc[0];
        if (s_row[s] >= 0)
            for (int q = 0; q < 6; ++q) X[(size_t)col * ld + s_row[s] + q] = (T)acc[q + 1];
    }
}

// ------------------------------------------------------------ prefix sums
// offsets[0] = 0, offsets[i + 1] = offsets[i] + counts[i]; one block of 1024.
__global__ void pg_exclusive_scan(const int* counts, int n, long long* offsets, long long* total) {
    __shared__ long long part[1024];
    const int t = threadIdx.x;
    const long long chunk = (n + blockDim.x - 1) / blockDim.x;
    const long long b = t * chunk, e = min((long long)n, b + chunk);
    long long s = 0;
    for (long long i = b; i < e; ++i) s += counts[i];
    part[t] = s;
    __syncthreads();
    for (int o = 1; o < (int)blockDim.x; o <<= 1) {
        const long long v = t >= o ? part[t - o] : 0;
        __syncthreads();
        part[t] += v;
        __syncthreads();
    }
    long long run = part[t] - s;  // exclusive prefix of this chunk
    if (t == 0) offsets[0] = 0;
    for (long long i = b; i < e; ++i) {
        run += counts[i];
        offsets[i + 1] = run;
    }
    if (t == blockDim.x - 1) *total = part[t];
}

// ------------------------------------------------------------- launchers
void launch_exclusive_scan(const int* counts, int n, long long* offsets, long long* total, cudaStream_t st) {
    pg_exclusive_scan<<<1, 1024, 0, st>>>(counts, n, offsets, total);
}

void launch_nb_count(const DevBatch& B, int* counts, cudaStream_t st) {
    const int threads = 256, warps = threads / 32;
    pg_nb_count<<<(B.n_atoms + warps - 1) / warps, threads, 0, st>>>(B, counts);
}

void launch_nb_fill(const DevBatch& B, const long long* off, int* nb_j, double* nb_d, cudaStream_t st) {
    const int threads = 256, warps = threads / 32;
    pg_nb_fill<<<(B.n_atoms + warps - 1) / warps, threads, 0, st>>>(B, off, nb_j, nb_d);
}

template <typename T>
void launch_anlm(const DevModel& M, const DevBatch& B, const long long* nb_off, const int* nb_j, const double* nb_d,
                 const long long* a_off, double2* A, int max_k0, cudaStream_t st) {
    const int threads = 128, nw = threads / 32;
    const size_t slot = basis_slot_elems<T>(M.n_fn_max, M.n_ylm, M.maxl);
    const size_t smem = slot * nw * sizeof(T) + 16 + (size_t)max_k0 * sizeof(double2) + (2 * nw + 4) * sizeof(int) +
                        16 + ylm_table_size(M.n_ylm, M.maxl) * sizeof(T);
    PG_CUDA(cudaFuncSetAttribute(pg_anlm<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    pg_anlm<T><<<B.n_atoms, threads, smem, st>>>(M, B, nb_off, nb_j, nb_d, a_off, A);
}

template <typename T>
void launch_features_adjoint(const DevModel& M, const DevBatch& B, const long long* a_off, const double2* A,
                             const long long* d_off, T* D, const long long* g_off, void* G, int max_k,
                             cudaStream_t st) {
    const size_t smem = (size_t)max_k * sizeof(cplx<T>);
    PG_CUDA(cudaFuncSetAttribute(pg_features_adjoint<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    pg_features_adjoint<T><<<B.n_atoms, 256, smem, st>>>(M, B, a_off, A, d_off, D, g_off,
                                                         reinterpret_cast<cplx<T>*>(G));
}

size_t rows_smem_bytes(const DevModel& M, int chunk, int cap_ent, bool fp64) {
    const size_t ts = fp64 ? 8 : 4;
    const int nw = chunk / 32;
    const size_t slot = fp64 ? basis_slot_elems<double>(M.n_fn_max, M.n_ylm, M.maxl)
                             : basis_slot_elems<float>(M.n_fn_max, M.n_ylm, M.maxl);
    return (size_t)kRowsTR * 3 * chunk * ts + (size_t)cap_ent * (2 * ts + 4) + (size_t)chunk * (M.n_tp + 1) * 4 +
           16 + (size_t)ylm_table_size(M.n_ylm, M.maxl) * ts + 16 + slot * nw * ts + 16 +
           (size_t)nw * (4 * 8 + 3 * 4) + 16 + (size_t)7 * chunk * 8;
}

template <typename T>
void launch_rows(const DevModel& M, const DevBatch& B, const long long* nb_off, const int* nb_j, const double* nb_d,
                 const long long* d_off, const T* D, const long long* g_off, const void* G, const RowItem* items,
                 int n_items, const long long* f_row, int chunk, int n_chunks, int cap_ent, T* X, long long ld,
                 double* partial, cudaStream_t st) {
    const size_t smem = rows_smem_bytes(M, chunk, cap_ent, sizeof(T) == 8);
    PG_CUDA(cudaFuncSetAttribute(pg_rows<T, kRowsTR>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    dim3 grid(n_chunks, n_items);
    pg_rows<T, kRowsTR><<<grid, chunk, smem, st>>>(M, B, nb_off, nb_j, nb_d, d_off, D, g_off,
                                                   reinterpret_cast<const cplx<T>*>(G), items, f_row, cap_ent, X,
                                                   ld, partial);
}

template <typename T>
void launch_rows_reduce(int F, int n_st, const int* item_off, const double* partial, const long long* e_row,
                        const long long* s_row, T* X, long long ld, cudaStream_t st) {
    dim3 grid(n_st, (F + 255) / 256);
    pg_rows_reduce<T><<<grid, 256, 0, st>>>(F, item_off, partial, e_row, s_row, X, ld);
}

template void launch_anlm<double>(const DevModel&, const DevBatch&, const long long*, const int*, const double*,
                                  const long long*, double2*, int, cudaStream_t);
template void launch_anlm<float>(const DevModel&, const DevBatch&, const long long*, const int*, const double*,
                                 const long long*, double2*, int, cudaStream_t);
template void launch_features_adjoint<double>(const DevModel&, const DevBatch&, const long long*, const double2*,
                                              const long long*, double*, const long long*, void*, int,
                                              cudaStream_t);
template void launch_features_adjoint<float>(const DevModel&, const DevBatch&, const long long*, const double2*,
                                             const long long*, float*, const long long*, void*, int, cudaStream_t);
template void launch_rows<double>(const DevModel&, const DevBatch&, const long long*, const int*, const double*,
                                  const long long*, const double*, const long long*, const void*, const RowItem*,
                                  int, const long long*, int, int, int, double*, long long, double*, cudaStream_t);
template void launch_rows<float>(const DevModel&, const DevBatch&, const long long*, const int*, const double*,
                                 const long long*, const float*, const long long*, const void*, const RowItem*, int,
                                 const long long*, int, int, int, float*, long long, double*, cudaStream_t);
template void launch_rows_reduce<double>(int, int, const int*, const double*, const long long*, const long long*,
                                         double*, long long, cudaStream_t);
template void launch_rows_reduce<float>(int, int, const int*, const double*, const long long*, const long long*,
                                        float*, long long, cudaStream_t);

}  // namespace pg
