// Training rows of X on the GPU.
//
//   pg_nb_count / pg_nb_fill   full neighbour list of every atom of a batch
//   (+ pg_nb_order/pg_nb_disp) (NeighborFull, compute/neighbor_full.cpp:10-76):
//                              same (j, translation) order and bit-identical
//                              displacements (IEEE double, no contraction);
//                              structures of 1,024+ atoms search a cell list and
//                              order their candidates afterwards.
//   pg_anlm                    a_nlm for m <= 0 of every atom (local.cpp:62-114),
//                              sums over neighbours accumulated in FP64 (FP32
//                              kernel: float-float).
//   pg_features_adjoint        invariant features d_k of every atom and the
//                              sparse adjoint G_k[h] = d d_k / d a_h with the
//                              conjugate half folded in (features.cpp:155-248),
//                              stored in the X-row layout by type pair.
//   pg_nb_mirror               mirror index of every pair.
//   pg_rows_pairs              per centre: the derivatives dd_k/dd_p of its
//                              linear features for every pair (the pair bases
//                              contracted with the adjoint G), and their self
//                              and virial sums.
//   pg_rows                    force rows of X per target atom: the pair
//                              derivatives landing on it summed into its
//                              linear columns and weighted into its product
//                              columns (model.cpp:159-267).
//   pg_rows_es                 energy and stress rows per structure.
#include <cuda_runtime.h>

#include <climits>

#include "kernels.h"

namespace pg {

// ------------------------------------------------------------ K1 neighbours
// One warp per centre atom; candidates (j, t) in j-major order.  Only
// __dadd_rn/__dmul_rn are used so nothing is contracted into an FMA.
// Whether candidate (j, translation t) is a neighbour of i: the FP64
// squared distance r2 = dx^2 + dy^2 + dz^2 (dx = (pj - pi) + t, no
// contraction) satisfies tol2 < r2 < rc2.  FP32 decides every candidate
// whose FP32 squared distance is beyond the rounding margin on either side
// (prefilter_r2 above, inner_r2 below, and well above zero); the rest (a
// thin shell at the cutoff, near-coincident atoms) are decided in FP64.
__device__ __forceinline__ bool pair_in(const DevBatch& B, int i, int j, int t, double rc2, double tol2) {
    const float4 a = B.posf[i], b = B.posf[j], tt = B.transf[t];
    const float fx = b.x - a.x + tt.x, fy = b.y - a.y + tt.y, fz = b.z - a.z + tt.z;
    const float r2f = fx * fx + fy * fy + fz * fz;
    if (r2f > B.prefilter_r2) return false;
    if (r2f < B.inner_r2 && r2f > 1e-6f) return true;
    const double* pi = B.pos + 3 * (size_t)i;
    const double* pj = B.pos + 3 * (size_t)j;
    const double* tr = B.trans + 3 * (size_t)t;
    const double dx = __dadd_rn(__dadd_rn(pj[0], -pi[0]), tr[0]);
    const double dy = __dadd_rn(__dadd_rn(pj[1], -pi[1]), tr[1]);
    const double dz = __dadd_rn(__dadd_rn(pj[2], -pi[2]), tr[2]);
    const double r2 = __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
    return r2 < rc2 && r2 > tol2;
}

// List entry q of atom i from its key j_local * nt + t: the neighbour, the
// FP64 displacement (pj - pi) + t (the form the neighbour test uses) and its
// FP32 copy with the FP32 squared distance.
__device__ __forceinline__ void write_entry(const DevBatch& B, int i, int a0, int t0, int nt, long long key,
                                            long long q, int* nb_j, double* nb_d, float4* nb_df) {
    const int j = a0 + (int)(key / nt), t = t0 + (int)(key % nt);
    const double* pi = B.pos + 3 * (size_t)i;
    const double* pj = B.pos + 3 * (size_t)j;
    const double* tr = B.trans + 3 * (size_t)t;
    const double dx = __dadd_rn(__dadd_rn(pj[0], -pi[0]), tr[0]);
    const double dy = __dadd_rn(__dadd_rn(pj[1], -pi[1]), tr[1]);
    const double dz = __dadd_rn(__dadd_rn(pj[2], -pi[2]), tr[2]);
    nb_j[q] = j;
    nb_d[3 * q] = dx;
    nb_d[3 * q + 1] = dy;
    nb_d[3 * q + 2] = dz;
    const float x = (float)dx, y = (float)dy, z = (float)dz;
    nb_df[q] = make_float4(x, y, z, x * x + y * y + z * z);
}

// Cell-list candidates of atom i (structure with cell list c): for every
// translation u whose shifted sphere meets the atoms' fractional range, the
// atoms of the bins it covers.  Calls visit(k_in_cl_atoms_range...) through the
// bin ranges; the warp iterates bins uniformly and lanes take the atoms.
struct ClQuery {
    int lo[3], hi[3];
};
__device__ __forceinline__ bool cl_range(const DevBatch& B, int c, const double* fi, int4 n, ClQuery& q) {
    const int4 g = B.cl_grid[c];
    const double* geo = B.cl_geom + 9 * c;
    const int gd[3] = {g.x, g.y, g.z};
    const int nd[3] = {n.x, n.y, n.z};
    for (int d = 0; d < 3; ++d) {
        const double cq = fi[d] - nd[d];
        const double l = floor((cq - geo[6 + d] - geo[d]) * geo[3 + d]);
        const double h = floor((cq + geo[6 + d] - geo[d]) * geo[3 + d]);
        if (h < 0.0 || l > gd[d] - 1) return false;
        q.lo[d] = l < 0.0 ? 0 : (int)l;
        q.hi[d] = h > gd[d] - 1 ? gd[d] - 1 : (int)h;
    }
    return true;
}

__global__ void pg_nb_count(DevBatch B, int* counts, int* max_cl) {
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (warp >= B.n_atoms) return;
    const int i = warp;
    const int s = B.atom_st[i];
    const int a0 = B.st_atom_off[s], n = B.st_atom_off[s + 1] - a0;
    const int t0 = B.st_trans_off[s], nt = B.st_trans_off[s + 1] - t0;
    const double rc2 = __dmul_rn(B.cutoff, B.cutoff), tol2 = __dmul_rn(1e-10, 1e-10);
    int cnt = 0;
    const int c = B.st_cl[s];
    if (c >= 0) {
        const double fi[3] = {B.frac[3 * (size_t)i], B.frac[3 * (size_t)i + 1], B.frac[3 * (size_t)i + 2]};
        const int4 g = B.cl_grid[c];
        for (int u = 0; u < nt; ++u) {
            ClQuery q;
            if (!cl_range(B, c, fi, B.tn[t0 + u], q)) continue;
            for (int bz = q.lo[2]; bz <= q.hi[2]; ++bz)
                for (int by = q.lo[1]; by <= q.hi[1]; ++by)
                    for (int bx = q.lo[0]; bx <= q.hi[0]; ++bx) {
                        const int bin = g.w + (bz * g.y + by) * g.x + bx;
                        for (int k = B.cl_bin_start[bin] + lane; k < B.cl_bin_start[bin + 1]; k += 32)
                            cnt += pair_in(B, i, B.cl_atoms[k], t0 + u, rc2, tol2) ? 1 : 0;
                    }
        }
    } else {
        const int total = n * nt;  // candidates (j, t), j-major; n * nt < 2^31 (checked on the host)
        // lane q = j * nt + t walks the candidates with a carried (j, t) instead of dividing
        int j = lane / nt, t = lane % nt;
        const int dj = 32 / nt, dt = 32 % nt;
        for (int q = lane; q < total; q += 32) {
            cnt += pair_in(B, i, a0 + j, t0 + t, rc2, tol2) ? 1 : 0;
            j += dj;
            t += dt;
            if (t >= nt) {
                t -= nt;
                ++j;
            }
        }
    }
    for (int o = 16; o > 0; o >>= 1) cnt += __shfl_down_sync(0xffffffffu, cnt, o);
    if (lane == 0) {
        counts[i] = cnt;
        if (c >= 0) atomicMax(max_cl, cnt);
    }
}

// The kept candidates' keys j_local * nt + t: in (j, t) order for brute-force
// atoms (entries written by pg_nb_disp), unordered for cell-list atoms
// (ordered and written by pg_nb_order).
__global__ void pg_nb_fill(DevBatch B, const long long* offsets, long long* keys) {
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (warp >= B.n_atoms) return;
    const int i = warp;
    const int s = B.atom_st[i];
    const int a0 = B.st_atom_off[s], n = B.st_atom_off[s + 1] - a0;
    const int t0 = B.st_trans_off[s], nt = B.st_trans_off[s + 1] - t0;
    const double rc2 = __dmul_rn(B.cutoff, B.cutoff), tol2 = __dmul_rn(1e-10, 1e-10);
    long long w = offsets[i];
    const long long wend = offsets[i + 1];
    const int c = B.st_cl[s];
    if (c >= 0) {
        const double fi[3] = {B.frac[3 * (size_t)i], B.frac[3 * (size_t)i + 1], B.frac[3 * (size_t)i + 2]};
        const int4 g = B.cl_grid[c];
        for (int u = 0; u < nt; ++u) {
            ClQuery q;
            if (!cl_range(B, c, fi, B.tn[t0 + u], q)) continue;
            for (int bz = q.lo[2]; bz <= q.hi[2]; ++bz)
                for (int by = q.lo[1]; by <= q.hi[1]; ++by)
                    for (int bx = q.lo[0]; bx <= q.hi[0]; ++bx) {
                        const int bin = g.w + (bz * g.y + by) * g.x + bx;
                        const int kb = B.cl_bin_start[bin], ke = B.cl_bin_start[bin + 1];
                        for (int k0 = kb; k0 < ke; k0 += 32) {
                            const int k = k0 + lane;
                            int j = 0;
                            bool keep = false;
                            if (k < ke) {
                                j = B.cl_atoms[k];
                                keep = pair_in(B, i, j, t0 + u, rc2, tol2);
                            }
                            const unsigned m = __ballot_sync(0xffffffffu, keep);
                            if (keep) {
                                const long long p = w + __popc(m & ((1u << lane) - 1u));
                                if (p < wend) keys[p] = (long long)(j - a0) * nt + u;
                            }
                            w += __popc(m);
                        }
                    }
        }
        return;
    }
    const int total = n * nt;
    int j = lane / nt, t = lane % nt;
    const int dj = 32 / nt, dt = 32 % nt;
    for (int base = 0; base < total; base += 32) {
        const int q = base + lane;
        const int jq = j, tq = t;
        bool keep = false;
        if (q < total) keep = pair_in(B, i, a0 + j, t0 + t, rc2, tol2);
        j += dj;
        t += dt;
        if (t >= nt) {
            t -= nt;
            ++j;
        }
        const unsigned m = __ballot_sync(0xffffffffu, keep);
        if (keep) {
            const long long k = w + __popc(m & ((1u << lane) - 1u));
            if (k < wend) keys[k] = (long long)jq * nt + tq;
        }
        w += __popc(m);
    }
}

// Entries of the brute-force atoms from their keys (one warp per atom).
__global__ void pg_nb_disp(DevBatch B, const long long* offsets, const long long* keys, int* nb_j, double* nb_d,
                           float4* nb_df) {
    const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (i >= B.n_atoms) return;
    const int s = B.atom_st[i];
    if (B.st_cl[s] >= 0) return;
    const int a0 = B.st_atom_off[s];
    const int t0 = B.st_trans_off[s], nt = B.st_trans_off[s + 1] - t0;
    for (long long q = offsets[i] + lane; q < offsets[i + 1]; q += 32)
        write_entry(B, i, a0, t0, nt, keys[q], q, nb_j, nb_d, nb_df);
}

// Cell-list atoms: sort the candidate keys (block per atom, bitonic in shared
// memory) into the reference's (j, t) order and write the list entries, with
// the displacement recomputed exactly as the neighbour test forms it.
__global__ void pg_nb_order(DevBatch B, const long long* offsets, long long* keys, int* nb_j, double* nb_d,
                            float4* nb_df) {
    __shared__ long long sk[kCellListMaxPairs];
    const int i = blockIdx.x;
    const int s = B.atom_st[i];
    if (B.st_cl[s] < 0) return;
    const int a0 = B.st_atom_off[s];
    const int t0 = B.st_trans_off[s], nt = B.st_trans_off[s + 1] - t0;
    const long long o0 = offsets[i];
    const int m = (int)(offsets[i + 1] - o0);
    if (m > kCellListMaxPairs) return;  // rejected on the host before this launch
    int p2 = 1;
    while (p2 < m) p2 <<= 1;
    for (int q = threadIdx.x; q < p2; q += blockDim.x) sk[q] = q < m ? keys[o0 + q] : LLONG_MAX;
    __syncthreads();
    for (int k = 2; k <= p2; k <<= 1)
        for (int jj = k >> 1; jj > 0; jj >>= 1) {
            for (int q = threadIdx.x; q < p2; q += blockDim.x) {
                const int r = q ^ jj;
                if (r > q) {
                    const long long x = sk[q], y = sk[r];
                    const bool up = (q & k) == 0;
                    if ((x > y) == up) {
                        sk[q] = y;
                        sk[r] = x;
                    }
                }
            }
            __syncthreads();
        }
    for (int q = threadIdx.x; q < m; q += blockDim.x) {
        write_entry(B, i, a0, t0, nt, sk[q], o0 + q, nb_j, nb_d, nb_df);
        keys[o0 + q] = sk[q];  // entry q's key, for later refreshes of its displacement
    }
}

// Displacements of every list entry from its key, after the positions have
// moved (the evaluator's neighbour-list reuse; one warp per atom).
__global__ void pg_nb_refresh(DevBatch B, const long long* offsets, const long long* keys, int* nb_j, double* nb_d,
                              float4* nb_df) {
    const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (i >= B.n_atoms) return;
    const int s = B.atom_st[i];
    const int a0 = B.st_atom_off[s];
    const int t0 = B.st_trans_off[s], nt = B.st_trans_off[s + 1] - t0;
    for (long long q = offsets[i] + lane; q < offsets[i + 1]; q += 32)
        write_entry(B, i, a0, t0, nt, keys[q], q, nb_j, nb_d, nb_df);
}

// ---------------------------------------------------------------- K2 a_nlm
// Block per centre atom, pairs taken one type pair at a time: the pairs of
// that type pair are compacted into a list (256 at a time) and taken up to 32
// at a time (a super-chunk).  The block builds their bases at once into
// shared memory (thread = pair and two Legendre columns, ylm_column, or pair
// and radial functions): Y_lm [pair][key] and f_n [pair][n].  Then every
// thread adds f_n Y_lm over the super-chunk's pairs into the heads of that
// type pair it owns: partial sums over 8 pairs in T, each added to the long
// (FP64, or float-float) total.
constexpr int kAnlmChunk = 32;  // pairs per a_nlm super-chunk
template <typename T>
__global__ void __launch_bounds__(256) pg_anlm(DevModel M, DevBatch B, const long long* nb_off, const int* nb_j,
                                               const double* nb_d, const long long* a_off, cplx<T>* A) {
    constexpr int NW = 8, PS = kAnlmChunk, TPP = 256 / PS;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ int s_list[256], s_wcnt[NW];
    const int i = blockIdx.x;
    const int t1 = B.types[i];
    const DevType& ty = M.types[t1];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int NY = M.n_ylm, NF = M.n_fn_max, L = M.maxl;
    // per head: running sums of the real and imaginary parts (16 bytes)
    LongSum<T>* acc = reinterpret_cast<LongSum<T>*>(smem_raw);
    cplx<T>* Yt = reinterpret_cast<cplx<T>*>(acc + 2 * (size_t)ty.K0);  // [PS][NY]
    T* rad = reinterpret_cast<T*>(Yt + (size_t)PS * NY);                // [PS][NF]
    T* s_tab = rad + (size_t)PS * NF;
    load_ylm_tab<T>(M.ylm_tab, s_tab, M.n_ylm, M.maxl);
    const YlmTab<T> tab = ylm_tab_view<T>(s_tab, M.n_ylm, M.maxl);
    for (int h = threadIdx.x; h < 2 * ty.K0; h += blockDim.x) acc[h] = LongSum<T>();
    const long long p0 = nb_off[i];
    const int np = (int)(nb_off[i + 1] - p0);
    for (int tp = 0; tp < M.n_tp; ++tp) {
        const int q0 = ty.tp_head_off[tp], nh = ty.tp_head_off[tp + 1] - q0;
        if (nh == 0) continue;  // the type pair is not one of this centre type's
        const int nfn = M.tp_nfn[tp];
        for (int r0 = 0; r0 < np; r0 += 256) {
            // compact the pairs of tp among r0 .. r0 + 255, in list order
            const int r = r0 + threadIdx.x;
            const bool f = r < np && M.type_pairs[t1 * M.n_type + B.types[nb_j[p0 + r]]] == tp;
            const unsigned m = __ballot_sync(0xffffffffu, f);
            if (lane == 0) s_wcnt[warp] = __popc(m);
            __syncthreads();
            int before = 0, c = 0;
            for (int w = 0; w < NW; ++w) {
                before += w < warp ? s_wcnt[w] : 0;
                c += s_wcnt[w];
            }
            if (f) s_list[before + __popc(m & ((1u << lane) - 1u))] = r;
            __syncthreads();
            for (int k0 = 0; k0 < c; k0 += PS) {
                const int n = min(PS, c - k0);
                // bases: thread t of pair p builds Legendre columns (a, L - a) for
                // a = t, t + TPP, .. (2a <= L), then radial functions t, t + TPP, ..
                {
                    const int p = threadIdx.x / TPP, t = threadIdx.x % TPP;
                    T dx = 0, dy = 0, dz = 0, dis = 1;
                    const bool ok = p < n && pair_geometry<T>(M, B, nb_d, p0 + s_list[k0 + p], dx, dy, dz, dis);
                    T* rows = reinterpret_cast<T*>(Yt + (size_t)p * NY);
                    if (M.gtinv) {
                        const YlmDir<T> dir = ylm_dir<T>(dx, dy, dz, dis);
                        for (int a = t; 2 * a <= L; a += TPP)
                            for (int side = 0; side < 2; ++side) {
                                const int mp = side ? L - a : a;
                                if (side && mp == a) break;
                                if (ok) {
                                    ylm_column<T, false>(mp, L, tab, dir, rows, 2);
                                } else {
                                    for (int l = mp; l <= L; ++l) {
                                        rows[2 * (l * (l + 1) / 2 + l - mp)] = (T)0;
                                        rows[2 * (l * (l + 1) / 2 + l - mp) + 1] = (T)0;
                                    }
                                }
                            }
                    } else if (t == 0) {
                        rows[0] = ok ? (T)1 : (T)0;
                        rows[1] = (T)0;
                    }
                    for (int q = t; q < nfn; q += TPP) {
                        T fn = 0, fnd;
                        if (ok) radial_one<T>(M, tp, q, dis, fn, fnd);
                        rad[p * NF + q] = fn;
                    }
                }
                __syncthreads();
                for (int q = threadIdx.x; q < nh; q += blockDim.x) {
                    const int h = ty.tp_heads[q0 + q];
                    const int nid = ty.head_nid[h], key = ty.head_key[h];
                    for (int w0 = 0; w0 < n; w0 += 8) {
                        T px = 0, py = 0;
                        for (int w = w0; w < min(n, w0 + 8); ++w) {
                            const T fw = rad[w * NF + nid];
                            if (!(fw >= (T)1e-20)) continue;
                            const cplx<T> y = Yt[(size_t)w * NY + key];
                            px += fw * y.re;
                            py += fw * y.im;
                        }
                        acc[2 * h].add(px);
                        acc[2 * h + 1].add(py);
                    }
                }
                __syncthreads();
            }
        }
    }
    cplx<T>* out = A + a_off[i];
    for (int h = threadIdx.x; h < ty.K0; h += blockDim.x) out[h] = {acc[2 * h].value(), acc[2 * h + 1].value()};
}

// ----------------------------------------------- K4 features and adjoint G
// Block per centre.  Windowed warp sums: a warp evaluates kAdjWin terms of its
// 32 outputs at a time (all lanes, whatever output a term belongs to; the
// packed codes and coefficients of the window are requested together, so that
// their L2 latency overlaps), then each lane adds its own output's terms from
// the window, in list order.  (A rank of 32 adjoint slots holds about 130
// terms in the binary l_max 8 model: 128-term windows in FP32; the FP64 kernel,
// with its slower products, gains from 256.)
template <typename T>
constexpr int adj_win() { return sizeof(T) == 4 ? 128 : 256; }
template <typename T>
__global__ void __launch_bounds__(256, sizeof(T) == 4 ? 4 : 3) pg_features_adjoint(DevModel M, DevBatch B, const long long* a_off,
                                                           const cplx<T>* A, const long long* d_off, T* D,
                                                           const long long* g_off, cplx<T>* G) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    constexpr int NW = 8, kWin = adj_win<T>(), kU = kWin / 32;
    const int i = blockIdx.x;
    const int t1 = B.types[i];
    const DevType& ty = M.types[t1];
    cplx<T>* a = reinterpret_cast<cplx<T>*>(smem_raw);
    cplx<T>* s_v = a + ty.K;  // [NW][kWin]
    load_full_a<T>(ty, A + a_off[i], a);
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    cplx<T>* win = s_v + (size_t)warp * kWin;
    // feature values d_k = sum_q coeff_q Re(prod a[ids_q])
    const int nl = ty.n_lin;
    const T* vcoef = reinterpret_cast<const T*>(ty.vcoef);
    T* Di = D + d_off[i];
    for (int k0 = 32 * warp; k0 < nl; k0 += 32 * NW) {
        const int k = k0 + lane;
        const int tb = ty.val_off[k0], te = ty.val_off[min(k0 + 32, nl)];
        const int ms = k < nl ? ty.val_off[k] : te, me = k < nl ? ty.val_off[k + 1] : te;
        T v = 0;
        for (int w0 = tb; w0 < te; w0 += kWin) {
            int4 c4[kU];
            T cf[kU];
#pragma unroll
            for (int u = 0; u < kU; ++u) {
                const int t = min(w0 + 32 * u + lane, te - 1);
                c4[u] = ty.vcode[t];
                cf[u] = vcoef[t];
            }
#pragma unroll
            for (int u = 0; u < kU; ++u)
                if (w0 + 32 * u + lane < te) win[32 * u + lane].re = cf[u] * packed_term_product<T>(c4[u], a).re;
            __syncwarp();
            const int lo = max(ms, w0), hi = min(me, w0 + kWin);
            for (int t = lo; t < hi; ++t) v += win[t - w0].re;
            __syncwarp();
        }
        if (k < nl) Di[k] = v;
    }
    // adjoint entries in the X-row layout (rank-major groups of bundles per
    // type pair; padding slots hold zero), warp per rank of 32 slots
    cplx<T>* Gi = G + g_off[i];
    const T* coef = reinterpret_cast<const T*>(ty.tcoef);
    for (int rk = warp; rk < ty.lay_size / 32; rk += NW) {
        const int slot = 32 * rk + lane;
        const int tb = ty.slot_toff[32 * rk], te = ty.slot_toff[32 * rk + 32];
        const int ms = ty.slot_toff[slot], me = ty.slot_toff[slot + 1];
        cplx<T> g = {(T)0, (T)0};
        for (int w0 = tb; w0 < te; w0 += kWin) {
            int4 c4[kU];
            T cf[kU];
#pragma unroll
            for (int u = 0; u < kU; ++u) {
                const int t = min(w0 + 32 * u + lane, te - 1);
                c4[u] = ty.tcode[t];
                cf[u] = coef[t];
            }
#pragma unroll
            for (int u = 0; u < kU; ++u)
                if (w0 + 32 * u + lane < te) {
                    const cplx<T> p = packed_term_product<T>(c4[u], a);
                    cplx<T> v = {cf[u] * p.re, cf[u] * p.im};
                    if (c4[u].w >> 8) v.im = -v.im;
                    win[32 * u + lane] = v;
                }
            __syncwarp();
            const int lo = max(ms, w0), hi = min(me, w0 + kWin);
            for (int t = lo; t < hi; ++t) {
                const cplx<T> v = win[t - w0];
                g.re += v.re;
                g.im += v.im;
            }
            __syncwarp();
        }
        Gi[slot] = g;
    }
}

// --------------------------------------------------------------- K5 rows
// The force rows of X factor through the linear features d_k of each centre:
//   X_force[(j,c), col] = -sum_{p: i_p -> j, i_p != j} sum_{k in col} w_k,col(i_p) dd_k(i_p)/dd_p,c
//                         + [j = i] sum_{k in col} w_k,col(i) sum_{p in list(i), j_p != i} dd_k(i)/dd_p,c,
// where w_k,col(i) is the product of the other features of the column and
// dd_k(i)/dd_p = sum_e Re(G_e(i) . dphi_(h_e)(d_p)/dd_p) over the adjoint
// entries of k (model.cpp:159-267 builds the same rows column by column).
//   pg_nb_mirror    index of the mirror (j -> i, -d) of every pair (i -> j, d)
//   pg_rows_pairs   stage A, per centre: dd_k/dd_p for every pair p, stored at
//                   the slot of its mirror (so the pairs landing on a target are
//                   contiguous), plus the self and virial sums DS
//   pg_rows         stage B, per target block: expansion into the columns
//   pg_rows_es      energy and stress rows, per structure

// Mirror of every pair: entry (b -> a, d) pairs with (a -> b, -d).  The
// translation set is symmetric and displacements are formed without
// contraction, so -d is bit-identical.  Optionally also the group slot of the
// pair: the first entry of b in a's list.  One warp per atom.
__global__ void pg_nb_mirror(int n_atoms, const long long* nb_off, const int* nb_j, const double* nb_d,
                             long long* mirror, long long* gslot, int* missing) {
    const int b = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (b >= n_atoms) return;
    for (long long q = nb_off[b] + lane; q < nb_off[b + 1]; q += 32) {
        const int a = nb_j[q];
        const double dx = nb_d[3 * q], dy = nb_d[3 * q + 1], dz = nb_d[3 * q + 2];
        long long lo = nb_off[a], hi = nb_off[a + 1];
        while (lo < hi) {
            const long long mid = (lo + hi) >> 1;
            if (nb_j[mid] < b) lo = mid + 1;
            else hi = mid;
        }
        if (gslot) gslot[q] = lo;  // first entry of b in a's list: the slot of the group (b, a)
        long long m = -1;
        for (long long p = lo; p < nb_off[a + 1] && nb_j[p] == b; ++p)
            if (nb_d[3 * p] == -dx && nb_d[3 * p + 1] == -dy && nb_d[3 * p + 2] == -dz) {
                m = p;
                break;
            }
        mirror[q] = m;
        if (m < 0) atomicAdd(missing, 1);
    }
}

// Stage A.  Block per centre atom i of a force structure; its pairs are
// ordered by type pair (stably, so the images of a neighbour stay
// consecutive).  The entries of feature k by a type pair share one radial
// function n (host/flat_tables.h), so with phi_h(d) = f_n(r) Y_lm(d/r) the
// derivative by pair p factors into
//   dd_k/dd_p,c = f_n(r_p) S_k,c(p) + f_n'(r_p) (d_p,c / r_p) T_k(p),
//   T_k(p) = sum_e Re(G_e(i) Y_(key e)(p)),  S_k,c(p) = sum_e Re(G_e(i) dY_(key e)(p)/dd_c).
// The pairs of one type pair are taken up to `ps` at a time (a super-chunk):
// the block builds their bases at once into shared memory, a table of the
// Y_lm and their gradients (8 values per key; thread = pair and two Legendre
// columns, ylm_column) and of the radial functions (f_n, f_n' d_x/r,
// f_n' d_y/r, f_n' d_z/r; thread = pair and n).  Then each warp takes groups
// of 32 bundles (lane = two features with the same key sequence) and runs
// over the group's entries once per NW pairs of the super-chunk, one table
// row per pair and rank serving both features.  The entries of the centre are
// stored by type pair, rank-major in groups (pg_features_adjoint), so the
// lanes read them coalesced with equal loop lengths and most ranks name one
// key for all 32 lanes: a shared-memory broadcast.
// The images of one neighbour j are summed and stored once, at the group slot
// (the first entry of i in j's list), indexed by feature position, so stage B
// reads one vector per (centre, target).  The centre's DS vectors are
// accumulated per type pair, also by feature position, in registers over a
// super-chunk:
//   DS[i][tp][c][x]   = sum_{p of tp, j_p != i} dd_k/dd_p,c         (self rows)
//   DS[i][tp][3+q][x] = sum_{p of tp} d_p,b(q) dd_k/dd_p,a(q)       (virial)
// with k = perm_tp[x] and (a, b)(q) = (x,x) (y,y) (z,z) (x,y) (y,z) (z,x).

// Eight consecutive values of a 16-byte-aligned shared-memory row.
__device__ __forceinline__ void load_row8(const float* p, float (&v)[8]) {
    const float4 a = reinterpret_cast<const float4*>(p)[0], b = reinterpret_cast<const float4*>(p)[1];
    v[0] = a.x;
    v[1] = a.y;
    v[2] = a.z;
    v[3] = a.w;
    v[4] = b.x;
    v[5] = b.y;
    v[6] = b.z;
    v[7] = b.w;
}
__device__ __forceinline__ void load_row8(const double* p, double (&v)[8]) {
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const double2 a = reinterpret_cast<const double2*>(p)[q];
        v[2 * q] = a.x;
        v[2 * q + 1] = a.y;
    }
}
__device__ __forceinline__ void load_row4(const float* p, float (&v)[4]) {
    const float4 a = *reinterpret_cast<const float4*>(p);
    v[0] = a.x;
    v[1] = a.y;
    v[2] = a.z;
    v[3] = a.w;
}
__device__ __forceinline__ void load_row4(const double* p, double (&v)[4]) {
    const double2 a = reinterpret_cast<const double2*>(p)[0], b = reinterpret_cast<const double2*>(p)[1];
    v[0] = a.x;
    v[1] = a.y;
    v[2] = b.x;
    v[3] = b.y;
}

// Two consecutive values at an 8- (FP32) or 16-byte (FP64) aligned address.
__device__ __forceinline__ void load_pair(const float* p, float (&v)[2]) {
    const float2 a = *reinterpret_cast<const float2*>(p);
    v[0] = a.x;
    v[1] = a.y;
}
__device__ __forceinline__ void load_pair(const double* p, double (&v)[2]) {
    const double2 a = *reinterpret_cast<const double2*>(p);
    v[0] = a.x;
    v[1] = a.y;
}
__device__ __forceinline__ void store_pair(float* p, const float (&v)[2]) {
    *reinterpret_cast<float2*>(p) = make_float2(v[0], v[1]);
}
__device__ __forceinline__ void store_pair(double* p, const double (&v)[2]) {
    *reinterpret_cast<double2*>(p) = make_double2(v[0], v[1]);
}

template <typename T>
__global__ void __launch_bounds__(kRowsThreads, sizeof(T) == 4 ? 2 : 1)
    pg_rows_pairs(DevModel M, DevBatch B, const long long* nb_off, const int* nb_j, const double* nb_d,
                  const long long* gslot, const long long* s_off, const long long* g_off, const cplx<T>* G,
                  const long long* f_row, int* order, T* Dp, T* DS, int ps) {
    constexpr int NW = kRowsThreads / 32;
    static_assert(NW == 8, "a contraction step takes 8 pairs");
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ int s_wcnt[NW], s_tpoff[kMaxTypePairs + 1];
    __shared__ int s_flag[kMaxSuperChunk];  // ok | self << 1 | flush << 2 | fresh << 3
    __shared__ long long s_slot[kMaxSuperChunk];
    const int i = blockIdx.x;
    if (f_row[B.atom_st[i]] < 0) return;
    const int t1 = B.types[i];
    const DevType& ty = M.types[t1];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int NL = M.max_lin, NY = M.n_ylm, NF = M.n_fn_max, L = M.maxl;
    // Y_lm table [key][pair][8] (Y, dY/dx, dY/dy, dY/dz as re, im): the rows of
    // the pairs of a step sit at fixed offsets from their key's row; the key
    // stride is padded by 16 or 32 bytes so that lanes reading different keys
    // of one pair hit different banks
    const int KS = ps * 8 + 4;
    T* tab = reinterpret_cast<T*>(smem_raw);  // [NY][KS]
    T* rad = tab + (size_t)NY * KS;           // [ps][NF][4]: f, f' x/r, f' y/r, f' z/r
    T* geo = rad + (size_t)ps * NF * 4;       // [ps][4]: d_x, d_y, d_z, 0 for an image of the centre (else 1)
    T* s_tab = geo + (size_t)ps * 4;
    load_ylm_tab<T>(M.ylm_tab, s_tab, M.n_ylm, M.maxl);
    const long long p0 = nb_off[i], p1 = nb_off[i + 1];
    const int np = (int)(p1 - p0);
    int* ord = order + p0;
    // stable order of the pairs by type pair
    int cursor = 0;
    for (int tp = 0; tp < M.n_tp; ++tp) {
        if (threadIdx.x == 0) s_tpoff[tp] = cursor;
        for (int r0 = 0; r0 < np; r0 += blockDim.x) {
            const int r = r0 + threadIdx.x;
            const bool f = r < np && M.type_pairs[t1 * M.n_type + B.types[nb_j[p0 + r]]] == tp;
            const unsigned m = __ballot_sync(0xffffffffu, f);
            if (lane == 0) s_wcnt[warp] = __popc(m);
            __syncthreads();
            int before = 0, total = 0;
            for (int w = 0; w < NW; ++w) {
                before += w < warp ? s_wcnt[w] : 0;
                total += s_wcnt[w];
            }
            if (f) ord[cursor + before + __popc(m & ((1u << lane) - 1u))] = r;
            cursor += total;
            __syncthreads();
        }
    }
    if (threadIdx.x == 0) s_tpoff[M.n_tp] = cursor;
    __syncthreads();
    const YlmTab<T> ytab = ylm_tab_view<T>(s_tab, M.n_ylm, M.maxl);
    const cplx<T>* Gi = G + g_off[i];
    const int npos = ty.n_pos;
    T* dsa = DS + s_off[i];  // [type pair of the centre type][9][n_pos], feature positions of that pair
    for (int q = threadIdx.x; q < 9 * npos * ty.n_tpl; q += blockDim.x) dsa[q] = (T)0;
    const int tpp = kRowsThreads / ps;  // threads per pair building the Y_lm table
    for (int tp = 0; tp < M.n_tp; ++tp) {
        const int r_end = s_tpoff[tp + 1];
        if (ty.tpl[tp] < 0 || r_end == s_tpoff[tp]) continue;  // no heads of tp: zero derivatives
        const int nfn = M.tp_nfn[tp];
        const int* pos_nid = ty.tp_pos_nid + (size_t)tp * npos;
        T* ds = dsa + (size_t)ty.tpl[tp] * 9 * npos;
        for (int sc0 = s_tpoff[tp]; sc0 < r_end; sc0 += ps) {
            const int nsc = min(ps, r_end - sc0);
            const int nsc8 = (nsc + NW - 1) / NW * NW;  // whole contraction steps; pairs past nsc are zero
            // ---- bases of the super-chunk, thread t of pair p (tpp threads a pair):
            // threads 0 .. ny-1 build Legendre columns (a, L - a), a = t, t + tpp,
            // .. (2a <= L); the others the radial functions and the pair's flags.
            // Per step of NW pairs, the running image sums are stored at a
            // group's last image or the step's end ("flush"), and stored rather
            // than added when the group's first image is in this step ("fresh";
            // runs of images are contiguous).
            {
                const int p = threadIdx.x / tpp, t = threadIdx.x - (threadIdx.x / tpp) * tpp;
                const int ny = M.gtinv ? min(tpp, L / 2 + 1) : 1;
                const int nfree = tpp - ny;
                T dx = 0, dy = 0, dz = 0, dis = 1;
                bool ok = false;
                long long q = p0;
                if (p < nsc) {
                    q = p0 + ord[sc0 + p];
                    ok = pair_geometry<T>(M, B, nb_d, q, dx, dy, dz, dis);
                }
                if (p < nsc && t == tpp - 1) {
                    const int j = nb_j[q];
                    geo[4 * p] = dx;
                    geo[4 * p + 1] = dy;
                    geo[4 * p + 2] = dz;
                    geo[4 * p + 3] = j == i ? (T)0 : (T)1;
                    const int step = p / NW * NW;
                    const bool last = q + 1 == p1 || nb_j[q + 1] != j;
                    const bool flush = last || p == min(step + NW, nsc) - 1;
                    bool fresh = false;
                    for (int v = p; v >= step; --v) {
                        const long long qv = p0 + ord[sc0 + v];
                        if (qv == p0 || nb_j[qv - 1] != nb_j[qv]) {
                            fresh = true;
                            break;
                        }
                    }
                    s_flag[p] = (ok ? 1 : 0) | (j == i ? 2 : 0) | (flush ? 4 : 0) | (fresh ? 8 : 0);
                    s_slot[p] = gslot[q];
                }
                if (p < nsc8) {
                    T* rows = tab + (size_t)p * 8;
                    if (!M.gtinv) {
                        if (t == 0)
                            for (int v = 0; v < 8; ++v) rows[v] = (v == 0 && ok) ? (T)1 : (T)0;
                    } else if (t < ny) {
                        const YlmDir<T> dir = ylm_dir<T>(dx, dy, dz, dis);
                        for (int a = t; 2 * a <= L; a += ny)
                            for (int side = 0; side < 2; ++side) {
                                const int mp = side ? L - a : a;
                                if (side && mp == a) break;
                                if (ok) {
                                    ylm_column<T>(mp, L, ytab, dir, rows, KS);
                                } else {
                                    for (int l = mp; l <= L; ++l)
                                        for (int v = 0; v < 8; ++v) rows[(size_t)KS * (l * (l + 1) / 2 + l - mp) + v] = (T)0;
                                }
                            }
                    }
                    // radial functions n of this thread: the free threads share them
                    // (all threads when none is free)
                    const int r0t = nfree > 0 ? t - ny : t, rstep = nfree > 0 ? nfree : tpp;
                    if (r0t >= 0) {
                        const T invr = (T)1 / dis;
                        for (int n = r0t; n < nfn; n += rstep) {
                            T* o = rad + ((size_t)p * NF + n) * 4;
                            if (ok) {
                                T f, fd;
                                radial_one<T>(M, tp, n, dis, f, fd);
                                o[0] = f;
                                o[1] = fd * (dx * invr);
                                o[2] = fd * (dy * invr);
                                o[3] = fd * (dz * invr);
                            } else {
                                o[0] = o[1] = o[2] = o[3] = (T)0;
                            }
                        }
                    }
                }
            }
            __syncthreads();
            // ---- contraction: warp = group of 32 bundles, lane = bundle (two
            // features with the same keys, positions xa and xa + 1); the group's
            // entries are read rank-major (coalesced) and one table row per pair
            // and rank serves both features
            const int ng = ty.n_groups;
            static_assert(NW == kLayWarps, "the group schedule is laid out for the block's warps");
            for (int k = 0; k < ty.n_rounds; ++k) {
                // groups past the last of tp have no entries and are not scheduled:
                // zero derivatives, nothing stored (stage B reads positions below tp_nnz only)
                const int grp = ty.lay_sched[((size_t)tp * ty.n_rounds + k) * NW + warp];
                if (grp < 0) continue;
                const int base = ty.lay_grp_base[tp * ng + grp], cnt = ty.lay_grp_cnt[tp * ng + grp];
                const int xa = 64 * grp + 2 * lane;
                const int nid0 = pos_nid[xa], nid1 = pos_nid[xa + 1];
                // the DS sums of both features, over the super-chunk
                T sv[9][2];
#pragma unroll
                for (int v = 0; v < 9; ++v) load_pair(ds + (size_t)v * npos + xa, sv[v]);
                for (int s0 = 0; s0 < nsc; s0 += NW) {
                    const T* tab0 = tab + (size_t)s0 * 8;
                    // per pair and feature: T, S_x, S_y, S_z
                    T acc[NW][2][4];
#pragma unroll
                    for (int w = 0; w < NW; ++w)
#pragma unroll
                        for (int f = 0; f < 2; ++f) acc[w][f][0] = acc[w][f][1] = acc[w][f][2] = acc[w][f][3] = (T)0;
                    // entries are loaded kPrefetch ranks ahead of the one contracted
                    constexpr int kPrefetch = 2;
                    cplx<T> ga[kPrefetch], gb[kPrefetch];
                    int kq[kPrefetch];
#pragma unroll
                    for (int s = 0; s < kPrefetch; ++s) {
                        ga[s] = gb[s] = {(T)0, (T)0};
                        kq[s] = 0;
                        if (s < cnt) {
                            ga[s] = Gi[base + 64 * s + lane];
                            gb[s] = Gi[base + 64 * s + 32 + lane];
                            kq[s] = ty.lay_key[base + 64 * s + lane];
                        }
                    }
                    for (int r0 = 0; r0 < cnt; r0 += kPrefetch) {
#pragma unroll
                        for (int s = 0; s < kPrefetch; ++s) {
                            const int r = r0 + s;
                            if (r >= cnt) break;
                            const T are = ga[s].re, aim = -ga[s].im, bre = gb[s].re, bim = -gb[s].im;
                            const T* row = tab0 + (size_t)KS * kq[s];
                            if (r + kPrefetch < cnt) {
                                const int sl = base + 64 * (r + kPrefetch) + lane;
                                ga[s] = Gi[sl];
                                gb[s] = Gi[sl + 32];
                                kq[s] = ty.lay_key[sl];
                            }
#pragma unroll
                            for (int w = 0; w < NW; ++w) {
                                T v[8];
                                load_row8(row + 8 * w, v);
#pragma unroll
                                for (int c = 0; c < 4; ++c) {
                                    acc[w][0][c] = fma(aim, v[2 * c + 1], fma(are, v[2 * c], acc[w][0][c]));
                                    acc[w][1][c] = fma(bim, v[2 * c + 1], fma(bre, v[2 * c], acc[w][1][c]));
                                }
                            }
                        }
                    }
                    // ---- per pair: derivatives of both features, image sums, DS sums
                    // (an out-of-range pair has a zero table: its terms vanish)
                    const int n = min(NW, nsc - s0);
                    T run[3][2] = {{0, 0}, {0, 0}, {0, 0}};
#pragma unroll
                    for (int w = 0; w < NW; ++w) {
                        if (w >= n) break;
                        const int pw = s0 + w;
                        const int fl = s_flag[pw];
                        T dg[4], r0v[4], r1v[4];
                        load_row4(geo + 4 * pw, dg);
                        load_row4(rad + ((size_t)pw * NF + nid0) * 4, r0v);
                        load_row4(rad + ((size_t)pw * NF + nid1) * 4, r1v);
                        T a[3][2];
#pragma unroll
                        for (int c = 0; c < 3; ++c) {
                            a[c][0] = fma(r0v[0], acc[w][0][1 + c], r0v[1 + c] * acc[w][0][0]);
                            a[c][1] = fma(r1v[0], acc[w][1][1 + c], r1v[1 + c] * acc[w][1][0]);
                        }
#pragma unroll
                        for (int f = 0; f < 2; ++f) {
                            sv[0][f] = fma(dg[3], a[0][f], sv[0][f]);
                            sv[1][f] = fma(dg[3], a[1][f], sv[1][f]);
                            sv[2][f] = fma(dg[3], a[2][f], sv[2][f]);
                            sv[3][f] = fma(dg[0], a[0][f], sv[3][f]);
                            sv[4][f] = fma(dg[1], a[1][f], sv[4][f]);
                            sv[5][f] = fma(dg[2], a[2][f], sv[5][f]);
                            sv[6][f] = fma(dg[1], a[0][f], sv[6][f]);
                            sv[7][f] = fma(dg[2], a[1][f], sv[7][f]);
                            sv[8][f] = fma(dg[0], a[2][f], sv[8][f]);
#pragma unroll
                            for (int c = 0; c < 3; ++c) run[c][f] += a[c][f];
                        }
                        if (fl & 4) {
                            T* o = Dp + (size_t)s_slot[pw] * 3 * NL + xa;
#pragma unroll
                            for (int c = 0; c < 3; ++c) {
                                if (fl & 8) {
                                    store_pair(o + (size_t)c * NL, run[c]);
                                } else {
                                    T old[2];
                                    load_pair(o + (size_t)c * NL, old);
                                    old[0] += run[c][0];
                                    old[1] += run[c][1];
                                    store_pair(o + (size_t)c * NL, old);
                                }
                                run[c][0] = run[c][1] = (T)0;
                            }
                        }
                    }
                }
#pragma unroll
                for (int v = 0; v < 9; ++v) store_pair(ds + (size_t)v * npos + xa, sv[v]);
            }
            __syncthreads();
        }
    }
}

// Stage B.  Force rows of one target atom j (block per target, X zeroed
// beforehand).  A centre type contributes to its own columns only: a linear
// column of feature k receives -sum_i dd_k(i)/dd_(i->j) over the centres i of
// that type with images on j (the runs of j's list; their group vectors sit
// at the runs' first slots, by feature position), and a product column
// d_a d_b (d_c) receives -sum_i (d_b dd_a + d_a dd_b ...) with centre i's
// features as weights.  The groups of one centre type are listed in shared
// memory first; the linear part is a coalesced column sum of their vectors
// over the positions with entries (each thread owns S positions per slab).
// When the three rows of j (F x 3 values) fit in shared memory (SROW), they
// are summed there and written to X once at the end (plain stores, no
// read-modify-write of X), and the product columns of two features are
// summed by role (QP: thread = (column, differentiated feature with data),
// weight x group-vector value, in the same pass over the groups; the two
// roles of a column are added in separate phases).  Otherwise each
// contribution is added to X in place and the product columns are gathered
// per column (thread per column) in the same pass when one slab covers the
// positions, else in a pass of their own.  The self rows add the centre's DS
// vectors to its own type's columns.  Every X element has one writer at a
// time (per type, per phase), and types and phases are taken in order, so
// the sums are deterministic.
__device__ __forceinline__ void unpack_col(int2 c, int& k0, int& k1, int& k2, int& w) {
    k0 = c.x & 0xffff;
    k1 = (c.x >> 16) & 0xffff;
    k2 = c.y & 0xffff;
    w = (c.y >> 16) & 0xffff;
}

// Recipe of product column p of a centre type for stage B: the column, its
// features k0, k1 (, k2) with their positions x in the group vectors of the
// type pair, and which positions lie below nnz (the others hold no data: their
// derivatives vanish).  False when the column has no such position.
struct ProdCol {
    int col, k0, k1, k2, w, x0, x1, x2;
    bool b0, b1, b2;
};
__device__ __forceinline__ bool prod_col(const DevType& ty, const int* ipos, int nnz, int p, ProdCol& pc) {
    pc.col = ty.prod_col[p];
    unpack_col(ty.col_pack[pc.col], pc.k0, pc.k1, pc.k2, pc.w);
    pc.x0 = ipos[pc.k0];
    pc.x1 = ipos[pc.k1];
    pc.x2 = pc.w > 2 ? ipos[pc.k2] : 0;
    pc.b0 = pc.x0 < nnz;
    pc.b1 = pc.x1 < nnz;
    pc.b2 = pc.w > 2 && pc.x2 < nnz;
    return pc.b0 || pc.b1 || pc.b2;
}
// v += the column's derivative from one group vector src (3 x NL), with the
// centre's features Di as weights.
template <typename T>
__device__ __forceinline__ void prod_col_add(const ProdCol& pc, const T* src, const T* Di, int NL, T (&v)[3]) {
    T w0, w1, w2 = 0;
    if (pc.w == 2) {
        w0 = Di[pc.k1];
        w1 = Di[pc.k0];
    } else {
        w0 = Di[pc.k1] * Di[pc.k2];
        w1 = Di[pc.k0] * Di[pc.k2];
        w2 = Di[pc.k0] * Di[pc.k1];
    }
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        const T s0 = pc.b0 ? src[c * NL + pc.x0] : (T)0, s1 = pc.b1 ? src[c * NL + pc.x1] : (T)0;
        v[c] += w0 * s0 + w1 * s1;
        if (pc.b2) v[c] += w2 * src[c * NL + pc.x2];
    }
}

// Four consecutive values from a 16-byte-aligned address (FP32: one float4;
// FP64: two double2).
__device__ __forceinline__ void load_vec4(const float* p, float (&v)[4]) {
    const float4 a = __ldg(reinterpret_cast<const float4*>(p));
    v[0] = a.x;
    v[1] = a.y;
    v[2] = a.z;
    v[3] = a.w;
}
__device__ __forceinline__ void load_vec4(const double* p, double (&v)[4]) {
    const double2 a = __ldg(reinterpret_cast<const double2*>(p)), b = __ldg(reinterpret_cast<const double2*>(p) + 1);
    v[0] = a.x;
    v[1] = a.y;
    v[2] = b.x;
    v[3] = b.y;
}

// Rows r0 .. r0 + 2 of column col of X (or of the block's copy s_x when SROW)
// minus v (plus v when add).
template <bool SROW, typename T>
__device__ __forceinline__ void sub_row3(T* s_x, T* X, long long ld, long long r0, int col, const T (&v)[3],
                                         bool add = false) {
    const T sg = add ? (T)1 : (T)-1;
    if (SROW) {
        T* o = s_x + 3 * col;
        o[0] += sg * v[0];
        o[1] += sg * v[1];
        o[2] += sg * v[2];
    } else {
        T* o = X + (size_t)col * ld + r0;
        o[0] += sg * v[0];
        o[1] += sg * v[1];
        o[2] += sg * v[2];
    }
}

template <typename T, bool SROW, bool QP>
__global__ void __launch_bounds__(kRowsThreads, sizeof(T) == 4 ? 5 : 1) pg_rows(DevModel M, DevBatch B, const long long* nb_off,
                                                        const int* nb_j, const long long* d_off, const T* D,
                                                        const T* Dp, const long long* s_off, const T* DS,
                                                        const long long* f_row, T* X, long long ld) {
    constexpr int S = 4;  // positions per thread per slab
    const int gj = blockIdx.x;
    const int s = B.atom_st[gj];
    if (f_row[s] < 0) return;
    const int sa0 = B.st_atom_off[s];
    const int tj = B.types[gj];
    const long long r0 = f_row[s] + 3LL * (gj - sa0);
    const long long q0 = nb_off[gj], qe = nb_off[gj + 1];
    const int NL = M.max_lin;
    // the groups of j's list (runs of one neighbour i != j) of one centre type,
    // listed kSeg pairs of the list at a time: a group's vector sits at its
    // first pair, so a group that crosses a segment is taken in the first one
    constexpr int kSeg = 1024;
    __shared__ int s_list[kSeg];
    __shared__ long long s_doff[kSeg];  // d_off of each group's centre (its features weight the product columns)
    __shared__ int s_wcnt[kRowsThreads / 32];
    // the three rows of j by column ([col][3]) when SROW
    extern __shared__ __align__(16) unsigned char s_x_raw[];
    T* s_x = reinterpret_cast<T*>(s_x_raw);
    if (SROW) {
        for (int q = threadIdx.x; q < 3 * M.F; q += blockDim.x) s_x[q] = (T)0;
        __syncthreads();
    }
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int tc = 0; tc < M.n_type; ++tc) {
        const DevType& ty = M.types[tc];
        const int nl = ty.n_lin;
        const int tp = M.type_pairs[tc * M.n_type + tj];
        const int* perm = ty.tp_perm + (size_t)tp * ty.n_pos;
        const int* ipos = ty.tp_ipos + (size_t)tp * nl;
        const int nnz = ty.tp_nnz[tp];  // the group vectors hold positions below nnz; the rest vanish
        if (nnz == 0) continue;
        for (long long sb = q0; sb < qe; sb += kSeg) {
            const long long se = min(sb + kSeg, qe);
            int n = 0;
            for (long long w0 = sb; w0 < se; w0 += blockDim.x) {
                const long long q = w0 + threadIdx.x;
                bool head = false;
                int gi = 0;
                if (q < se) {
                    gi = nb_j[q];
                    head = gi != gj && (q == q0 || nb_j[q - 1] != gi) && B.types[gi] == tc;
                }
                const unsigned m = __ballot_sync(0xffffffffu, head);
                if (lane == 0) s_wcnt[warp] = __popc(m);
                __syncthreads();
                int before = 0, total = 0;
                for (int w = 0; w < kRowsThreads / 32; ++w) {
                    before += w < warp ? s_wcnt[w] : 0;
                    total += s_wcnt[w];
                }
                if (head) {
                    const int k = n + before + __popc(m & ((1u << lane) - 1u));
                    s_list[k] = (int)(q - sb);
                    s_doff[k] = d_off[gi];
                }
                n += total;
                __syncthreads();
            }
            // linear columns: sum of the group vectors.  Product columns of two
            // features: thread = role (column, differentiated feature with data
            // in tp), summed in the same pass over the groups (first slab) and
            // added to the column in two phases.  Otherwise, when one slab covers
            // the positions and a thread per product column suffices, the
            // product columns are gathered in the same pass, while the group
            // vector is in L1; else in a pass of their own.
            // (QP: all centre types have such roles and the rows are in shared
            // memory, chosen at launch: in X itself, the roles' and positions'
            // separate adds would each be a read-modify-write of X)
            constexpr bool qp = QP;
            const int qn = qp ? ty.prod_qn[tp] : 0;
            const bool has_q = (int)threadIdx.x < qn;
            // the role's position and weight feature; its column and phase are read after the pass
            int2 qr = make_int2(0, 0);
            if (has_q) qr = *reinterpret_cast<const int2*>(ty.prod_q + (size_t)tp * kRowsThreads + threadIdx.x);
            T qv[3] = {0, 0, 0};
            const bool fuse = qp || (nnz <= S * (int)blockDim.x && ty.n_prod <= (int)blockDim.x);
            ProdCol pc;
            const bool has_pc = !qp && fuse && (int)threadIdx.x < ty.n_prod && prod_col(ty, ipos, nnz, threadIdx.x, pc);
            T pv[3] = {0, 0, 0};
            // thread = S consecutive positions of a slab, read as one vector per
            // Cartesian component (the group vectors' stride NL is a multiple of 4)
            for (int slab = 0; slab < nnz; slab += S * blockDim.x) {
                const int xb = slab + S * (int)threadIdx.x;
                T acc[S][3];
#pragma unroll
                for (int m = 0; m < S; ++m) acc[m][0] = acc[m][1] = acc[m][2] = (T)0;
#pragma unroll 4
                for (int k = 0; k < n; ++k) {
                    const long long q = sb + s_list[k];
                    const T* src = Dp + (size_t)q * 3 * NL;
                    if (xb < nnz) {
#pragma unroll
                        for (int c = 0; c < 3; ++c) {
                            T v[S];
                            load_vec4(src + (size_t)c * NL + xb, v);
#pragma unroll
                            for (int m = 0; m < S; ++m) acc[m][c] += v[m];
                        }
                    }
                    if (has_pc) prod_col_add(pc, src, D + s_doff[k], NL, pv);
                    if (has_q && slab == 0) {
                        const T wq = D[s_doff[k] + qr.y];
#pragma unroll
                        for (int c = 0; c < 3; ++c) qv[c] += wq * src[(size_t)c * NL + qr.x];
                    }
                }
#pragma unroll
                for (int m = 0; m < S; ++m) {
                    const int x = xb + m;
                    if (x >= nnz || perm[x] < 0) continue;  // past the positions with data, or a hole
                    const int col = ty.lin_col[perm[x]];
                    if (col < 0) continue;
                    sub_row3<SROW>(s_x, X, ld, r0, col, acc[m]);
                }
            }
            if (has_pc) sub_row3<SROW>(s_x, X, ld, r0, pc.col, pv);
            if (qp) {
                // roles of phase 0, then of phase 1 (the second feature of a
                // column): one writer per column at a time; a square column's
                // one role counts twice
                int2 cw = make_int2(0, 0);
                if (has_q) cw = reinterpret_cast<const int2*>(ty.prod_q + (size_t)tp * kRowsThreads + threadIdx.x)[1];
                if (has_q && (cw.y & 1) == 0) {
                    const T m = (cw.y & 2) ? (T)2 : (T)1;
                    const T v[3] = {m * qv[0], m * qv[1], m * qv[2]};
                    sub_row3<SROW>(s_x, X, ld, r0, cw.x, v);
                }
                __syncthreads();
                if (has_q && (cw.y & 1) == 1) sub_row3<SROW>(s_x, X, ld, r0, cw.x, qv);
            }
            // product columns, own pass
            for (int p = threadIdx.x; !fuse && p < ty.n_prod; p += blockDim.x) {
                if (!prod_col(ty, ipos, nnz, p, pc)) continue;
                T v[3] = {0, 0, 0};
                for (int k = 0; k < n; ++k) {
                    const long long q = sb + s_list[k];
                    prod_col_add(pc, Dp + (size_t)q * 3 * NL, D + s_doff[k], NL, v);
                }
                sub_row3<SROW>(s_x, X, ld, r0, pc.col, v);
            }
            // before the list is rebuilt; a column shared by several types is
            // also updated type by type
            __syncthreads();
        }
    }
    // self rows: the target as a centre (type tj), its DS self vectors (per type
    // pair, by position).  With product roles (QP): per type pair, thread =
    // position for the linear columns (contiguous DS reads), then thread = role
    // for the product columns (phases apart); else thread = feature / column.
    const DevType& ty = M.types[tj];
    const int nl = ty.n_lin, npos = ty.n_pos;
    const T* Di = D + d_off[gj];
    const T* dsa = DS + s_off[gj];
    if (QP) {
        for (int l = 0; l < ty.n_tpl; ++l) {
            const int tpl = ty.tpl_tp[l];
            const int* pm = ty.tp_perm + (size_t)tpl * npos;
            const T* ds = dsa + (size_t)l * 9 * npos;
            for (int x = threadIdx.x; x < ty.tp_nnz[tpl]; x += blockDim.x) {
                const int k = pm[x];
                if (k < 0) continue;
                const int col = ty.lin_col[k];
                if (col < 0) continue;
                const T v[3] = {ds[x], ds[npos + x], ds[2 * npos + x]};
                sub_row3<SROW>(s_x, X, ld, r0, col, v, true);
            }
            const bool has_q = (int)threadIdx.x < ty.prod_qn[tpl];
            int4 qr = make_int4(0, 0, 0, 0);
            T v[3] = {0, 0, 0};
            if (has_q) {
                qr = ty.prod_q[(size_t)tpl * kRowsThreads + threadIdx.x];
                const T wq = ((qr.w & 2) ? (T)2 : (T)1) * Di[qr.y];
#pragma unroll
                for (int c = 0; c < 3; ++c) v[c] = wq * ds[(size_t)c * npos + qr.x];
            }
            if (has_q && (qr.w & 1) == 0) sub_row3<SROW>(s_x, X, ld, r0, qr.z, v, true);
            __syncthreads();
            if (has_q && (qr.w & 1) == 1) sub_row3<SROW>(s_x, X, ld, r0, qr.z, v, true);
            __syncthreads();
        }
    }
    for (int k = threadIdx.x; !QP && k < nl; k += blockDim.x) {
        const int col = ty.lin_col[k];
        if (col < 0) continue;
        T v0 = 0, v1 = 0, v2 = 0;
        for (int l = 0; l < ty.n_tpl; ++l) {
            const T* ds = dsa + (size_t)l * 9 * npos;
            const int x = ty.tp_ipos[(size_t)ty.tpl_tp[l] * nl + k];
            v0 += ds[x];
            v1 += ds[npos + x];
            v2 += ds[2 * npos + x];
        }
        const T v[3] = {v0, v1, v2};
        sub_row3<SROW>(s_x, X, ld, r0, col, v, true);
    }
    __syncthreads();
    for (int p = threadIdx.x; !QP && p < ty.n_prod; p += blockDim.x) {
        const int col = ty.prod_col[p];
        int k0, k1, k2, w;
        unpack_col(ty.col_pack[col], k0, k1, k2, w);
        T w0, w1, w2 = 0;
        if (w == 2) {
            w0 = Di[k1];
            w1 = Di[k0];
        } else {
            w0 = Di[k1] * Di[k2];
            w1 = Di[k0] * Di[k2];
            w2 = Di[k0] * Di[k1];
        }
        T v[3] = {0, 0, 0};
        for (int l = 0; l < ty.n_tpl; ++l) {
            const T* ds = dsa + (size_t)l * 9 * npos;
            const int* ip = ty.tp_ipos + (size_t)ty.tpl_tp[l] * nl;
            const int x0 = ip[k0], x1 = ip[k1], x2 = w > 2 ? ip[k2] : 0;
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                v[c] += w0 * ds[(size_t)c * npos + x0] + w1 * ds[(size_t)c * npos + x1];
                if (w > 2) v[c] += w2 * ds[(size_t)c * npos + x2];
            }
        }
        sub_row3<SROW>(s_x, X, ld, r0, col, v, true);
    }
    if (SROW) {
        __syncthreads();
        // three consecutive threads a column: a warp's stores cover about ten
        // columns' 12-byte runs
        for (int q = threadIdx.x; q < 3 * M.F; q += blockDim.x) {
            const int col = q / 3;
            X[(size_t)col * ld + r0 + (q - 3 * col)] = s_x[q];
        }
    }
}

// Energy and stress rows, block per structure:
//   X[e_row, col] = sum_i poly_col(d(i)),
//   X[s_row + q, col] = -sum_i sum_{k in col} w_k,col(i) DS[i][3+q][k].
// A linear column (one feature k, w = 1) is a plain sum over the structure's
// atoms of its centre type: energies with thread = features k, t + 256 r
// (r < kEsFeat) held in registers while the atoms go by (each atom's feature
// row read contiguously); stresses per type pair of the centre type with
// thread = feature positions x, t + 256 r (the DS rows are stored by position
// and read contiguously; partial sums over four atoms in T), each position's
// sum added to its feature's column.
// Product columns: thread = column, weights from the atom's features.  Every
// sum runs over the atoms in order in a long accumulator (FP64, or float-float
// in the FP32 kernel) and is added to X (zeroed per batch) type pair by type
// pair and type by type, since a column can belong to the features of several
// centre types (those of a type pair): deterministic.
constexpr int kEsThreads = 256, kEsFeat = 4;
template <typename T>
__global__ void __launch_bounds__(kEsThreads) pg_rows_es(DevModel M, DevBatch B, const long long* d_off, const T* D,
                                                         const long long* s_off, const T* DS, const long long* e_row,
                                                         const long long* f_row, const long long* s_row, T* X,
                                                         long long ld) {
    const int s = blockIdx.x;
    const bool force = f_row[s] >= 0 && s_row[s] >= 0;
    const int a0 = B.st_atom_off[s], a1 = B.st_atom_off[s + 1];
    T* xe = X + e_row[s];
    T* xs = force ? X + s_row[s] : nullptr;
    for (int tc = 0; tc < M.n_type; ++tc) {
        const DevType& ty = M.types[tc];
        const int nl = ty.n_lin, ntpl = ty.n_tpl, npos = ty.n_pos;
        // ---- linear columns: energies
        for (int kb = 0; kb < nl; kb += kEsThreads * kEsFeat) {
            LongSum<T> acc[kEsFeat];
            int kk[kEsFeat];
#pragma unroll
            for (int r = 0; r < kEsFeat; ++r) kk[r] = kb + threadIdx.x + r * kEsThreads;
            for (int i = a0; i < a1; ++i) {
                if (B.types[i] != tc) continue;
                const T* Di = D + d_off[i];
#pragma unroll
                for (int r = 0; r < kEsFeat; ++r)
                    if (kk[r] < nl) acc[r].add(Di[kk[r]]);
            }
#pragma unroll
            for (int r = 0; r < kEsFeat; ++r) {
                if (kk[r] >= nl) continue;
                const int col = ty.lin_col[kk[r]];
                if (col >= 0) xe[(size_t)col * ld] += (T)acc[r].value();
            }
        }
        // ---- linear columns: stresses, type pair by type pair (positions past
        // tp_nnz hold no derivatives)
        for (int l = 0; force && l < ntpl; ++l) {
            __syncthreads();  // the previous type pair's additions to a column are done
            const int tp = ty.tpl_tp[l];
            const int nnz = ty.tp_nnz[tp];
            const int* perm = ty.tp_perm + (size_t)tp * npos;
            for (int xb = 0; xb < nnz; xb += kEsThreads * kEsFeat) {
                // partial sums over kEsRun atoms in T, each added to the long sum
                constexpr int kEsRun = 4;
                LongSum<T> acc[kEsFeat][6];
                T part[kEsFeat][6];
#pragma unroll
                for (int r = 0; r < kEsFeat; ++r)
#pragma unroll
                    for (int q = 0; q < 6; ++q) part[r][q] = (T)0;
                int run = 0;
                for (int i = a0; i < a1; ++i) {
                    if (B.types[i] != tc) continue;
                    const T* ds = DS + s_off[i] + ((size_t)l * 9 + 3) * npos;
#pragma unroll
                    for (int r = 0; r < kEsFeat; ++r) {
                        const int x = xb + threadIdx.x + r * kEsThreads;
                        if (x < nnz)
#pragma unroll
                            for (int q = 0; q < 6; ++q) part[r][q] -= ds[(size_t)q * npos + x];
                    }
                    if (++run == kEsRun) {
                        run = 0;
#pragma unroll
                        for (int r = 0; r < kEsFeat; ++r)
#pragma unroll
                            for (int q = 0; q < 6; ++q) {
                                acc[r][q].add(part[r][q]);
                                part[r][q] = (T)0;
                            }
                    }
                }
#pragma unroll
                for (int r = 0; r < kEsFeat; ++r)
#pragma unroll
                    for (int q = 0; q < 6; ++q) acc[r][q].add(part[r][q]);
#pragma unroll
                for (int r = 0; r < kEsFeat; ++r) {
                    const int x = xb + threadIdx.x + r * kEsThreads;
                    if (x >= nnz || perm[x] < 0) continue;
                    const int col = ty.lin_col[perm[x]];
                    if (col < 0) continue;
#pragma unroll
                    for (int q = 0; q < 6; ++q) xs[(size_t)col * ld + q] += (T)acc[r][q].value();
                }
            }
        }
        // ---- product columns
        for (int p = threadIdx.x; p < ty.n_prod; p += kEsThreads) {
            const int col = ty.prod_col[p];
            int k0, k1, k2, w;
            unpack_col(ty.col_pack[col], k0, k1, k2, w);
            LongSum<T> acc[7];
            for (int i = a0; i < a1; ++i) {
                if (B.types[i] != tc) continue;
                const T* Di = D + d_off[i];
                T w0, w1, w2 = 0, e;
                if (w == 2) {
                    w0 = Di[k1];
                    w1 = Di[k0];
                    e = Di[k0] * Di[k1];
                } else {
                    w0 = Di[k1] * Di[k2];
                    w1 = Di[k0] * Di[k2];
                    w2 = Di[k0] * Di[k1];
                    e = Di[k0] * Di[k1] * Di[k2];
                }
                acc[0].add(e);
                if (!force) continue;
                const T* dsi = DS + s_off[i] + 3 * (size_t)npos;
                for (int l = 0; l < ntpl; ++l) {
                    const T* ds = dsi + (size_t)l * 9 * npos;
                    const int* ip = ty.tp_ipos + (size_t)ty.tpl_tp[l] * nl;
                    const int x0 = ip[k0], x1 = ip[k1], x2 = w > 2 ? ip[k2] : 0;
#pragma unroll
                    for (int q = 0; q < 6; ++q) {
                        T v = w0 * ds[(size_t)q * npos + x0] + w1 * ds[(size_t)q * npos + x1];
                        if (w > 2) v += w2 * ds[(size_t)q * npos + x2];
                        acc[1 + q].add(-v);
                    }
                }
            }
            xe[(size_t)col * ld] += (T)acc[0].value();
            if (force)
#pragma unroll
                for (int q = 0; q < 6; ++q) xs[(size_t)col * ld + q] += (T)acc[1 + q].value();
        }
        // a column shared by several centre types receives their sums type by type
        __syncthreads();
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

void launch_nb_count(const DevBatch& B, int* counts, int* max_cl, cudaStream_t st) {
    const int threads = 256, warps = threads / 32;
    pg_nb_count<<<(B.n_atoms + warps - 1) / warps, threads, 0, st>>>(B, counts, max_cl);
}

void launch_nb_fill(const DevBatch& B, const long long* off, int* nb_j, double* nb_d, float4* nb_df, long long* keys,
                    bool any_cl, cudaStream_t st) {
    const int threads = 256, warps = threads / 32;
    pg_nb_fill<<<(B.n_atoms + warps - 1) / warps, threads, 0, st>>>(B, off, keys);
    if (any_cl) pg_nb_order<<<B.n_atoms, 256, 0, st>>>(B, off, keys, nb_j, nb_d, nb_df);
    pg_nb_disp<<<(B.n_atoms + warps - 1) / warps, threads, 0, st>>>(B, off, keys, nb_j, nb_d, nb_df);
}

void launch_nb_refresh(const DevBatch& B, const long long* off, const long long* keys, int* nb_j, double* nb_d,
                       float4* nb_df, cudaStream_t st) {
    const int threads = 256, warps = threads / 32;
    if (B.n_atoms > 0)
        pg_nb_refresh<<<(B.n_atoms + warps - 1) / warps, threads, 0, st>>>(B, off, keys, nb_j, nb_d, nb_df);
}

template <typename T>
void launch_anlm(const DevModel& M, const DevBatch& B, const long long* nb_off, const int* nb_j, const double* nb_d,
                 const long long* a_off, void* A, int max_k0, cudaStream_t st) {
    const int threads = 256;
    const size_t smem = (size_t)max_k0 * 2 * sizeof(LongSum<T>) + (size_t)kAnlmChunk * M.n_ylm * sizeof(cplx<T>) +
                        (size_t)kAnlmChunk * M.n_fn_max * sizeof(T) + ylm_table_size(M.n_ylm, M.maxl) * sizeof(T);
    PG_CUDA(cudaFuncSetAttribute(pg_anlm<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    pg_anlm<T><<<B.n_atoms, threads, smem, st>>>(M, B, nb_off, nb_j, nb_d, a_off, reinterpret_cast<cplx<T>*>(A));
}

template <typename T>
void launch_features_adjoint(const DevModel& M, const DevBatch& B, const long long* a_off, const void* A,
                             const long long* d_off, T* D, const long long* g_off, void* G, int max_k,
                             cudaStream_t st) {
    const size_t smem = ((size_t)max_k + 8 * adj_win<T>()) * sizeof(cplx<T>);
    PG_CUDA(cudaFuncSetAttribute(pg_features_adjoint<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    pg_features_adjoint<T><<<B.n_atoms, 256, smem, st>>>(M, B, a_off, reinterpret_cast<const cplx<T>*>(A), d_off, D, g_off,
                                                         reinterpret_cast<cplx<T>*>(G));
}

// Pairs per stage-A super-chunk: 32, or fewer (16, 8) where the tables of 32
// pairs would not leave room for two blocks per SM (FP32) or one (FP64).
int rows_pairs_chunk(const DevModel& M, bool fp64) {
    const size_t budget = fp64 ? 200 * 1024 : 110 * 1024;
    int ps = kMaxSuperChunk;
    while (ps > 8 && rows_pairs_smem_bytes(M, fp64, ps) > budget) ps /= 2;
    return ps;
}

size_t rows_pairs_smem_bytes(const DevModel& M, bool fp64, int ps) {
    const size_t ts = fp64 ? 8 : 4;
    return (size_t)M.n_ylm * (ps * 8 + 4) * ts + (size_t)ps * M.n_fn_max * 4 * ts + (size_t)ps * 4 * ts +
           (size_t)ylm_table_size(M.n_ylm, M.maxl) * ts;
}

void launch_nb_mirror(int n_atoms, const long long* nb_off, const int* nb_j, const double* nb_d, long long* mirror,
                      long long* gslot, int* missing, cudaStream_t st) {
    const int threads = 256;
    pg_nb_mirror<<<(int)(((long long)n_atoms * 32 + threads - 1) / threads), threads, 0, st>>>(
        n_atoms, nb_off, nb_j, nb_d, mirror, gslot, missing);
}

template <typename T>
void launch_rows_pairs(const DevModel& M, const DevBatch& B, const long long* nb_off, const int* nb_j,
                       const double* nb_d, const long long* gslot, const long long* s_off, const long long* g_off,
                       const void* G, const long long* f_row, int* order, T* Dp, T* DS, cudaStream_t st) {
    const int ps = rows_pairs_chunk(M, sizeof(T) == 8);
    const size_t smem = rows_pairs_smem_bytes(M, sizeof(T) == 8, ps);
    PG_CUDA(cudaFuncSetAttribute(pg_rows_pairs<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    pg_rows_pairs<T><<<B.n_atoms, kRowsThreads, smem, st>>>(M, B, nb_off, nb_j, nb_d, gslot, s_off, g_off,
                                                           reinterpret_cast<const cplx<T>*>(G), f_row, order, Dp, DS,
                                                           ps);
}

template <typename T>
void launch_rows(const DevModel& M, const DevBatch& B, const long long* nb_off, const int* nb_j,
                 const long long* d_off, const T* D, const T* Dp, const long long* s_off, const T* DS,
                 const long long* f_row, T* X, long long ld, cudaStream_t st) {
    // the three rows of a target in shared memory when they fit beside the lists
    // at the kernel's occupancy (FP32: five blocks an SM; FP64: one)
    const size_t rows3 = 3 * sizeof(T) * (size_t)M.F;
    const bool srow = rows3 <= (sizeof(T) == 4 ? 31 * 1024 + 512 : 200 * 1024);
    bool qp = srow;
    for (int t = 0; t < M.n_type; ++t) qp = qp && M.types[t].prod_qok;
    auto go = [&](auto kernel, size_t smem) {
        PG_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        kernel<<<B.n_atoms, kRowsThreads, smem, st>>>(M, B, nb_off, nb_j, d_off, D, Dp, s_off, DS, f_row, X, ld);
    };
    if (srow)
        qp ? go(pg_rows<T, true, true>, rows3) : go(pg_rows<T, true, false>, rows3);
    else
        qp ? go(pg_rows<T, false, true>, 0) : go(pg_rows<T, false, false>, 0);
}

template <typename T>
void launch_rows_es(const DevModel& M, const DevBatch& B, const long long* d_off, const T* D, const long long* s_off,
                    const T* DS, const long long* e_row, const long long* f_row, const long long* s_row, T* X,
                    long long ld, cudaStream_t st) {
    if (B.n_st > 0)
        pg_rows_es<T><<<B.n_st, kEsThreads, 0, st>>>(M, B, d_off, D, s_off, DS, e_row, f_row, s_row, X, ld);
}

template void launch_anlm<double>(const DevModel&, const DevBatch&, const long long*, const int*, const double*,
                                  const long long*, void*, int, cudaStream_t);
template void launch_anlm<float>(const DevModel&, const DevBatch&, const long long*, const int*, const double*,
                                 const long long*, void*, int, cudaStream_t);
template void launch_features_adjoint<double>(const DevModel&, const DevBatch&, const long long*, const void*,
                                              const long long*, double*, const long long*, void*, int,
                                              cudaStream_t);
template void launch_features_adjoint<float>(const DevModel&, const DevBatch&, const long long*, const void*,
                                             const long long*, float*, const long long*, void*, int, cudaStream_t);
template void launch_rows_pairs<double>(const DevModel&, const DevBatch&, const long long*, const int*,
                                        const double*, const long long*, const long long*, const long long*,
                                        const void*, const long long*, int*, double*, double*, cudaStream_t);
template void launch_rows_pairs<float>(const DevModel&, const DevBatch&, const long long*, const int*,
                                       const double*, const long long*, const long long*, const long long*,
                                       const void*, const long long*, int*, float*, float*, cudaStream_t);
template void launch_rows<double>(const DevModel&, const DevBatch&, const long long*, const int*, const long long*,
                                  const double*, const double*, const long long*, const double*, const long long*,
                                  double*, long long, cudaStream_t);
template void launch_rows<float>(const DevModel&, const DevBatch&, const long long*, const int*, const long long*,
                                 const float*, const float*, const long long*, const float*, const long long*,
                                 float*, long long, cudaStream_t);
template void launch_rows_es<double>(const DevModel&, const DevBatch&, const long long*, const double*,
                                     const long long*, const double*, const long long*, const long long*,
                                     const long long*, double*, long long, cudaStream_t);
template void launch_rows_es<float>(const DevModel&, const DevBatch&, const long long*, const float*,
                                    const long long*, const float*, const long long*, const long long*,
                                    const long long*, float*, long long, cudaStream_t);

}  // namespace pg
