// Device-side views of the model tables and of a batch of structures, and the
// warp-cooperative pair basis (radial functions, Y_lm for m <= 0 and their
// gradients) shared by the training and evaluation kernels.
#pragma once

#include <cstdint>

#include "host/flat_tables.h"

namespace pg {

constexpr int kMaxTypes = 8;
constexpr double kPiD = 3.1415926535897932384626433832795;

template <typename T>
struct cplx {
    T re, im;
};
template <typename T>
__device__ __forceinline__ cplx<T> cmul(cplx<T> a, cplx<T> b) {
    return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re};
}
template <typename T>
__device__ __forceinline__ T creal_mul(cplx<T> a, cplx<T> b) {
    return a.re * b.re - a.im * b.im;
}

// Product of the a entries of one term, left to right.
template <typename T>
__device__ inline cplx<T> term_product(const FlatTerm& t, const cplx<T>* a) {
    if (t.n == 0) return {(T)1, (T)0};
    cplx<T> v = a[t.ids[0]];
    for (int q = 1; q < t.n; ++q) v = cmul(v, a[t.ids[q]]);
    return v;
}

// Re(prod a[ids]) in the reference's association (polymlp_products.cpp:21-37).
template <typename T>
__device__ inline T term_product_real(const FlatTerm& t, const cplx<T>* a) {
    const int n = t.n;
    if (n == 0) return (T)1;
    if (n == 1) return a[t.ids[0]].re;
    if (n == 2) return creal_mul(a[t.ids[0]], a[t.ids[1]]);
    if (n == 3) return creal_mul(cmul(a[t.ids[0]], a[t.ids[1]]), a[t.ids[2]]);
    if (n == 4) return creal_mul(cmul(cmul(a[t.ids[1]], a[t.ids[2]]), a[t.ids[3]]), a[t.ids[0]]);
    cplx<T> v = a[t.ids[1]];
    for (int q = 2; q < n; ++q) v = cmul(v, a[t.ids[q]]);
    return creal_mul(v, a[t.ids[0]]);
}

// Windowed warp sums.  A warp owns 32 outputs whose terms are contiguous in
// a term list (output l's terms are [off_l, off_l+1)): the terms are evaluated
// 32 at a time by all lanes, whatever output they belong to, into a window
// s_v of kTermWin values; then each lane adds its own output's terms from the
// window, in list order.  This balances outputs with unequal term counts.
constexpr int kTermWin = 128;

struct DevType {
    int K, K0, n_lin;
    const int *head_nid, *head_key, *head_m;
    const int *full_src, *full_is_conj;
    const double* full_cc;
    const float* full_cc_f;    // FP32 copy of full_cc
    const int* val_off;
    const FlatTerm* val_terms;
    const int *col_ncomp, *comp_k;
    const int2* col_pack;      // per column: k0 | k1 << 16, k2 | count << 16 (its up to three linear features)
    int n_prod;                // columns that are products of two or three features of this type
    const int *lin_col, *prod_col;  // per feature: its linear column (-1: none); the product columns
    // Force rows of the product columns when all are products of two features
    // (prod_q): per type pair tp of this centre type, prod_qn[tp] (<= the row
    // kernel's block size) roles, one per (column, differentiated feature k with
    // data in tp): prod_q[tp][t] = {position of k, the other feature (weight),
    // column, phase | 2 * (square column)}.  A role sums weight x group-vector
    // value over the centres; phase 0 and 1 roles of a column are added apart.
    int prod_qok;
    const int* prod_qn;
    const int4* prod_q;
    const int *tp_head_off, *tp_heads;  // heads of each type pair (CSR over type pairs)
    // X-row layout of the adjoint entries by type pair (host/flat_tables.h)
    int n_groups, lay_size, n_tpl, n_pos;  // n_pos: feature positions per type pair (host/flat_tables.h)
    int n_rounds;                          // rounds of the stage-A group schedule lay_sched
    const int* lay_sched;
    const int *lay_key, *lay_grp_base, *lay_grp_cnt, *tp_perm, *tp_ipos, *tpl, *tpl_tp;
    const int* tp_pos_nid;  // per type pair and position: the radial function of the feature's entries
    const int* tp_nnz;      // per type pair: feature positions with entries (the first ones)
    // adjoint terms in X-row slot order: slot s owns terms slot_toff[s] ..
    // slot_toff[s + 1]; per term the full a ids (16 bits each, two per word in
    // x, y, z), n | conj << 8 in w, and its coefficient (T of the model; the
    // sign of the entry's conjugate head folded into conjugate terms)
    const int* slot_toff;
    const int4* tcode;
    const void* tcoef;
    // feature-value terms packed like tcode (val_off order), coefficients in T
    const int4* vcode;
    const void* vcoef;
};

// Product of the a ids of a packed term (ids 16 bits each, two per word in x,
// y, z; n in the low byte of w), in the order of term_product.
// Products of two and three factors (nearly all terms of the gtinv models up
// to order 4) take their own short paths.
template <typename T>
__device__ __forceinline__ cplx<T> packed_term_product(const int4 c4, const cplx<T>* a) {
    const int n = c4.w & 0xff;
    if (n == 2) return cmul(a[c4.x & 0xffff], a[(c4.x >> 16) & 0xffff]);
    if (n == 3) return cmul(cmul(a[c4.x & 0xffff], a[(c4.x >> 16) & 0xffff]), a[c4.y & 0xffff]);
    const int id[6] = {c4.x & 0xffff, (c4.x >> 16) & 0xffff, c4.y & 0xffff,
                       (c4.y >> 16) & 0xffff, c4.z & 0xffff, (c4.z >> 16) & 0xffff};
    cplx<T> p = {(T)1, (T)0};
    if (n > 0) p = a[id[0]];
#pragma unroll
    for (int q = 1; q < 6; ++q)
        if (q < n) p = cmul(p, a[id[q]]);
    return p;
}

// Feature values d_k = sum_q coeff_q Re(prod a[ids_q]) of one centre, one
// warp per 32 consecutive features (windowed warp sums over the packed value
// terms vcode/vcoef; a window's codes are requested together).
template <typename T>
__device__ __forceinline__ void warp_feature_values(const DevType& ty, const cplx<T>* a, T* out, cplx<T>* s_v,
                                                    int warp, int n_warps, int lane) {
    constexpr int kU = kTermWin / 32;
    const T* vcoef = reinterpret_cast<const T*>(ty.vcoef);
    for (int k0 = 32 * warp; k0 < ty.n_lin; k0 += 32 * n_warps) {
        const int k = k0 + lane;
        const int tb = ty.val_off[k0], te = ty.val_off[min(k0 + 32, ty.n_lin)];
        const int ms = k < ty.n_lin ? ty.val_off[k] : te, me = k < ty.n_lin ? ty.val_off[k + 1] : te;
        T v = 0;
        for (int w0 = tb; w0 < te; w0 += kTermWin) {
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
                if (w0 + 32 * u + lane < te) s_v[32 * u + lane].re = cf[u] * packed_term_product<T>(c4[u], a).re;
            __syncwarp();
            const int lo = max(ms, w0), hi = min(me, w0 + kTermWin);
            for (int t = lo; t < hi; ++t) v += s_v[t - w0].re;
            __syncwarp();
        }
        if (k < ty.n_lin) out[k] = v;
    }
}

template <typename T>
__device__ __forceinline__ T full_cc_of(const DevType& ty, int f);
template <>
__device__ __forceinline__ double full_cc_of<double>(const DevType& ty, int f) { return ty.full_cc[f]; }
template <>
__device__ __forceinline__ float full_cc_of<float>(const DevType& ty, int f) { return ty.full_cc_f[f]; }

// All K a_nlm of a centre (smem a) from its K0 no-conjugate ones (A, in T):
// a conjugate entry is cc * conj(its source).
template <typename T>
__device__ __forceinline__ void load_full_a(const DevType& ty, const cplx<T>* A, cplx<T>* a) {
    for (int f = threadIdx.x; f < ty.K; f += blockDim.x) {
        const cplx<T> s = A[ty.full_src[f]];
        if (ty.full_is_conj[f]) {
            const T cc = full_cc_of<T>(ty, f);
            a[f] = {cc * s.re, -cc * s.im};
        } else {
            a[f] = s;
        }
    }
}

struct DevModel {
    int n_type, n_tp, F, n_fn_max, maxl, n_ylm, gtinv;
    int max_k0, max_lin;  // largest K0 and feature-position count n_pos (a multiple of 4) over the centre types
    int max_k0tp;         // largest number of heads of one type pair
    double cutoff;
    const int* type_pairs;
    const int* tp_nfn;
    const double *tp_beta, *tp_mu;
    // FP32 copies for the FP32 kernels; rc2_safe_f: a squared distance
    // whose FP32 value lies below it is surely inside the cutoff in FP64
    float cutoff_f, rc2_safe_f;
    const float *tp_beta_f, *tp_mu_f;
    // Legendre/Y_lm constants (ylm_table_size doubles), see ylm_tables()
    const double* ylm_tab;
    DevType types[kMaxTypes];
};

// Constants of the normalised associated Legendre recursion and of the Y_lm
// gradients, which depend on (l, m) only:
//   A[lm], B[lm]  recursion coefficients for m <= l - 2,
//   D1[lm]        sqrt((l - m)(l + m + 1)) for m < l,
//   C1[l] = -sqrt(1 + 0.5 / l), C2[m] = sqrt(2m + 3), D0[l] = sqrt(l (l + 1) / 2),
//   DEC[idx]      (l, m') of the m <= 0 index idx = l(l+1)/2 + l - m'.
// Layout: A | B | D1 | DEC (n_ylm each) | C1 | C2 | D0 (maxl + 1 each).
__host__ __device__ inline int ylm_table_size(int n_ylm, int maxl) { return 4 * n_ylm + 3 * (maxl + 1); }

template <typename T>
struct YlmTab {
    const T *A, *B, *D1, *C1, *C2, *D0;
    const int* DEC;
};

template <typename T>
__device__ inline YlmTab<T> ylm_tab_view(const T* base, int n_ylm, int maxl) {
    YlmTab<T> t;
    t.A = base;
    t.B = base + n_ylm;
    t.D1 = base + 2 * n_ylm;
    t.DEC = reinterpret_cast<const int*>(base + 3 * n_ylm);
    t.C1 = base + 4 * n_ylm;
    t.C2 = t.C1 + maxl + 1;
    t.D0 = t.C2 + maxl + 1;
    return t;
}

// Copy the constants into shared memory as T (the DEC entries keep their bits).
template <typename T>
__device__ inline void load_ylm_tab(const double* src, T* dst, int n_ylm, int maxl) {
    const int n = ylm_table_size(n_ylm, maxl);
    for (int q = threadIdx.x; q < n; q += blockDim.x) {
        if (q >= 3 * n_ylm && q < 4 * n_ylm) {
            reinterpret_cast<int*>(dst + 3 * n_ylm)[q - 3 * n_ylm] = (int)src[q];
        } else {
            dst[q] = (T)src[q];
        }
    }
}

// Basis of one pair image, in shared memory, computed by one warp.
template <typename T>
struct BasisView {
    T* fn;         // [n_fn_max]
    T* fnd;        // [n_fn_max]
    cplx<T>* Y;    // [n_ylm]
    cplx<T>* dY;   // [3][n_ylm]
    T* P;          // [n_ylm + 2] scratch
    T* Q;          // [n_ylm + 2] scratch
    T* cs;         // [maxl + 1] cos(m phi)
    T* sn;         // [maxl + 1] sin(m phi)
};

template <typename T>
__host__ __device__ inline size_t basis_slot_elems(int n_fn_max, int n_ylm, int maxl) {
    // counted in units of T
    return (size_t)2 * n_fn_max + 2 * (size_t)n_ylm * 4 + 2 * ((size_t)n_ylm + 2) + 2 * ((size_t)maxl + 1);
}

template <typename T>
__device__ inline BasisView<T> basis_view(T* base, int n_fn_max, int n_ylm, int maxl) {
    BasisView<T> v;
    v.fn = base;
    v.fnd = base + n_fn_max;
    v.Y = reinterpret_cast<cplx<T>*>(base + 2 * n_fn_max);
    v.dY = v.Y + n_ylm;
    v.P = base + 2 * n_fn_max + 2 * (size_t)n_ylm * 4;
    v.Q = v.P + n_ylm + 2;
    v.cs = v.Q + n_ylm + 2;
    v.sn = v.cs + maxl + 1;
    return v;
}

__device__ __forceinline__ int lmi(int l, int m) { return l * (l + 1) / 2 + m; }

// Model constants in the precision T of a kernel (no FP64 work in FP32 kernels).
template <typename T>
__device__ __forceinline__ T model_cutoff(const DevModel& M);
template <>
__device__ __forceinline__ double model_cutoff<double>(const DevModel& M) { return M.cutoff; }
template <>
__device__ __forceinline__ float model_cutoff<float>(const DevModel& M) { return M.cutoff_f; }
template <typename T>
__device__ __forceinline__ T model_beta(const DevModel& M, int q);
template <>
__device__ __forceinline__ double model_beta<double>(const DevModel& M, int q) { return M.tp_beta[q]; }
template <>
__device__ __forceinline__ float model_beta<float>(const DevModel& M, int q) { return M.tp_beta_f[q]; }
template <typename T>
__device__ __forceinline__ T model_mu(const DevModel& M, int q);
template <>
__device__ __forceinline__ double model_mu<double>(const DevModel& M, int q) { return M.tp_mu[q]; }
template <>
__device__ __forceinline__ float model_mu<float>(const DevModel& M, int q) { return M.tp_mu_f[q]; }

// Sum in T with a long result: FP64 for T = double; for T = float a
// float-float pair (Knuth's TwoSum keeps the rounding error of every addition
// in lo), about 48 significant bits without FP64 instructions.
template <typename T>
struct LongSum {
    double v = 0.0;
    __device__ __forceinline__ void add(double x) { v += x; }
    __device__ __forceinline__ double value() const { return v; }
    __device__ __forceinline__ void merge(const LongSum& o) { v += o.v; }
};
template <>
struct LongSum<float> {
    float hi = 0.f, lo = 0.f;
    __device__ __forceinline__ void add(float x) {
        const float s = __fadd_rn(hi, x);
        const float bb = __fsub_rn(s, hi);
        const float e = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bb)), __fsub_rn(x, bb));
        hi = s;
        lo = __fadd_rn(lo, e);
    }
    __device__ __forceinline__ float value() const { return __fadd_rn(hi, lo); }
    __device__ __forceinline__ void merge(const LongSum& o) {
        add(o.hi);
        lo = __fadd_rn(lo, o.lo);
    }
};

// Radial functions of one type pair at distance dis
// (polymlp_basis_function.h:16-43, polymlp_functions_interface.cpp:41-62).
template <typename T, bool DERIV>
__device__ __noinline__ void warp_radial(const DevModel& M, int tp, T dis, BasisView<T> B, int lane) {
    const int nfn = M.tp_nfn[tp];
    const T r = dis;
    const T rc = model_cutoff<T>(M);
    const T v1 = (T)kPiD / rc;
    const T v2 = v1 * r;
    T fc, fcd = 0;
    if (DERIV) {
        fc = (T)0.5 * (cos(v2) + (T)1.0);
        fcd = (T)-0.5 * v1 * sin(v2);
    } else {
        fc = (T)0.5 * (cos((T)kPiD * r / rc) + (T)1.0);
    }
    for (int q = lane; q < nfn; q += 32) {
        const T beta = model_beta<T>(M, tp * M.n_fn_max + q);
        const T mu = model_mu<T>(M, tp * M.n_fn_max + q);
        const T x = r - mu;
        const T bf = exp(-beta * x * x);
        B.fn[q] = bf * fc;
        if (DERIV) B.fnd[q] = (T)-2.0 * beta * x * bf * fc + bf * fcd;
    }
}

// Y_lm (m <= 0, index l(l+1)/2 + l + m) and gradients of the unit vector
// (x, y, z)/r, following the normalised associated Legendre recursion of
// polymlp_spherical_harmonics.cpp:27-209 (Limpanuparb & Milthorpe,
// arXiv:1410.1748), with the (l, m) constants read from a table.  Lane m
// computes the Legendre column m; lanes then fill the (l, m) table.
template <typename T, bool DERIV>
__device__ __noinline__ void warp_ylm(int maxl, int n_ylm, const YlmTab<T>& tab, T x, T y, T z, T r, BasisView<T> B,
                                int lane) {
    const T ct = z / r;
    const T rho = hypot(x, y);
    const T cp = rho > (T)0 ? x / rho : (T)1;
    const T sp = rho > (T)0 ? y / rho : (T)0;
    const T st = sqrt((T)1 - ct * ct);
    const T s2pi = (T)0.39894228040143267794;
    const T sq3 = (T)1.7320508075688772935, sq32 = (T)1.2247448713915890491;
    const int L = maxl;
    if (lane <= L) {
        const int m = lane;
        T pmm, qmm;
        if (m == 0) {
            pmm = s2pi;
            qmm = 0;
        } else {
            pmm = -st * sq32 * s2pi;
            qmm = -sq32 * s2pi;
            for (int l = 2; l <= m; ++l) {
                const T c1 = tab.C1[l] * st;
                pmm = c1 * pmm;
                qmm = c1 * qmm;
            }
        }
        B.P[lmi(m, m)] = pmm;
        B.Q[lmi(m, m)] = qmm;
        if (m + 1 <= L) {
            T p1, q1;
            if (m == 0) {
                p1 = ct * sq3 * s2pi;
                q1 = 0;
            } else {
                const T c2 = tab.C2[m] * ct;
                p1 = c2 * pmm;
                q1 = c2 * qmm;
            }
            B.P[lmi(m + 1, m)] = p1;
            B.Q[lmi(m + 1, m)] = q1;
            T p2 = pmm, q2 = qmm;
            for (int l = m + 2; l <= L; ++l) {
                const T alm = tab.A[lmi(l, m)], blm = tab.B[lmi(l, m)];
                const T p = alm * (ct * p1 + blm * p2);
                const T q = alm * (ct * q1 + blm * q2);
                B.P[lmi(l, m)] = p;
                B.Q[lmi(l, m)] = q;
                p2 = p1;
                q2 = q1;
                p1 = p;
                q1 = q;
            }
        }
        // cos(m phi), sin(m phi) by the Chebyshev recurrence
        T c1 = 1, c2 = cp, s1 = 0, s2 = -sp;
        const T tc = (T)2 * c2;
        for (int mp = 1; mp <= m; ++mp) {
            const T s = tc * s1 - s2, c = tc * c1 - c2;
            c2 = c1;
            c1 = c;
            s2 = s1;
            s1 = s;
        }
        B.cs[m] = c1;
        B.sn[m] = s1;
    }
    if (lane == 0) {
        B.P[n_ylm] = 0;
        B.Q[n_ylm] = 0;
        B.P[n_ylm + 1] = 0;
        B.Q[n_ylm + 1] = 0;
    }
    __syncwarp();
    const T h = (T)0.5 * (T)1.41421356237309504880;
    const T invr = (T)1 / r;
    for (int idx = lane; idx < n_ylm; idx += 32) {
        const int dec = tab.DEC[idx];
        const int l = dec & 0xff, mp = dec >> 8;  // m = -mp
        if (mp == 0) {
            B.Y[idx] = {B.P[lmi(l, 0)] * h, (T)0};
            if (DERIV) {
                const T qv = (l == 0) ? B.Q[1] : B.Q[lmi(l, 1)];
                const T common = qv * st * invr * tab.D0[l];
                B.dY[idx] = {common * ct * cp, (T)0};
                B.dY[n_ylm + idx] = {common * ct * sp, (T)0};
                B.dY[2 * n_ylm + idx] = {-common * st, (T)0};
            }
        } else {
            const T sign = (mp & 1) ? (T)-1 : (T)1;
            const T c = B.cs[mp], s = B.sn[mp];
            const T tmp = sign * B.P[lmi(l, mp)] * h;
            B.Y[idx] = {tmp * c, -(tmp * s)};
            if (DERIV) {
                const cplx<T> common = {c * h * invr, s * h * invr};
                const T qlm = B.Q[lmi(l, mp)];
                T dth = (T)mp * ct * qlm;
                if (mp != l) dth += tab.D1[lmi(l, mp)] * B.Q[lmi(l, mp + 1)] * st;
                const T dph = (T)mp * qlm;  // imaginary
                cplx<T> ax = cmul(common, cplx<T>{dth * ct * cp, -dph * sp});
                cplx<T> ay = cmul(common, cplx<T>{dth * ct * sp, dph * cp});
                cplx<T> az = {-common.re * dth * st, -common.im * dth * st};
                B.dY[idx] = {sign * ax.re, -sign * ax.im};
                B.dY[n_ylm + idx] = {sign * ay.re, -sign * ay.im};
                B.dY[2 * n_ylm + idx] = {sign * az.re, -sign * az.im};
            }
        }
    }
}

// One radial function q of type pair tp and its derivative at distance r, in
// the operation order of warp_radial (for one thread).
template <typename T>
__device__ __forceinline__ void radial_one(const DevModel& M, int tp, int q, T r, T& fn, T& fnd) {
    const T rc = model_cutoff<T>(M);
    const T v1 = (T)kPiD / rc;
    const T v2 = v1 * r;
    const T fc = (T)0.5 * (cos(v2) + (T)1.0);
    const T fcd = (T)-0.5 * v1 * sin(v2);
    const T beta = model_beta<T>(M, tp * M.n_fn_max + q);
    const T mu = model_mu<T>(M, tp * M.n_fn_max + q);
    const T x = r - mu;
    const T bf = exp(-beta * x * x);
    fn = bf * fc;
    fnd = (T)-2.0 * beta * x * bf * fc + bf * fcd;
}

// Direction terms of Y_lm shared by the columns of one pair.
template <typename T>
struct YlmDir {
    T ct, st, cp, sp, invr;
};
template <typename T>
__device__ __forceinline__ YlmDir<T> ylm_dir(T x, T y, T z, T r) {
    YlmDir<T> d;
    d.ct = z / r;
    const T rho = hypot(x, y);
    d.cp = rho > (T)0 ? x / rho : (T)1;
    d.sp = rho > (T)0 ? y / rho : (T)0;
    d.st = sqrt((T)1 - d.ct * d.ct);
    d.invr = (T)1 / r;
    return d;
}

// Column m' = mp of Y_lm (keys (l, -mp), l = mp .. L; key k = l(l+1)/2 + l - mp
// at rows + ks k: with DERIV 8 values, Y, dY/dx, dY/dy, dY/dz as (re, im);
// else Y alone) for one thread.  The same recursion and constants as warp_ylm
// (the normalised associated Legendre recursion of
// polymlp_spherical_harmonics.cpp:27-209), run down column mp, with the Q
// recursion of column mp + 1 in lock step for the theta derivative, so that
// no (l, m) scratch table is needed.
template <typename T, bool DERIV = true>
__device__ __noinline__ void ylm_column(int mp, int L, const YlmTab<T>& tab, const YlmDir<T>& d, T* rows, int ks) {
    const T s2pi = (T)0.39894228040143267794;
    const T sq3 = (T)1.7320508075688772935, sq32 = (T)1.2247448713915890491;
    const T h = (T)0.5 * (T)1.41421356237309504880;
    const T ct = d.ct, st = d.st, cp = d.cp, sp = d.sp, invr = d.invr;
    // diagonals P_mp,mp, Q_mp,mp and Q_mp+1,mp+1
    T pmm, qmm;
    if (mp == 0) {
        pmm = s2pi;
        qmm = 0;
    } else {
        pmm = -st * sq32 * s2pi;
        qmm = -sq32 * s2pi;
        for (int l = 2; l <= mp; ++l) {
            const T c1 = tab.C1[l] * st;
            pmm = c1 * pmm;
            qmm = c1 * qmm;
        }
    }
    T qn_mm = 0;  // Q_mp+1,mp+1
    if (mp + 1 <= L) qn_mm = (mp + 1 == 1) ? -sq32 * s2pi : (tab.C1[mp + 1] * st) * qmm;
    // cos(mp phi), sin(mp phi) by the Chebyshev recurrence
    T cs = 1, c2 = cp, sn = 0, s2 = -sp;
    {
        const T tc = (T)2 * c2;
        for (int q = 1; q <= mp; ++q) {
            const T s = tc * sn - s2, c = tc * cs - c2;
            c2 = cs;
            cs = c;
            s2 = sn;
            sn = s;
        }
    }
    const T sign = (mp & 1) ? (T)-1 : (T)1;
    const cplx<T> common = {cs * h * invr, sn * h * invr};
    T p1 = 0, p2 = 0, q1 = 0, q2 = 0;     // column mp: values at l - 1, l - 2
    T n1 = 0, n2 = 0;                     // column mp + 1 (Q only)
    for (int l = mp; l <= L; ++l) {
        T p, q, qn;
        if (l == mp) {
            p = pmm;
            q = qmm;
            qn = 0;
        } else if (l == mp + 1) {
            if (mp == 0) {
                p = ct * sq3 * s2pi;
                q = 0;
            } else {
                const T c2m = tab.C2[mp] * ct;
                p = c2m * p1;
                q = c2m * q1;
            }
            qn = qn_mm;
        } else {
            const T alm = tab.A[lmi(l, mp)], blm = tab.B[lmi(l, mp)];
            p = alm * (ct * p1 + blm * p2);
            q = alm * (ct * q1 + blm * q2);
            if (l == mp + 2) {
                qn = (tab.C2[mp + 1] * ct) * n1;
            } else {
                const T aln = tab.A[lmi(l, mp + 1)], bln = tab.B[lmi(l, mp + 1)];
                qn = aln * (ct * n1 + bln * n2);
            }
        }
        p2 = p1;
        p1 = p;
        q2 = q1;
        q1 = q;
        n2 = n1;
        n1 = qn;
        T* o = rows + (size_t)ks * (l * (l + 1) / 2 + l - mp);
        if (!DERIV) {
            const T tmp = mp == 0 ? p * h : sign * p * h;
            o[0] = mp == 0 ? tmp : tmp * cs;
            o[1] = mp == 0 ? (T)0 : -(tmp * sn);
            continue;
        }
        if (mp == 0) {
            const T qv = (l == 0) ? (T)0 : qn;
            const T c0 = qv * st * invr * tab.D0[l];
            o[0] = p * h;
            o[1] = 0;
            o[2] = c0 * ct * cp;
            o[3] = 0;
            o[4] = c0 * ct * sp;
            o[5] = 0;
            o[6] = -c0 * st;
            o[7] = 0;
        } else {
            const T tmp = sign * p * h;
            T dth = (T)mp * ct * q;
            if (mp != l) dth += tab.D1[lmi(l, mp)] * qn * st;
            const T dph = (T)mp * q;
            const cplx<T> ax = cmul(common, cplx<T>{dth * ct * cp, -dph * sp});
            const cplx<T> ay = cmul(common, cplx<T>{dth * ct * sp, dph * cp});
            const cplx<T> az = {-common.re * dth * st, -common.im * dth * st};
            o[0] = tmp * cs;
            o[1] = -(tmp * sn);
            o[2] = sign * ax.re;
            o[3] = -sign * ax.im;
            o[4] = sign * ay.re;
            o[5] = -sign * ay.im;
            o[6] = sign * az.re;
            o[7] = -sign * az.im;
        }
    }
}

}  // namespace pg
