// CPU oracle: see oracle.h.  TEST INFRASTRUCTURE ONLY.
//
// Restates the reference algorithm (sekocha/pypolymlp) in plain C++:
//   neighbour lists       compute/neighbor_full.cpp:10-76, neighbor_half.cpp:10-179
//   radial functions      polymlp/polymlp_basis_function.h:16-43,
//                         polymlp/polymlp_functions_interface.cpp:11-86
//   spherical harmonics   polymlp/polymlp_spherical_harmonics.cpp:27-209
//   a_nlm + derivatives   compute/local.cpp:62-217, compute/local_pair.cpp:58-123
//   features/derivatives  polymlp/polymlp_features.cpp:155-248, polymlp_products.cpp
//   polynomial X rows     compute/model.cpp:39-267, compute/py_model.cpp:10-56
//   evaluator             compute/polymlp_eval.cpp:24-403, polymlp/polymlp_potential.cpp:235-295
// The derivative arrays are dense over all atoms of a structure, as in the
// reference, so timing this code times the reference algorithm.
#include "oracle.h"

#include <omp.h>

#include <cmath>
#include <complex>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

#include "cell.h"
#include "model_tables.h"
#include "params.h"

using cd = std::complex<double>;

namespace {

thread_local std::string g_err;
constexpr double kPi = 3.1415926535897932384626433832795;

template <class F>
int guarded(F&& f) {
    try {
        f();
        return 0;
    } catch (const std::exception& e) {
        g_err = e.what();
    } catch (...) {
        g_err = "unknown error";
    }
    return 1;
}

// ---------------------------------------------------------------- radial
// f_n(r) = exp(-beta (r - mu)^2) * 0.5 (cos(pi r / rc) + 1) and derivative.
void radial_d(double dis, double cutoff, const pg::FeatureParams& fp, const std::vector<int>& ns, double* fn,
              double* fnd) {
    double fc = 0.0, fcd = 0.0;
    if (dis < cutoff) {
        const double v1 = kPi / cutoff, v2 = v1 * dis;
        fc = 0.5 * (std::cos(v2) + 1.0);
        fcd = -0.5 * v1 * std::sin(v2);
    }
    for (size_t q = 0; q < ns.size(); ++q) {
        const double beta = fp.params[ns[q]][0], mu = fp.params[ns[q]][1];
        const double dx = dis - mu;
        const double bf = std::exp(-beta * dx * dx);
        const double bfd = -2.0 * beta * dx * bf;
        fn[q] = bf * fc;
        fnd[q] = bfd * fc + bf * fcd;
    }
}

void radial(double dis, double cutoff, const pg::FeatureParams& fp, const std::vector<int>& ns, double* fn) {
    const double fc = dis < cutoff ? 0.5 * (std::cos(kPi * dis / cutoff) + 1.0) : 0.0;
    for (size_t q = 0; q < ns.size(); ++q) {
        const double beta = fp.params[ns[q]][0], mu = fp.params[ns[q]][1];
        const double dx = dis - mu;
        fn[q] = std::exp(-beta * dx * dx) * fc;
    }
}

// ---------------------------------------------------------------- Y_lm
// Normalised associated Legendre functions P_l^m and P_l^m / sin(theta),
// m >= 0, index l(l+1)/2 + m (Limpanuparb & Milthorpe, arXiv:1410.1748).
inline int lmi(int l, int m) { return l * (l + 1) / 2 + m; }

void legendre(int lmax, double ct, std::vector<double>& p, std::vector<double>* q) {
    const int n = (lmax + 1) * (lmax + 2) / 2;
    p.assign(n + 1, 0.0);
    if (q) q->assign(n + 1, 0.0);
    const double s2pi = 0.39894228040143267794;
    p[0] = s2pi;
    if (lmax == 0) return;
    const double st = std::sqrt(1.0 - ct * ct);
    p[lmi(1, 0)] = ct * 1.7320508075688772935 * s2pi;
    p[lmi(1, 1)] = -st * 1.2247448713915890491 * s2pi;
    if (q) (*q)[lmi(1, 1)] = -1.2247448713915890491 * s2pi;
    for (int l = 2; l <= lmax; ++l) {
        const double c1 = -std::sqrt(1.0 + 0.5 / l) * st;
        const double c2 = std::sqrt(2.0 * (l - 1.0) + 3.0) * ct;
        p[lmi(l, l)] = c1 * p[lmi(l - 1, l - 1)];
        p[lmi(l, l - 1)] = c2 * p[lmi(l - 1, l - 1)];
        if (q) {
            (*q)[lmi(l, l)] = c1 * (*q)[lmi(l - 1, l - 1)];
            (*q)[lmi(l, l - 1)] = c2 * (*q)[lmi(l - 1, l - 1)];
        }
    }
    for (int l = 2; l <= lmax; ++l) {
        const double ls = l * l, lm1s = (l - 1) * (l - 1);
        for (int m = 0; m <= l - 2; ++m) {
            const double ms = m * m;
            const double alm = std::sqrt((4.0 * ls - 1.0) / (ls - ms));
            const double blm = -std::sqrt((lm1s - ms) / (4.0 * lm1s - 1.0));
            p[lmi(l, m)] = alm * (ct * p[lmi(l - 1, m)] + blm * p[lmi(l - 2, m)]);
            if (q) (*q)[lmi(l, m)] = alm * (ct * (*q)[lmi(l - 1, m)] + blm * (*q)[lmi(l - 2, m)]);
        }
    }
}

// Y_lm for m <= 0 at index l(l+1)/2 + l + m.
void ylm_only(double x, double y, double z, int lmax, std::vector<cd>& Y) {
    const double r = std::sqrt(x * x + y * y + z * z);
    const double ct = z / r;
    const double rho = std::hypot(x, y);
    const double cp = rho > 0.0 ? x / rho : 1.0, sp = rho > 0.0 ? y / rho : 0.0;
    std::vector<double> p;
    legendre(lmax, ct, p, nullptr);
    Y.assign((lmax + 1) * (lmax + 2) / 2, cd(0.0, 0.0));
    const double h = 0.5 * M_SQRT2;
    for (int l = 0; l <= lmax; ++l) Y[lmi(l, 0) + l] = p[lmi(l, 0)] * h;
    double c1 = 1.0, c2 = cp, s1 = 0.0, s2 = -sp;
    const double tc = 2.0 * c2;
    double sign = -1.0;
    for (int mp = 1; mp <= lmax; ++mp) {
        const double s = tc * s1 - s2, c = tc * c1 - c2;
        c2 = c1;
        c1 = c;
        s2 = s1;
        s1 = s;
        for (int l = mp; l <= lmax; ++l) Y[lmi(l, -mp) + l] = (sign * p[lmi(l, mp)] * h) * cd(c, -s);
        sign *= -1.0;
    }
}

void ylm_deriv(double r, double x, double y, double z, int lmax, std::vector<cd>& Y, std::vector<cd>& Yx,
               std::vector<cd>& Yy, std::vector<cd>& Yz) {
    const double ct = z / r;
    const double rho = std::hypot(x, y);
    const double cp = rho > 0.0 ? x / rho : 1.0, sp = rho > 0.0 ? y / rho : 0.0;
    std::vector<double> p, q;
    legendre(lmax, ct, p, &q);
    const int n = (lmax + 1) * (lmax + 2) / 2;
    Y.assign(n, cd());
    Yx.assign(n, cd());
    Yy.assign(n, cd());
    Yz.assign(n, cd());
    const double st = std::sqrt(1.0 - ct * ct);
    const double invr = 1.0 / r;
    const double h = 0.5 * M_SQRT2;
    for (int l = 0; l <= lmax; ++l) {
        const int idx = lmi(l, 0) + l;
        Y[idx] = p[lmi(l, 0)] * h;
        const double common = q[lmi(l, 1)] * st * invr * std::sqrt(0.5 * l * (l + 1));
        Yx[idx] = common * ct * cp;
        Yy[idx] = common * ct * sp;
        Yz[idx] = -common * st;
    }
    double c1 = 1.0, c2 = cp, s1 = 0.0, s2 = -sp;
    const double tc = 2.0 * c2;
    double sign = -1.0;
    for (int mp = 1; mp <= lmax; ++mp) {
        const double s = tc * s1 - s2, c = tc * c1 - c2;
        c2 = c1;
        c1 = c;
        s2 = s1;
        s1 = s;
        for (int l = mp; l <= lmax; ++l) {
            const int idx = lmi(l, -mp) + l;
            Y[idx] = (sign * p[lmi(l, mp)] * h) * cd(c, -s);
            const cd common = cd(c, s) * h * invr;
            double dth = mp * ct * q[lmi(l, mp)];
            if (mp != l) dth += std::sqrt((double)((l - mp) * (l + mp + 1))) * q[lmi(l, mp + 1)] * st;
            const cd dph(0.0, mp * q[lmi(l, mp)]);
            Yx[idx] = sign * std::conj(common * (dth * ct * cp - dph * sp));
            Yy[idx] = sign * std::conj(common * (dth * ct * sp + dph * cp));
            Yz[idx] = sign * std::conj(-common * dth * st);
        }
        sign *= -1.0;
    }
}

// ---------------------------------------------------------------- neighbours
struct NList {
    std::vector<int> off, nb;
    std::vector<double> d;  // 3 per entry: pos[j] - pos[i] + t
};

NList neighbor_full(const double* axis, const double* pos, int n, double cutoff) {
    const auto ct = pg::cell_translations(axis, pos, n, cutoff);
    const double tol_sq = 1e-10 * 1e-10, rc2 = cutoff * cutoff;
    NList L;
    L.off.assign(n + 1, 0);
    for (int i = 0; i < n; ++i) {
        for (int j = 0; j < n; ++j) {
            const double dx0 = ct.pos[j][0] - ct.pos[i][0];
            const double dy0 = ct.pos[j][1] - ct.pos[i][1];
            const double dz0 = ct.pos[j][2] - ct.pos[i][2];
            for (const auto& t : ct.trans) {
                const double dx = dx0 + t[0], dy = dy0 + t[1], dz = dz0 + t[2];
                const double r2 = dx * dx + dy * dy + dz * dz;
                if (r2 < rc2 && r2 > tol_sq) {
                    L.nb.push_back(j);
                    L.d.insert(L.d.end(), {dx, dy, dz});
                }
            }
        }
        L.off[i + 1] = (int)L.nb.size();
    }
    return L;
}

NList neighbor_half(const double* axis, const double* pos, int n, double cutoff) {
    const auto ct = pg::cell_translations(axis, pos, n, cutoff);
    const double tol = 1e-10, tol_sq = tol * tol, rc2 = cutoff * cutoff;
    NList L;
    L.off.assign(n + 1, 0);
    for (int i = 0; i < n; ++i) {
        for (int j = 0; j < i; ++j) {
            const double dx0 = ct.pos[j][0] - ct.pos[i][0];
            const double dy0 = ct.pos[j][1] - ct.pos[i][1];
            const double dz0 = ct.pos[j][2] - ct.pos[i][2];
            for (const auto& t : ct.trans) {
                const double dx = dx0 + t[0], dy = dy0 + t[1], dz = dz0 + t[2];
                const double r2 = dx * dx + dy * dy + dz * dz;
                if (r2 < rc2 && r2 > tol_sq) {
                    L.nb.push_back(j);
                    L.d.insert(L.d.end(), {dx, dy, dz});
                }
            }
        }
        for (const auto& t : ct.trans) {
            const double dx = t[0], dy = t[1], dz = t[2];
            const double r2 = dx * dx + dy * dy + dz * dz;
            if (r2 < rc2 && r2 > tol_sq) {
                bool keep;
                if (dz >= tol) keep = true;
                else if (std::fabs(dz) < tol && dy >= tol) keep = true;
                else if (std::fabs(dz) < tol && std::fabs(dy) < tol && dx >= tol) keep = true;
                else keep = false;
                if (keep) {
                    L.nb.push_back(i);
                    L.d.insert(L.d.end(), {dx, dy, dz});
                }
            }
        }
        L.off[i + 1] = (int)L.nb.size();
    }
    return L;
}

// neighbor_half.cpp:126-179
NList half_to_full(const NList& H, int n) {
    std::vector<int> deg(n, 0);
    for (int i = 0; i < n; ++i) {
        deg[i] += H.off[i + 1] - H.off[i];
        for (int k = H.off[i]; k < H.off[i + 1]; ++k) ++deg[H.nb[k]];
    }
    NList F;
    F.off.assign(n + 1, 0);
    for (int i = 0; i < n; ++i) F.off[i + 1] = F.off[i] + deg[i];
    F.nb.assign(F.off[n], 0);
    F.d.assign(3 * (size_t)F.off[n], 0.0);
    std::vector<int> pos(F.off.begin(), F.off.end() - 1);
    for (int i = 0; i < n; ++i)
        for (int k = H.off[i]; k < H.off[i + 1]; ++k) {
            const int j = H.nb[k];
            int a = pos[i]++;
            F.nb[a] = j;
            for (int c = 0; c < 3; ++c) F.d[3 * a + c] = H.d[3 * k + c];
            a = pos[j]++;
            F.nb[a] = i;
            for (int c = 0; c < 3; ++c) F.d[3 * a + c] = -H.d[3 * k + c];
        }
    return F;
}

// ---------------------------------------------------------------- products
inline double prod_real(const cd& a, const cd& b) { return a.real() * b.real() - a.imag() * b.imag(); }

// polymlp_products.cpp:21-37
double product_real(const std::vector<int>& ids, const std::vector<cd>& a) {
    const size_t n = ids.size();
    if (n == 4) return prod_real(a[ids[1]] * a[ids[2]] * a[ids[3]], a[ids[0]]);
    if (n == 3) return prod_real(a[ids[0]] * a[ids[1]], a[ids[2]]);
    if (n == 2) return prod_real(a[ids[0]], a[ids[1]]);
    if (n == 1) return a[ids[0]].real();
    if (n == 0) return 1.0;
    cd v = a[ids[1]];
    for (size_t i = 2; i < n; ++i) v *= a[ids[i]];
    return prod_real(v, a[ids[0]]);
}

template <class T>
T product(const std::vector<int>& ids, const std::vector<T>& a) {
    if (ids.empty()) return T(1.0);
    T v = a[ids[0]];
    for (size_t i = 1; i < ids.size(); ++i) v *= a[ids[i]];
    return v;
}

struct Model {
    pg::ModelTables mt;
    explicit Model(const pg_feature_params* p) : mt(pg::build_model_tables(pg::feature_params_from_abi(p))) {}
};

// ---------------------------------------------------------------- X rows
// One structure: Model::run (model.cpp:39-88) with Local::gtinv_d / LocalPair::pair_d.
void structure_rows(const pg::ModelTables& mt, const double* axis, const double* pos, const int* types, int N,
                    bool force, double* x, int64_t ld, int64_t e_row, int64_t f_row, int64_t s_row) {
    const auto& fp = mt.fp;
    const int F = mt.n_features;
    const NList L = neighbor_full(axis, pos, N, fp.cutoff);
    std::vector<double> xe(F, 0.0);
    std::vector<double> xf(force ? (size_t)3 * N * F : 0, 0.0);  // [col][3N]
    std::vector<double> xs(force ? (size_t)6 * F : 0, 0.0);     // [col][6]
    std::vector<double> fn(fp.params.size()), fnd(fp.params.size());
    std::vector<cd> Y, Yx, Yy, Yz;
    const double tol = 1e-20;
    for (int a1 = 0; a1 < N; ++a1) {
        const int t1 = types[a1];
        const auto& tt = mt.types[t1];
        const int nlin = (int)tt.lin_index.size();
        std::vector<double> d(nlin, 0.0);
        std::vector<double> dfx, dfy, dfz, dfs;  // [feature][N] and [feature][6]
        if (force) {
            dfx.assign((size_t)nlin * N, 0.0);
            dfy.assign((size_t)nlin * N, 0.0);
            dfz.assign((size_t)nlin * N, 0.0);
            dfs.assign((size_t)nlin * 6, 0.0);
        }
        if (fp.gtinv) {
            const int K = (int)tt.full.size();
            std::vector<cd> a(K, cd());
            std::vector<cd> ax, ay, az, as;
            if (force) {
                ax.assign((size_t)K * N, cd());
                ay.assign((size_t)K * N, cd());
                az.assign((size_t)K * N, cd());
                as.assign((size_t)K * 6, cd());
            }
            for (int k = L.off[a1]; k < L.off[a1 + 1]; ++k) {
                const int j = L.nb[k];
                const double dx = L.d[3 * k], dy = L.d[3 * k + 1], dz = L.d[3 * k + 2];
                const double dis = std::sqrt(dx * dx + dy * dy + dz * dz);
                if (dis >= fp.cutoff) continue;
                const int tp = mt.type_pairs[t1][types[j]];
                const auto& ns = mt.tp_to_n[tp];
                if (force) {
                    radial_d(dis, fp.cutoff, fp, ns, fn.data(), fnd.data());
                    ylm_deriv(dis, dx, dy, dz, fp.maxl, Y, Yx, Yy, Yz);
                } else {
                    radial(dis, fp.cutoff, fp, ns, fn.data());
                    ylm_only(dx, dy, dz, fp.maxl, Y);
                }
                for (const auto& e : tt.noconj) {
                    if (e.tp != tp) continue;
                    const double f = fn[e.n_id];
                    if (!force) {
                        if (!(std::fabs(f) > tol)) continue;
                        a[e.ilocal_id] += f * Y[e.ylm_key];
                        continue;
                    }
                    if (f < tol) continue;
                    const int id = e.ilocal_id;
                    a[id] += f * Y[e.ylm_key];
                    const cd d1 = fnd[e.n_id] * Y[e.ylm_key] / dis;
                    const cd vx = d1 * dx + f * Yx[e.ylm_key];
                    const cd vy = d1 * dy + f * Yy[e.ylm_key];
                    const cd vz = d1 * dz + f * Yz[e.ylm_key];
                    ax[(size_t)id * N + a1] += vx;
                    ay[(size_t)id * N + a1] += vy;
                    az[(size_t)id * N + a1] += vz;
                    ax[(size_t)id * N + j] -= vx;
                    ay[(size_t)id * N + j] -= vy;
                    az[(size_t)id * N + j] -= vz;
                    as[(size_t)id * 6 + 0] -= vx * dx;
                    as[(size_t)id * 6 + 1] -= vy * dy;
                    as[(size_t)id * 6 + 2] -= vz * dz;
                    as[(size_t)id * 6 + 3] -= vx * dy;
                    as[(size_t)id * 6 + 4] -= vy * dz;
                    as[(size_t)id * 6 + 5] -= vz * dx;
                }
            }
            for (const auto& e : tt.full) {
                if (!e.conj) continue;
                const int i1 = e.ilocal_id, i2 = e.ilocal_conj_id;
                a[i1] = e.cc * std::conj(a[i2]);
                if (force) {
                    for (int q = 0; q < N; ++q) {
                        ax[(size_t)i1 * N + q] = e.cc * std::conj(ax[(size_t)i2 * N + q]);
                        ay[(size_t)i1 * N + q] = e.cc * std::conj(ay[(size_t)i2 * N + q]);
                        az[(size_t)i1 * N + q] = e.cc * std::conj(az[(size_t)i2 * N + q]);
                    }
                    for (int q = 0; q < 6; ++q) as[(size_t)i1 * 6 + q] = e.cc * std::conj(as[(size_t)i2 * 6 + q]);
                }
            }
            for (int f = 0; f < nlin; ++f) {
                double v = 0.0;
                for (const auto& s : tt.value_terms[f]) v += s.coeff * product_real(s.ids, a);
                d[f] = v;
            }
            if (force) {
                for (int f = 0; f < nlin; ++f)
                    for (const auto& s : tt.deriv_terms[f]) {
                        const cd val = s.coeff * product<cd>(s.rest, a);
                        const size_t h = (size_t)s.head;
                        for (int q = 0; q < N; ++q) {
                            dfx[(size_t)f * N + q] += prod_real(val, ax[h * N + q]);
                            dfy[(size_t)f * N + q] += prod_real(val, ay[h * N + q]);
                            dfz[(size_t)f * N + q] += prod_real(val, az[h * N + q]);
                        }
                        for (int q = 0; q < 6; ++q) dfs[(size_t)f * 6 + q] += prod_real(val, as[h * 6 + q]);
                    }
            }
        } else {
            // pair features (local_pair.cpp:17-123)
            for (int k = L.off[a1]; k < L.off[a1 + 1]; ++k) {
                const int j = L.nb[k];
                const double dx = L.d[3 * k], dy = L.d[3 * k + 1], dz = L.d[3 * k + 2];
                const double dis = std::sqrt(dx * dx + dy * dy + dz * dz);
                if (dis >= fp.cutoff) continue;
                const int tp = mt.type_pairs[t1][types[j]];
                const auto& ns = mt.tp_to_n[tp];
                if (force) radial_d(dis, fp.cutoff, fp, ns, fn.data(), fnd.data());
                else radial(dis, fp.cutoff, fp, ns, fn.data());
                for (const auto& e : tt.ntp) {
                    if (e.tp != tp) continue;
                    const int id = e.ilocal_id;
                    d[id] += fn[e.n_id];
                    if (!force) continue;
                    const double vx = fnd[e.n_id] * dx / dis, vy = fnd[e.n_id] * dy / dis,
                                 vz = fnd[e.n_id] * dz / dis;
                    dfx[(size_t)id * N + a1] += vx;
                    dfy[(size_t)id * N + a1] += vy;
                    dfz[(size_t)id * N + a1] += vz;
                    dfx[(size_t)id * N + j] -= vx;
                    dfy[(size_t)id * N + j] -= vy;
                    dfz[(size_t)id * N + j] -= vz;
                    dfs[(size_t)id * 6 + 0] -= vx * dx;
                    dfs[(size_t)id * 6 + 1] -= vy * dy;
                    dfs[(size_t)id * 6 + 2] -= vz * dz;
                    dfs[(size_t)id * 6 + 3] -= vx * dy;
                    dfs[(size_t)id * 6 + 4] -= vy * dz;
                    dfs[(size_t)id * 6 + 5] -= vz * dx;
                }
            }
        }
        // model_polynomial (model.cpp:159-267)
        for (const auto& p : tt.poly) {
            const int col = p.col;
            const size_t n = p.local_ids.size();
            const int c1 = p.local_ids[0];
            const int c2 = n > 1 ? p.local_ids[1] : 0, c3 = n > 2 ? p.local_ids[2] : 0;
            double w1 = 1.0, w2 = 0.0, w3 = 0.0;
            if (n == 1) {
                xe[col] += d[c1];
            } else if (n == 2) {
                xe[col] += d[c1] * d[c2];
                w1 = d[c2];
                w2 = d[c1];
            } else {
                xe[col] += d[c1] * d[c2] * d[c3];
                w1 = d[c2] * d[c3];
                w2 = d[c1] * d[c3];
                w3 = d[c1] * d[c2];
            }
            if (!force) continue;
            double* xfc = &xf[(size_t)col * 3 * N];
            for (int q = 0; q < N; ++q) {
                const double* srcs[3] = {dfx.data(), dfy.data(), dfz.data()};
                for (int c = 0; c < 3; ++c) {
                    const double* s = srcs[c];
                    double v;
                    if (n == 1) v = s[(size_t)c1 * N + q];
                    else if (n == 2) v = w1 * s[(size_t)c1 * N + q] + w2 * s[(size_t)c2 * N + q];
                    else v = w1 * s[(size_t)c1 * N + q] + w2 * s[(size_t)c2 * N + q] + w3 * s[(size_t)c3 * N + q];
                    xfc[3 * q + c] += v;
                }
            }
            for (int q = 0; q < 6; ++q) {
                double v;
                if (n == 1) v = dfs[(size_t)c1 * 6 + q];
                else if (n == 2) v = w1 * dfs[(size_t)c1 * 6 + q] + w2 * dfs[(size_t)c2 * 6 + q];
                else v = w1 * dfs[(size_t)c1 * 6 + q] + w2 * dfs[(size_t)c2 * 6 + q] + w3 * dfs[(size_t)c3 * 6 + q];
                xs[(size_t)col * 6 + q] += v;
            }
        }
    }
    for (int c = 0; c < F; ++c) x[e_row + c * ld] = xe[c];
    if (force)
        for (int c = 0; c < F; ++c) {
            for (int r = 0; r < 3 * N; ++r) x[f_row + r + c * ld] = xf[(size_t)c * 3 * N + r];
            for (int r = 0; r < 6; ++r) x[s_row + r + c * ld] = xs[(size_t)c * 6 + r];
        }
}

// ---------------------------------------------------------------- evaluator
struct Eval {
    pg::ModelTables mt;
    std::vector<std::vector<std::vector<pg::PotTerm>>> pot;  // [type][head] terms, coeffs x2
};

// Evaluator for one structure (polymlp_eval.cpp:24-403).
void eval_structure(const Eval& ev, const double* axis, const double* pos, const int* types, int N, double& energy,
                    double* forces, double* stress, bool omp) {
    const auto& mt = ev.mt;
    const auto& fp = mt.fp;
    const NList H = neighbor_half(axis, pos, N, fp.cutoff);
    const NList Fl = half_to_full(H, N);
    const int nfn = (int)fp.params.size();
    // per-atom adjoints (prod_sum_e, prod_sum_f)
    std::vector<std::vector<cd>> pse(N), psf(N);
    std::vector<std::vector<double>> pse_r(N), psf_r(N);
#pragma omp parallel for schedule(guided) if (omp)
    for (int i = 0; i < N; ++i) {
        const int t1 = types[i];
        const auto& tt = mt.types[t1];
        std::vector<double> fn(nfn);
        std::vector<cd> Y;
        std::vector<double> feat(tt.lin_index.size(), 0.0);
        if (fp.gtinv) {
            const int K = (int)tt.full.size();
            std::vector<double> ar(tt.noconj.size(), 0.0), ai(tt.noconj.size(), 0.0);
            for (int k = Fl.off[i]; k < Fl.off[i + 1]; ++k) {
                const int j = Fl.nb[k];
                const double dx = -Fl.d[3 * k], dy = -Fl.d[3 * k + 1], dz = -Fl.d[3 * k + 2];
                const double dis = std::sqrt(dx * dx + dy * dy + dz * dz);
                if (dis >= fp.cutoff) continue;
                const int tp = mt.type_pairs[t1][types[j]];
                radial(dis, fp.cutoff, fp, mt.tp_to_n[tp], fn.data());
                ylm_only(dx, dy, dz, fp.maxl, Y);
                for (size_t q = 0; q < tt.noconj.size(); ++q) {
                    const auto& e = tt.noconj[q];
                    if (e.tp != tp) continue;
                    const double f = fn[e.n_id];
                    if (f < 1e-20) continue;
                    const cd v = f * Y[e.ylm_key];
                    ar[q] += v.real();
                    ai[q] += v.imag();
                }
            }
            std::vector<cd> a(K, cd());
            for (size_t q = 0; q < tt.noconj.size(); ++q) {
                const auto& e = tt.noconj[q];
                a[e.ilocal_id] = cd(ar[q], ai[q]);
                a[e.ilocal_conj_id] = cd(e.cc * ar[q], -e.cc * ai[q]);
            }
            for (size_t f = 0; f < feat.size(); ++f) {
                double v = 0.0;
                for (const auto& s : tt.value_terms[f]) v += s.coeff * product_real(s.ids, a);
                feat[f] = v;
            }
            std::vector<double> pf(tt.prod_features.size());
            for (size_t q = 0; q < pf.size(); ++q) pf[q] = product<double>(tt.prod_features[q], feat);
            std::vector<cd> pd(tt.prod_deriv.size());
            for (size_t q = 0; q < pd.size(); ++q) pd[q] = product<cd>(tt.prod_deriv[q], a);
            const auto& terms = ev.pot[t1];
            pse[i].assign(terms.size(), cd());
            psf[i].assign(terms.size(), cd());
            for (size_t h = 0; h < terms.size(); ++h) {
                double er = 0, ei = 0, fr = 0, fi = 0;
                for (const auto& pt : terms[h]) {
                    const double fv = pf[pt.prod_features_id];
                    const double se = fv * pt.coeff_e, sf = fv * pt.coeff_f;
                    const cd dv = pd[pt.prod_id];
                    er += dv.real() * se;
                    ei += dv.imag() * se;
                    fr += dv.real() * sf;
                    fi += dv.imag() * sf;
                }
                pse[i][h] = cd(er, ei);
                psf[i][h] = cd(fr, fi);
            }
        } else {
            std::vector<double> antp(tt.ntp.size(), 0.0);
            for (int k = Fl.off[i]; k < Fl.off[i + 1]; ++k) {
                const int j = Fl.nb[k];
                const double dx = -Fl.d[3 * k], dy = -Fl.d[3 * k + 1], dz = -Fl.d[3 * k + 2];
                const double dis = std::sqrt(dx * dx + dy * dy + dz * dz);
                if (dis >= fp.cutoff) continue;
                const int tp = mt.type_pairs[t1][types[j]];
                radial(dis, fp.cutoff, fp, mt.tp_to_n[tp], fn.data());
                for (const auto& e : tt.ntp)
                    if (e.tp == tp) antp[e.ilocal_id] += fn[e.n_id];
            }
            for (size_t f = 0; f < feat.size(); ++f) feat[f] = antp[tt.value_terms[f][0].ids[0]];
            std::vector<double> pf(tt.prod_features.size());
            for (size_t q = 0; q < pf.size(); ++q) pf[q] = product<double>(tt.prod_features[q], feat);
            const auto& terms = ev.pot[t1];
            pse_r[i].assign(terms.size(), 0.0);
            psf_r[i].assign(terms.size(), 0.0);
            for (size_t h = 0; h < terms.size(); ++h) {
                double se = 0, sf = 0;
                for (const auto& pt : terms[h]) {
                    const double v = pf[pt.prod_features_id];
                    se += pt.coeff_e * v;
                    sf += pt.coeff_f * v;
                }
                pse_r[i][h] = 0.5 * se;
                psf_r[i][h] = 0.5 * sf;
            }
        }
    }
    // pair loop over the half list
    std::vector<std::vector<double>> ea(N), fxa(N), fya(N), fza(N);
    for (int i = 0; i < N; ++i) {
        const int m = H.off[i + 1] - H.off[i];
        ea[i].assign(m, 0.0);
        fxa[i].assign(m, 0.0);
        fya[i].assign(m, 0.0);
        fza[i].assign(m, 0.0);
    }
#pragma omp parallel for schedule(guided) if (omp)
    for (int i = 0; i < N; ++i) {
        const int t1 = types[i];
        const auto& tt = mt.types[t1];
        std::vector<double> fn(nfn), fnd(nfn);
        std::vector<cd> Y, Yx, Yy, Yz;
        for (int k = H.off[i]; k < H.off[i + 1]; ++k) {
            const int jj = k - H.off[i];
            const int j = H.nb[k];
            const double dx = -H.d[3 * k], dy = -H.d[3 * k + 1], dz = -H.d[3 * k + 2];
            const double dis = std::sqrt(dx * dx + dy * dy + dz * dz);
            if (dis >= fp.cutoff) continue;
            const int tp = mt.type_pairs[t1][types[j]];
            radial_d(dis, fp.cutoff, fp, mt.tp_to_n[tp], fn.data(), fnd.data());
            if (fp.gtinv) {
                ylm_deriv(dis, dx, dy, dz, fp.maxl, Y, Yx, Yy, Yz);
                double e = 0, fx = 0, fy = 0, fz = 0;
                for (const auto& a : tt.noconj) {
                    if (a.tp != tp) continue;
                    const double f = fn[a.n_id];
                    if (f < 1e-20) continue;
                    const cd val = f * Y[a.ylm_key];
                    const cd d1 = fnd[a.n_id] * Y[a.ylm_key] / dis;
                    const cd vx = -(d1 * dx + f * Yx[a.ylm_key]);
                    const cd vy = -(d1 * dy + f * Yy[a.ylm_key]);
                    const cd vz = -(d1 * dz + f * Yz[a.ylm_key]);
                    const cd se = pse[i][a.ilocal_noconj_id] + pse[j][a.jlocal_noconj_id] * a.sign_j;
                    const cd sf = psf[i][a.ilocal_noconj_id] + psf[j][a.jlocal_noconj_id] * a.sign_j;
                    const double factor = (a.m == 0) ? 0.5 : 1.0;
                    const cd sse = se * factor, ssf = sf * factor;
                    e += prod_real(val, sse);
                    fx += prod_real(vx, ssf);
                    fy += prod_real(vy, ssf);
                    fz += prod_real(vz, ssf);
                }
                ea[i][jj] = e;
                fxa[i][jj] = fx;
                fya[i][jj] = fy;
                fza[i][jj] = fz;
            } else {
                double e = 0, f = 0;
                for (const auto& a : tt.ntp) {
                    if (a.tp != tp) continue;
                    e += fn[a.n_id] * (pse_r[i][a.ilocal_id] + pse_r[j][a.jlocal_id]);
                    f += fnd[a.n_id] * (psf_r[i][a.ilocal_id] + psf_r[j][a.jlocal_id]);
                }
                f *= -1.0 / dis;
                ea[i][jj] = e;
                fxa[i][jj] = f * dx;
                fya[i][jj] = f * dy;
                fza[i][jj] = f * dz;
            }
        }
    }
    // collect_properties (polymlp_eval.cpp:293-335)
    energy = 0.0;
    for (int i = 0; i < 3 * N; ++i) forces[i] = 0.0;
    for (int q = 0; q < 6; ++q) stress[q] = 0.0;
    for (int i = 0; i < N; ++i)
        for (int k = H.off[i]; k < H.off[i + 1]; ++k) {
            const int jj = k - H.off[i];
            const int j = H.nb[k];
            const double dx = -H.d[3 * k], dy = -H.d[3 * k + 1], dz = -H.d[3 * k + 2];
            const double dis = std::sqrt(dx * dx + dy * dy + dz * dz);
            if (dis >= fp.cutoff) continue;
            energy += ea[i][jj];
            const double fx = fxa[i][jj], fy = fya[i][jj], fz = fza[i][jj];
            forces[3 * i] += fx;
            forces[3 * i + 1] += fy;
            forces[3 * i + 2] += fz;
            forces[3 * j] -= fx;
            forces[3 * j + 1] -= fy;
            forces[3 * j + 2] -= fz;
            stress[0] += dx * fx;
            stress[1] += dy * fy;
            stress[2] += dz * fz;
            stress[3] += dx * fy;
            stress[4] += dy * fz;
            stress[5] += dz * fx;
        }
}

std::vector<int64_t> atom_offsets(const pg_structures* st) {
    std::vector<int64_t> off(st->n_st + 1, 0);
    for (int s = 0; s < st->n_st; ++s) off[s + 1] = off[s] + st->n_atoms[s];
    return off;
}

}  // namespace

extern "C" {

int or_last_error(char* buf, size_t len) {
    if (len) {
        std::strncpy(buf, g_err.c_str(), len - 1);
        buf[len - 1] = 0;
    }
    return 0;
}

int or_n_features(const pg_feature_params* p, int* n) {
    return guarded([&] { *n = Model(p).mt.n_features; });
}

int or_features_x(const pg_feature_params* p, const pg_structures* st, const int64_t* e_row, const int64_t* f_row,
                  const int64_t* s_row, double* x, int64_t ld, int n_threads) {
    return guarded([&] {
        const Model m(p);
        const auto off = atom_offsets(st);
        std::string err;
        const int nt = n_threads > 0 ? n_threads : omp_get_max_threads();
#pragma omp parallel for schedule(guided, 1) num_threads(nt)
        for (int s = 0; s < st->n_st; ++s) {
            try {
                structure_rows(m.mt, st->axis + 9 * (size_t)s, st->positions + 3 * off[s], st->types + off[s],
                               st->n_atoms[s], f_row[s] >= 0, x, ld, e_row[s], f_row[s], s_row[s]);
            } catch (const std::exception& e) {
#pragma omp critical
                err = e.what();
            }
        }
        if (!err.empty()) throw std::runtime_error(err);
    });
}

int or_eval(const pg_feature_params* p, const double* coeffs, int n_coeffs, const pg_structures* st, double* energy,
            double* forces, double* stress, int n_threads) {
    return guarded([&] {
        Eval ev;
        ev.mt = pg::build_model_tables(pg::feature_params_from_abi(p));
        std::vector<double> c2(coeffs, coeffs + n_coeffs);
        for (auto& c : c2) c *= 2.0;  // PolymlpEval stores 2 * coeffs (polymlp_eval.cpp:17)
        ev.pot = pg::build_potential_terms(ev.mt, c2);
        const auto off = atom_offsets(st);
        if (n_threads > 0) omp_set_num_threads(n_threads);
        for (int s = 0; s < st->n_st; ++s)
            eval_structure(ev, st->axis + 9 * (size_t)s, st->positions + 3 * off[s], st->types + off[s],
                           st->n_atoms[s], energy[s], forces + 3 * off[s], stress + 6 * s, n_threads != 1);
    });
}

int or_neighbor_list(const pg_structures* st, int s, double cutoff, int half, int64_t* n_entries, int* offsets,
                     int* neighbors, double* diffs) {
    return guarded([&] {
        const auto off = atom_offsets(st);
        const NList L = half ? neighbor_half(st->axis + 9 * (size_t)s, st->positions + 3 * off[s], st->n_atoms[s], cutoff)
                             : neighbor_full(st->axis + 9 * (size_t)s, st->positions + 3 * off[s], st->n_atoms[s], cutoff);
        *n_entries = (int64_t)L.nb.size();
        if (!offsets) return;
        std::memcpy(offsets, L.off.data(), L.off.size() * sizeof(int));
        std::memcpy(neighbors, L.nb.data(), L.nb.size() * sizeof(int));
        std::memcpy(diffs, L.d.data(), L.d.size() * sizeof(double));
    });
}

int or_translations(const pg_structures* st, int s, double cutoff, int* n_trans, double* trans,
                    double* positions_rev) {
    return guarded([&] {
        const auto off = atom_offsets(st);
        const auto ct = pg::cell_translations(st->axis + 9 * (size_t)s, st->positions + 3 * off[s], st->n_atoms[s], cutoff);
        *n_trans = (int)ct.trans.size();
        if (trans)
            for (size_t k = 0; k < ct.trans.size(); ++k)
                for (int c = 0; c < 3; ++c) trans[3 * k + c] = ct.trans[k][c];
        if (positions_rev)
            for (size_t i = 0; i < ct.pos.size(); ++i)
                for (int c = 0; c < 3; ++c) positions_rev[3 * i + c] = ct.pos[i][c];
    });
}

int or_fn(double dis, double cutoff, int n_fn, const double* params, double* fn, double* fn_d) {
    return guarded([&] {
        pg::FeatureParams fp;
        std::vector<int> ns;
        for (int n = 0; n < n_fn; ++n) {
            fp.params.push_back({params[2 * n], params[2 * n + 1]});
            ns.push_back(n);
        }
        radial_d(dis, cutoff, fp, ns, fn, fn_d);
    });
}

int or_ylm(double r, double x, double y, double z, int lmax, double* ylm, double* ylm_dx, double* ylm_dy,
           double* ylm_dz) {
    return guarded([&] {
        std::vector<cd> Y, Yx, Yy, Yz;
        ylm_deriv(r, x, y, z, lmax, Y, Yx, Yy, Yz);
        for (size_t k = 0; k < Y.size(); ++k) {
            ylm[2 * k] = Y[k].real();
            ylm[2 * k + 1] = Y[k].imag();
            ylm_dx[2 * k] = Yx[k].real();
            ylm_dx[2 * k + 1] = Yx[k].imag();
            ylm_dy[2 * k] = Yy[k].real();
            ylm_dy[2 * k + 1] = Yy[k].imag();
            ylm_dz[2 * k] = Yz[k].real();
            ylm_dz[2 * k + 1] = Yz[k].imag();
        }
    });
}

}  // extern "C"

// ---------------------------------------------------------------- PolymlpAPI surface
// The per-type steps of PolymlpAPI on given order parameters, for the
// reference's own unit tests (tests/test_cxx/test_polymlp_api*.py).
namespace {

std::vector<cd> complex_in(const double* a, size_t n) {
    std::vector<cd> v(n);
    for (size_t i = 0; i < n; ++i) v[i] = cd(a[2 * i], a[2 * i + 1]);
    return v;
}

const pg::TypeTables& type_tables(const pg::ModelTables& mt, int type) {
    if (type < 0 || type >= (int)mt.types.size()) throw std::runtime_error("type out of range");
    return mt.types[type];
}

}  // namespace

int or_api_sizes(const pg_feature_params* p, int type, int* sizes) {
    return guarded([&] {
        const Model m(p);
        const auto& tt = type_tables(m.mt, type);
        sizes[0] = (int)tt.full.size();
        sizes[1] = (int)tt.noconj.size();
        sizes[2] = (int)tt.ntp.size();
        sizes[3] = (int)tt.lin_index.size();
        sizes[4] = (int)(m.mt.fp.gtinv ? tt.noconj.size() : tt.ntp.size());
    });
}

// m of each no-conjugate a_nlm entry, in the input order of or_api_conjugate
int or_api_noconj_m(const pg_feature_params* p, int type, int* m) {
    return guarded([&] {
        const Model mo(p);
        const auto& tt = type_tables(mo.mt, type);
        for (size_t q = 0; q < tt.noconj.size(); ++q) m[q] = tt.noconj[q].m;
    });
}

// compute_anlmtp_conjugate (polymlp_api.cpp:62-80)
int or_api_conjugate(const pg_feature_params* p, int type, const double* re, const double* im, double* a) {
    return guarded([&] {
        const Model m(p);
        const auto& tt = type_tables(m.mt, type);
        std::vector<cd> out(tt.full.size(), cd());
        for (size_t q = 0; q < tt.noconj.size(); ++q) {
            const auto& e = tt.noconj[q];
            out[e.ilocal_id] = cd(re[q], im[q]);
            out[e.ilocal_conj_id] = cd(e.cc * re[q], -e.cc * im[q]);
        }
        for (size_t i = 0; i < out.size(); ++i) {
            a[2 * i] = out[i].real();
            a[2 * i + 1] = out[i].imag();
        }
    });
}

// Features::compute_features (polymlp_features.cpp:155-206)
int or_api_features(const pg_feature_params* p, int type, const double* a, double* out) {
    return guarded([&] {
        const Model m(p);
        const auto& tt = type_tables(m.mt, type);
        if (m.mt.fp.gtinv) {
            const auto av = complex_in(a, tt.full.size());
            for (size_t f = 0; f < tt.lin_index.size(); ++f) {
                double v = 0.0;
                for (const auto& s : tt.value_terms[f]) v += s.coeff * product_real(s.ids, av);
                out[f] = v;
            }
        } else {
            for (size_t f = 0; f < tt.lin_index.size(); ++f) out[f] = a[tt.value_terms[f][0].ids[0]];
        }
    });
}

// Features::compute_features_deriv (polymlp_features.cpp:208-248), gtinv
int or_api_features_deriv(const pg_feature_params* p, int type, const double* a, const double* dax,
                          const double* day, const double* daz, const double* das, int n_col, double* ox,
                          double* oy, double* oz, double* os) {
    return guarded([&] {
        const Model m(p);
        if (!m.mt.fp.gtinv) throw std::runtime_error("feature derivatives from a_nlm need a gtinv model");
        const auto& tt = type_tables(m.mt, type);
        const size_t K = tt.full.size(), nl = tt.lin_index.size();
        const auto av = complex_in(a, K);
        const auto vx = complex_in(dax, K * n_col), vy = complex_in(day, K * n_col), vz = complex_in(daz, K * n_col);
        const auto vs = complex_in(das, K * 6);
        std::fill(ox, ox + nl * n_col, 0.0);
        std::fill(oy, oy + nl * n_col, 0.0);
        std::fill(oz, oz + nl * n_col, 0.0);
        std::fill(os, os + nl * 6, 0.0);
        for (size_t f = 0; f < nl; ++f)
            for (const auto& s : tt.deriv_terms[f]) {
                const cd val = s.coeff * product<cd>(s.rest, av);
                const size_t h = (size_t)s.head;
                for (int q = 0; q < n_col; ++q) {
                    ox[f * n_col + q] += prod_real(val, vx[h * n_col + q]);
                    oy[f * n_col + q] += prod_real(val, vy[h * n_col + q]);
                    oz[f * n_col + q] += prod_real(val, vz[h * n_col + q]);
                }
                for (int q = 0; q < 6; ++q) os[f * 6 + q] += prod_real(val, vs[h * 6 + q]);
            }
    });
}

// Potential::compute_sum_of_prod_anlmtp / _antp (polymlp_potential.cpp:203-295);
// coefficients as the reference's parser returns them (twice the stored ones)
int or_api_sum_of_prod(const pg_feature_params* p, const double* coeffs, int n_coeffs, int type, const double* a,
                       double* pe, double* pf) {
    return guarded([&] {
        const Model m(p);
        const auto& tt = type_tables(m.mt, type);
        const auto terms = pg::build_potential_terms(m.mt, std::vector<double>(coeffs, coeffs + n_coeffs));
        const auto& heads = terms[type];
        std::vector<double> feat(tt.lin_index.size());
        if (or_api_features(p, type, a, feat.data()) != 0) throw std::runtime_error("feature values failed");
        std::vector<double> pfv(tt.prod_features.size());
        for (size_t q = 0; q < pfv.size(); ++q) pfv[q] = product<double>(tt.prod_features[q], feat);
        if (m.mt.fp.gtinv) {
            const auto av = complex_in(a, tt.full.size());
            std::vector<cd> pd(tt.prod_deriv.size());
            for (size_t q = 0; q < pd.size(); ++q) pd[q] = product<cd>(tt.prod_deriv[q], av);
            for (size_t h = 0; h < heads.size(); ++h) {
                cd se, sf;
                for (const auto& pt : heads[h]) {
                    se += pd[pt.prod_id] * (pfv[pt.prod_features_id] * pt.coeff_e);
                    sf += pd[pt.prod_id] * (pfv[pt.prod_features_id] * pt.coeff_f);
                }
                pe[2 * h] = se.real();
                pe[2 * h + 1] = se.imag();
                pf[2 * h] = sf.real();
                pf[2 * h + 1] = sf.imag();
            }
        } else {
            std::vector<double> av(a, a + tt.ntp.size());
            std::vector<double> pd(tt.prod_deriv.size());
            for (size_t q = 0; q < pd.size(); ++q) pd[q] = product<double>(tt.prod_deriv[q], av);
            for (size_t h = 0; h < heads.size(); ++h) {
                double se = 0.0, sf = 0.0;
                for (const auto& pt : heads[h]) {
                    const double v = pfv[pt.prod_features_id] * pd[pt.prod_id];
                    se += pt.coeff_e * v;
                    sf += pt.coeff_f * v;
                }
                pe[h] = 0.5 * se;
                pf[h] = 0.5 * sf;
            }
        }
    });
}
