// C ABI over the reference's own C++ (compiled unmodified from its sources by
// oracle/Makefile into oracle/_ref/).  Test infrastructure only: it is used to
// pin the oracle and to generate golden fixtures in a container that holds
// the reference sources.  The glue here (structure loop and row layout)
// follows PyModel (src/pypolymlp/cxx/src/compute/py_model.cpp:10-56),
// PyPropertiesFast (src/pypolymlp/cxx/src/compute/py_properties_fast.cpp:19-56)
// and PyFeaturesAttr (src/pypolymlp/cxx/src/compute/py_features_attr.cpp:11).
#include <cstring>
#include <stdexcept>
#include <string>

#include "compute/model.h"
#include "compute/neighbor_cell.h"
#include "compute/neighbor_full.h"
#include "compute/neighbor_half.h"
#include "compute/polymlp_eval.h"
#include <sstream>

#include "polymlp/polymlp_api.h"
#include "polymlp/polymlp_parse_potential.h"
#include "polymlp/polymlp_parse_potential_legacy.h"
#include "polymlp/polymlp_read_gtinv.h"
#include "polymlp_gb300.h"

namespace {

thread_local std::string g_err;

feature_params to_fp(const pg_feature_params* p) {
    feature_params fp;
    fp.n_type = p->n_type;
    fp.force = false;
    fp.params.clear();
    for (int n = 0; n < p->n_fn; ++n) fp.params.push_back({p->pair_params[2 * n], p->pair_params[2 * n + 1]});
    fp.params_conditional.assign(p->n_type, vector2i(p->n_type));
    for (int i = 0; i < p->n_type; ++i)
        for (int j = i; j < p->n_type; ++j) {
            const int k = i * p->n_type + j;
            fp.params_conditional[i][j] =
                vector1i(p->cond_values + p->cond_offsets[k], p->cond_values + p->cond_offsets[k + 1]);
        }
    fp.cutoff = p->cutoff;
    fp.pair_type = "gaussian";
    fp.feature_type = p->feature_type ? "gtinv" : "pair";
    fp.model_type = p->model_type;
    fp.maxp = p->max_p;
    fp.maxl = p->max_l;
    size_t vpos = 0;
    for (int c = 0; c < p->n_lcomb; ++c) {
        vector1i lc(p->lcomb_values + p->lcomb_offsets[c], p->lcomb_values + p->lcomb_offsets[c + 1]);
        const int order = (int)lc.size();
        vector2i lms;
        vector1d coeffs;
        for (int q = p->lmseq_offsets[c]; q < p->lmseq_offsets[c + 1]; ++q) {
            lms.emplace_back(p->lmseq_values + vpos, p->lmseq_values + vpos + order);
            vpos += order;
            coeffs.push_back(p->lm_coeffs[q]);
        }
        fp.l_comb.push_back(lc);
        fp.lm_array.push_back(lms);
        fp.lm_coeffs.push_back(coeffs);
    }
    return fp;
}

void structure(const pg_structures* st, int s, int64_t off, vector2d& axis, vector2d& pos, vector1i& types) {
    const int n = st->n_atoms[s];
    axis.assign(3, vector1d(3));
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) axis[a][b] = st->axis[(size_t)s * 9 + a * 3 + b];
    pos.assign(3, vector1d(n));
    types.assign(n, 0);
    for (int i = 0; i < n; ++i) {
        for (int c = 0; c < 3; ++c) pos[c][i] = st->positions[(off + i) * 3 + c];
        types[i] = st->types[off + i];
    }
}

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

}  // namespace

extern "C" {

int ref_last_error(char* buf, size_t len) {
    if (len) {
        std::strncpy(buf, g_err.c_str(), len - 1);
        buf[len - 1] = 0;
    }
    return 0;
}

int ref_n_features(const pg_feature_params* p, int* n) {
    return guarded([&] {
        PolymlpAPI api;
        api.set_features(to_fp(p));
        *n = api.get_n_variables();
    });
}

int ref_features_x(const pg_feature_params* p, const pg_structures* st, const int64_t* e_row,
                   const int64_t* f_row, const int64_t* s_row, double* x, int64_t ld) {
    return guarded([&] {
        const feature_params fp = to_fp(p);
        Model mod(fp);
        const int nf = mod.get_n_features();
        std::vector<int64_t> off(st->n_st + 1, 0);
        for (int s = 0; s < st->n_st; ++s) off[s + 1] = off[s] + st->n_atoms[s];
#pragma omp parallel for schedule(guided, 1)
        for (int s = 0; s < st->n_st; ++s) {
            vector2d axis, pos;
            vector1i types;
            structure(st, s, off[s], axis, pos, types);
            NeighborFull neigh(axis, pos, fp.cutoff);
            Eigen::VectorXd xe;
            Eigen::MatrixXd xf, xs;
            const bool force = f_row[s] >= 0;
            mod.run(neigh, types, force, xe, xf, xs);
            for (int c = 0; c < nf; ++c) x[e_row[s] + c * ld] = xe(c);
            if (force) {
                for (int c = 0; c < nf; ++c) {
                    for (int r = 0; r < xf.rows(); ++r) x[f_row[s] + r + c * ld] = xf(r, c);
                    for (int r = 0; r < 6; ++r) x[s_row[s] + r + c * ld] = xs(r, c);
                }
            }
        }
    });
}

int ref_eval(const pg_feature_params* p, const double* coeffs, int n_coeffs, const pg_structures* st,
             double* energy, double* forces, double* stress) {
    return guarded([&] {
        const feature_params fp = to_fp(p);
        PolymlpEval ev(fp, vector1d(coeffs, coeffs + n_coeffs));
        int64_t off = 0;
        for (int s = 0; s < st->n_st; ++s) {
            vector2d axis, pos;
            vector1i types;
            structure(st, s, off, axis, pos, types);
            NeighborHalf neigh(axis, pos, fp.cutoff, true);
            double e;
            vector2d f;
            vector1d sv;
            ev.eval(types, neigh, true, e, f, sv);
            energy[s] = e;
            for (int i = 0; i < st->n_atoms[s]; ++i)
                for (int c = 0; c < 3; ++c) forces[(off + i) * 3 + c] = f[i][c];
            for (int c = 0; c < 6; ++c) stress[s * 6 + c] = sv[c];
            off += st->n_atoms[s];
        }
    });
}

int ref_neighbor_list(const pg_structures* st, int s, double cutoff, int half, int64_t* n_entries,
                      int* offsets, int* neighbors, double* diffs) {
    return guarded([&] {
        int64_t off = 0;
        for (int q = 0; q < s; ++q) off += st->n_atoms[q];
        vector2d axis, pos;
        vector1i types;
        structure(st, s, off, axis, pos, types);
        const int n = st->n_atoms[s];
        auto fill = [&](auto& neigh) {
            int64_t total = 0;
            for (int i = 0; i < n; ++i) total += neigh.size(i);
            *n_entries = total;
            if (!offsets) return;
            int64_t k = 0;
            offsets[0] = 0;
            for (int i = 0; i < n; ++i) {
                auto [b, e] = neigh.range(i);
                for (int q = b; q < e; ++q) {
                    neighbors[k] = neigh.neighbor_atom(q);
                    neigh.diff(q, diffs[3 * k], diffs[3 * k + 1], diffs[3 * k + 2]);
                    ++k;
                }
                offsets[i + 1] = (int)k;
            }
        };
        if (half) {
            NeighborHalf nh(axis, pos, cutoff, false);
            fill(nh);
        } else {
            NeighborFull nf(axis, pos, cutoff);
            fill(nf);
        }
    });
}

int ref_translations(const pg_structures* st, int s, double cutoff, int* n_trans, double* trans,
                     double* positions_rev) {
    return guarded([&] {
        int64_t off = 0;
        for (int q = 0; q < s; ++q) off += st->n_atoms[q];
        vector2d axis, pos;
        vector1i types;
        structure(st, s, off, axis, pos, types);
        NeighborCell cell(axis, pos, cutoff);
        const auto& t = cell.get_translations();
        *n_trans = (int)t.size();
        if (trans)
            for (size_t k = 0; k < t.size(); ++k)
                for (int c = 0; c < 3; ++c) trans[3 * k + c] = t[k][c];
        if (positions_rev) {
            const auto& pr = cell.get_positions_cartesian();
            for (int i = 0; i < st->n_atoms[s]; ++i)
                for (int c = 0; c < 3; ++c) positions_rev[3 * i + c] = pr[c][i];
        }
    });
}

// Readgtinv (src/pypolymlp/cxx/src/polymlp/polymlp_read_gtinv.cpp:12): sizes[0..3] =
// n_lcomb, n_l values, n_m-combinations, n_m values.  NULL arrays query sizes.
int ref_readgtinv(int order, const int* maxl, int n_maxl, int version, int* sizes, int* lcomb_offsets,
                  int* lcomb_values, int* lmseq_offsets, int* lmseq_values, double* coeffs) {
    return guarded([&] {
        Readgtinv rg(order, vector1i(maxl, maxl + n_maxl), version);
        const auto& lc = rg.get_l_comb();
        const auto& lm = rg.get_lm_seq();
        const auto& cf = rg.get_lm_coeffs();
        int nl = 0, nm = 0, nmv = 0;
        for (size_t c = 0; c < lc.size(); ++c) {
            nl += (int)lc[c].size();
            nm += (int)lm[c].size();
            for (const auto& v : lm[c]) nmv += (int)v.size();
        }
        sizes[0] = (int)lc.size();
        sizes[1] = nl;
        sizes[2] = nm;
        sizes[3] = nmv;
        if (!lcomb_offsets) return;
        int il = 0, im = 0, imv = 0;
        lcomb_offsets[0] = 0;
        lmseq_offsets[0] = 0;
        for (size_t c = 0; c < lc.size(); ++c) {
            for (int l : lc[c]) lcomb_values[il++] = l;
            lcomb_offsets[c + 1] = il;
            for (size_t q = 0; q < lm[c].size(); ++q) {
                for (int v : lm[c][q]) lmseq_values[imv++] = v;
                coeffs[im++] = cf[c][q];
            }
            lmseq_offsets[c + 1] = im;
        }
    });
}

// FeaturesAttr::get_type_pairs (py_features_attr.cpp:19): n_type x n_type, row-major.
int ref_type_pairs(const pg_feature_params* p, int* out) {
    return guarded([&] {
        const feature_params fp = to_fp(p);
        PolymlpAPI api;
        api.set_model_parameters(fp);
        const auto& tps = api.get_maps().type_pairs;
        for (size_t a = 0; a < tps.size(); ++a)
            for (size_t b = 0; b < tps[a].size(); ++b) out[a * tps.size() + b] = tps[a][b];
    });
}

// FeaturesAttr-equivalent sizes and ids (py_features_attr.cpp:11-45).
int ref_feature_attrs(const pg_feature_params* p, int* n_linear, int* radial_ids, int* gtinv_ids,
                      int* n_tcomb_values, int* tcomb_offsets, int* tcomb_values, int* n_poly,
                      int* n_poly_values, int* poly_offsets, int* poly_values) {
    return guarded([&] {
        const feature_params fp = to_fp(p);
        PolymlpAPI api;
        api.set_model_parameters(fp);
        const auto& modelp = api.get_model_params();
        auto& maps = api.get_maps();
        vector1i rad, gt;
        vector2i tc, poly;
        if (fp.feature_type == "pair") {
            for (const auto& ntp : maps.ntp_attrs) {
                rad.push_back(ntp.n);
                tc.push_back({ntp.tp});
            }
        } else {
            const auto& lts = modelp.get_linear_terms();
            const auto& tcs = modelp.get_tp_combs();
            for (const auto& lt : lts) {
                rad.push_back(lt.n);
                gt.push_back(lt.lm_comb_id);
                tc.push_back(tcs[lt.order][lt.tp_comb_id]);
            }
        }
        for (const auto& c : modelp.get_comb2()) poly.push_back(c);
        for (const auto& c : modelp.get_comb3()) poly.push_back(c);
        int ntv = 0, npv = 0;
        for (const auto& v : tc) ntv += (int)v.size();
        for (const auto& v : poly) npv += (int)v.size();
        *n_linear = (int)rad.size();
        *n_tcomb_values = ntv;
        *n_poly = (int)poly.size();
        *n_poly_values = npv;
        if (!radial_ids) return;
        int k = 0;
        tcomb_offsets[0] = 0;
        for (size_t i = 0; i < rad.size(); ++i) {
            radial_ids[i] = rad[i];
            if (gtinv_ids) gtinv_ids[i] = gt.empty() ? -1 : gt[i];
            for (int v : tc[i]) tcomb_values[k++] = v;
            tcomb_offsets[i + 1] = k;
        }
        k = 0;
        poly_offsets[0] = 0;
        for (size_t i = 0; i < poly.size(); ++i) {
            for (int v : poly[i]) poly_values[k++] = v;
            poly_offsets[i + 1] = k;
        }
    });
}

// A polymlp.yaml (legacy = 0) or polymlp.lammps (legacy = 1) file read by the
// reference's own parsers (polymlp/polymlp_parse_potential.cpp:214-257,
// polymlp/polymlp_parse_potential_legacy.cpp), summarised as text lines
// "key v1 v2 ..." in buf: elements, cutoff, pair_type, feature_type,
// model_type, max_p, max_l, n_l_comb (the invariant tables it derived),
// params (pairs of Gaussian parameters), cond i j ids... per type pair,
// coeffs (as the parser returns them: 2 x the file's values), mass.
int ref_parse_potential(const char* file, int legacy, char* buf, size_t len) {
    return guarded([&] {
        feature_params fp;
        vector1d coeffs, mass;
        std::vector<std::string> ele;
        if (legacy)
            parse_polymlp_legacy(file, fp, coeffs, ele, mass);
        else
            parse_polymlp(file, fp, coeffs, ele, mass);
        std::ostringstream o;
        o.precision(17);
        o << "elements";
        for (const auto& e : ele) o << " " << e;
        o << "\ncutoff " << fp.cutoff << "\npair_type " << fp.pair_type << "\nfeature_type " << fp.feature_type
          << "\nmodel_type " << fp.model_type << "\nmax_p " << fp.maxp << "\nmax_l " << fp.maxl
          << "\nn_l_comb " << fp.l_comb.size() << "\nparams";
        for (const auto& p : fp.params) o << " " << p[0] << " " << p[1];
        o << "\n";
        for (size_t i = 0; i < fp.params_conditional.size(); ++i)
            for (size_t j = i; j < fp.params_conditional[i].size(); ++j) {
                o << "cond " << i << " " << j;
                for (int v : fp.params_conditional[i][j]) o << " " << v;
                o << "\n";
            }
        o << "coeffs";
        for (double c : coeffs) o << " " << c;
        o << "\nmass";
        for (double m : mass) o << " " << m;
        o << "\n";
        const std::string t = o.str();
        if (t.size() + 1 > len) throw std::runtime_error("summary buffer too small");
        std::memcpy(buf, t.c_str(), t.size() + 1);
    });
}

}  // extern "C"

// PolymlpAPI::parse_polymlp_file + compute_sum_of_prod_anlmtp
// (polymlp_api.cpp:20-32, polymlp_potential.cpp:235-289): a (interleaved re/im,
// the type's full a_nlm order) -> prod_sum_e / prod_sum_f (interleaved, *n heads).
extern "C" int ref_api_sum_of_prod(const char* file, const char* ele0, const char* ele1, int type, const double* a, int K,
                        double* pe, double* pf, int* n) {
    return guarded([&] {
        PolymlpAPI api;
        std::vector<std::string> ele{ele0, ele1};
        vector1d mass{1.0, 1.0};
        api.parse_polymlp_file(file, ele, mass);
        vector1dc av(K);
        for (int i = 0; i < K; ++i) av[i] = dc(a[2 * i], a[2 * i + 1]);
        vector1dc e, f;
        api.compute_sum_of_prod_anlmtp(av, type, e, f);
        *n = (int)e.size();
        for (size_t i = 0; i < e.size(); ++i) {
            pe[2 * i] = e[i].real();
            pe[2 * i + 1] = e[i].imag();
            pf[2 * i] = f[i].real();
            pf[2 * i + 1] = f[i].imag();
        }
    });
}
