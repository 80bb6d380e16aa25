// Host-side model tables: see model_tables.h for the reference files whose
// setup this restates.  Every ordering rule that decides a column of X or a
// local index of a_nlm is kept as in the reference; merge order inside a
// feature (an unordered_map in the reference) only changes summation order.
#include "model_tables.h"

#include <algorithm>
#include <set>
#include <stdexcept>
#include <utility>

namespace pg {
namespace {

std::vector<int> erase_one(const std::vector<int>& v, size_t idx) {
    std::vector<int> out;
    out.reserve(v.size() ? v.size() - 1 : 0);
    for (size_t i = 0; i < v.size(); ++i)
        if (i != idx) out.push_back(v[i]);
    std::sort(out.begin(), out.end());
    return out;
}

std::vector<int> sorted_intersection(std::vector<int> a, std::vector<int> b) {
    std::sort(a.begin(), a.end());
    std::sort(b.begin(), b.end());
    std::vector<int> c;
    std::set_intersection(a.begin(), a.end(), b.begin(), b.end(), std::back_inserter(c));
    return c;
}

// True if every type pair in tps contains type t (polymlp_model_params_gtinv.cpp:10).
bool type_in_all_pairs(const std::vector<int>& tps, const std::vector<std::vector<int>>& type_pairs,
                       int t) {
    const auto& row = type_pairs[t];
    for (int tp : tps)
        if (std::find(row.begin(), row.end(), tp) == row.end()) return false;
    return true;
}

// All sequences of length r over [0, n) in lexicographic order.
// Keys ascending, each with the sum of its values in the order given (as an
// ordered map's operator[] += would give).
template <typename K>
std::vector<std::pair<K, double>> merge_keys(std::vector<std::pair<K, double>> v) {
    std::stable_sort(v.begin(), v.end(), [](const auto& a, const auto& b) { return a.first < b.first; });
    std::vector<std::pair<K, double>> out;
    for (auto& e : v) {
        if (out.empty() || out.back().first != e.first) out.push_back({std::move(e.first), 0.0});
        out.back().second += e.second;
    }
    return out;
}

// Up to six ints, ordered and compared as a std::vector<int> of them would be
// (lexicographically, a prefix first): the keys of one feature term.
struct SmallKey {
    static constexpr size_t kCap = 6;
    std::array<int, kCap> v{};
    int n = 0;
    void push(int x) { v[n++] = x; }
    void sort() {  // insertion sort: at most six values
        for (int i = 1; i < n; ++i) {
            const int x = v[i];
            int j = i - 1;
            for (; j >= 0 && v[j] > x; --j) v[j + 1] = v[j];
            v[j + 1] = x;
        }
    }
    SmallKey erase(int i) const {
        SmallKey k;
        for (int j = 0; j < n; ++j)
            if (j != i) k.push(v[j]);
        return k;
    }
    std::vector<int> vec() const { return std::vector<int>(v.begin(), v.begin() + n); }
    bool operator<(const SmallKey& o) const {
        return std::lexicographical_compare(v.begin(), v.begin() + n, o.v.begin(), o.v.begin() + o.n);
    }
    bool operator==(const SmallKey& o) const { return n == o.n && std::equal(v.begin(), v.begin() + n, o.v.begin()); }
    bool operator!=(const SmallKey& o) const { return !(*this == o); }
};

// Ascending distinct keys (as an ordered set's iteration).
std::vector<std::vector<int>> sorted_unique(std::vector<std::vector<int>> v) {
    std::sort(v.begin(), v.end());
    v.erase(std::unique(v.begin(), v.end()), v.end());
    return v;
}

void all_sequences(int n, int r, std::vector<int>& cur, std::vector<std::vector<int>>& out) {
    if ((int)cur.size() == r) {
        out.push_back(cur);
        return;
    }
    for (int i = 0; i < n; ++i) {
        cur.push_back(i);
        all_sequences(n, r, cur, out);
        cur.pop_back();
    }
}

struct Builder {
    const FeatureParams& fp;
    ModelTables mt;
    int n_fn = 0;
    std::vector<std::vector<int>> n_to_tp;
    std::vector<std::vector<int>> tpn_to_n_id;
    // (n, lm, tp) -> global and (global, type) -> local, dense (-1: none)
    std::vector<int> nlmtp_global, global_local;
    std::vector<int> global_to_global_conj;

    int& nlmtp_to_global(int n, int lm, int tp) {
        return nlmtp_global[((size_t)n * mt.n_lm + lm) * mt.n_type_pairs + tp];
    }
    int nlmtp_at(int n, int lm, int tp) {
        if (n < 0 || n >= n_fn || lm < 0 || lm >= mt.n_lm || tp < 0 || tp >= mt.n_type_pairs ||
            nlmtp_to_global(n, lm, tp) < 0)
            throw std::runtime_error("internal: no order parameter for (n, lm, tp)");
        return nlmtp_to_global(n, lm, tp);
    }
    int& global_to_local(int g, int t) { return global_local[(size_t)g * fp.n_type + t]; }
    int local_at(int g, int t) {
        if (g < 0 || (size_t)g * fp.n_type >= global_local.size() || global_to_local(g, t) < 0)
            throw std::runtime_error("internal: no local index for (global, type)");
        return global_to_local(g, t);
    }
    std::vector<std::vector<int>> comb1_indices, comb2_indices, comb3_indices;

    explicit Builder(const FeatureParams& f) : fp(f) { mt.fp = f; }

    void type_pairs() {
        const int nt = fp.n_type;
        mt.type_pairs.assign(nt, std::vector<int>(nt, 0));
        int tp = 0;
        for (int i = 0; i < nt; ++i)
            for (int j = i; j < nt; ++j) {
                mt.type_pairs[i][j] = mt.type_pairs[j][i] = tp;
                mt.tp_to_types.push_back({i, j});
                mt.tp_to_n.push_back(fp.cond[i][j]);
                ++tp;
            }
        mt.n_type_pairs = tp;
        n_fn = (int)fp.params.size();
        n_to_tp.assign(n_fn, {});
        tpn_to_n_id.assign(tp, std::vector<int>(n_fn, 0));
        for (int t = 0; t < tp; ++t) {
            int id = 0;
            for (int n : mt.tp_to_n[t]) {
                if (n < 0 || n >= n_fn) throw std::runtime_error("pair_params_conditional index out of range");
                n_to_tp[n].push_back(t);
                tpn_to_n_id[t][n] = id++;
            }
        }
    }

    // polymlp_mapping.cpp:83-137 (pair)
    void pair_maps() {
        mt.types.assign(fp.n_type, TypeTables());
        std::vector<Ntp> global;
        int gid = 0;
        for (int tp = 0; tp < mt.n_type_pairs; ++tp)
            for (int n : mt.tp_to_n[tp]) {
                Ntp a;
                a.n = n;
                a.n_id = tpn_to_n_id[tp][n];
                a.tp = tp;
                a.global_id = gid++;
                global.push_back(a);
            }
        global_local.assign(global.size() * fp.n_type, -1);
        for (const auto& a : global) {
            const int t1 = mt.tp_to_types[a.tp][0], t2 = mt.tp_to_types[a.tp][1];
            const int l1 = (int)mt.types[t1].ntp.size(), l2 = (int)mt.types[t2].ntp.size();
            Ntp b = a;
            b.ilocal_id = l1;
            b.jlocal_id = l2;
            mt.types[t1].ntp.push_back(b);
            global_to_local(a.global_id, t1) = l1;
            if (t1 != t2) {
                Ntp c = a;
                c.ilocal_id = l2;
                c.jlocal_id = l1;
                mt.types[t2].ntp.push_back(c);
                global_to_local(a.global_id, t2) = l2;
            }
        }
        // linear features: one per ntp, in global ntp order (polymlp_features_utils.cpp:25)
        mt.n_linear = (int)global.size();
        comb1_indices.assign(fp.n_type, {});
        for (const auto& a : global)
            for (int t = 0; t < fp.n_type; ++t)
                if (type_in_all_pairs({a.tp}, mt.type_pairs, t)) comb1_indices[t].push_back(a.global_id);
        for (const auto& a : global) {
            const int t1 = mt.tp_to_types[a.tp][0], t2 = mt.tp_to_types[a.tp][1];
            for (int q = 0; q < (t1 == t2 ? 1 : 2); ++q) {
                const int t = q == 0 ? t1 : t2;
                auto& tt = mt.types[t];
                const int loc = local_at(a.global_id, t);
                tt.value_terms.push_back({Term{1.0, {loc}}});
                tt.deriv_terms.push_back({DerivTerm{1.0, loc, {}}});
                tt.feature_order.push_back(1);
            }
        }
        // polynomial combos (polymlp_model_params_polynomial.cpp:28-48,108-164)
        if (fp.model_type > 2) throw std::runtime_error("Polymlp: Model type error (pair features need model_type <= 2).");
        if (fp.maxp > 3) throw std::runtime_error("Polymlp: maxp must be smaller than or equal to 3.");
        std::vector<int> iarray;
        if (fp.model_type == 2)
            for (int n = 0; n < mt.n_linear; ++n) iarray.push_back(n);
        comb2_indices.assign(fp.n_type, {});
        comb3_indices.assign(fp.n_type, {});
        if (fp.model_type > 1) {
            auto append = [&](const std::vector<int>& tps, const std::vector<int>& comb,
                              std::vector<std::vector<int>>& target,
                              std::vector<std::vector<int>>& target_idx) {
                bool match = false;
                const int ic = (int)target.size();
                for (int t = 0; t < fp.n_type; ++t)
                    if (type_in_all_pairs(tps, mt.type_pairs, t)) {
                        target_idx[t].push_back(ic);
                        match = true;
                    }
                if (match) target.push_back(comb);
            };
            if (fp.maxp > 1)
                for (size_t i1 = 0; i1 < iarray.size(); ++i1)
                    for (size_t i2 = 0; i2 <= i1; ++i2)
                        append({global[iarray[i1]].tp, global[iarray[i2]].tp}, {iarray[i2], iarray[i1]},
                               mt.comb2, comb2_indices);
            if (fp.maxp > 2)
                for (size_t i1 = 0; i1 < iarray.size(); ++i1)
                    for (size_t i2 = 0; i2 <= i1; ++i2)
                        for (size_t i3 = 0; i3 <= i2; ++i3)
                            append({global[iarray[i1]].tp, global[iarray[i2]].tp, global[iarray[i3]].tp},
                                   {iarray[i3], iarray[i2], iarray[i1]}, mt.comb3, comb3_indices);
        }
    }

    // polymlp_mapping.cpp:247-279, 139-227
    void gtinv_maps() {
        mt.types.assign(fp.n_type, TypeTables());
        struct LmAttr {
            int l, m, ylm_key;
            bool conj;
            double cc, sign_j;
        };
        std::vector<LmAttr> lm_attrs;
        for (int l = 0; l <= fp.maxl; ++l) {
            const double sign_j = (l % 2 == 0) ? 1.0 : -1.0;
            for (int m = -l; m <= l; ++m) {
                const double cc = (m % 2 == 0) ? 1.0 : -1.0;
                LmAttr a;
                a.l = l;
                a.m = m;
                a.cc = cc;
                a.sign_j = sign_j;
                if (m < 1) {
                    a.ylm_key = (l + 3) * l / 2 + m;
                    a.conj = false;
                } else {
                    a.ylm_key = (l + 3) * l / 2 - m;
                    a.conj = true;
                }
                lm_attrs.push_back(a);
            }
        }
        mt.n_lm = (int)lm_attrs.size();
        mt.n_ylm = (fp.maxl + 1) * (fp.maxl + 2) / 2;

        std::vector<Nlmtp> global;
        int gid = 0;
        nlmtp_global.assign((size_t)n_fn * mt.n_lm * mt.n_type_pairs, -1);
        for (int n = 0; n < n_fn; ++n) {
            const auto& tp_n = n_to_tp[n];
            for (int lm = 0; lm < mt.n_lm; ++lm) {
                const auto& la = lm_attrs[lm];
                const int conj_subtract = 2 * la.m * (int)tp_n.size();
                for (int tp : tp_n) {
                    Nlmtp a;
                    a.n = n;
                    a.n_id = tpn_to_n_id[tp][n];
                    a.l = la.l;
                    a.m = la.m;
                    a.lm = lm;
                    a.ylm_key = la.ylm_key;
                    a.conj = la.conj;
                    a.cc = la.cc;
                    a.sign_j = la.sign_j;
                    a.tp = tp;
                    a.global_id = gid;
                    a.global_conj_id = gid - conj_subtract;
                    nlmtp_to_global(n, lm, tp) = gid;
                    global.push_back(a);
                    ++gid;
                }
            }
        }
        global_to_global_conj.resize(global.size());
        for (const auto& a : global) global_to_global_conj[a.global_id] = a.global_conj_id;
        global_local.assign(global.size() * fp.n_type, -1);

        for (const auto& a : global) {
            const int t1 = mt.tp_to_types[a.tp][0], t2 = mt.tp_to_types[a.tp][1];
            auto& T1 = mt.types[t1];
            auto& T2 = mt.types[t2];
            const int l1 = (int)T1.full.size(), l2 = (int)T2.full.size();
            const int nc1 = (int)T1.noconj.size(), nc2 = (int)T2.noconj.size();
            Nlmtp b = a;
            b.ilocal_id = l1;
            b.ilocal_noconj_id = nc1;
            b.jlocal_noconj_id = nc2;
            T1.full.push_back(b);
            if (!a.conj) T1.noconj.push_back(b);
            global_to_local(a.global_id, t1) = l1;
            if (t1 != t2) {
                Nlmtp c = a;
                c.ilocal_id = l2;
                c.ilocal_noconj_id = nc2;
                c.jlocal_noconj_id = nc1;
                T2.full.push_back(c);
                if (!a.conj) T2.noconj.push_back(c);
                global_to_local(a.global_id, t2) = l2;
            }
        }
        for (int t = 0; t < fp.n_type; ++t) {
            for (auto& a : mt.types[t].full) a.ilocal_conj_id = local_at(a.global_conj_id, t);
            for (auto& a : mt.types[t].noconj) a.ilocal_conj_id = local_at(a.global_conj_id, t);
        }
    }

    // polymlp_model_params_gtinv.cpp:33-151
    void gtinv_linear_terms() {
        if (fp.l_comb.empty()) throw std::runtime_error("gtinv features need a non-empty l_comb");
        const int gtinv_order = (int)fp.l_comb.back().size();
        const int ntp = mt.n_type_pairs;
        mt.tp_combs.assign(gtinv_order + 1, {});
        for (int order = 1; order <= gtinv_order; ++order) {
            std::vector<std::vector<int>> perm;
            std::vector<int> cur;
            all_sequences(ntp, order, cur, perm);
            for (const auto& p : perm)
                for (int t = 0; t < fp.n_type; ++t)
                    if (type_in_all_pairs(p, mt.type_pairs, t)) {
                        mt.tp_combs[order].push_back(p);
                        break;
                    }
        }
        std::vector<std::vector<std::vector<int>>> nonzero_n(gtinv_order + 1);
        for (int order = 1; order <= gtinv_order; ++order)
            for (const auto& comb : mt.tp_combs[order]) {
                std::vector<int> inter;
                for (size_t k = 0; k < comb.size(); ++k)
                    inter = (k == 0) ? mt.tp_to_n[comb[k]] : sorted_intersection(inter, mt.tp_to_n[comb[k]]);
                nonzero_n[order].push_back(inter);
            }
        std::vector<std::vector<LinearTerm>> by_n(n_fn);
        for (size_t lmc = 0; lmc < fp.l_comb.size(); ++lmc) {
            const auto& lc = fp.l_comb[lmc];
            const int order = (int)lc.size();
            if (order > gtinv_order) throw std::runtime_error("l_comb order exceeds gtinv order");
            const auto& ref = mt.tp_combs[order];
            std::set<std::vector<std::pair<int, int>>> uniq;
            for (const auto& comb : ref) {
                std::vector<std::pair<int, int>> v;
                for (size_t j = 0; j < comb.size(); ++j) v.push_back({lc[j], comb[j]});
                std::sort(v.begin(), v.end());
                uniq.insert(v);
            }
            for (const auto& lt : uniq) {
                std::vector<int> comb;
                for (const auto& p : lt) comb.push_back(p.second);
                const int comb_id = (int)(std::find(ref.begin(), ref.end(), comb) - ref.begin());
                std::vector<int> t1a;
                for (int t = 0; t < fp.n_type; ++t)
                    if (type_in_all_pairs(comb, mt.type_pairs, t)) t1a.push_back(t);
                for (int n : nonzero_n[order][comb_id]) {
                    LinearTerm lt1;
                    lt1.n = n;
                    lt1.lm_comb_id = (int)lmc;
                    lt1.tp_comb_id = comb_id;
                    lt1.order = order;
                    lt1.type1 = t1a;
                    by_n[n].push_back(lt1);
                }
            }
        }
        for (const auto& v : by_n)
            for (const auto& lt1 : v) mt.linear_terms.push_back(lt1);
        mt.n_linear = (int)mt.linear_terms.size();
    }

    // polymlp_model_params_polynomial.cpp:51-82,167-268
    void gtinv_polynomial_combos() {
        if (fp.model_type > 4) throw std::runtime_error("Polymlp: Model type error.");
        if (fp.maxp > 3) throw std::runtime_error("Polymlp: maxp must be smaller than or equal to 3.");
        std::vector<int> iarray;
        if (fp.model_type == 2) {
            for (int n = 0; n < mt.n_linear; ++n) iarray.push_back(n);
        } else if (fp.model_type > 2) {
            const int max_order = (fp.model_type == 3) ? 1 : 2;
            for (int n = 0; n < mt.n_linear; ++n)
                if (mt.linear_terms[n].order <= max_order) iarray.push_back(n);
        }
        comb1_indices.assign(fp.n_type, {});
        comb2_indices.assign(fp.n_type, {});
        comb3_indices.assign(fp.n_type, {});
        for (int i = 0; i < mt.n_linear; ++i)
            for (int t : mt.linear_terms[i].type1) comb1_indices[t].push_back(i);
        if (fp.model_type <= 1) return;
        auto intersect_types = [&](std::initializer_list<int> ids) {
            std::vector<int> inter;
            bool first = true;
            for (int id : ids) {
                const auto& t1 = mt.linear_terms[id].type1;
                if (first) {
                    inter = t1;
                    first = false;
                } else {
                    std::vector<int> tmp;
                    std::set_intersection(inter.begin(), inter.end(), t1.begin(), t1.end(),
                                          std::back_inserter(tmp));
                    inter = tmp;
                }
            }
            return inter;
        };
        if (fp.maxp > 1)
            for (size_t i1 = 0; i1 < iarray.size(); ++i1)
                for (size_t i2 = 0; i2 <= i1; ++i2) {
                    auto inter = intersect_types({iarray[i1], iarray[i2]});
                    if (inter.empty()) continue;
                    const int ic = (int)mt.comb2.size();
                    mt.comb2.push_back({iarray[i2], iarray[i1]});
                    for (int t : inter) comb2_indices[t].push_back(ic);
                }
        if (fp.maxp > 2)
            for (size_t i1 = 0; i1 < iarray.size(); ++i1)
                for (size_t i2 = 0; i2 <= i1; ++i2)
                    for (size_t i3 = 0; i3 <= i2; ++i3) {
                        auto inter = intersect_types({iarray[i1], iarray[i2], iarray[i3]});
                        if (inter.empty()) continue;
                        const int ic = (int)mt.comb3.size();
                        mt.comb3.push_back({iarray[i3], iarray[i2], iarray[i1]});
                        for (int t : inter) comb3_indices[t].push_back(ic);
                    }
    }


    // polymlp_features_utils.cpp:48-132: linear gtinv features of each type,
    // with the representative (id or conjugate-id) product used for values.
    void gtinv_features() {
        for (const auto& lt : mt.linear_terms) {
            const auto& tp_comb = mt.tp_combs[lt.order][lt.tp_comb_id];
            const auto& lm_list = fp.lm_array.at(lt.lm_comb_id);
            const auto& coeffs = fp.lm_coeffs.at(lt.lm_comb_id);
            if (lm_list.empty()) throw std::runtime_error("internal: an invariant without terms");
            for (int t : lt.type1) {
                // per term: its globals g1 (sorted), the conjugate's g2 (sorted),
                // the representative min(g1, g2), and their local indices
                std::vector<std::pair<SmallKey, double>> vm;
                std::vector<std::pair<std::pair<int, SmallKey>, double>> dm;
                vm.reserve(lm_list.size());
                dm.reserve(lm_list.size() * lm_list[0].size());
                auto& pd = prod_deriv_keys[t];
                for (size_t i = 0; i < lm_list.size(); ++i) {
                    if (lm_list[i].size() > SmallKey::kCap) throw std::runtime_error("gtinv order must be 1..6");
                    SmallKey g1, g2, l1, lr;
                    for (size_t k = 0; k < lm_list[i].size(); ++k) g1.push(nlmtp_at(lt.n, lm_list[i][k], tp_comb[k]));
                    g1.sort();
                    for (int k = 0; k < g1.n; ++k) g2.push(global_to_global_conj[g1.v[k]]);
                    g2.sort();
                    const SmallKey& r = (g2 < g1) ? g2 : g1;
                    for (int k = 0; k < g1.n; ++k) {
                        l1.push(local_at(g1.v[k], t));
                        lr.push(local_at(r.v[k], t));
                    }
                    vm.push_back({lr, coeffs[i]});
                    for (int k = 0; k < l1.n; ++k) dm.push_back({{l1.v[k], l1.erase(k)}, coeffs[i]});
                }
                auto& tt = mt.types[t];
                tt.feature_order.push_back((int)lm_list[0].size());
                // merge identical representative products (mapped features)
                std::vector<Term> vterms;
                for (const auto& kv : merge_keys(std::move(vm))) vterms.push_back(Term{kv.second, kv.first.vec()});
                tt.value_terms.push_back(std::move(vterms));
                // derivative terms merged by (head, rest), sorted by head then rest
                // (the rests are the erase-one keys of the feature's terms: prod_deriv
                // candidates, distinct per feature)
                std::vector<DerivTerm> dterms;
                const size_t pd0 = pd.size();
                for (const auto& kv : merge_keys(std::move(dm))) {
                    dterms.push_back(DerivTerm{kv.second, kv.first.first, kv.first.second.vec()});
                    pd.push_back(kv.first.second);
                }
                std::sort(pd.begin() + pd0, pd.end());
                pd.erase(std::unique(pd.begin() + pd0, pd.end()), pd.end());
                tt.deriv_terms.push_back(std::move(dterms));
            }
        }
    }

    // per type: the erase-one keys of every (unmerged) feature term (prod_deriv candidates)
    std::vector<std::vector<SmallKey>> prod_deriv_keys;

    void finalize_types() {
        for (int t = 0; t < fp.n_type; ++t) {
            auto& tt = mt.types[t];
            tt.lin_index = comb1_indices[t];
            std::map<int, int> map1;
            for (size_t k = 0; k < tt.lin_index.size(); ++k) {
                map1[tt.lin_index[k]] = (int)k;
                tt.poly.push_back(PolyTerm{tt.lin_index[k], {(int)k}});
            }
            for (int i : comb2_indices[t])
                tt.poly.push_back(PolyTerm{mt.n_linear + i, {map1.at(mt.comb2[i][0]), map1.at(mt.comb2[i][1])}});
            for (int i : comb3_indices[t])
                tt.poly.push_back(PolyTerm{mt.n_linear + (int)mt.comb2.size() + i,
                                           {map1.at(mt.comb3[i][0]), map1.at(mt.comb3[i][1]),
                                            map1.at(mt.comb3[i][2])}});
            // prod_deriv keys: every erase-one key of every term (features.cpp:92)
            if (fp.gtinv) {
                auto& pd = prod_deriv_keys[t];
                std::sort(pd.begin(), pd.end());
                pd.erase(std::unique(pd.begin(), pd.end()), pd.end());
                tt.prod_deriv.clear();
                for (const auto& k : pd) tt.prod_deriv.push_back(k.vec());
            } else {
                tt.prod_deriv.clear();
                if (!tt.ntp.empty()) tt.prod_deriv.push_back(std::vector<int>{});
            }
            std::vector<std::vector<int>> pf;
            for (const auto& p : tt.poly)
                for (size_t i = 0; i < p.local_ids.size(); ++i) pf.push_back(erase_one(p.local_ids, i));
            tt.prod_features = sorted_unique(std::move(pf));
            if (tt.lin_index.size() != tt.value_terms.size())
                throw std::runtime_error("internal: feature count mismatch");
        }
        mt.n_features = mt.n_linear + (int)mt.comb2.size() + (int)mt.comb3.size();
    }
};

}  // namespace

ModelTables build_model_tables(const FeatureParams& fp) {
    if (fp.n_type <= 0) throw std::runtime_error("n_type must be positive");
    if ((int)fp.cond.size() != fp.n_type) throw std::runtime_error("pair_params_conditional has wrong shape");
    Builder b(fp);
    b.type_pairs();
    b.prod_deriv_keys.assign(fp.n_type, {});
    if (fp.gtinv) {
        b.gtinv_maps();
        b.gtinv_linear_terms();
        b.gtinv_polynomial_combos();
        b.gtinv_features();
    } else {
        b.pair_maps();
    }
    b.finalize_types();
    return std::move(b.mt);
}

// polymlp_potential.cpp:47-157 restated.
std::vector<std::vector<std::vector<PotTerm>>> build_potential_terms(const ModelTables& mt,
                                                                    const std::vector<double>& pot) {
    if ((int)pot.size() != mt.n_features) throw std::runtime_error("coefficient vector has wrong length");
    std::vector<std::vector<std::vector<PotTerm>>> out(mt.fp.n_type);
    for (int t = 0; t < mt.fp.n_type; ++t) {
        const auto& tt = mt.types[t];
        std::map<std::vector<int>, int> pd_id, pf_id;
        for (size_t i = 0; i < tt.prod_deriv.size(); ++i) pd_id[tt.prod_deriv[i]] = (int)i;
        for (size_t i = 0; i < tt.prod_features.size(); ++i) pf_id[tt.prod_features[i]] = (int)i;
        // (head, prod_id, pf_id) -> (coeff_e, coeff_f)
        std::map<std::array<int, 3>, std::array<double, 2>> acc;
        for (const auto& p : tt.poly) {
            int n_prods = 0;
            for (int k : p.local_ids) n_prods += tt.feature_order[k];
            for (size_t i = 0; i < p.local_ids.size(); ++i) {
                const int head_term = p.local_ids[i];
                const int pfid = pf_id.at(erase_one(p.local_ids, i));
                // The merged derivative terms carry sum(coeff) per (head, rest),
                // which equals the reference's per-term accumulation.
                for (const auto& dt : tt.deriv_terms[head_term]) {
                    if (mt.fp.gtinv && tt.full[dt.head].conj) continue;
                    const double coeff_f = pot[p.col] * dt.coeff;
                    const double coeff_e = coeff_f / double(n_prods);
                    const int pdid = pd_id.at(dt.rest);
                    auto& a = acc[{dt.head, pdid, pfid}];
                    a[0] += coeff_e;
                    a[1] += coeff_f;
                }
            }
        }
        const int n_heads = mt.fp.gtinv ? (int)tt.noconj.size() : (int)tt.ntp.size();
        out[t].assign(n_heads, {});
        for (const auto& kv : acc) {
            int head = kv.first[0];
            if (mt.fp.gtinv) head = tt.full[head].ilocal_noconj_id;
            out[t][head].push_back(PotTerm{kv.second[0], kv.second[1], kv.first[1], kv.first[2]});
        }
        for (auto& v : out[t])
            std::sort(v.begin(), v.end(), [](const PotTerm& a, const PotTerm& b) {
                if (a.prod_id != b.prod_id) return a.prod_id < b.prod_id;
                return a.prod_features_id < b.prod_features_id;
            });
    }
    return out;
}

FeatureAttrs feature_attrs(const ModelTables& mt) {
    FeatureAttrs a;
    if (!mt.fp.gtinv) {
        // ntp attributes in global (type pair, radial) order
        for (int tp = 0; tp < mt.n_type_pairs; ++tp)
            for (int n : mt.tp_to_n[tp]) {
                a.radial_ids.push_back(n);
                a.tcomb_ids.push_back({tp});
            }
    } else {
        for (const auto& lt : mt.linear_terms) {
            a.radial_ids.push_back(lt.n);
            a.gtinv_ids.push_back(lt.lm_comb_id);
            a.tcomb_ids.push_back(mt.tp_combs[lt.order][lt.tp_comb_id]);
        }
    }
    for (const auto& c : mt.comb2) a.polynomial_ids.push_back(c);
    for (const auto& c : mt.comb3) a.polynomial_ids.push_back(c);
    return a;
}

}  // namespace pg
