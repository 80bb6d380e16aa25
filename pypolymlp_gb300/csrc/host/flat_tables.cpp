// Flattening of ModelTables for device upload (see flat_tables.h).
#include "flat_tables.h"

#include <algorithm>
#include <array>
#include <cmath>
#include <map>
#include <stdexcept>

namespace pg {
namespace {

FlatTerm make_term(double coeff, const std::vector<int>& ids, int conj) {
    if ((int)ids.size() > kMaxOrder) throw std::runtime_error("product order exceeds the supported maximum (6)");
    FlatTerm t{};
    t.coeff = coeff;
    t.n = (int)ids.size();
    t.conj = conj;
    for (int i = 0; i < kMaxOrder; ++i) t.ids[i] = i < t.n ? ids[i] : 0;
    return t;
}

// Depth-first packing of the costs (taken in descending order) into nb bins of
// capacity cap; bins of equal load are tried once per item.  False when none
// exists or after `budget` nodes.
bool pack_dfs(const std::vector<int>& cost, const std::vector<int>& order, size_t t, int cap, std::vector<int>& load,
              std::vector<int>& bin, long& budget) {
    if (t == order.size()) return true;
    if (--budget < 0) return false;
    const int i = order[t];
    for (size_t b = 0; b < load.size(); ++b) {
        if (load[b] + cost[i] > cap) continue;
        bool seen = false;
        for (size_t e = 0; e < b && !seen; ++e) seen = load[e] == load[b];
        if (seen) continue;
        load[b] += cost[i];
        bin[i] = (int)b;
        if (pack_dfs(cost, order, t + 1, cap, load, bin, budget)) return true;
        load[b] -= cost[i];
    }
    return false;
}

// Bins (warps) for the costs (groups) with a small largest load: longest first
// to the least-loaded bin, then an exact search for each smaller largest load
// down to the lower bound (bounded in nodes; the best packing found is kept).
std::vector<int> pack_groups(const std::vector<int>& cost, int nb) {
    std::vector<int> order(cost.size());
    for (size_t i = 0; i < order.size(); ++i) order[i] = (int)i;
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return cost[a] > cost[b]; });
    std::vector<int> bin(cost.size(), 0), load(nb, 0);
    for (int i : order) {
        const int b = (int)(std::min_element(load.begin(), load.end()) - load.begin());
        load[b] += cost[i];
        bin[i] = b;
    }
    int best = *std::max_element(load.begin(), load.end());
    long total = 0;
    int top = 0;
    for (int c : cost) {
        total += c;
        top = std::max(top, c);
    }
    const int lower = std::max(top, (int)((total + nb - 1) / nb));
    for (int cap = lower; cap < best; ++cap) {
        std::vector<int> l2(nb, 0), b2(cost.size(), 0);
        long budget = 200000;
        if (pack_dfs(cost, order, 0, cap, l2, b2, budget)) {
            bin = b2;
            break;
        }
    }
    return bin;
}

}  // namespace

FlatModel flatten_model(const ModelTables& mt) {
    FlatModel fm;
    const auto& fp = mt.fp;
    fm.n_type = fp.n_type;
    fm.n_tp = mt.n_type_pairs;
    fm.n_features = mt.n_features;
    fm.gtinv = fp.gtinv;
    fm.cutoff = fp.cutoff;
    fm.maxl = fp.gtinv ? fp.maxl : 0;
    fm.n_ylm = fp.gtinv ? (fp.maxl + 1) * (fp.maxl + 2) / 2 : 1;
    for (int i = 0; i < fp.n_type; ++i)
        for (int j = 0; j < fp.n_type; ++j) fm.type_pairs.push_back(mt.type_pairs[i][j]);
    fm.n_fn_max = 1;
    for (const auto& ns : mt.tp_to_n) fm.n_fn_max = std::max<int>(fm.n_fn_max, (int)ns.size());
    fm.tp_beta.assign((size_t)fm.n_tp * fm.n_fn_max, 0.0);
    fm.tp_mu.assign((size_t)fm.n_tp * fm.n_fn_max, 0.0);
    for (int tp = 0; tp < fm.n_tp; ++tp) {
        fm.tp_nfn.push_back((int)mt.tp_to_n[tp].size());
        for (size_t q = 0; q < mt.tp_to_n[tp].size(); ++q) {
            fm.tp_beta[(size_t)tp * fm.n_fn_max + q] = fp.params[mt.tp_to_n[tp][q]][0];
            fm.tp_mu[(size_t)tp * fm.n_fn_max + q] = fp.params[mt.tp_to_n[tp][q]][1];
        }
    }
    const int F = mt.n_features;
    fm.types.resize(fp.n_type);
    for (int t = 0; t < fp.n_type; ++t) {
        const auto& tt = mt.types[t];
        auto& ft = fm.types[t];
        ft.n_lin = (int)tt.lin_index.size();
        // heads and conj completion
        if (fp.gtinv) {
            ft.K = (int)tt.full.size();
            ft.K0 = (int)tt.noconj.size();
            for (const auto& e : tt.noconj) {
                ft.head_tp.push_back(e.tp);
                ft.head_nid.push_back(e.n_id);
                ft.head_key.push_back(e.ylm_key);
                ft.head_m.push_back(e.m);
                ft.head_l.push_back(e.l);
                ft.head_full.push_back(e.ilocal_id);
                ft.head_jloc.push_back(e.jlocal_noconj_id);
                ft.head_signj.push_back(e.sign_j);
            }
            ft.full_src.assign(ft.K, 0);
            ft.full_cc.assign(ft.K, 1.0);
            ft.full_is_conj.assign(ft.K, 0);
            std::vector<int> full_to_head(ft.K, -1);
            for (int h = 0; h < ft.K0; ++h) full_to_head[tt.noconj[h].ilocal_id] = h;
            for (const auto& e : tt.full) {
                if (e.conj) {
                    ft.full_src[e.ilocal_id] = full_to_head.at(e.ilocal_conj_id);
                    ft.full_cc[e.ilocal_id] = e.cc;
                    ft.full_is_conj[e.ilocal_id] = 1;
                } else {
                    ft.full_src[e.ilocal_id] = full_to_head.at(e.ilocal_id);
                }
            }
            // value terms
            ft.val_off.push_back(0);
            for (int k = 0; k < ft.n_lin; ++k) {
                for (const auto& s : tt.value_terms[k]) ft.val_terms.push_back(make_term(s.coeff, s.ids, 0));
                ft.val_off.push_back((int)ft.val_terms.size());
            }
            // G entries: per feature, group deriv terms by folded head
            ft.ent_off.push_back(0);
            ft.term_off.push_back(0);
            for (int k = 0; k < ft.n_lin; ++k) {
                // key: (type pair of the head, head)
                std::map<std::pair<int, int>, std::vector<FlatTerm>> by_head;
                for (const auto& d : tt.deriv_terms[k]) {
                    const auto& fe = tt.full[d.head];
                    const int h = fe.conj ? full_to_head.at(fe.ilocal_conj_id) : full_to_head.at(d.head);
                    by_head[{tt.noconj[h].tp, h}].push_back(make_term(d.coeff, d.rest, fe.conj ? 1 : 0));
                }
                std::vector<int> tpo(mt.n_type_pairs + 1, 0);
                for (auto& kv : by_head) {
                    ft.ent_head.push_back(kv.first.second);
                    for (auto& term : kv.second) ft.g_terms.push_back(term);
                    ft.term_off.push_back((int)ft.g_terms.size());
                    tpo[kv.first.first + 1]++;
                }
                for (int t = 0; t < mt.n_type_pairs; ++t) tpo[t + 1] += tpo[t];
                for (int t = 0; t <= mt.n_type_pairs; ++t) ft.ent_tp_off.push_back(ft.ent_off.back() + tpo[t]);
                ft.ent_off.push_back((int)ft.ent_head.size());
            }
        } else {
            ft.K = ft.K0 = (int)tt.ntp.size();
            for (const auto& e : tt.ntp) {
                ft.head_tp.push_back(e.tp);
                ft.head_nid.push_back(e.n_id);
                ft.head_key.push_back(0);
                ft.head_m.push_back(0);
                ft.head_l.push_back(0);
                ft.head_full.push_back(e.ilocal_id);
                ft.head_jloc.push_back(e.jlocal_id);
                ft.head_signj.push_back(1.0);
            }
            ft.full_src.resize(ft.K);
            for (int h = 0; h < ft.K; ++h) ft.full_src[h] = h;
            ft.full_cc.assign(ft.K, 1.0);
            ft.full_is_conj.assign(ft.K, 0);
            ft.val_off.push_back(0);
            ft.ent_off.push_back(0);
            ft.term_off.push_back(0);
            for (int k = 0; k < ft.n_lin; ++k) {
                const int h = tt.value_terms[k][0].ids[0];
                ft.val_terms.push_back(make_term(1.0, {h}, 0));
                ft.val_off.push_back((int)ft.val_terms.size());
                const int e0 = (int)ft.ent_head.size();
                ft.ent_head.push_back(h);
                ft.g_terms.push_back(make_term(1.0, {}, 0));
                ft.term_off.push_back((int)ft.g_terms.size());
                for (int t = 0; t <= mt.n_type_pairs; ++t) ft.ent_tp_off.push_back(t <= tt.ntp[h].tp ? e0 : e0 + 1);
                ft.ent_off.push_back((int)ft.ent_head.size());
            }
        }
        // column recipes over all F columns
        ft.col_ncomp.assign(F, 0);
        ft.comp_k.assign((size_t)F * 3, -1);
        ft.comp_w.assign((size_t)F * 6, -1);
        ft.col_nent.assign(F, 0);
        for (const auto& p : tt.poly) {
            const int n = (int)p.local_ids.size();
            ft.col_ncomp[p.col] = n;
            for (int c = 0; c < n; ++c) {
                ft.comp_k[(size_t)p.col * 3 + c] = p.local_ids[c];
                int q = 0;
                for (int o = 0; o < n; ++o)
                    if (o != c) ft.comp_w[((size_t)p.col * 3 + c) * 2 + q++] = p.local_ids[o];
                const int k = p.local_ids[c];
                ft.col_nent[p.col] += ft.ent_off[k + 1] - ft.ent_off[k];
            }
        }
        for (int c = 0; c < F; ++c) fm.max_nent_col = std::max(fm.max_nent_col, ft.col_nent[c]);
        // evaluator tables: entry -> feature, head -> entries, type pair -> heads, feature -> columns
        ft.ent_k.assign(ft.ent_head.size(), 0);
        for (int k = 0; k < ft.n_lin; ++k)
            for (int e = ft.ent_off[k]; e < ft.ent_off[k + 1]; ++e) ft.ent_k[e] = k;
        std::vector<std::vector<int>> by_head(ft.K0);
        for (size_t e = 0; e < ft.ent_head.size(); ++e) by_head[ft.ent_head[e]].push_back((int)e);
        ft.head_ent_off.assign(1, 0);
        for (const auto& v : by_head) {
            ft.head_ent.insert(ft.head_ent.end(), v.begin(), v.end());
            ft.head_ent_off.push_back((int)ft.head_ent.size());
        }
        ft.tp_head_off.assign(1, 0);
        for (int tp = 0; tp < mt.n_type_pairs; ++tp) {
            for (int h = 0; h < ft.K0; ++h)
                if (ft.head_tp[h] == tp) ft.tp_heads.push_back(h);
            ft.tp_head_off.push_back((int)ft.tp_heads.size());
        }
        std::vector<std::vector<std::array<int, 3>>> kc(ft.n_lin);
        for (const auto& p : tt.poly) {
            const int n = (int)p.local_ids.size();
            for (int c = 0; c < n; ++c) {
                std::array<int, 3> r{p.col, -1, -1};
                int q = 1;
                for (int o = 0; o < n; ++o)
                    if (o != c) r[q++] = p.local_ids[o];
                kc[p.local_ids[c]].push_back(r);
            }
        }
        ft.kcol_off.assign(1, 0);
        for (const auto& v : kc) {
            for (const auto& r : v) {
                ft.kcol_col.push_back(r[0]);
                ft.kcol_o1.push_back(r[1]);
                ft.kcol_o2.push_back(r[2]);
            }
            ft.kcol_off.push_back((int)ft.kcol_col.size());
        }
        // X-row entry layout by type pair (see flat_tables.h)
        {
            const int ntp = mt.n_type_pairs, nl = ft.n_lin;
            // per type pair: the key sequence of every feature, the features in
            // layout order and the bundles (two features with equal keys, or one)
            std::vector<std::vector<std::vector<int>>> keys(ntp, std::vector<std::vector<int>>(nl));
            std::vector<std::vector<std::array<int, 2>>> bundles(ntp);
            std::vector<std::vector<int>> rest(ntp);  // features without entries of tp
            ft.n_groups = 0;
            ft.n_pos = 0;
            for (int tp = 0; tp < ntp; ++tp) {
                for (int k = 0; k < nl; ++k) {
                    const int e0 = ft.ent_tp_off[(size_t)k * (ntp + 1) + tp];
                    const int e1 = ft.ent_tp_off[(size_t)k * (ntp + 1) + tp + 1];
                    for (int e = e0; e < e1; ++e) {
                        const int h = ft.ent_head[e];
                        if (ft.head_nid[h] != ft.head_nid[ft.ent_head[e0]])
                            throw std::runtime_error("internal: a feature mixes radial functions within a type pair");
                        keys[tp][k].push_back(ft.head_key[h]);
                    }
                }
                const auto& kt = keys[tp];
                std::vector<int> order(nl);
                for (int k = 0; k < nl; ++k) order[k] = k;
                std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
                    if (kt[a].size() != kt[b].size()) return kt[a].size() > kt[b].size();
                    return kt[a] < kt[b];
                });
                for (size_t q = 0; q < order.size();) {
                    const int k = order[q];
                    if (kt[k].empty()) {
                        rest[tp].push_back(k);
                        ++q;
                    } else if (q + 1 < order.size() && kt[order[q + 1]] == kt[k]) {
                        bundles[tp].push_back({k, order[q + 1]});
                        q += 2;
                    } else {
                        bundles[tp].push_back({k, -1});
                        ++q;
                    }
                }
                const int ng = ((int)bundles[tp].size() + 31) / 32;
                ft.n_groups = std::max(ft.n_groups, ng);
                ft.n_pos = std::max(ft.n_pos, 64 * ng + (int)rest[tp].size());
            }
            ft.n_pos = std::max(4, (ft.n_pos + 3) & ~3);
            const int np = ft.n_pos, ng = ft.n_groups;
            ft.tp_perm.assign((size_t)ntp * np, -1);
            ft.tp_ipos.assign((size_t)ntp * nl, 0);
            ft.tp_pos_nid.assign((size_t)ntp * np, 0);
            ft.lay_grp_base.assign((size_t)ntp * ng, 0);
            ft.lay_grp_cnt.assign((size_t)ntp * ng, 0);
            ft.tp_nnz.assign(ntp, 0);
            ft.tpl.assign(ntp, -1);
            for (int tp = 0; tp < ntp; ++tp) {
                if (ft.tp_head_off[tp + 1] > ft.tp_head_off[tp]) {
                    ft.tpl[tp] = (int)ft.tpl_tp.size();
                    ft.tpl_tp.push_back(tp);
                }
                const auto& kt = keys[tp];
                const auto& bt = bundles[tp];
                const int ngt = ((int)bt.size() + 31) / 32;
                auto place = [&](int k, int x) {
                    ft.tp_perm[(size_t)tp * np + x] = k;
                    ft.tp_ipos[(size_t)tp * nl + k] = x;
                    if (!kt[k].empty())
                        ft.tp_pos_nid[(size_t)tp * np + x] =
                            ft.head_nid[ft.ent_head[ft.ent_tp_off[(size_t)k * (ntp + 1) + tp]]];
                };
                for (size_t t = 0; t < bt.size(); ++t) {
                    const int x = 64 * (int)(t / 32) + 2 * (int)(t % 32);
                    place(bt[t][0], x);
                    if (bt[t][1] >= 0) place(bt[t][1], x + 1);
                }
                for (size_t q = 0; q < rest[tp].size(); ++q) place(rest[tp][q], 64 * ngt + (int)q);
                ft.tp_nnz[tp] = 64 * ngt;
                for (int g = 0; g < ngt; ++g) {
                    const int c = (int)kt[bt[32 * g][0]].size();
                    ft.lay_grp_base[(size_t)tp * ng + g] = (int)ft.lay_ent.size();
                    ft.lay_grp_cnt[(size_t)tp * ng + g] = c;
                    for (int r = 0; r < c; ++r) {
                        // a zero entry names the key of lane 0's entry (same address: a broadcast)
                        const int key0 = kt[bt[32 * g][0]][r];
                        for (int half = 0; half < 2; ++half)
                            for (int l = 0; l < 32; ++l) {
                                const size_t t = 32 * (size_t)g + l;
                                const int k = t < bt.size() ? bt[t][half] : -1;
                                int e = -1;
                                if (k >= 0 && r < (int)kt[k].size()) e = ft.ent_tp_off[(size_t)k * (ntp + 1) + tp] + r;
                                const int k0 = t < bt.size() ? bt[t][0] : -1;
                                ft.lay_ent.push_back(e);
                                ft.lay_key.push_back((k0 >= 0 && r < (int)kt[k0].size()) ? kt[k0][r] : key0);
                            }
                    }
                }
            }
            ft.lay_size = (int)ft.lay_ent.size();
            // warp schedule of the groups (a group costs its ranks plus about
            // three ranks of epilogue): the smallest largest warp load found
            std::vector<std::vector<std::vector<int>>> lists(ntp, std::vector<std::vector<int>>(kLayWarps));
            ft.n_rounds = 0;
            for (int tp = 0; tp < ntp; ++tp) {
                std::vector<int> gs;
                for (int g = 0; g < ng; ++g)
                    if (ft.lay_grp_cnt[(size_t)tp * ng + g] > 0) gs.push_back(g);
                std::stable_sort(gs.begin(), gs.end(), [&](int a, int b) {
                    return ft.lay_grp_cnt[(size_t)tp * ng + a] > ft.lay_grp_cnt[(size_t)tp * ng + b];
                });
                std::vector<int> cost;
                for (int g : gs) cost.push_back(ft.lay_grp_cnt[(size_t)tp * ng + g] + 3);
                const std::vector<int> wof = pack_groups(cost, kLayWarps);
                for (size_t q = 0; q < gs.size(); ++q) lists[tp][wof[q]].push_back(gs[q]);
                for (int w = 0; w < kLayWarps; ++w) ft.n_rounds = std::max(ft.n_rounds, (int)lists[tp][w].size());
            }
            ft.lay_sched.assign((size_t)ntp * ft.n_rounds * kLayWarps, -1);
            for (int tp = 0; tp < ntp; ++tp)
                for (int w = 0; w < kLayWarps; ++w)
                    for (size_t k = 0; k < lists[tp][w].size(); ++k)
                        ft.lay_sched[((size_t)tp * ft.n_rounds + k) * kLayWarps + w] = lists[tp][w][k];
            // product-column roles of stage B
            {
                const int F = (int)ft.col_ncomp.size();
                bool ok = true;
                for (int c = 0; c < F; ++c) ok = ok && ft.col_ncomp[c] <= 2;
                ft.prod_qn.assign(ntp, 0);
                ft.prod_q.assign((size_t)ntp * kRowRoles * 4, 0);
                for (int tp = 0; ok && tp < ntp; ++tp) {
                    const int nnz = ft.tp_nnz[tp];
                    const int* ipos = ft.tp_ipos.data() + (size_t)tp * nl;
                    std::vector<std::array<int, 4>> r;
                    for (int c = 0; c < F; ++c) {
                        if (ft.col_ncomp[c] != 2) continue;
                        const int k0 = ft.comp_k[(size_t)c * 3], k1 = ft.comp_k[(size_t)c * 3 + 1];
                        if (k0 == k1) {
                            if (ipos[k0] < nnz) r.push_back({ipos[k0], k0, c, 2});
                        } else {
                            if (ipos[k0] < nnz) r.push_back({ipos[k0], k1, c, 0});
                            if (ipos[k1] < nnz) r.push_back({ipos[k1], k0, c, 1});
                        }
                    }
                    if ((int)r.size() > kRowRoles) {
                        ok = false;
                        break;
                    }
                    // by position: the lanes of a warp read few distinct group-vector values
                    std::stable_sort(r.begin(), r.end(), [](const std::array<int, 4>& a, const std::array<int, 4>& b) {
                        return a[0] < b[0];
                    });
                    ft.prod_qn[tp] = (int)r.size();
                    for (size_t t = 0; t < r.size(); ++t)
                        for (int v = 0; v < 4; ++v) ft.prod_q[((size_t)tp * kRowRoles + t) * 4 + v] = r[t][v];
                }
                ft.prod_qok = ok ? 1 : 0;
                if (!ok) std::fill(ft.prod_qn.begin(), ft.prod_qn.end(), 0);
            }
        }
    }
    // Legendre / Y_lm constants, computed in IEEE double with the reference's
    // expressions (polymlp_spherical_harmonics.cpp:95-196).
    {
        const int L = fm.maxl, n = fm.n_ylm;
        auto lmi = [](int l, int m) { return l * (l + 1) / 2 + m; };
        std::vector<double> t(4 * n + 3 * (L + 1), 0.0);
        for (int l = 0; l <= L; ++l) {
            const double ls = l * l, lm1s = (l - 1) * (l - 1);
            for (int m = 0; m <= l; ++m) {
                const double ms = m * m;
                if (m <= l - 2) {
                    t[lmi(l, m)] = std::sqrt((4.0 * ls - 1.0) / (ls - ms));
                    t[n + lmi(l, m)] = -std::sqrt((lm1s - ms) / (4.0 * lm1s - 1.0));
                }
                if (m < l) t[2 * n + lmi(l, m)] = std::sqrt((double)((l - m) * (l + m + 1)));
                // DEC: index l(l+1)/2 + l - m' for m' = m
                t[3 * n + lmi(l, 0) + l - m] = (double)(l | (m << 8));
            }
            t[4 * n + l] = l >= 2 ? -std::sqrt(1.0 + 0.5 / l) : 0.0;
            t[4 * n + (L + 1) + l] = std::sqrt(2.0 * l + 3.0);
            t[4 * n + 2 * (L + 1) + l] = std::sqrt(0.5 * l * (l + 1));
        }
        fm.ylm_tab = t;
    }
    return fm;
}

}  // namespace pg
