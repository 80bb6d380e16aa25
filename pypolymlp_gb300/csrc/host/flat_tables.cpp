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

// Rows of the head-space gradient tile for the nh heads of one type pair.
// The force-row contraction reads, per rank of a 32-feature group, the rows of
// the heads that the group's entries of that rank name; row r sits in
// shared-memory bank set r mod 8, so heads read together should have distinct
// rows mod 8 (same head: broadcast, no conflict).  `ranks` lists the distinct
// heads (0..nh-1) read together.  Greedy colouring (most-read heads first,
// each to the class that least raises the ranks' largest class), then one
// pass of pairwise swaps that lower the sum over ranks of the largest class;
// class c gets rows c, c + 8, ...  Returns the row of each head.
std::vector<int> colour_head_rows(int nh, const std::vector<std::vector<int>>& ranks) {
    constexpr int kC = 8;
    std::vector<std::vector<int>> ranks_of(nh);
    for (size_t r = 0; r < ranks.size(); ++r)
        for (int u : ranks[r]) ranks_of[u].push_back((int)r);
    std::vector<std::array<int, kC>> cls(ranks.size());
    for (auto& a : cls) a.fill(0);
    auto largest = [&](int r) { return *std::max_element(cls[r].begin(), cls[r].end()); };
    std::vector<int> cap(kC, 0), col(nh, 0), order(nh);
    for (int u = 0; u < nh; ++u) {
        cap[u % kC]++;
        order[u] = u;
    }
    std::stable_sort(order.begin(), order.end(),
                     [&](int a, int b) { return ranks_of[a].size() > ranks_of[b].size(); });
    for (int u : order) {
        long best = -1;
        int bc = 0;
        for (int c = 0; c < kC; ++c) {
            if (cap[c] == 0) continue;
            long cost = 0;
            for (int r : ranks_of[u]) cost += (cls[r][c] + 1 > largest(r) ? 16 : 0) + cls[r][c];
            if (best < 0 || cost < best) {
                best = cost;
                bc = c;
            }
        }
        col[u] = bc;
        cap[bc]--;
        for (int r : ranks_of[u]) cls[r][bc]++;
    }
    auto move = [&](int u, int from, int to) {
        for (int r : ranks_of[u]) {
            cls[r][from]--;
            cls[r][to]++;
        }
    };
    std::vector<int> touched;
    for (int a = 0; a < nh; ++a)
        for (int b = a + 1; b < nh; ++b) {
            const int ca = col[a], cb = col[b];
            if (ca == cb || ranks_of[a].empty()) continue;
            touched.assign(ranks_of[a].begin(), ranks_of[a].end());
            touched.insert(touched.end(), ranks_of[b].begin(), ranks_of[b].end());
            std::sort(touched.begin(), touched.end());
            touched.erase(std::unique(touched.begin(), touched.end()), touched.end());
            long before = 0, after = 0;
            for (int r : touched) before += largest(r);
            move(a, ca, cb);
            move(b, cb, ca);
            for (int r : touched) after += largest(r);
            if (after < before) {
                col[a] = cb;
                col[b] = ca;
            } else {
                move(a, cb, ca);
                move(b, ca, cb);
            }
        }
    std::vector<int> next(kC), row(nh);
    for (int c = 0; c < kC; ++c) next[c] = c;
    for (int u = 0; u < nh; ++u) {
        row[u] = next[col[u]];
        next[col[u]] += kC;
    }
    return row;
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
            ft.n_groups = (nl + 31) / 32;
            std::vector<int> hpos_of(ft.K0, 0);
            for (int tp = 0; tp < ntp; ++tp)
                for (int q = ft.tp_head_off[tp]; q < ft.tp_head_off[tp + 1]; ++q)
                    hpos_of[ft.tp_heads[q]] = q - ft.tp_head_off[tp];
            ft.tp_perm.assign((size_t)ntp * nl, 0);
            ft.tp_ipos.assign((size_t)ntp * nl, 0);
            ft.lay_grp_base.assign((size_t)ntp * ft.n_groups, 0);
            ft.lay_grp_cnt.assign((size_t)ntp * ft.n_groups, 0);
            ft.tp_nnz.assign(ntp, 0);
            ft.tpl.assign(ntp, -1);
            ft.tp_head_row.assign(ft.tp_heads.size(), 0);
            for (int tp = 0; tp < ntp; ++tp) {
                if (ft.tp_head_off[tp + 1] > ft.tp_head_off[tp]) {
                    ft.tpl[tp] = (int)ft.tpl_tp.size();
                    ft.tpl_tp.push_back(tp);
                }
                auto cnt = [&](int k) {
                    return ft.ent_tp_off[(size_t)k * (ntp + 1) + tp + 1] - ft.ent_tp_off[(size_t)k * (ntp + 1) + tp];
                };
                std::vector<int> order(nl);
                for (int k = 0; k < nl; ++k) order[k] = k;
                std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return cnt(a) > cnt(b); });
                for (int x = 0; x < nl; ++x) {
                    ft.tp_perm[(size_t)tp * nl + x] = order[x];
                    ft.tp_ipos[(size_t)tp * nl + order[x]] = x;
                    if (cnt(order[x]) > 0) ft.tp_nnz[tp] = x + 1;
                }
                const size_t tp_base = ft.lay_ent.size();
                std::vector<std::vector<int>> ranks;
                for (int g = 0; g < ft.n_groups; ++g) {
                    const int c = cnt(order[32 * g]);
                    ft.lay_grp_base[(size_t)tp * ft.n_groups + g] = (int)ft.lay_ent.size();
                    ft.lay_grp_cnt[(size_t)tp * ft.n_groups + g] = c;
                    for (int r = 0; r < c; ++r) {
                        std::vector<int> heads;
                        for (int l = 0; l < 32; ++l) {
                            const int x = 32 * g + l;
                            int e = -1;
                            if (x < nl && r < cnt(order[x])) e = ft.ent_tp_off[(size_t)order[x] * (ntp + 1) + tp] + r;
                            ft.lay_ent.push_back(e);
                            ft.lay_hpos.push_back(e >= 0 ? hpos_of[ft.ent_head[e]] : 0);
                            if (e >= 0) heads.push_back(hpos_of[ft.ent_head[e]]);
                        }
                        std::sort(heads.begin(), heads.end());
                        heads.erase(std::unique(heads.begin(), heads.end()), heads.end());
                        ranks.push_back(std::move(heads));
                    }
                }
                // head -> row of the gradient tile; a zero entry reads the row of
                // its rank's first entry (lane 0 holds the group's largest feature)
                const int q0 = ft.tp_head_off[tp], nh = ft.tp_head_off[tp + 1] - q0;
                const std::vector<int> row = colour_head_rows(nh, ranks);
                for (int q = 0; q < nh; ++q) ft.tp_head_row[q0 + q] = row[q];
                for (size_t s = tp_base; s < ft.lay_ent.size(); s += 32) {
                    const int first = row[ft.lay_hpos[s]];
                    for (int l = 0; l < 32; ++l)
                        ft.lay_hpos[s + l] = ft.lay_ent[s + l] >= 0 ? row[ft.lay_hpos[s + l]] : first;
                }
            }
            ft.lay_size = (int)ft.lay_ent.size();
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
