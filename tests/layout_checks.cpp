// Invariants of the host-built X-row layout tables (flat_tables.cpp), checked on
// the CPU by tests/test_layout_tables.py: tp_perm and tp_ipos are inverse (holes
// aside); the features with entries of a type pair sit below tp_nnz, in bundles
// (positions 64g + 2l and 64g + 2l + 1) of equal key sequences, with entry counts
// non-increasing in bundle order; all entries of a feature by one type pair name
// one radial function, tp_pos_nid at its position; slots hold the r-th entries
// of their features and name the key of lane l's first feature, or lane 0's
// past its entries; the slots cover every entry once; and the ranks read few
// distinct keys (the mean over ranks is reported and bounded by 4); the warp
// schedule names every group with entries once, its largest warp load no
// worse than longest-first; the product-column roles of
// stage B cover each (column, differentiated feature with data) once, one role
// per column and phase, by position.  Returns 0
// and a summary, or 1 and the first violation, in msg.
#include <algorithm>
#include <cstdio>
#include <functional>
#include <set>
#include <vector>

#include "host/flat_tables.h"
#include "host/params.h"

extern "C" int check_layout(const pg_feature_params* p, char* msg, int n_msg) {
    using namespace pg;
    const FlatModel fm = flatten_model(build_model_tables(feature_params_from_abi(p)));
    const int ntp = fm.n_tp;
    long ranks = 0, distinct = 0, slots = 0, entries = 0, roles = 0, role_types = 0, sched_load = 0, lpt_load = 0;
    for (size_t t = 0; t < fm.types.size(); ++t) {
        const FlatType& ft = fm.types[t];
        const int nl = ft.n_lin, ng = ft.n_groups, np = ft.n_pos;
        if (np < nl || np % 4) {
            snprintf(msg, n_msg, "type %zu: n_pos %d for %d features", t, np, nl);
            return 1;
        }
        std::vector<int> seen(ft.ent_head.size(), 0);
        for (int tp = 0; tp < ntp; ++tp) {
            auto e0 = [&](int k) { return ft.ent_tp_off[(size_t)k * (ntp + 1) + tp]; };
            auto cnt = [&](int k) { return k < 0 ? 0 : ft.ent_tp_off[(size_t)k * (ntp + 1) + tp + 1] - e0(k); };
            auto key = [&](int k, int r) { return ft.head_key[ft.ent_head[e0(k) + r]]; };
            const int* perm = ft.tp_perm.data() + (size_t)tp * np;
            const int nnz = ft.tp_nnz[tp];
            if (nnz % 64 || nnz > np) {
                snprintf(msg, n_msg, "type %zu tp %d: tp_nnz %d", t, tp, nnz);
                return 1;
            }
            std::vector<int> hits(nl, 0);
            for (int x = 0; x < np; ++x) {
                const int k = perm[x];
                if (k < 0) continue;
                if (k >= nl || hits[k]++ || ft.tp_ipos[(size_t)tp * nl + k] != x) {
                    snprintf(msg, n_msg, "type %zu tp %d: position %d and feature %d disagree", t, tp, x, k);
                    return 1;
                }
                if ((cnt(k) > 0) != (x < nnz)) {
                    snprintf(msg, n_msg, "type %zu tp %d: feature %d with %d entries at position %d (nnz %d)", t,
                             tp, k, cnt(k), x, nnz);
                    return 1;
                }
                for (int e = e0(k); e < e0(k) + cnt(k); ++e)
                    if (ft.head_nid[ft.ent_head[e]] != ft.tp_pos_nid[(size_t)tp * np + x]) {
                        snprintf(msg, n_msg, "type %zu tp %d feature %d: entry %d names radial %d, position %d", t,
                                 tp, k, e, ft.head_nid[ft.ent_head[e]], ft.tp_pos_nid[(size_t)tp * np + x]);
                        return 1;
                    }
            }
            for (int k = 0; k < nl; ++k)
                if (hits[k] != 1) {
                    snprintf(msg, n_msg, "type %zu tp %d: feature %d at %d positions", t, tp, k, hits[k]);
                    return 1;
                }
            std::vector<int> sched(ng, 0);
            for (int q = 0; q < ft.n_rounds * kLayWarps; ++q) {
                const int g = ft.lay_sched[(size_t)tp * ft.n_rounds * kLayWarps + q];
                if (g >= ng || (g >= 0 && sched[g]++)) {
                    snprintf(msg, n_msg, "type %zu tp %d: schedule entry %d names group %d", t, tp, q, g);
                    return 1;
                }
            }
            for (int g = 0; g < ng; ++g)
                if (sched[g] != (ft.lay_grp_cnt[(size_t)tp * ng + g] > 0 ? 1 : 0)) {
                    snprintf(msg, n_msg, "type %zu tp %d: group %d scheduled %d times", t, tp, g, sched[g]);
                    return 1;
                }
            // the largest warp load (a group costs its ranks + 3) is no worse than
            // longest-first to the least-loaded warp
            {
                std::vector<int> load(kLayWarps, 0), lpt(kLayWarps, 0), cost;
                for (int q = 0; q < ft.n_rounds * kLayWarps; ++q) {
                    const int g = ft.lay_sched[(size_t)tp * ft.n_rounds * kLayWarps + q];
                    if (g >= 0) load[q % kLayWarps] += ft.lay_grp_cnt[(size_t)tp * ng + g] + 3;
                }
                for (int g = 0; g < ng; ++g)
                    if (ft.lay_grp_cnt[(size_t)tp * ng + g] > 0) cost.push_back(ft.lay_grp_cnt[(size_t)tp * ng + g] + 3);
                std::sort(cost.begin(), cost.end(), std::greater<int>());
                for (int c : cost) *std::min_element(lpt.begin(), lpt.end()) += c;
                const int ms = *std::max_element(load.begin(), load.end()), ml = *std::max_element(lpt.begin(), lpt.end());
                if (ms > ml) {
                    snprintf(msg, n_msg, "type %zu tp %d: largest warp load %d, longest-first %d", t, tp, ms, ml);
                    return 1;
                }
                sched_load += ms;
                lpt_load += ml;
            }
            int prev = 1 << 30;
            for (int g = 0; g < ng; ++g) {
                const int base = ft.lay_grp_base[(size_t)tp * ng + g], c = ft.lay_grp_cnt[(size_t)tp * ng + g];
                if (64 * g >= nnz) {
                    if (c != 0) {
                        snprintf(msg, n_msg, "type %zu tp %d group %d past tp_nnz has entries", t, tp, g);
                        return 1;
                    }
                    continue;
                }
                if (c != cnt(perm[64 * g])) {
                    snprintf(msg, n_msg, "type %zu tp %d group %d: count %d is not lane 0's", t, tp, g, c);
                    return 1;
                }
                for (int l = 0; l < 32; ++l) {
                    const int ka = perm[64 * g + 2 * l], kb = perm[64 * g + 2 * l + 1];
                    if (kb >= 0 && (ka < 0 || cnt(ka) != cnt(kb))) {
                        snprintf(msg, n_msg, "type %zu tp %d group %d lane %d: bundle partner unlike", t, tp, g, l);
                        return 1;
                    }
                    for (int r = 0; kb >= 0 && r < cnt(kb); ++r)
                        if (key(ka, r) != key(kb, r)) {
                            snprintf(msg, n_msg, "type %zu tp %d group %d lane %d: bundle keys differ", t, tp, g, l);
                            return 1;
                        }
                    if (ka >= 0) {
                        if (cnt(ka) > prev) {
                            snprintf(msg, n_msg, "type %zu tp %d group %d lane %d: counts not descending", t, tp, g, l);
                            return 1;
                        }
                        prev = cnt(ka);
                    }
                }
                for (int r = 0; r < c; ++r) {
                    const int s0 = base + 64 * r;
                    std::set<int> keys;
                    for (int h = 0; h < 2; ++h)
                        for (int l = 0; l < 32; ++l) {
                            const int k = perm[64 * g + 2 * l + h], ka = perm[64 * g + 2 * l];
                            const int e = ft.lay_ent[s0 + 32 * h + l];
                            const int want_e = r < cnt(k) ? e0(k) + r : -1;
                            if (e != want_e) {
                                snprintf(msg, n_msg, "type %zu tp %d group %d rank %d slot %d: entry %d, expected %d",
                                         t, tp, g, r, 32 * h + l, e, want_e);
                                return 1;
                            }
                            const int want = r < cnt(ka) ? key(ka, r) : ft.lay_key[s0];
                            if (ft.lay_key[s0 + 32 * h + l] != want) {
                                snprintf(msg, n_msg, "type %zu tp %d group %d rank %d slot %d: key %d, expected %d",
                                         t, tp, g, r, 32 * h + l, ft.lay_key[s0 + 32 * h + l], want);
                                return 1;
                            }
                            if (e >= 0) {
                                seen[e]++;
                                ++entries;
                            }
                            if (h == 0) keys.insert(want);
                        }
                    distinct += (long)keys.size();
                    slots += 64;
                    ++ranks;
                }
            }
        }
        for (size_t e = 0; e < seen.size(); ++e)
            if (seen[e] != 1) {
                snprintf(msg, n_msg, "type %zu: entry %zu is in %d slots", t, e, seen[e]);
                return 1;
            }
        // product-column roles of stage B: with prod_qok, every (column of two
        // features, differentiated feature with data in tp) has one role naming
        // its position and the other feature, a column has at most one role per
        // phase, and the roles run by position
        const int F = (int)ft.col_ncomp.size();
        bool two = true;
        for (int c = 0; c < F; ++c) two = two && ft.col_ncomp[c] <= 2;
        if (ft.prod_qok && !two) {
            snprintf(msg, n_msg, "type %zu: product roles with a column of three features", t);
            return 1;
        }
        for (int tp = 0; ft.prod_qok && tp < ntp; ++tp) {
            const int nq = ft.prod_qn[tp], nnz = ft.tp_nnz[tp];
            const int* ipos = ft.tp_ipos.data() + (size_t)tp * nl;
            if (nq > kRowRoles) {
                snprintf(msg, n_msg, "type %zu tp %d: %d roles", t, tp, nq);
                return 1;
            }
            std::set<std::pair<int, int>> want, got, phase_col;
            for (int c = 0; c < F; ++c) {
                if (ft.col_ncomp[c] != 2) continue;
                const int k0 = ft.comp_k[(size_t)c * 3], k1 = ft.comp_k[(size_t)c * 3 + 1];
                if (ipos[k0] < nnz) want.insert({c, k0});
                if (ipos[k1] < nnz) want.insert({c, k1});
            }
            int prev = -1;
            for (int q = 0; q < nq; ++q) {
                const int* r = ft.prod_q.data() + ((size_t)tp * kRowRoles + q) * 4;
                const int x = r[0], kw = r[1], c = r[2], ph = r[3] & 1, sq = r[3] >> 1;
                const int k = x >= 0 && x < np ? ft.tp_perm[(size_t)tp * np + x] : -1;
                const bool col_ok = c >= 0 && c < F && ft.col_ncomp[c] == 2;
                const int k0 = col_ok ? ft.comp_k[(size_t)c * 3] : -2, k1 = col_ok ? ft.comp_k[(size_t)c * 3 + 1] : -2;
                const bool pair_ok = col_ok && ((ph == 0 && k == k0 && kw == k1) || (ph == 1 && k == k1 && kw == k0));
                if (x >= nnz || k < 0 || !pair_ok || sq != (k0 == k1 ? 1 : 0) || (sq && ph) || x < prev ||
                    !got.insert({c, k}).second || !phase_col.insert({c, ph}).second) {
                    snprintf(msg, n_msg, "type %zu tp %d: role %d (position %d, weight %d, column %d, flags %d)", t, tp,
                             q, x, kw, c, r[3]);
                    return 1;
                }
                prev = x;
            }
            if (got != want) {
                snprintf(msg, n_msg, "type %zu tp %d: %zu roles, %zu expected", t, tp, got.size(), want.size());
                return 1;
            }
            roles += nq;
        }
        role_types += ft.prod_qok;
    }
    if (ranks > 0 && distinct > 4 * ranks) {
        snprintf(msg, n_msg, "ranks read %.2f distinct keys on average", (double)distinct / ranks);
        return 1;
    }
    snprintf(msg, n_msg,
             "ranks %ld, distinct keys per rank %.2f, slot efficiency %.3f, product roles %ld (%ld of %zu types), "
             "largest warp loads %ld (longest-first %ld)",
             ranks, ranks ? (double)distinct / ranks : 0.0, slots ? (double)entries / slots : 0.0, roles, role_types,
             fm.types.size(), sched_load, lpt_load);
    return 0;
}
