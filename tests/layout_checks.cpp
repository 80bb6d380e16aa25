// Invariants of the host-built X-row layout tables (flat_tables.cpp), checked on
// the CPU by tests/test_layout_tables.py: the gradient-tile rows of each type
// pair are a permutation, entries name the row of their head, zero entries
// repeat their rank's lane-0 row, the positions with entries of a type pair come
// first (tp_nnz of them), and the colouring does not raise the bank-set load of
// a rank above the uncoloured order.  Returns 0 and a summary, or 1 and the
// first violation, in msg.
#include <algorithm>
#include <cstdio>
#include <map>
#include <set>
#include <vector>

#include "host/flat_tables.h"
#include "host/params.h"

namespace {

// largest number of distinct rows of one bank set (row mod 8) among `rows`
int bank_load(const std::vector<int>& rows) {
    std::map<int, std::set<int>> cls;
    for (int r : rows) cls[r % 8].insert(r);
    int m = 0;
    for (const auto& kv : cls) m = std::max(m, (int)kv.second.size());
    return m;
}

}  // namespace

extern "C" int check_layout(const pg_feature_params* p, char* msg, int n_msg) {
    using namespace pg;
    const FlatModel fm = flatten_model(build_model_tables(feature_params_from_abi(p)));
    const int ntp = fm.n_tp;
    long coloured = 0, plain = 0, ranks = 0;
    for (size_t t = 0; t < fm.types.size(); ++t) {
        const FlatType& ft = fm.types[t];
        const int nl = ft.n_lin, ng = ft.n_groups;
        for (int tp = 0; tp < ntp; ++tp) {
            const int q0 = ft.tp_head_off[tp], nh = ft.tp_head_off[tp + 1] - q0;
            std::vector<int> pos_of(ft.K0, -1), row_of(ft.K0, -1), seen(nh, 0);
            for (int q = 0; q < nh; ++q) {
                const int r = ft.tp_head_row[q0 + q];
                if (r < 0 || r >= nh || seen[r]++) {
                    snprintf(msg, n_msg, "type %zu tp %d: head rows are not a permutation", t, tp);
                    return 1;
                }
                pos_of[ft.tp_heads[q0 + q]] = q;
                row_of[ft.tp_heads[q0 + q]] = r;
            }
            auto cnt = [&](int k) {
                return ft.ent_tp_off[(size_t)k * (ntp + 1) + tp + 1] - ft.ent_tp_off[(size_t)k * (ntp + 1) + tp];
            };
            int nnz = 0;
            for (int x = 0; x < nl; ++x)
                if (cnt(ft.tp_perm[(size_t)tp * nl + x]) > 0) nnz = x + 1;
            for (int x = 0; x < nnz; ++x)
                if (cnt(ft.tp_perm[(size_t)tp * nl + x]) == 0) {
                    snprintf(msg, n_msg, "type %zu tp %d: a position without entries before the last with", t, tp);
                    return 1;
                }
            if (nnz != ft.tp_nnz[tp]) {
                snprintf(msg, n_msg, "type %zu tp %d: tp_nnz %d, expected %d", t, tp, ft.tp_nnz[tp], nnz);
                return 1;
            }
            for (int g = 0; g < ng; ++g) {
                const int base = ft.lay_grp_base[(size_t)tp * ng + g], c = ft.lay_grp_cnt[(size_t)tp * ng + g];
                for (int r = 0; r < c; ++r) {
                    std::vector<int> rows_c, rows_p;
                    const int s0 = base + 32 * r;
                    if (ft.lay_ent[s0] < 0) {
                        snprintf(msg, n_msg, "type %zu tp %d group %d rank %d: lane 0 holds no entry", t, tp, g, r);
                        return 1;
                    }
                    for (int l = 0; l < 32; ++l) {
                        const int e = ft.lay_ent[s0 + l];
                        const int want = e >= 0 ? row_of[ft.ent_head[e]] : ft.lay_hpos[s0];
                        if (ft.lay_hpos[s0 + l] != want) {
                            snprintf(msg, n_msg, "type %zu tp %d group %d rank %d lane %d: row %d, expected %d", t,
                                     tp, g, r, l, ft.lay_hpos[s0 + l], want);
                            return 1;
                        }
                        if (e >= 0) {
                            rows_c.push_back(row_of[ft.ent_head[e]]);
                            rows_p.push_back(pos_of[ft.ent_head[e]]);
                        }
                    }
                    coloured += bank_load(rows_c);
                    plain += bank_load(rows_p);
                    ++ranks;
                }
            }
        }
    }
    if (coloured > plain) {
        snprintf(msg, n_msg, "colouring raised the bank-set load: %ld > %ld over %ld ranks", coloured, plain, ranks);
        return 1;
    }
    snprintf(msg, n_msg, "ranks %ld, bank-set load coloured %ld, uncoloured %ld", ranks, coloured, plain);
    return 0;
}
