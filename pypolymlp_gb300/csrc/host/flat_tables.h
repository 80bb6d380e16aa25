// Flat (device-uploadable) form of the model tables.
//
// Naming: K = full a_nlm entries of a centre type, K0 = no-conjugate entries
// (m <= 0), "head" = a no-conjugate entry.  For each linear feature k of a
// type the adjoint vector G_k[h] = d(feature k)/d(a_h) (conjugate heads folded
// into their m <= 0 partner) is stored sparsely as "G entries".
#pragma once

#include <cstdint>
#include <vector>

#include "model_tables.h"

namespace pg {

constexpr int kMaxOrder = 6;  // gtinv order supported by the reference tables

// One product term: coeff * prod(a[ids[0..n)]) (ids: full local ids).
struct FlatTerm {
    double coeff;
    int n;
    int conj;  // G terms: 1 if the term's head is the conjugate of the entry's head
    int ids[kMaxOrder];
};

struct FlatType {
    int K = 0, K0 = 0, n_lin = 0;
    // heads (K0): meta for basis lookup and the evaluator
    std::vector<int> head_tp, head_nid, head_key, head_m, head_l, head_full, head_jloc;
    std::vector<double> head_signj;
    // conj completion of full entries: src head index and cc (cc = 0 for heads)
    std::vector<int> full_src;
    std::vector<double> full_cc;
    std::vector<int> full_is_conj;
    // value terms per linear feature (CSR)
    std::vector<int> val_off;
    std::vector<FlatTerm> val_terms;
    // G entries per linear feature (CSR over features), head per entry, terms per entry (CSR)
    std::vector<int> ent_off, ent_head, term_off;
    // per linear feature k: (n_tp + 1) offsets of its entries by type pair
    // (entries of a feature are sorted by type pair, then head)
    std::vector<int> ent_tp_off;
    std::vector<FlatTerm> g_terms;
    // per column (all F columns): recipe components.  comp_k[col*3+c] is the
    // local linear feature (-1 = unused); comp_w[(col*3+c)*2+q] are the
    // feature indices whose product weights the component (-1 = none).
    std::vector<int> col_ncomp, comp_k, comp_w;
    // per column: number of G entries (sum over its components), for smem sizing
    std::vector<int> col_nent;
    // evaluator tables
    std::vector<int> ent_k;                 // linear feature of each G entry
    std::vector<int> head_ent_off, head_ent; // per head (K0): entries with that head (CSR)
    std::vector<int> tp_head_off, tp_heads;  // per type pair: heads of that pair (CSR)
    // per linear feature k: polynomial columns containing it (CSR): column and the
    // (up to two) other features whose product weights d(col)/d(d_k); -1 = none
    std::vector<int> kcol_off, kcol_col, kcol_o1, kcol_o2;
    // X-row layout of the adjoint entries, per type pair tp of this centre
    // type: the features are ordered by their number of entries of tp
    // (descending; tp_perm[tp][x] is the feature at position x, tp_ipos the
    // inverse) and taken 32 at a time (group g = positions 32g .. 32g+31);
    // group g stores its entries rank-major: slot lay_grp_base[tp][g] + 32 r +
    // lane holds the r-th entry of the feature at position 32g + lane
    // (lay_ent = -1 where that feature has fewer entries: a zero entry).
    // n_groups = ceil(n_lin / 32); lay_grp_cnt[tp][g] = entries of the group's
    // first (largest) feature.  lay_hpos is the row of the entry's head in the
    // per-type-pair gradient tile: tp_head_row[q] for the tp_heads entry q, rows
    // coloured so that the heads one rank reads fall in distinct bank sets; a
    // zero entry repeats the row of its rank's lane 0.
    // tp_nnz[tp]: positions with entries of tp (they come first); the
    // derivatives of the other features by a pair of tp vanish.
    int n_groups = 0, lay_size = 0;
    std::vector<int> lay_ent, lay_hpos, lay_grp_base, lay_grp_cnt, tp_perm, tp_ipos, tp_head_row, tp_nnz;
    // type pairs with heads for this centre type: local index or -1, and back
    std::vector<int> tpl, tpl_tp;
};

struct FlatModel {
    int n_type = 0, n_tp = 0, n_features = 0, n_fn_max = 0, maxl = 0, n_ylm = 0;
    bool gtinv = true;
    double cutoff = 0.0;
    std::vector<int> type_pairs;        // n_type*n_type
    std::vector<int> tp_nfn;            // radial functions per type pair
    std::vector<double> tp_beta, tp_mu; // [tp*n_fn_max + n_id]
    std::vector<FlatType> types;
    int max_nent_col = 0;               // max G entries of a single column (any type)
    std::vector<double> ylm_tab;        // Legendre / Y_lm constants (device_model.cuh layout)
};

FlatModel flatten_model(const ModelTables& mt);

}  // namespace pg
