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
constexpr int kLayWarps = 8;  // warps of a stage-A block (the contraction's group schedule)
constexpr int kRowRoles = 256;  // threads of a stage-B block: the most product-column roles of a type pair

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
    // type.  The entries of feature k by type pair tp all name one radial
    // function, tp_pos_nid[tp][x] at the feature's position x, so the force
    // derivative by a pair d of tp factors into
    //   dd_k/dd = f_n(r) sum_e Re(G_e grad Y_e) + f_n'(r) d/r sum_e Re(G_e Y_e),
    // sums over the Y_lm keys of the entries.  The features with entries of tp
    // are ordered by their number of entries (descending), then by their key
    // sequence, and taken two at a time into bundles of two features with the
    // same key sequence (or one, when the next feature's keys differ), so that
    // one table row of a key serves both.  Bundle t = 32 g + l sits in group g,
    // lane l: its features at positions 64 g + 2 l and 64 g + 2 l + 1 (holes,
    // tp_perm = -1, where a bundle has one feature or the group is not full).
    // The features without entries of tp follow at 64 n_g(tp) onwards, and
    // positions run to n_pos (all type pairs; a multiple of 4); tp_perm[tp][x]
    // is the feature at position x, tp_ipos[tp][k] the position of feature k.
    // Group g stores its entries rank-major: slots lay_grp_base[tp][g] + 64 r
    // + l and + 32 + l hold the r-th entries of the two features of lane l
    // (lay_ent = -1 for a hole or a feature with fewer entries: a zero entry).
    // n_groups = the most groups of any type pair; lay_grp_cnt[tp][g] = entries
    // of the group's first (largest) feature, 0 for groups past the last.
    // lay_key is the Y_lm key of the lane's entries of the rank (both slots); a
    // lane past its feature's entries repeats the key of lane 0, so the lanes
    // of a rank read few distinct keys.  tp_nnz[tp] = 64 n_g(tp): the positions
    // that can hold derivatives of tp; the others' derivatives vanish.
    // lay_sched[tp][k][w] (n_rounds x kLayWarps per type pair): the k-th group
    // of warp w in stage A, or -1; the packing with the smallest largest warp
    // load found (a group costs its ranks + 3).
    int n_groups = 0, lay_size = 0, n_pos = 0, n_rounds = 0;
    std::vector<int> lay_ent, lay_key, lay_grp_base, lay_grp_cnt, tp_perm, tp_ipos, tp_pos_nid, tp_nnz, lay_sched;
    // Product-column roles of stage B (prod_qok: every product column of this
    // type is a product of two features and each type pair has at most
    // kRowRoles roles).  Per type pair tp, prod_qn[tp] roles, one per (column,
    // differentiated feature k with a position below tp_nnz):
    // prod_q[(tp * kRowRoles + t) * 4 + {0,1,2,3}] = {position of k, the other
    // feature (the weight), column, phase | 2 * (square column)}, by position.
    // A column's phase-0 role is its first feature's, phase 1 its second's.
    int prod_qok = 0;
    std::vector<int> prod_qn, prod_q;
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
