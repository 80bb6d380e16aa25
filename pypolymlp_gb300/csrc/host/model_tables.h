// Host-side model tables for the polynomial MLP hot path.
//
// The tables fix the column order of X and the index maps that the CUDA
// kernels (and the CPU oracle) consume.  They restate the setup that the
// reference performs in
//   src/pypolymlp/cxx/src/polymlp/polymlp_mapping.cpp            (Mapping)
//   src/pypolymlp/cxx/src/polymlp/polymlp_model_params_gtinv.cpp (uniq_gtinv_type)
//   src/pypolymlp/cxx/src/polymlp/polymlp_model_params_polynomial.cpp
//   src/pypolymlp/cxx/src/polymlp/polymlp_features_utils.cpp
//   src/pypolymlp/cxx/src/polymlp/polymlp_features_mapping_utils.cpp
//   src/pypolymlp/cxx/src/polymlp/polymlp_features_polynomial.cpp
//   src/pypolymlp/cxx/src/polymlp/polymlp_potential.cpp           (Potential)
// with the same ordering rules (std::set iteration, n-major linear terms),
// and flattens the result into plain arrays for device upload.
#pragma once

#include <array>
#include <cstdint>
#include <map>
#include <string>
#include <vector>

namespace pg {

// Mirrors the reference's feature_params (polymlp_mlpcpp.h:55).
struct FeatureParams {
    int n_type = 1;
    bool gtinv = true;          // feature_type: "gtinv" (true) or "pair" (false)
    int model_type = 2;
    int maxp = 2;
    int maxl = 0;
    double cutoff = 6.0;
    std::vector<std::array<double, 2>> params;          // (beta, mu) per radial n
    std::vector<std::vector<std::vector<int>>> cond;    // cond[i][j] (i<=j): active n
    std::vector<std::vector<std::vector<int>>> lm_array; // per l_comb: m-combos as l*l+l+m
    std::vector<std::vector<int>> l_comb;
    std::vector<std::vector<double>> lm_coeffs;
};

// One (n, l, m, tp) element of the order parameters a_nlm for a centre type.
struct Nlmtp {
    int n = 0, n_id = 0, l = 0, m = 0, lm = 0, ylm_key = 0, tp = 0;
    bool conj = false;
    double cc = 1.0, sign_j = 1.0;
    int global_id = 0, global_conj_id = 0;
    int ilocal_id = 0, ilocal_noconj_id = 0, jlocal_noconj_id = 0, ilocal_conj_id = 0;
};

struct Ntp {
    int n = 0, n_id = 0, tp = 0, global_id = 0, ilocal_id = 0, jlocal_id = 0;
};

struct LinearTerm {
    int n = 0, lm_comb_id = 0, tp_comb_id = 0, order = 0;
    std::vector<int> type1;
};

// A product term coeff * prod(a[ids]) (ids are local full ids of a type).
struct Term {
    double coeff = 0.0;
    std::vector<int> ids;
};

// One derivative term: coeff * a[head] * prod(a[rest]).
struct DerivTerm {
    double coeff = 0.0;
    int head = 0;
    std::vector<int> rest;
};

struct PolyTerm {
    int col = 0;                 // global column of X
    std::vector<int> local_ids;  // local linear-feature indices (1..3)
};

struct PotTerm {
    double coeff_e = 0.0, coeff_f = 0.0;
    int prod_id = 0, prod_features_id = 0;
};

struct TypeTables {
    // gtinv: full (K) and no-conjugate (K0) order-parameter lists
    std::vector<Nlmtp> full, noconj;
    // pair: radial order parameters
    std::vector<Ntp> ntp;
    // linear features of this type (global linear index, in column order)
    std::vector<int> lin_index;
    // per linear feature: value terms (representative ids) and derivative terms
    std::vector<std::vector<Term>> value_terms;
    std::vector<std::vector<DerivTerm>> deriv_terms;
    // per linear feature: polynomial degree in a (size of its product terms)
    std::vector<int> feature_order;
    // polynomial terms (all columns that this type contributes to)
    std::vector<PolyTerm> poly;
    // prod_deriv keys (reference: Features::prod_deriv) and polynomial keys
    std::vector<std::vector<int>> prod_deriv;
    std::vector<std::vector<int>> prod_features;
};

struct ModelTables {
    FeatureParams fp;
    int n_type_pairs = 0;
    std::vector<std::vector<int>> type_pairs;   // [t1][t2] -> tp
    std::vector<std::array<int, 2>> tp_to_types;
    std::vector<std::vector<int>> tp_to_n;
    int n_lm = 0;                                // (maxl+1)^2
    int n_ylm = 0;                               // (maxl+1)(maxl+2)/2 (m <= 0)
    std::vector<LinearTerm> linear_terms;        // gtinv only
    std::vector<std::vector<std::vector<int>>> tp_combs;  // [order][id] -> tps
    int n_linear = 0;
    std::vector<std::vector<int>> comb2, comb3;
    int n_features = 0;
    std::vector<TypeTables> types;
};

// Build every table.  Throws std::runtime_error on invalid settings (where
// the reference calls exit(8)).
ModelTables build_model_tables(const FeatureParams& fp);

// Feature attributes as FeaturesAttr returns them
// (src/pypolymlp/cxx/src/compute/py_features_attr.cpp:11-60): per linear
// feature its radial id, invariant id (-1 for pair features) and type
// combination (type-pair ids); then the polynomial columns as lists of linear
// ids (second order, then third order).
struct FeatureAttrs {
    std::vector<int> radial_ids, gtinv_ids;
    std::vector<std::vector<int>> tcomb_ids, polynomial_ids;
};
FeatureAttrs feature_attrs(const ModelTables& mt);

// Evaluator terms (reference Potential::set_terms_using_mapping).  For gtinv
// the heads are no-conjugate local ids; for pair they are ntp local ids.
// Coefficients are used as given (the reference's 2x factor is applied by
// the caller).
std::vector<std::vector<std::vector<PotTerm>>> build_potential_terms(
    const ModelTables& mt, const std::vector<double>& pot);

}  // namespace pg
