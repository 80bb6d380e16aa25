/*
 * CPU oracle for the polynomial-MLP hot path.  TEST INFRASTRUCTURE ONLY:
 * only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may
 * load it, and only as the checker or the timed CPU baseline.  The product
 * (libpolymlp_gb300.so) never links or calls it.
 *
 * It restates, in plain C++ with OpenMP, the reference algorithm of
 * sekocha/pypolymlp for this path (file:line citations in oracle.cpp):
 * neighbour lists, radial functions and spherical harmonics, a_nlm and its
 * dense derivatives, invariant features and their derivatives, the
 * polynomial X rows, and the adjoint energy/force/stress evaluator.
 * It shares the host model-table builder with the product; that builder is
 * pinned separately against the compiled reference (feature counts,
 * attributes and X columns).
 */
#ifndef POLYMLP_ORACLE_H
#define POLYMLP_ORACLE_H

#include "polymlp_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

int or_last_error(char* buf, size_t len);
int or_n_features(const pg_feature_params* fp, int* n);
int or_features_x(const pg_feature_params* fp, const pg_structures* st, const int64_t* e_row,
                  const int64_t* f_row, const int64_t* s_row, double* x, int64_t ld, int n_threads);
int or_eval(const pg_feature_params* fp, const double* coeffs, int n_coeffs, const pg_structures* st,
            double* energy, double* forces, double* stress, int n_threads);
int or_neighbor_list(const pg_structures* st, int structure, double cutoff, int half, int64_t* n_entries,
                     int* offsets, int* neighbors, double* diffs);
int or_translations(const pg_structures* st, int structure, double cutoff, int* n_trans, double* trans,
                    double* positions_rev);
/* get_fn (radial functions and derivatives) and get_ylm (m <= 0 harmonics and
 * gradients, interleaved re/im) for single arguments. */
int or_fn(double dis, double cutoff, int n_fn, const double* params, double* fn, double* fn_d);
int or_ylm(double r, double x, double y, double z, int lmax, double* ylm, double* ylm_dx, double* ylm_dy,
           double* ylm_dz);

/* PolymlpAPI test surface (src/pypolymlp/cxx/src/polymlp/polymlp_api.cpp:62-190,
 * polymlp_features.cpp:155-248, polymlp_potential.cpp:203-295) for one atom
 * type; complex arrays interleave re/im.  sizes: [full a_nlm K, no-conjugate
 * K0, a_ntp, linear features, potential heads]. */
int or_api_sizes(const pg_feature_params* fp, int type, int* sizes);
int or_api_noconj_m(const pg_feature_params* fp, int type, int* m);
int or_api_conjugate(const pg_feature_params* fp, int type, const double* re, const double* im, double* a);
int or_api_features(const pg_feature_params* fp, int type, const double* a, double* out);
int or_api_features_deriv(const pg_feature_params* fp, int type, const double* a, const double* dax,
                          const double* day, const double* daz, const double* das, int n_col, double* ox,
                          double* oy, double* oz, double* os);
int or_api_sum_of_prod(const pg_feature_params* fp, const double* coeffs, int n_coeffs, int type, const double* a,
                       double* pe, double* pf);

#ifdef __cplusplus
}
#endif

#endif
