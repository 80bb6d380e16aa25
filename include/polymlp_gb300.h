/*
 * polymlp_gb300.h - C ABI of libpolymlp_gb300.so, the GB300 (sm_103a) hot path
 * of the polynomial machine-learning potential (pypolymlp).
 *
 * Every entry point returns 0 on success and a non-zero status on failure;
 * pg_last_error() returns the message of the last failure on this thread.
 * No entry point calls exit(), and none takes or returns torch types.
 * Buffers are caller-owned; host pointers unless a function says otherwise.
 *
 * Reference interfaces that these entry points replace are cited per
 * function (paths inside sekocha/pypolymlp).
 */
#ifndef POLYMLP_GB300_H
#define POLYMLP_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/*
 * Model settings.  Mirrors struct feature_params
 * (src/pypolymlp/cxx/src/polymlp/polymlp_mlpcpp.h:55), which the reference
 * fills from params.as_dict() in convert_params_dict_to_feature_params
 * (src/pypolymlp/cxx/src/compute/py_params.cpp:11).
 */
typedef struct pg_feature_params {
    int n_type;
    int feature_type;          /* 0 = "pair", 1 = "gtinv" */
    int model_type;            /* 1..4 */
    int max_p;                 /* 1..3 */
    int max_l;
    double cutoff;
    int n_fn;                  /* number of radial functions */
    const double* pair_params; /* n_fn x 2, row-major (beta, mu) */
    const int* cond_offsets;   /* n_type*n_type + 1 offsets; entry (i, j), i <= j, row-major */
    const int* cond_values;    /* active radial indices of each type pair */
    int n_lcomb;               /* gtinv: number of l combinations */
    const int* lcomb_offsets;  /* n_lcomb + 1 */
    const int* lcomb_values;   /* l values of each combination */
    const int* lmseq_offsets;  /* n_lcomb + 1, cumulative number of m-combinations */
    const int* lmseq_values;   /* per m-combination: order entries, each l*l+l+m */
    const double* lm_coeffs;   /* one coefficient per m-combination */
} pg_feature_params;

/*
 * A batch of periodic structures.  axis: n_st x 3 x 3 row-major, columns are
 * the lattice vectors (as PolymlpStructure.axis).  positions: Cartesian,
 * atom-major (sum(n_atoms) x 3).  types: sum(n_atoms) type indices.
 */
typedef struct pg_structures {
    int n_st;
    const int* n_atoms;
    const double* axis;
    const double* positions;
    const int* types;
} pg_structures;

typedef struct pg_model pg_model;
typedef struct pg_gram pg_gram;
typedef struct pg_eval pg_eval;
typedef struct pg_batch pg_batch;

enum { PG_FP64 = 0, PG_MIXED = 1 };

/* Message of the last failure on the calling thread (truncated to len). */
int pg_last_error(char* buf, size_t len);

/* Number of visible CUDA devices (0 when none); fails if the runtime is unusable. */
int pg_device_count(int* count);

/*
 * Model tables.  Replaces Model(fp) / PolymlpAPI::set_features
 * (src/pypolymlp/cxx/src/compute/model.cpp:11,
 *  src/pypolymlp/cxx/src/polymlp/polymlp_api.cpp:44).
 */
int pg_model_create(const pg_feature_params* fp, pg_model** out);
int pg_model_destroy(pg_model* m);
int pg_model_n_features(const pg_model* m, int* n_features);

/*
 * Feature attributes, as FeaturesAttr
 * (src/pypolymlp/cxx/src/compute/py_features_attr.cpp:11).  Sizes are written
 * to *n_linear (radial/gtinv/tcomb entries), *n_tcomb_values (flattened type
 * combinations) and *n_poly_values (flattened polynomial ids); pass NULL
 * arrays to query sizes.
 */
int pg_model_feature_attrs(const pg_model* m, int* n_linear, int* radial_ids, int* gtinv_ids,
                           int* n_tcomb_values, int* tcomb_offsets, int* tcomb_values,
                           int* n_poly, int* n_poly_values, int* poly_offsets, int* poly_values);

/*
 * The same attributes from the feature parameters alone, host only (no
 * device, no model handle), as the FeaturesAttr constructor
 * (src/pypolymlp/cxx/src/compute/py_features_attr.cpp:11-41).  type_pairs, if
 * non-NULL, receives the n_type x n_type type-pair ids, row-major
 * (FeaturesAttr::get_type_pairs).  gtinv_ids are -1 for pair features.
 */
int pg_feature_attrs(const pg_feature_params* fp, int* n_linear, int* radial_ids, int* gtinv_ids,
                     int* n_tcomb_values, int* tcomb_offsets, int* tcomb_values, int* n_poly,
                     int* n_poly_values, int* poly_offsets, int* poly_values, int* type_pairs);

/*
 * X rows of a batch of structures, as PotentialModel
 * (src/pypolymlp/cxx/src/compute/py_model.cpp:10-56 with Model::run,
 *  src/pypolymlp/cxx/src/compute/model.cpp:39).  For structure s, the energy
 * row is e_row[s]; if f_row[s] >= 0 the 3*n_atoms force rows start there
 * (atom-major x, y, z) and the 6 stress rows (xx, yy, zz, xy, yz, zx) start at
 * s_row[s].  x is column-major with leading dimension ld (>= every row used);
 * rows of this batch are overwritten, other rows are untouched.
 * precision: PG_FP64 or PG_MIXED (FP32 features, FP64 sums over neighbours).
 */
int pg_features_x(pg_model* m, const pg_structures* st, const int64_t* e_row,
                  const int64_t* f_row, const int64_t* s_row, double* x, int64_t ld,
                  int precision);

/*
 * The CUDA stream (a cudaStream_t, passed as void*) on which the calling
 * host thread's later calls issue their device work; NULL (the default) is
 * the legacy default stream.  Per host thread, as the reference's objects are
 * used one per thread (pybind11_mlp.cpp holds the GIL).  Every entry point
 * returns once its results are on the host, so the stream orders the
 * library's work against the caller's own work on it.  The allocation-free
 * solve (pg_solve_ridge_noalloc) always uses the legacy default stream.  No
 * reference counterpart (the reference has no device work).
 */
int pg_set_stream(void* stream);
int pg_get_stream(void** stream);

/*
 * Work figures of a model, for roofline accounting (no reference
 * counterpart): atom types, largest l, radial functions per type pair,
 * k0_pair[a * n_type + b] = a_nlm heads (m <= 0 entries) of a centre of type
 * a over its type-b neighbours (n_type^2; NULL to skip) and n_terms[a] =
 * product terms of the feature values and their adjoint for type a (n_type;
 * NULL to skip).
 */
int pg_model_work(const pg_model* m, int* n_type, int* max_l, int* n_radial, int* k0_pair, int64_t* n_terms);

/*
 * Force-row work of a model, for roofline accounting (no reference
 * counterpart): per centre type a and neighbour type b (n_type^2 each),
 * n_entries = adjoint entries by that type pair (the stage-A contraction per
 * pair) and n_positions = linear features with such entries.
 */
int pg_model_xrow_work(const pg_model* m, int* n_entries, int* n_positions);

/*
 * Fused regression assembly: X rows are generated on the device, weighted,
 * and summed into X^T X, X^T y, y^T y and the column sums of the (unweighted)
 * energy rows, without X leaving the GPU.  Replaces the sequential loop of
 * calc_xtx_xty (src/pypolymlp/mlp_dev/core/data_sequential.py:25-152) with its
 * numpy x.T @ x (src/pypolymlp/mlp_dev/core/utils_sequential.py:94).
 * w and y are per-row weights and weighted targets of this batch in the row
 * layout given by e_row/f_row/s_row (relative to the batch, ld = n_rows).
 */
int pg_gram_create(pg_model* m, int precision, pg_gram** out);
int pg_gram_destroy(pg_gram* g);
int pg_gram_accumulate(pg_gram* g, const pg_structures* st, const int64_t* e_row,
                       const int64_t* f_row, const int64_t* s_row, int64_t n_rows,
                       const double* w, const double* y);
/* Zero the sums of a pg_gram (same model and precision). */
int pg_gram_reset(pg_gram* g);
/* Results (host): xtx F x F (full symmetric), xty F, yty, xe_sum F, xe_sq_sum F, n_rows. */
int pg_gram_result(pg_gram* g, double* xtx, double* xty, double* yty, double* xe_sum,
                   double* xe_sq_sum, int64_t* n_rows_total);

/*
 * A batch staged on the device: structures (with translations and wrapped
 * positions from the host), row layout, weights and weighted targets.  The
 * same arguments as pg_gram_accumulate; pg_gram_accumulate_batch then does
 * only device work (neighbour lists, rows, X^T X, ...), so a batch can be
 * assembled repeatedly with its inputs resident in HBM.
 */
int pg_batch_create(pg_model* m, const pg_structures* st, const int64_t* e_row, const int64_t* f_row,
                    const int64_t* s_row, int64_t n_rows, const double* w, const double* y, int precision,
                    pg_batch** out);
int pg_batch_destroy(pg_batch* b);
/*
 * Neighbour pairs of the force structures of a batch by centre type and
 * neighbour type (counts[a * n_type + b], n_type^2 entries), from the
 * neighbour lists of its last pg_gram_accumulate_batch (zero before).
 */
int pg_batch_pair_counts(pg_batch* b, int n_type, int64_t* counts);
int pg_gram_accumulate_batch(pg_gram* g, pg_batch* b);
/*
 * X^T X of one host block X (n_rows x n_features, column-major, leading
 * dimension ld), on the device: the `xtx += x.T @ x` of calc_xtx_xty
 * (mlp_dev/core/data_sequential.py:145-152) for a block that is already
 * materialised.  PG_FP64: FP64 products and sums; PG_MIXED: X rounded to FP32,
 * then per 1,024-row segment and column split into four BF16 fixed-point
 * slices (28 bits of the segment's column maximum); 13 slice products on the
 * tensor cores with exact FP32 partial sums and float-float segment sums give
 * the Gram of those rows to ~1e-12.  xtx is F x F (full, symmetric).
 */
int pg_gram_xtx(const double* x, int64_t n_rows, int n_features, int64_t ld, int precision, double* xtx);

/*
 * Weighted residuals R = y - X C of a staged batch for n_coef (<= 16)
 * coefficient vectors C (F x n_coef, column-major, in X's own column scaling),
 * with the rows regenerated at the pg_gram's precision and accumulated in
 * FP64.  Writes X^T R (F x n_coef) and the sums of R^2 over energy, force and
 * stress rows (3 x n_coef, kind-major).  Used for the iterative refinement of
 * a fit (r = X^T (y - X c)) and for test-set RMSEs from residuals.
 */
int pg_batch_residual(pg_gram* g, pg_batch* b, const double* coefs, int n_coef, double* xtr, double* sq,
                      int64_t* n_rows);

/*
 * Ridge solve for every alpha on the device, as solver_ridge
 * (src/pypolymlp/mlp_dev/standard/solvers.py:48-84) with LAPACK posv: for each
 * alpha, Cholesky of xtx + alpha*I and two triangular solves.  All alphas are
 * factored together (one set of launches, no host round trip per alpha).
 * xtx (F x F) and xty (F) are host arrays; coefs is F x n_alpha column-major.
 * info[i] != 0 marks a failed factorisation, for which the column is filled
 * with 1e30.
 */
int pg_solve_ridge(int n_features, const double* xtx, const double* xty, const double* alphas,
                   int n_alpha, double* coefs, int* info);
/*
 * The same with one right-hand side per alpha: rhs is F x n_alpha
 * (column-major), column i solved with xtx + alphas[i]*I.  Iterative
 * refinement of a fit solves for per-alpha residuals; no reference
 * counterpart (posv's right-hand side, solvers.py:21-46, is the same X^T y for
 * every alpha).
 */
int pg_solve_ridge_rhs(int n_features, const double* xtx, const double* rhs, const double* alphas,
                       int n_alpha, double* coefs, int* info);

/*
 * Ridge solve that allocates no memory.  No counterpart in the reference: it
 * exists for callers that cannot allocate device memory at the point where
 * they solve - a host framework or inference server whose own allocator owns
 * the GPU's memory, or a loop that must never enter the allocator.  The
 * caller passes device buffers:
 * d_xtx (F x F, column-major, symmetric), d_xty (F) and d_coefs (F, written);
 * *info (host) is 0, or column + 1 of a failed factorisation (then d_coefs is
 * filled with 1e30), as for pg_solve_ridge with one alpha.  The factor is
 * built in a fixed device array inside the library: n_features must be at
 * most 1024 (larger sizes are rejected with an error), and each GPU that loads
 * the library keeps that array (about 8 MiB) until the process exits.  The
 * first call on a device looks up the array's address (cudaGetSymbolAddress).
 * All calls on a device share the array and it keeps the last call's
 * contents, so calls whose GPU work overlaps (other threads or streams) race.
 * Work is issued on the default stream and the call returns when it is done.
 */
int pg_solve_ridge_noalloc(int n_features, const double* d_xtx, const double* d_xty, double alpha,
                           double* d_coefs, int* info);

/*
 * Energy / force / stress evaluation, as PotentialPropertiesFast
 * (src/pypolymlp/cxx/src/compute/py_properties_fast.cpp:10-77 with
 *  PolymlpEval::eval, src/pypolymlp/cxx/src/compute/polymlp_eval.cpp:24).
 * coeffs are already divided by the column scales (as in polymlp.yaml).
 * energy: n_st; forces: sum(n_atoms) x 3 (atom-major); stress: n_st x 6 in
 * eV per cell (xx, yy, zz, xy, yz, zx).
 */
int pg_eval_create(const pg_feature_params* fp, const double* coeffs, int n_coeffs, int precision,
                   pg_eval** out);
int pg_eval_destroy(pg_eval* e);
int pg_eval_run(pg_eval* e, const pg_structures* st, double* energy, double* forces,
                double* stress);

/*
 * Repeated evaluation of the same atoms at new positions (molecular dynamics,
 * the ASE calculator's loop, calculator/utils/ase_calculator.py:63, and the
 * autograd wrapper).  pg_eval_bind stages the structures once and builds
 * their neighbour lists with cutoff + skin; pg_eval_update takes the atoms'
 * new Cartesian positions (same order as bound, sum(n_atoms) x 3) and only
 * refreshes the kept entries' displacements, unless some atom has moved more
 * than skin / 2 since the lists were built, when it rebuilds them (*rebuilt =
 * 1).  The cell, atom counts and types stay those bound.
 * pg_eval_bound_energy: energies only (no pair gradients: the forward pass of
 * E); pg_eval_bound_run: energies, forces and stresses (recomputing a_nlm:
 * the backward pass).  Results equal pg_eval_run's on the same positions up
 * to summation order.  pg_eval_workspace_bytes: device bytes the evaluator
 * holds (lists, a_nlm, adjoint and per-pair gradients; no per-atom
 * derivative arrays).  No reference counterpart (the reference rebuilds its
 * neighbour list per call).
 */
int pg_eval_bind(pg_eval* e, const pg_structures* st, double skin);
int pg_eval_update(pg_eval* e, const double* positions, int* rebuilt);
int pg_eval_bound_energy(pg_eval* e, double* energy);
int pg_eval_bound_run(pg_eval* e, double* energy, double* forces, double* stress);
int pg_eval_workspace_bytes(const pg_eval* e, int64_t* bytes);

/*
 * Per-kernel timing with CUDA events on the launching stream.  pg_profile_read
 * synchronises the device and returns, per kernel name, the summed launch
 * durations (ms) and launch counts recorded since the previous read; names are
 * NUL-separated in the names buffer.
 */
int pg_profile_enable(int on);
int pg_profile_read(char* names, size_t names_len, double* ms, int* launches, int max_names, int* n_names);

/*
 * Neighbour lists (test surface, as NeighborFull / NeighborHalf,
 * src/pypolymlp/cxx/src/compute/neighbor_full.cpp:10,
 * src/pypolymlp/cxx/src/compute/neighbor_half.cpp:10).  For one structure:
 * offsets (n_atoms + 1), neighbour index and displacement pos[j] - pos[i] + t
 * (3 per entry).  Pass NULL arrays to query *n_entries first.
 */
int pg_neighbor_list(const pg_structures* st, int structure, double cutoff, int half,
                     int64_t* n_entries, int* offsets, int* neighbors, double* diffs);

#ifdef __cplusplus
}
#endif

#endif /* POLYMLP_GB300_H */
