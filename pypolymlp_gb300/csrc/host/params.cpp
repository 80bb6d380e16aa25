// Unpacks pg_feature_params (the flat form of the reference's feature_params,
// filled in src/pypolymlp/cxx/src/compute/py_params.cpp:11-60).
#include "params.h"

#include <stdexcept>
#include <string>

namespace pg {

FeatureParams feature_params_from_abi(const pg_feature_params* p) {
    if (!p) throw std::runtime_error("null feature params");
    if (p->n_type < 1 || p->n_type > 64) throw std::runtime_error("n_type out of range");
    if (p->n_fn < 1) throw std::runtime_error("no radial functions (pair_params is empty)");
    if (!(p->cutoff > 0.0)) throw std::runtime_error("cutoff must be positive");
    if (p->feature_type != 0 && p->feature_type != 1) throw std::runtime_error("unknown feature_type");
    if (p->max_l < 0 || p->max_l > 20) throw std::runtime_error("max_l out of range");
    FeatureParams fp;
    fp.n_type = p->n_type;
    fp.gtinv = p->feature_type == 1;
    fp.model_type = p->model_type;
    fp.maxp = p->max_p;
    fp.maxl = p->max_l;
    fp.cutoff = p->cutoff;
    for (int n = 0; n < p->n_fn; ++n) fp.params.push_back({p->pair_params[2 * n], p->pair_params[2 * n + 1]});
    fp.cond.assign(p->n_type, std::vector<std::vector<int>>(p->n_type));
    for (int i = 0; i < p->n_type; ++i)
        for (int j = i; j < p->n_type; ++j) {
            const int k = i * p->n_type + j;
            for (int q = p->cond_offsets[k]; q < p->cond_offsets[k + 1]; ++q) {
                const int n = p->cond_values[q];
                if (n < 0 || n >= p->n_fn) throw std::runtime_error("pair_params_conditional index out of range");
                fp.cond[i][j].push_back(n);
            }
        }
    if (fp.gtinv) {
        size_t vpos = 0;  // running offset into lmseq_values (orders differ per l_comb)
        for (int c = 0; c < p->n_lcomb; ++c) {
            std::vector<int> lc(p->lcomb_values + p->lcomb_offsets[c], p->lcomb_values + p->lcomb_offsets[c + 1]);
            const int order = (int)lc.size();
            if (order < 1 || order > 6) throw std::runtime_error("gtinv order must be 1..6");
            for (int l : lc)
                if (l < 0 || l > p->max_l) throw std::runtime_error("l in l_comb exceeds max_l");
            std::vector<std::vector<int>> lms;
            std::vector<double> cf;
            for (int q = p->lmseq_offsets[c]; q < p->lmseq_offsets[c + 1]; ++q) {
                std::vector<int> mc(p->lmseq_values + vpos, p->lmseq_values + vpos + order);
                vpos += order;
                for (int k = 0; k < order; ++k) {
                    const int l = lc[k], lm = mc[k];
                    if (lm < l * l || lm > l * l + 2 * l) throw std::runtime_error("lm_seq entry inconsistent with l_comb");
                }
                lms.push_back(mc);
                cf.push_back(p->lm_coeffs[q]);
            }
            fp.l_comb.push_back(lc);
            fp.lm_array.push_back(lms);
            fp.lm_coeffs.push_back(cf);
        }
        if (fp.l_comb.empty()) throw std::runtime_error("gtinv features need l_comb");
    }
    return fp;
}

}  // namespace pg
