// C ABI of libpolymlp_gb300.so (declared in include/polymlp_gb300.h): model
// creation, X rows, neighbour lists.  The regression assembly, solver and
// evaluator entry points live in gram.cu, solve.cu and eval.cu.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <memory>
#include <map>
#include <mutex>
#include <numeric>

#include "host/cell.h"
#include "host/params.h"
#include "kernels.h"
#include "model.h"

namespace pg {

static thread_local std::string g_last_error;
void set_last_error(const std::string& msg) { g_last_error = msg; }

static thread_local cudaStream_t g_stream = nullptr;
cudaStream_t current_stream() { return g_stream; }

// ------------------------------------------------------------ profiler
namespace {
struct ProfRec {
    std::string name;
    cudaEvent_t a, b;
};
std::mutex g_prof_mu;
bool g_prof_on = std::getenv("PG_PROFILE") != nullptr;
std::vector<ProfRec> g_prof;
}  // namespace

ProfScope::ProfScope(const char* name, cudaStream_t st) : name_(name), st_(st) {
    if (!g_prof_on) return;
    cudaEventCreate(&a_);
    cudaEventCreate(&b_);
    cudaEventRecord(a_, st_);
}

ProfScope::~ProfScope() {
    if (!a_) return;
    cudaEventRecord(b_, st_);
    std::lock_guard<std::mutex> lk(g_prof_mu);
    g_prof.push_back(ProfRec{name_, a_, b_});
}

// ------------------------------------------------------------ DeviceModel
void DeviceModel::build(const FlatModel& fm, bool fp64) {
    if (fm.n_type > kMaxTypes) throw std::runtime_error("at most 8 atom types are supported on the device");
    bufs.clear();
    bufs.reserve(64 * kMaxTypes);
    auto up = [&](const auto& v) -> const void* {
        bufs.emplace_back();
        upload(bufs.back(), v);
        return bufs.back().template as<void>();
    };
    dm = DevModel{};
    dm.n_type = fm.n_type;
    dm.n_tp = fm.n_tp;
    dm.F = fm.n_features;
    dm.n_fn_max = fm.n_fn_max;
    dm.maxl = fm.maxl;
    dm.n_ylm = fm.n_ylm;
    dm.gtinv = fm.gtinv ? 1 : 0;
    dm.cutoff = fm.cutoff;
    dm.max_k0 = dm.max_lin = dm.max_k0tp = 1;
    for (const auto& ft : fm.types) {
        dm.max_k0 = std::max(dm.max_k0, ft.K0);
        dm.max_lin = std::max(dm.max_lin, ft.n_pos);
        for (int tp = 0; tp < fm.n_tp; ++tp)
            dm.max_k0tp = std::max(dm.max_k0tp, ft.tp_head_off[tp + 1] - ft.tp_head_off[tp]);
    }
    // the stride of the group vectors: a multiple of 4, so that stage B reads them as vectors
    dm.max_lin = (dm.max_lin + 3) & ~3;
    const int F = fm.n_features;
    const size_t smem_limit = 227 * 1024;
    if (rows_pairs_smem_bytes(dm, fp64, rows_pairs_chunk(dm, fp64)) > smem_limit)
        throw std::runtime_error("model too large for the pg_rows_pairs shared-memory layout");
    if (fm.n_tp > kMaxTypePairs) throw std::runtime_error("at most 64 type pairs are supported");
    dm.type_pairs = (const int*)up(fm.type_pairs);
    dm.tp_nfn = (const int*)up(fm.tp_nfn);
    dm.tp_beta = (const double*)up(fm.tp_beta);
    dm.tp_mu = (const double*)up(fm.tp_mu);
    dm.tp_beta_f = (const float*)up(std::vector<float>(fm.tp_beta.begin(), fm.tp_beta.end()));
    dm.tp_mu_f = (const float*)up(std::vector<float>(fm.tp_mu.begin(), fm.tp_mu.end()));
    dm.cutoff_f = (float)fm.cutoff;
    // FP32 squared distances carry a relative error below 1e-6
    dm.rc2_safe_f = (float)(fm.cutoff * fm.cutoff * (1.0 - 1e-5));
    dm.ylm_tab = (const double*)up(fm.ylm_tab);
    for (int t = 0; t < fm.n_type; ++t) {
        const FlatType& ft = fm.types[t];
        DevType& d = dm.types[t];
        d.K = ft.K;
        d.K0 = ft.K0;
        d.n_lin = ft.n_lin;
        d.head_nid = (const int*)up(ft.head_nid);
        d.head_key = (const int*)up(ft.head_key);
        d.head_m = (const int*)up(ft.head_m);
        d.full_src = (const int*)up(ft.full_src);
        d.full_is_conj = (const int*)up(ft.full_is_conj);
        d.full_cc = (const double*)up(ft.full_cc);
        d.full_cc_f = (const float*)up(std::vector<float>(ft.full_cc.begin(), ft.full_cc.end()));
        d.val_off = (const int*)up(ft.val_off);
        d.val_terms = (const FlatTerm*)up(ft.val_terms);
        d.col_ncomp = (const int*)up(ft.col_ncomp);
        d.comp_k = (const int*)up(ft.comp_k);
        std::vector<int2> pack(F);
        if (ft.n_lin >= 65536) throw std::runtime_error("too many linear features for the packed column recipes");
        for (int c = 0; c < F; ++c) {
            const int nc = ft.col_ncomp[c];
            if (nc > 3) throw std::runtime_error("polynomial order above 3 is not supported");
            int k[3] = {0, 0, 0};
            for (int q = 0; q < nc; ++q) k[q] = ft.comp_k[(size_t)c * 3 + q];
            pack[c] = make_int2(k[0] | (k[1] << 16), k[2] | (nc << 16));
        }
        d.col_pack = (const int2*)up(pack);
        std::vector<int> lin(ft.n_lin, -1), prod;
        for (int c = 0; c < F; ++c) {
            if (ft.col_ncomp[c] == 1) {
                const int k = ft.comp_k[(size_t)c * 3];
                if (lin[k] >= 0) throw std::runtime_error("internal: two linear columns for one feature");
                lin[k] = c;
            } else if (ft.col_ncomp[c] >= 2) {
                prod.push_back(c);
            }
        }
        d.n_prod = (int)prod.size();
        d.lin_col = (const int*)up(lin);
        d.prod_col = (const int*)up(prod);
        // product-column roles of stage B (host tables: 4 ints a role)
        static_assert(kRowRoles == kRowsThreads, "a stage-B thread per product-column role");
        d.prod_qok = ft.prod_qok;
        d.prod_qn = (const int*)up(ft.prod_qn);
        d.prod_q = (const int4*)up(ft.prod_q);
        d.n_groups = ft.n_groups;
        d.n_pos = ft.n_pos;
        d.lay_size = ft.lay_size;
        d.n_tpl = (int)ft.tpl_tp.size();
        d.lay_key = (const int*)up(ft.lay_key);
        d.lay_grp_base = (const int*)up(ft.lay_grp_base);
        d.lay_grp_cnt = (const int*)up(ft.lay_grp_cnt);
        d.lay_sched = (const int*)up(ft.lay_sched);
        d.n_rounds = ft.n_rounds;
        d.tp_perm = (const int*)up(ft.tp_perm);
        d.tp_ipos = (const int*)up(ft.tp_ipos);
        d.tp_pos_nid = (const int*)up(ft.tp_pos_nid);
        d.tp_nnz = (const int*)up(ft.tp_nnz);
        d.tpl = (const int*)up(ft.tpl);
        d.tpl_tp = (const int*)up(ft.tpl_tp);
        d.tp_head_off = (const int*)up(ft.tp_head_off);
        d.tp_heads = (const int*)up(ft.tp_heads);
        // adjoint terms in slot order, for pg_features_adjoint
        if (ft.K >= 65536) throw std::runtime_error("too many a_nlm entries for the packed term ids");
        std::vector<int> slot_toff(ft.lay_size + 1, 0);
        std::vector<int4> tcode;
        std::vector<double> tcoef;
        for (int sl = 0; sl < ft.lay_size; ++sl) {
            const int e = ft.lay_ent[sl];
            if (e >= 0) {
                const double cc = (ft.head_m[ft.ent_head[e]] & 1) ? -1.0 : 1.0;
                for (int q = ft.term_off[e]; q < ft.term_off[e + 1]; ++q) {
                    const FlatTerm& t = ft.g_terms[q];
                    int id[6] = {0, 0, 0, 0, 0, 0};
                    for (int r = 0; r < t.n; ++r) id[r] = t.ids[r];
                    tcode.push_back(make_int4(id[0] | (id[1] << 16), id[2] | (id[3] << 16), id[4] | (id[5] << 16),
                                              t.n | (t.conj << 8)));
                    tcoef.push_back(t.conj ? cc * t.coeff : t.coeff);
                }
            }
            slot_toff[sl + 1] = (int)tcode.size();
        }
        d.slot_toff = (const int*)up(slot_toff);
        d.tcode = (const int4*)up(tcode);
        if (fp64) {
            d.tcoef = up(tcoef);
        } else {
            d.tcoef = up(std::vector<float>(tcoef.begin(), tcoef.end()));
        }
        // feature-value terms in the same packed form (feature k owns val_off[k] ..)
        std::vector<int4> vcode;
        std::vector<double> vcoef;
        for (const FlatTerm& t : ft.val_terms) {
            int id[6] = {0, 0, 0, 0, 0, 0};
            for (int r = 0; r < t.n; ++r) id[r] = t.ids[r];
            vcode.push_back(make_int4(id[0] | (id[1] << 16), id[2] | (id[3] << 16), id[4] | (id[5] << 16), t.n));
            vcoef.push_back(t.coeff);
        }
        d.vcode = (const int4*)up(vcode);
        if (fp64) {
            d.vcoef = up(vcoef);
        } else {
            d.vcoef = up(std::vector<float>(vcoef.begin(), vcoef.end()));
        }
    }
}

// ------------------------------------------------------------ DeviceBatch
void DeviceBatch::upload_structures(const pg_structures* st, int s_begin, int s_end, double cutoff) {
    n_st = s_end - s_begin;
    long long off0 = 0;
    for (int s = 0; s < s_begin; ++s) off0 += st->n_atoms[s];
    st_atom_off.assign(1, 0);
    st_trans_off.assign(1, 0);
    types.clear();
    atom_st.clear();
    trans.clear();
    pos.clear();
    std::vector<int> st_cl, cl_bin_start(1, 0), cl_atoms;
    std::vector<int4> cl_grid, tn;
    std::vector<double> cl_geom, frac;
    n_cl = 0;
    long long a = off0;
    for (int s = s_begin; s < s_end; ++s) {
        const int n = st->n_atoms[s];
        if (n < 0) throw std::runtime_error("negative atom count");
        for (int i = 0; i < n; ++i) {
            const int t = st->types[a + i];
            if (t < 0) throw std::runtime_error("negative atom type");
        }
        const CellTranslations ct = cell_translations(st->axis + 9 * (size_t)s, st->positions + 3 * a, n, cutoff);
        for (const auto& t : ct.trans) trans.insert(trans.end(), t.begin(), t.end());
        for (const auto& t : ct.tn) tn.push_back(make_int4(t[0], t[1], t[2], 0));
        // fractional coordinates (all atoms; used by cell-list structures)
        double inv[3][3];
        {
            const double(&m)[3][3] = ct.axis;
            const double det = m[0][0] * (m[1][1] * m[2][2] - m[1][2] * m[2][1]) -
                               m[0][1] * (m[1][0] * m[2][2] - m[1][2] * m[2][0]) +
                               m[0][2] * (m[1][0] * m[2][1] - m[1][1] * m[2][0]);
            inv[0][0] = (m[1][1] * m[2][2] - m[1][2] * m[2][1]) / det;
            inv[0][1] = (m[0][2] * m[2][1] - m[0][1] * m[2][2]) / det;
            inv[0][2] = (m[0][1] * m[1][2] - m[0][2] * m[1][1]) / det;
            inv[1][0] = (m[1][2] * m[2][0] - m[1][0] * m[2][2]) / det;
            inv[1][1] = (m[0][0] * m[2][2] - m[0][2] * m[2][0]) / det;
            inv[1][2] = (m[0][2] * m[1][0] - m[0][0] * m[1][2]) / det;
            inv[2][0] = (m[1][0] * m[2][1] - m[1][1] * m[2][0]) / det;
            inv[2][1] = (m[0][1] * m[2][0] - m[0][0] * m[2][1]) / det;
            inv[2][2] = (m[0][0] * m[1][1] - m[0][1] * m[1][0]) / det;
        }
        const size_t f0 = frac.size();
        for (int i = 0; i < n; ++i)
            for (int r = 0; r < 3; ++r)
                frac.push_back(inv[r][0] * ct.pos[i][0] + inv[r][1] * ct.pos[i][1] + inv[r][2] * ct.pos[i][2]);
        if (n >= kCellListMinAtoms) {
            // bins of at least rc in each direction over the atoms' fractional range; a
            // sphere of radius rc spans at most rc / h_d in fractional coordinate d
            // (h_d the cell height across the other two lattice vectors)
            double fmin[3], fmax[3], h[3], scale[3], rq[3];
            int g[3];
            const double(&m)[3][3] = ct.axis;
            const double vol = std::fabs(m[0][0] * (m[1][1] * m[2][2] - m[1][2] * m[2][1]) -
                                         m[0][1] * (m[1][0] * m[2][2] - m[1][2] * m[2][0]) +
                                         m[0][2] * (m[1][0] * m[2][1] - m[1][1] * m[2][0]));
            for (int d = 0; d < 3; ++d) {
                const int e = (d + 1) % 3, f = (d + 2) % 3;
                const double cx = m[1][e] * m[2][f] - m[2][e] * m[1][f];
                const double cy = m[2][e] * m[0][f] - m[0][e] * m[2][f];
                const double cz = m[0][e] * m[1][f] - m[1][e] * m[0][f];
                h[d] = vol / std::sqrt(cx * cx + cy * cy + cz * cz);
                fmin[d] = 1e300;
                fmax[d] = -1e300;
                for (int i = 0; i < n; ++i) {
                    fmin[d] = std::min(fmin[d], frac[f0 + 3 * i + d]);
                    fmax[d] = std::max(fmax[d], frac[f0 + 3 * i + d]);
                }
                const double span = fmax[d] - fmin[d] + 1e-9;
                g[d] = std::max(1, std::min(256, (int)std::floor(h[d] * span / cutoff)));
                scale[d] = g[d] / span;
                rq[d] = cutoff / h[d] * (1.0 + 1e-9) + 1e-12;
            }
            const int nb = g[0] * g[1] * g[2];
            std::vector<std::vector<int>> bins(nb);
            for (int i = 0; i < n; ++i) {
                int bi[3];
                for (int d = 0; d < 3; ++d)
                    bi[d] = std::min(g[d] - 1, std::max(0, (int)std::floor((frac[f0 + 3 * i + d] - fmin[d]) * scale[d])));
                bins[(bi[2] * g[1] + bi[1]) * g[0] + bi[0]].push_back((int)(pos.size() / 3) + i);
            }
            st_cl.push_back(n_cl++);
            cl_grid.push_back(make_int4(g[0], g[1], g[2], (int)cl_bin_start.size() - 1));
            for (int d = 0; d < 3; ++d) cl_geom.push_back(fmin[d]);
            for (int d = 0; d < 3; ++d) cl_geom.push_back(scale[d]);
            for (int d = 0; d < 3; ++d) cl_geom.push_back(rq[d]);
            for (const auto& b : bins) {
                cl_atoms.insert(cl_atoms.end(), b.begin(), b.end());
                cl_bin_start.push_back((int)cl_atoms.size());
            }
        } else {
            st_cl.push_back(-1);
        }
        for (int i = 0; i < n; ++i) {
            pos.insert(pos.end(), ct.pos[i].begin(), ct.pos[i].end());
            types.push_back(st->types[a + i]);
            atom_st.push_back(s - s_begin);
        }
        st_atom_off.push_back(st_atom_off.back() + n);
        st_trans_off.push_back((int)(trans.size() / 3));
        if ((long long)n * (st_trans_off.back() - st_trans_off[st_trans_off.size() - 2]) >= (1LL << 31))
            throw std::runtime_error("structure too large: atoms x lattice translations must stay below 2^31");
        a += n;
    }
    n_atoms = st_atom_off.back();
    coord_max = 0.0;
    std::vector<float4> posf(pos.size() / 3), transf(trans.size() / 3);
    for (size_t q = 0; q < posf.size(); ++q) {
        posf[q] = make_float4((float)pos[3 * q], (float)pos[3 * q + 1], (float)pos[3 * q + 2], 0.f);
        for (int c = 0; c < 3; ++c) coord_max = std::max(coord_max, std::fabs(pos[3 * q + c]));
    }
    for (size_t q = 0; q < transf.size(); ++q) {
        transf[q] = make_float4((float)trans[3 * q], (float)trans[3 * q + 1], (float)trans[3 * q + 2], 0.f);
        for (int c = 0; c < 3; ++c) coord_max = std::max(coord_max, std::fabs(trans[3 * q + c]));
    }
    upload(d_posf, posf);
    upload(d_transf, transf);
    upload(d_st_cl, st_cl);
    upload(d_cl_grid, cl_grid);
    upload(d_cl_geom, cl_geom);
    upload(d_cl_bin_start, cl_bin_start);
    upload(d_cl_atoms, cl_atoms);
    upload(d_frac, frac);
    upload(d_tn, tn);
    if (d_maxcnt.bytes() == 0) d_maxcnt.alloc(sizeof(int));
    upload(d_st_atom_off, st_atom_off);
    upload(d_st_trans_off, st_trans_off);
    upload(d_trans, trans);
    upload(d_pos, pos);
    upload(d_types, types);
    upload(d_atom_st, atom_st);
    d_counts.reserve(sizeof(int) * std::max(1, n_atoms));
    d_nb_off.reserve(sizeof(long long) * (n_atoms + 1));
    d_total.reserve(sizeof(long long));
}

// Count candidates, scan on the device, then fill in the reference's order.
void DeviceBatch::build_neighbors(double cutoff, cudaStream_t stream) {
    const DevBatch B = view(cutoff);
    if (n_atoms == 0) {
        n_pairs = 0;
        nb_off.assign(1, 0);
        PG_CUDA(cudaMemsetAsync(d_nb_off.as<void>(), 0, sizeof(long long), stream));
        return;
    }
    PG_CUDA(cudaMemsetAsync(d_maxcnt.as<void>(), 0, sizeof(int), stream));
    {
        ProfScope ps("pg_nb_count", stream);
        launch_nb_count(B, d_counts.as<int>(), d_maxcnt.as<int>(), stream);
    }
    launch_exclusive_scan(d_counts.as<int>(), n_atoms, d_nb_off.as<long long>(), d_total.as<long long>(), stream);
    long long total = 0;
    int maxcnt = 0;
    PG_CUDA(cudaMemcpyAsync(&total, d_total.as<long long>(), sizeof(long long), cudaMemcpyDeviceToHost, stream));
    PG_CUDA(cudaMemcpyAsync(&maxcnt, d_maxcnt.as<int>(), sizeof(int), cudaMemcpyDeviceToHost, stream));
    PG_CUDA(cudaStreamSynchronize(stream));
    if (maxcnt > kCellListMaxPairs)
        throw std::runtime_error("more than 4096 neighbours of one atom in a large structure");
    n_pairs = total;
    d_nb_j.reserve(sizeof(int) * std::max<long long>(1, n_pairs));
    d_nb_d.reserve(sizeof(double) * 3 * std::max<long long>(1, n_pairs));
    d_keys.reserve(sizeof(long long) * std::max<long long>(1, n_pairs));
    d_nb_df.reserve(sizeof(float4) * std::max<long long>(1, n_pairs));
    ProfScope ps("pg_nb_fill", stream);
    launch_nb_fill(B, d_nb_off.as<long long>(), d_nb_j.as<int>(), d_nb_d.as<double>(), d_nb_df.as<float4>(),
                   d_keys.as<long long>(), n_cl > 0, stream);
}

void DeviceBatch::stage(const pg_structures* st, int s_begin, int s_end, double cutoff, cudaStream_t stream) {
    upload_structures(st, s_begin, s_end, cutoff);
    build_neighbors(cutoff, stream);
}

void DeviceBatch::host_offsets() {
    nb_off.assign(n_atoms + 1, 0);
    copy_d2h(nb_off.data(), d_nb_off.as<long long>(), sizeof(long long) * (n_atoms + 1));
}

DevBatch DeviceBatch::view(double cutoff) const {
    DevBatch B;
    B.n_st = n_st;
    B.n_atoms = n_atoms;
    B.st_atom_off = d_st_atom_off.as<int>();
    B.st_trans_off = d_st_trans_off.as<int>();
    B.trans = d_trans.as<double>();
    B.pos = d_pos.as<double>();
    B.types = d_types.as<int>();
    B.atom_st = d_atom_st.as<int>();
    B.posf = d_posf.as<float4>();
    B.transf = d_transf.as<float4>();
    B.st_cl = d_st_cl.as<int>();
    B.cl_grid = d_cl_grid.as<int4>();
    B.cl_geom = d_cl_geom.as<double>();
    B.cl_bin_start = d_cl_bin_start.as<int>();
    B.cl_atoms = d_cl_atoms.as<int>();
    B.frac = d_frac.as<double>();
    B.tn = d_tn.as<int4>();
    B.nb_df = d_nb_df.as<float4>();
    B.cutoff = cutoff;
    // FP32 differences of coordinates up to L carry an error below 4 L 2^-24 per
    // component, so |r2_f32 - r2| < 2 rc (12 L 2^-24) + O(L^2 2^-48) + the FP32
    // rounding of r2; the margin below covers that with a factor > 10
    const double L = std::max(1.0, coord_max);
    B.prefilter_r2 = (float)(cutoff * cutoff * (1.0 + 1e-4) + 1e-5 * L * (cutoff + L) + 1e-3);
    B.inner_r2 = (float)std::max(0.0, cutoff * cutoff * (1.0 - 1e-4) - 1e-5 * L * (cutoff + L) - 1e-3);
    return B;
}

// ------------------------------------------------------------ Model
Model::Model(const pg_feature_params* p)
    : tables(build_model_tables(feature_params_from_abi(p))), flat(flatten_model(tables)) {
    int dev = 0;
    PG_CUDA(cudaGetDevice(&dev));
    dev64.build(flat, true);
    dev32.build(flat, false);
    s_missing.alloc(sizeof(int));
    zero_async(s_missing.as<void>(), sizeof(int));
    max_k = max_k0 = 1;
    for (const auto& ft : flat.types) {
        max_k = std::max(max_k, ft.K);
        max_k0 = std::max(max_k0, ft.K0);
    }
}

// Per-atom storage offsets of a staged batch: a_nlm (K0), features (n_lin),
// adjoint entries in the X-row layout (lay_size), self/virial vectors
// (9 x n_pos feature positions per type pair of the centre type).
void Model::atom_offsets(const DeviceBatch& b, AtomOffsets& o) const {
    o.a_off.resize(b.n_atoms);
    o.d_off.resize(b.n_atoms);
    o.g_off.resize(b.n_atoms);
    o.s_off.resize(b.n_atoms);
    o.a_tot = o.d_tot = o.g_tot = o.s_tot = 0;
    for (int i = 0; i < b.n_atoms; ++i) {
        const auto& ft = flat.types[b.types[i]];
        o.a_off[i] = o.a_tot;
        o.d_off[i] = o.d_tot;
        o.g_off[i] = o.g_tot;
        o.s_off[i] = o.s_tot;
        o.a_tot += ft.K0;
        o.d_tot += ft.n_lin;
        o.g_tot += ft.lay_size;
        o.s_tot += 9LL * ft.n_pos * (long long)ft.tpl_tp.size();
    }
}

size_t Model::bytes_per_atom(bool fp64, double mean_pairs) const {
    const size_t ts = fp64 ? 8 : 4;
    size_t mx = 0;
    for (const auto& ft : flat.types) {
        // a_nlm, features, self/virial vectors (9 per feature) and G
        const size_t b = (size_t)ft.K0 * 16 + (size_t)ft.n_lin * ts + (size_t)ft.n_pos * ts * 9 * ft.tpl_tp.size() +
                         (size_t)ft.lay_size * 2 * ts;
        mx = std::max(mx, b);
    }
    size_t max_lin = 1;
    for (const auto& ft : flat.types) max_lin = std::max<size_t>(max_lin, ft.n_pos);
    // per pair: index, key, FP64 and FP32 displacements, mirror, group slot, order and
    // the pair derivatives (3 per feature); X rows
    return mx + (size_t)(mean_pairs * (72.0 + 3.0 * max_lin * ts)) + (size_t)flat.n_features * 3 * ts;
}

// Per-batch plan: per-atom storage offsets and pg_rows work items.
void Model::plan_rows(const DeviceBatch& b, RowPlan& plan) const {
    AtomOffsets o;
    atom_offsets(b, o);
    plan.a_tot = o.a_tot;
    plan.d_tot = o.d_tot;
    plan.g_tot = o.g_tot;
    plan.s_tot = o.s_tot;
    upload(plan.d_a_off, o.a_off);
    upload(plan.d_d_off, o.d_off);
    upload(plan.d_g_off, o.g_off);
    upload(plan.d_s_off, o.s_off);
}

// Rows of one uploaded batch into Xd (device, column-major, leading dim ld), in
// the batch-local row layout given by e_row/f_row/s_row (device arrays):
// neighbour lists, a_nlm, features + adjoint, force/stress rows, energy/stress sums.
template <typename T>
void Model::run_rows(DeviceBatch& b, const RowPlan& plan, const long long* d_e_row, const long long* d_f_row,
                     const long long* d_s_row, T* Xd, long long ld, cudaStream_t stream) {
    const bool fp64 = sizeof(T) == 8;
    const DeviceModel& dmod = fp64 ? dev64 : dev32;
    b.build_neighbors(flat.cutoff, stream);
    const DevBatch B = b.view(flat.cutoff);
    s_A.reserve(2 * sizeof(T) * std::max<long long>(1, plan.a_tot));
    s_D.reserve(sizeof(T) * std::max<long long>(1, plan.d_tot));
    s_G.reserve(2 * sizeof(T) * std::max<long long>(1, plan.g_tot));
    if (b.n_atoms > 0) {
        {
            ProfScope ps("pg_anlm", stream);
            launch_anlm<T>(dmod.dm, B, b.d_nb_off.as<long long>(), b.d_nb_j.as<int>(), b.d_nb_d.as<double>(),
                           plan.d_a_off.as<long long>(), s_A.as<void>(), max_k0, stream);
        }
        {
            ProfScope ps("pg_features_adjoint", stream);
            launch_features_adjoint<T>(dmod.dm, B, plan.d_a_off.as<long long>(), s_A.as<void>(),
                                       plan.d_d_off.as<long long>(), s_D.as<T>(), plan.d_g_off.as<long long>(),
                                       s_G.as<void>(), max_k, stream);
        }
    }
    s_DS.reserve(sizeof(T) * std::max<long long>(1, plan.s_tot));
    s_mirror.reserve(sizeof(long long) * std::max<long long>(1, b.n_pairs));
    s_gslot.reserve(sizeof(long long) * std::max<long long>(1, b.n_pairs));
    s_order.reserve(sizeof(int) * std::max<long long>(1, b.n_pairs));
    s_Dp.reserve(3 * sizeof(T) * (size_t)dmod.dm.max_lin * std::max<long long>(1, b.n_pairs));
    PG_CUDA(cudaMemsetAsync(Xd, 0, sizeof(T) * (size_t)ld * flat.n_features, stream));
    if (b.n_atoms > 0) {
        {
            ProfScope ps("pg_nb_mirror", stream);
            launch_nb_mirror(b.n_atoms, b.d_nb_off.as<long long>(), b.d_nb_j.as<int>(), b.d_nb_d.as<double>(),
                             s_mirror.as<long long>(), s_gslot.as<long long>(), s_missing.as<int>(), stream);
        }
        {
            ProfScope ps("pg_rows_pairs", stream);
            launch_rows_pairs<T>(dmod.dm, B, b.d_nb_off.as<long long>(), b.d_nb_j.as<int>(), b.d_nb_d.as<double>(),
                                 s_gslot.as<long long>(), plan.d_s_off.as<long long>(), plan.d_g_off.as<long long>(),
                                 s_G.as<void>(), d_f_row, s_order.as<int>(), s_Dp.as<T>(), s_DS.as<T>(), stream);
        }
        {
            ProfScope ps("pg_rows", stream);
            launch_rows<T>(dmod.dm, B, b.d_nb_off.as<long long>(), b.d_nb_j.as<int>(), plan.d_d_off.as<long long>(),
                           s_D.as<T>(), s_Dp.as<T>(), plan.d_s_off.as<long long>(), s_DS.as<T>(), d_f_row, Xd, ld,
                           stream);
        }
    }
    if (b.n_st > 0) {
        ProfScope ps("pg_rows_es", stream);
        launch_rows_es<T>(dmod.dm, B, plan.d_d_off.as<long long>(), s_D.as<T>(), plan.d_s_off.as<long long>(),
                          s_DS.as<T>(), d_e_row, d_f_row, d_s_row, Xd, ld, stream);
    }
    PG_CUDA(cudaGetLastError());
}

template <typename T>
void Model::batch_rows(DeviceBatch& b, const long long* d_e_row, const long long* d_f_row,
                       const long long* d_s_row, T* Xd, long long ld, cudaStream_t stream) {
    RowPlan plan;
    plan_rows(b, plan);
    run_rows<T>(b, plan, d_e_row, d_f_row, d_s_row, Xd, ld, stream);
    PG_CUDA(cudaStreamSynchronize(stream));
    check_mirrors();
}

// A pair without its exact mirror would mean an asymmetric neighbour list
// (its force contribution is then dropped).  The counter accumulates over
// batches until read here, after the work that fed it has completed.
void Model::check_mirrors() {
    int missing = 0;
    copy_d2h(&missing, s_missing.as<int>(), sizeof(int));
    if (missing) {
        zero_async(s_missing.as<void>(), sizeof(int));
        throw std::runtime_error("internal: neighbour list is not symmetric");
    }
}

template void Model::run_rows<double>(DeviceBatch&, const RowPlan&, const long long*, const long long*,
                                      const long long*, double*, long long, cudaStream_t);
template void Model::run_rows<float>(DeviceBatch&, const RowPlan&, const long long*, const long long*,
                                     const long long*, float*, long long, cudaStream_t);
template void Model::batch_rows<double>(DeviceBatch&, const long long*, const long long*, const long long*, double*,
                                        long long, cudaStream_t);
template void Model::batch_rows<float>(DeviceBatch&, const long long*, const long long*, const long long*, float*,
                                       long long, cudaStream_t);

// Split [0, n_st) into batches whose staged data fits the device memory limit.  Pairs
// per atom are estimated from each cell's density: N / V * 4/3 pi rc^3, with a
// margin for clustering.
std::vector<std::pair<int, int>> Model::plan_batches(const pg_structures* st, bool fp64, size_t limit) const {
    std::vector<std::pair<int, int>> out;
    const double rc = flat.cutoff;
    const double sphere = 4.0 / 3.0 * 3.14159265358979323846 * rc * rc * rc;
    int s0 = 0;
    double acc = 0.0;
    for (int s = 0; s < st->n_st; ++s) {
        const double* a = st->axis + 9 * (size_t)s;  // row-major, columns are lattice vectors
        const double vol = std::fabs(a[0] * (a[4] * a[8] - a[5] * a[7]) - a[1] * (a[3] * a[8] - a[5] * a[6]) +
                                     a[2] * (a[3] * a[7] - a[4] * a[6]));
        const int n = st->n_atoms[s];
        const double pairs = vol > 0.0 ? 1.5 * n / vol * sphere + 8.0 : 300.0;
        const double bytes = (double)n * (double)bytes_per_atom(fp64, pairs);
        if (s > s0 && acc + bytes > (double)limit) {
            out.push_back({s0, s});
            s0 = s;
            acc = 0.0;
        }
        acc += bytes;
    }
    if (s0 < st->n_st) out.push_back({s0, st->n_st});
    return out;
}

size_t device_batch_bytes() {
    if (const char* e = std::getenv("PG_BATCH_BYTES")) return (size_t)std::atoll(e);
    size_t free_b = 0, total_b = 0;
    PG_CUDA(cudaMemGetInfo(&free_b, &total_b));
    return (size_t)(0.55 * (double)free_b);
}

__global__ void pg_f32_to_f64(const float* src, double* dst, size_t n) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        dst[i] = (double)src[i];
}

}  // namespace pg

using namespace pg;


extern "C" {

int pg_last_error(char* buf, size_t len) {
    if (buf && len) {
        std::strncpy(buf, g_last_error.c_str(), len - 1);
        buf[len - 1] = 0;
    }
    return 0;
}

int pg_set_stream(void* stream) {
    g_stream = static_cast<cudaStream_t>(stream);
    return 0;
}

int pg_get_stream(void** stream) {
    return guarded([&] {
        if (!stream) throw std::runtime_error("null argument");
        *stream = static_cast<void*>(g_stream);
    });
}

int pg_device_count(int* count) {
    return guarded([&] {
        int n = 0;
        cudaError_t e = cudaGetDeviceCount(&n);
        if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) n = 0;
        else if (e != cudaSuccess) throw std::runtime_error(cudaGetErrorString(e));
        *count = n;
    });
}

int pg_model_create(const pg_feature_params* fp, pg_model** out) {
    return guarded([&] {
        if (!out) throw std::runtime_error("null output handle");
        auto h = new pg_model;
        try {
            h->m = std::make_unique<Model>(fp);
        } catch (...) {
            delete h;
            throw;
        }
        *out = h;
    });
}

int pg_model_destroy(pg_model* m) {
    return guarded([&] { delete m; });
}

int pg_model_n_features(const pg_model* m, int* n) {
    return guarded([&] {
        if (!m) throw std::runtime_error("null model");
        *n = m->m->flat.n_features;
    });
}

namespace {

// Flattened FeatureAttrs into the caller's arrays (sizes always written;
// arrays filled when radial_ids is non-null).
void write_feature_attrs(const pg::ModelTables& mt, int* n_linear, int* radial_ids, int* gtinv_ids,
                         int* n_tcomb_values, int* tcomb_offsets, int* tcomb_values, int* n_poly,
                         int* n_poly_values, int* poly_offsets, int* poly_values) {
    if (!n_linear || !n_tcomb_values || !n_poly || !n_poly_values) throw std::runtime_error("null size output");
    const pg::FeatureAttrs a = pg::feature_attrs(mt);
    int ntv = 0, npv = 0;
    for (const auto& v : a.tcomb_ids) ntv += (int)v.size();
    for (const auto& v : a.polynomial_ids) npv += (int)v.size();
    *n_linear = (int)a.radial_ids.size();
    *n_tcomb_values = ntv;
    *n_poly = (int)a.polynomial_ids.size();
    *n_poly_values = npv;
    if (!radial_ids) return;
    if (!tcomb_offsets || !tcomb_values || !poly_offsets || !poly_values) throw std::runtime_error("null array output");
    int k = 0;
    tcomb_offsets[0] = 0;
    for (size_t i = 0; i < a.radial_ids.size(); ++i) {
        radial_ids[i] = a.radial_ids[i];
        if (gtinv_ids) gtinv_ids[i] = a.gtinv_ids.empty() ? -1 : a.gtinv_ids[i];
        for (int v : a.tcomb_ids[i]) tcomb_values[k++] = v;
        tcomb_offsets[i + 1] = k;
    }
    k = 0;
    poly_offsets[0] = 0;
    for (size_t i = 0; i < a.polynomial_ids.size(); ++i) {
        for (int v : a.polynomial_ids[i]) poly_values[k++] = v;
        poly_offsets[i + 1] = k;
    }
}

}  // namespace

int pg_model_feature_attrs(const pg_model* m, int* n_linear, int* radial_ids, int* gtinv_ids, int* n_tcomb_values,
                           int* tcomb_offsets, int* tcomb_values, int* n_poly, int* n_poly_values,
                           int* poly_offsets, int* poly_values) {
    return guarded([&] {
        if (!m) throw std::runtime_error("null model");
        write_feature_attrs(m->m->tables, n_linear, radial_ids, gtinv_ids, n_tcomb_values, tcomb_offsets,
                            tcomb_values, n_poly, n_poly_values, poly_offsets, poly_values);
    });
}

int pg_model_work(const pg_model* m, int* n_type, int* max_l, int* n_radial, int* k0_pair, int64_t* n_terms) {
    return guarded([&] {
        if (!m || !n_type || !max_l || !n_radial) throw std::runtime_error("null argument");
        const pg::FlatModel& fm = m->m->flat;
        *n_type = fm.n_type;
        *max_l = fm.maxl;
        *n_radial = fm.n_fn_max;
        for (int a = 0; a < fm.n_type; ++a) {
            const pg::FlatType& T = fm.types[a];
            if (k0_pair)
                for (int b = 0; b < fm.n_type; ++b) {
                    const int tp = fm.type_pairs[a * fm.n_type + b];
                    k0_pair[a * fm.n_type + b] =
                        (tp >= 0 && tp + 1 < (int)T.tp_head_off.size()) ? T.tp_head_off[tp + 1] - T.tp_head_off[tp] : 0;
                }
            if (n_terms) n_terms[a] = (int64_t)T.val_terms.size() + (int64_t)T.g_terms.size();
        }
    });
}

int pg_model_xrow_work(const pg_model* m, int* n_entries, int* n_positions) {
    return guarded([&] {
        if (!m || !n_entries || !n_positions) throw std::runtime_error("null argument");
        const pg::FlatModel& fm = m->m->flat;
        const int nt = fm.n_type, ntp = fm.n_tp;
        for (int a = 0; a < nt; ++a) {
            const pg::FlatType& T = fm.types[a];
            for (int b = 0; b < nt; ++b) {
                const int tp = fm.type_pairs[a * nt + b];
                int ne = 0, np = 0;
                for (int k = 0; tp >= 0 && k < T.n_lin; ++k) {
                    const int c = T.ent_tp_off[(size_t)k * (ntp + 1) + tp + 1] - T.ent_tp_off[(size_t)k * (ntp + 1) + tp];
                    ne += c;
                    np += c > 0;
                }
                n_entries[a * nt + b] = ne;
                n_positions[a * nt + b] = np;
            }
        }
    });
}

int pg_feature_attrs(const pg_feature_params* fp, int* n_linear, int* radial_ids, int* gtinv_ids,
                     int* n_tcomb_values, int* tcomb_offsets, int* tcomb_values, int* n_poly,
                     int* n_poly_values, int* poly_offsets, int* poly_values, int* type_pairs) {
    return guarded([&] {
        if (!fp) throw std::runtime_error("null feature params");
        const pg::ModelTables mt = pg::build_model_tables(pg::feature_params_from_abi(fp));
        write_feature_attrs(mt, n_linear, radial_ids, gtinv_ids, n_tcomb_values, tcomb_offsets, tcomb_values,
                            n_poly, n_poly_values, poly_offsets, poly_values);
        if (type_pairs)
            for (int a = 0; a < mt.fp.n_type; ++a)
                for (int b = 0; b < mt.fp.n_type; ++b) type_pairs[a * mt.fp.n_type + b] = mt.type_pairs[a][b];
    });
}

int pg_features_x(pg_model* mh, const pg_structures* st, const int64_t* e_row, const int64_t* f_row,
                  const int64_t* s_row, double* x, int64_t ld, int precision) {
    return guarded([&] {
        if (!mh || !st || !x) throw std::runtime_error("null argument");
        if (precision != PG_FP64 && precision != PG_MIXED) throw std::runtime_error("unknown precision");
        Model& m = *mh->m;
        const bool fp64 = precision == PG_FP64;
        const int F = m.flat.n_features;
        cudaStream_t stream = current_stream();
        const auto batches = m.plan_batches(st, fp64, device_batch_bytes());
        DeviceBatch b;
        DevBuf Xd, X64, d_e, d_f, d_s;
        for (const auto& bt : batches) {
            const int s0 = bt.first, s1 = bt.second, nb = s1 - s0;
            b.upload_structures(st, s0, s1, m.flat.cutoff);
            // batch-local row layout: energies, stresses, forces
            std::vector<long long> le(nb), lf(nb, -1), ls(nb, -1);
            long long r = nb;
            for (int q = 0; q < nb; ++q) le[q] = q;
            for (int q = 0; q < nb; ++q)
                if (f_row[s0 + q] >= 0) {
                    ls[q] = r;
                    r += 6;
                }
            for (int q = 0; q < nb; ++q)
                if (f_row[s0 + q] >= 0) {
                    lf[q] = r;
                    r += 3LL * st->n_atoms[s0 + q];
                }
            const long long rows = r;
            upload(d_e, le);
            upload(d_f, lf);
            upload(d_s, ls);
            Xd.reserve((size_t)rows * F * (fp64 ? 8 : 4));
            double* X64p;
            if (fp64) {
                m.batch_rows<double>(b, d_e.as<long long>(), d_f.as<long long>(), d_s.as<long long>(),
                                     Xd.as<double>(), rows, stream);
                X64p = Xd.as<double>();
            } else {
                m.batch_rows<float>(b, d_e.as<long long>(), d_f.as<long long>(), d_s.as<long long>(),
                                    Xd.as<float>(), rows, stream);
                X64.reserve((size_t)rows * F * 8);
                pg_f32_to_f64<<<1024, 256, 0, stream>>>(Xd.as<float>(), X64.as<double>(), (size_t)rows * F);
                X64p = X64.as<double>();
            }
            PG_CUDA(cudaGetLastError());
            // copy each local row range to the caller's rows (column-major)
            auto copy_rows = [&](long long src_row, long long dst_row, long long n_rows) {
                if (n_rows <= 0) return;
                PG_CUDA(cudaMemcpy2DAsync(x + dst_row, (size_t)ld * sizeof(double), X64p + src_row,
                                          (size_t)rows * sizeof(double), (size_t)n_rows * sizeof(double), F,
                                          cudaMemcpyDeviceToHost, stream));
            };
            auto contiguous = [&](const int64_t* rr, int width_kind) {
                long long expect = -1;
                for (int q = 0; q < nb; ++q) {
                    const long long w = width_kind == 0 ? 1 : (width_kind == 1 ? 6 : 3LL * st->n_atoms[s0 + q]);
                    if (width_kind != 0 && f_row[s0 + q] < 0) continue;
                    if (expect >= 0 && rr[s0 + q] != expect) return false;
                    expect = rr[s0 + q] + w;
                }
                return true;
            };
            if (contiguous(e_row, 0)) {
                copy_rows(0, e_row[s0], nb);
            } else {
                for (int q = 0; q < nb; ++q) copy_rows(le[q], e_row[s0 + q], 1);
            }
            const bool cs = contiguous(s_row, 1), cf = contiguous(f_row, 2);
            long long ns = 0, nfr = 0, first_s = -1, first_f = -1;
            for (int q = 0; q < nb; ++q)
                if (f_row[s0 + q] >= 0) {
                    if (first_s < 0) {
                        first_s = q;
                        first_f = q;
                    }
                    ns += 6;
                    nfr += 3LL * st->n_atoms[s0 + q];
                }
            if (first_s >= 0) {
                if (cs) copy_rows(ls[first_s], s_row[s0 + first_s], ns);
                else
                    for (int q = 0; q < nb; ++q)
                        if (f_row[s0 + q] >= 0) copy_rows(ls[q], s_row[s0 + q], 6);
                if (cf) copy_rows(lf[first_f], f_row[s0 + first_f], nfr);
                else
                    for (int q = 0; q < nb; ++q)
                        if (f_row[s0 + q] >= 0) copy_rows(lf[q], f_row[s0 + q], 3LL * st->n_atoms[s0 + q]);
            }
            PG_CUDA(cudaStreamSynchronize(stream));
        }
    });
}

int pg_profile_enable(int on) {
    return guarded([&] { g_prof_on = on != 0; });
}

// Sum of launch durations per kernel name since the last read: writes up to
// max_names entries ("name" NUL-separated in names, total ms and launches).
int pg_profile_read(char* names, size_t names_len, double* ms, int* launches, int max_names, int* n_names) {
    return guarded([&] {
        PG_CUDA(cudaDeviceSynchronize());
        std::map<std::string, std::pair<double, int>> agg;
        {
            std::lock_guard<std::mutex> lk(g_prof_mu);
            for (auto& r : g_prof) {
                float t = 0.f;
                cudaEventElapsedTime(&t, r.a, r.b);
                auto& e = agg[r.name];
                e.first += t;
                e.second += 1;
                cudaEventDestroy(r.a);
                cudaEventDestroy(r.b);
            }
            g_prof.clear();
        }
        int k = 0;
        size_t pos = 0;
        for (auto& kv : agg) {
            if (k >= max_names || pos + kv.first.size() + 1 > names_len) break;
            std::memcpy(names + pos, kv.first.c_str(), kv.first.size() + 1);
            pos += kv.first.size() + 1;
            ms[k] = kv.second.first;
            launches[k] = kv.second.second;
            ++k;
        }
        *n_names = k;
    });
}

int pg_neighbor_list(const pg_structures* st, int structure, double cutoff, int half, int64_t* n_entries,
                     int* offsets, int* neighbors, double* diffs) {
    return guarded([&] {
        if (half) throw std::runtime_error("half lists are built by the evaluator; use half = 0");
        if (structure < 0 || structure >= st->n_st) throw std::runtime_error("structure index out of range");
        DeviceBatch b;
        b.stage(st, structure, structure + 1, cutoff, current_stream());
        b.host_offsets();
        *n_entries = b.n_pairs;
        if (!offsets) return;
        for (int i = 0; i <= b.n_atoms; ++i) offsets[i] = (int)b.nb_off[i];
        std::vector<int> nj(b.n_pairs);
        if (b.n_pairs) {
            copy_d2h(nj.data(), b.d_nb_j.as<int>(), sizeof(int) * b.n_pairs);
            copy_d2h(diffs, b.d_nb_d.as<double>(), sizeof(double) * 3 * b.n_pairs);
        }
        for (long long k = 0; k < b.n_pairs; ++k) neighbors[k] = nj[k];  // batch holds one structure: local ids
    });
}

}  // extern "C"
