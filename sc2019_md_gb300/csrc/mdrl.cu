/*
 * mdrl.cu — host side of libmdrl: context, validation, buffer management, launches and the
 * CUDA-graph step.  Kernels live in mdrl_kernels.cuh.
 */
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstddef>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <map>
#include <mutex>
#include <set>
#include <tuple>
#include <cstring>
#include <string>
#include <vector>

#include "mdrl_ctx.cuh"
#include "mdrl_force_warp.cuh"

using namespace mdrl;

namespace mdrl {
static thread_local std::string g_last_error;
void set_error(const std::string &msg) { g_last_error = msg; }

/* The armed fault: calls whose text starts with g_fault_call count down g_fault_left; the one that
 * takes it to zero fails. */
static std::mutex g_fault_mu;
static std::string g_fault_call;
static int g_fault_left = 0;

void fault_arm_from_env(bool at_create) {
    std::lock_guard<std::mutex> lock(g_fault_mu);
    g_fault_call.clear();
    g_fault_left = 0;
    const char *v = getenv("MDRL_FAULT");
    if (!v || !*v) return;
    std::string spec(v);
    const bool create = spec.compare(0, 7, "create:") == 0;
    if (create) spec = spec.substr(7);
    if (create != at_create) return;
    int k = 1;
    const size_t at = spec.find('@');
    if (at != std::string::npos) {
        k = atoi(spec.c_str() + at + 1);
        spec = spec.substr(0, at);
    }
    if (spec.empty() || k < 1) return;
    g_fault_call = spec;
    g_fault_left = k;
}

bool fault_hit(const char *call_text) {
    std::lock_guard<std::mutex> lock(g_fault_mu);
    if (g_fault_left <= 0 || strncmp(call_text, g_fault_call.c_str(), g_fault_call.size()) != 0) return false;
    return --g_fault_left == 0;
}
}  // namespace mdrl

extern "C" const char *mdrl_version(void) { return "mdrl 0.1 (sm_103a)"; }

extern "C" void mdrl_halfshell_offsets(int *offsets) {
    static const int t[kHalfShellCells][3] = MDRL_HALFSHELL_OFFSETS;
    if (offsets) memcpy(offsets, t, sizeof(t));
}

extern "C" const char *mdrl_last_error(void) { return g_last_error.c_str(); }

extern "C" void mdrl_default_params(mdrl_params *p) {
    if (!p) return;
    memset(p, 0, sizeof(*p));
    p->box[0] = p->box[1] = p->box[2] = 25.5;
    p->cutoff = 8.5;
    p->ntypes = 1;
    p->sigma[0] = 3.4;
    p->epsilon[0] = 0.238;
    p->mass[0] = 39.95;
    p->coulomb_k = 0.0;
    p->table_order = 1;
    p->table_bins = 256;
    p->table_min_log2 = -2;
    p->eval = MDRL_EVAL_TABLE;
    p->arith = MDRL_ARITH_FMA;
    p->accum = MDRL_ACC_FIXED64;
    p->integrator = MDRL_INT_VELOCITY_VERLET;
    p->dt_fs = 2.0;
    p->flags = 0;
    p->device = 0;
}

static int ilog2i(int v) { int l = 0; while ((1 << l) < v) ++l; return l; }

mdrl_status mdrl::validate_params(const mdrl_params *p) {
    char buf[256];
    for (int d = 0; d < 3; ++d)
        if (!(p->box[d] > 0.0) || !std::isfinite(p->box[d])) {
            set_error("box edges must be positive and finite");
            return MDRL_ERR_INVALID_ARG;
        }
    if (!(p->cutoff > 0.0) || !std::isfinite(p->cutoff)) {
        set_error("cutoff must be positive");
        return MDRL_ERR_INVALID_ARG;
    }
    if (p->ntypes < 1 || p->ntypes > MDRL_MAX_TYPES) {
        set_error("ntypes must be in 1..16");
        return MDRL_ERR_INVALID_ARG;
    }
    for (int t = 0; t < p->ntypes; ++t)
        if (!(p->sigma[t] > 0) || !(p->epsilon[t] >= 0) || !(p->mass[t] > 0)) {
            snprintf(buf, sizeof buf, "type %d: sigma and mass must be positive, epsilon >= 0", t);
            set_error(buf);
            return MDRL_ERR_INVALID_ARG;
        }
    if (!std::isfinite(p->coulomb_k) || std::fabs(p->coulomb_k) > 1.0e30) {
        set_error("coulomb_k must be finite");
        return MDRL_ERR_INVALID_ARG;
    }
    if (p->table_order < 1 || p->table_order > 3) {
        set_error("table_order must be 1, 2 or 3");
        return MDRL_ERR_INVALID_ARG;
    }
    if (p->table_bins < 16 || p->table_bins > 4096 || (p->table_bins & (p->table_bins - 1))) {
        set_error("table_bins must be a power of two in 16..4096");
        return MDRL_ERR_INVALID_ARG;
    }
    if (p->table_min_log2 < -30 || p->table_min_log2 > 20) {
        set_error("table_min_log2 out of range");
        return MDRL_ERR_INVALID_ARG;
    }
    if (p->eval != MDRL_EVAL_TABLE && p->eval != MDRL_EVAL_DIRECT) {
        set_error("eval must be MDRL_EVAL_TABLE or MDRL_EVAL_DIRECT");
        return MDRL_ERR_INVALID_ARG;
    }
    if (p->arith != MDRL_ARITH_FMA && p->arith != MDRL_ARITH_SEPARATE) {
        set_error("arith must be MDRL_ARITH_FMA or MDRL_ARITH_SEPARATE");
        return MDRL_ERR_INVALID_ARG;
    }
    if (p->accum < MDRL_ACC_FIXED64 || p->accum > MDRL_ACC_KAHAN) {
        set_error("accum must be one of MDRL_ACC_*");
        return MDRL_ERR_INVALID_ARG;
    }
    if (p->integrator != MDRL_INT_VELOCITY_VERLET && p->integrator != MDRL_INT_EULER) {
        set_error("integrator must be MDRL_INT_VELOCITY_VERLET or MDRL_INT_EULER");
        return MDRL_ERR_INVALID_ARG;
    }
    if (!(p->dt_fs > 0.0) || !std::isfinite(p->dt_fs)) {
        set_error("dt_fs must be positive");
        return MDRL_ERR_INVALID_ARG;
    }
    if ((p->flags & MDRL_FLAG_EXACT_DIFF) && p->arith != MDRL_ARITH_FMA) {
        set_error("MDRL_FLAG_EXACT_DIFF needs MDRL_ARITH_FMA");
        return MDRL_ERR_INVALID_ARG;
    }
    return MDRL_OK;
}

/* Cell grid and geometry; RANGE when the half shell would be wrong (n < 3 or edge < rc). */
static mdrl_status setup_geometry(mdrl_ctx *c) {
    const mdrl_params &p = c->p;
    const float rcf = (float)p.cutoff;
    c->g.rc2 = rcf * rcf;
    for (int d = 0; d < 3; ++d) {
        const float L = (float)p.box[d];
        int nc = p.ncell[d] > 0 ? p.ncell[d] : (int)std::floor((double)L / (double)rcf);
        c->g.L[d] = L;
        c->g.h[d] = 0.5f * L;
        c->g.nc[d] = nc;
        c->g.edge[d] = nc > 0 ? (float)((double)L / (double)nc) : 0.0f;
    }
    return MDRL_OK;
}

static mdrl_status check_cells(mdrl_ctx *c) {
    char buf[256];
    for (int d = 0; d < 3; ++d) {
        if (c->g.nc[d] < 3) {
            snprintf(buf, sizeof buf,
                     "axis %d: %d cells; the half-shell traversal needs at least 3 cells of edge >= rc "
                     "per axis (box %.4f, rc %.4f)", d, c->g.nc[d], (double)c->g.L[d], c->p.cutoff);
            set_error(buf);
            return MDRL_ERR_RANGE;
        }
        if ((double)c->g.edge[d] < (double)(float)c->p.cutoff) {
            snprintf(buf, sizeof buf, "axis %d: cell edge %.6f is below the cutoff %.6f", d,
                     (double)c->g.edge[d], c->p.cutoff);
            set_error(buf);
            return MDRL_ERR_RANGE;
        }
    }
    const long long nc = (long long)c->g.nc[0] * c->g.nc[1] * c->g.nc[2];
    if (nc > (1LL << 24) || nc * kHalfShellCells > 2147483647LL) {
        set_error("too many cells");
        return MDRL_ERR_RANGE;
    }
    return MDRL_OK;
}

mdrl_status mdrl::upload_tables(mdrl_ctx *c) {
    const int nidx = c->nseg * c->bins;
    const int nc = c->order + 1;
    dfree(&c->d_f2); dfree(&c->d_e2); dfree(&c->d_f4); dfree(&c->d_e4); dfree(&c->d_fr); dfree(&c->d_fp2); dfree(&c->d_fc2);
    auto coef = [&](int f, int k, int idx) { return c->tab[((size_t)f * nc + k) * nidx + idx]; };
    if (c->order == 1) {
        std::vector<float2> f2((size_t)3 * nidx), e2((size_t)3 * nidx);
        std::vector<float4> fr((size_t)2 * nidx);
        for (int i = 0; i < nidx; ++i) {
            for (int f = 0; f < 3; ++f) {
                f2[(size_t)3 * i + f] = make_float2(coef(f, 0, i), coef(f, 1, i));
                e2[(size_t)3 * i + f] = make_float2(coef(3 + f, 0, i), coef(3 + f, 1, i));
            }
            fr[(size_t)2 * i] = make_float4(coef(0, 0, i), coef(0, 1, i), coef(1, 0, i), coef(1, 1, i));
            fr[(size_t)2 * i + 1] = make_float4(coef(2, 0, i), coef(2, 1, i), 0.0f, 0.0f);
        }
        MDRL_TRY(dalloc(&c->d_fr, fr.size()));
        MDRL_CUDA(cudaMemcpy(c->d_fr, fr.data(), sizeof(float4) * fr.size(), cudaMemcpyHostToDevice));
        MDRL_TRY(dalloc(&c->d_f2, f2.size()));
        MDRL_TRY(dalloc(&c->d_e2, e2.size()));
        MDRL_CUDA(cudaMemcpy(c->d_f2, f2.data(), sizeof(float2) * f2.size(), cudaMemcpyHostToDevice));
        MDRL_CUDA(cudaMemcpy(c->d_e2, e2.data(), sizeof(float2) * e2.size(), cudaMemcpyHostToDevice));
    } else {
        std::vector<float4> f4((size_t)3 * nidx), e4((size_t)3 * nidx);
        for (int i = 0; i < nidx; ++i)
            for (int f = 0; f < 3; ++f) {
                float a[4] = {0, 0, 0, 0}, b[4] = {0, 0, 0, 0};
                for (int k = 0; k < nc; ++k) { a[k] = coef(f, k, i); b[k] = coef(3 + f, k, i); }
                f4[(size_t)3 * i + f] = make_float4(a[0], a[1], a[2], a[3]);
                e4[(size_t)3 * i + f] = make_float4(b[0], b[1], b[2], b[3]);
            }
        if (nc == 3) {
            /* order 2 packed without padding for the one-warp-per-item kernel (36 bytes per index) */
            std::vector<float4> fp2((size_t)2 * nidx);
            std::vector<float> fc2((size_t)nidx);
            for (int i = 0; i < nidx; ++i) {
                fp2[(size_t)2 * i] = make_float4(coef(0, 0, i), coef(0, 1, i), coef(0, 2, i), coef(1, 0, i));
                fp2[(size_t)2 * i + 1] = make_float4(coef(1, 1, i), coef(1, 2, i), coef(2, 0, i), coef(2, 1, i));
                fc2[i] = coef(2, 2, i);
            }
            MDRL_TRY(dalloc(&c->d_fp2, fp2.size()));
            MDRL_TRY(dalloc(&c->d_fc2, fc2.size()));
            MDRL_CUDA(cudaMemcpy(c->d_fp2, fp2.data(), sizeof(float4) * fp2.size(), cudaMemcpyHostToDevice));
            MDRL_CUDA(cudaMemcpy(c->d_fc2, fc2.data(), sizeof(float) * fc2.size(), cudaMemcpyHostToDevice));
        }
        MDRL_TRY(dalloc(&c->d_f4, f4.size()));
        MDRL_TRY(dalloc(&c->d_e4, e4.size()));
        MDRL_CUDA(cudaMemcpy(c->d_f4, f4.data(), sizeof(float4) * f4.size(), cudaMemcpyHostToDevice));
        MDRL_CUDA(cudaMemcpy(c->d_e4, e4.data(), sizeof(float4) * e4.size(), cudaMemcpyHostToDevice));
    }
    /* per-type-pair multipliers */
    const int T = c->p.ntypes;
    std::vector<float4> pc((size_t)T * T);
    for (int k = 0; k < T * T; ++k) {
        if (c->raw)
            pc[k] = make_float4(1.0f, -1.0f, 1.0f, -1.0f);
        else
            pc[k] = make_float4(c->pcoef[4 * k], c->pcoef[4 * k + 1], c->pcoef[4 * k + 2], c->pcoef[4 * k + 3]);
    }
    MDRL_TRY(dalloc(&c->d_pcoef, pc.size()));
    MDRL_CUDA(cudaMemcpy(c->d_pcoef, pc.data(), sizeof(float4) * pc.size(), cudaMemcpyHostToDevice));
    return MDRL_OK;
}

TableDev mdrl::table_dev(const mdrl_ctx *c) {
    TableDev t;
    t.f2 = c->d_f2; t.e2 = c->d_e2; t.f4 = c->d_f4; t.e4 = c->d_e4; t.fr = c->d_fr; t.fp2 = c->d_fp2; t.fc2 = c->d_fc2;
    t.order = c->order; t.nseg = c->nseg; t.bins = c->bins; t.lb = ilog2i(c->bins);
    t.min_log2 = c->min_log2;
    t.r2min = std::ldexp(1.0f, c->min_log2);
    t.local = c->local ? 1 : 0;
    return t;
}

static int segments_for(float rc2, int min_log2) {
    int e;
    std::frexp(rc2, &e); /* rc2 = m * 2^e, m in [0.5, 1) -> floor(log2 rc2) = e - 1 */
    return (e - 1) - min_log2 + 1;
}

extern "C" mdrl_status mdrl_create(const mdrl_params *p, mdrl_ctx **out) {
    if (!p || !out) { set_error("null argument"); return MDRL_ERR_INVALID_ARG; }
    *out = nullptr;
    fault_arm_from_env(true);
    MDRL_TRY(validate_params(p));
    int ndev = 0;
    MDRL_CUDA(cudaGetDeviceCount(&ndev));
    if (p->device < 0 || p->device >= ndev) { set_error("device ordinal out of range"); return MDRL_ERR_INVALID_ARG; }
    MDRL_CUDA(cudaSetDevice(p->device));
    mdrl_ctx *c = new mdrl_ctx();
    c->p = *p;
    setup_geometry(c);
    c->order = p->table_order;
    c->bins = p->table_bins;
    c->min_log2 = p->table_min_log2;
    c->nseg = segments_for(c->g.rc2, c->min_log2);
    if (c->nseg < 1) {
        delete c;
        set_error("cutoff lies below the first table segment");
        return MDRL_ERR_RANGE;
    }
    c->ke = (float)p->coulomb_k;
    c->local = c->order >= 2;    /* the library's own order-2/3 tables are bin-local */
    fit_tables(c->order, c->nseg, c->bins, c->min_log2, 8, &c->tab, 0.0, c->local);
    mix_pair_coefficients(*p, &c->pcoef, nullptr);
    const double conv = 4.184e-4; /* (kcal/mol/A)/amu -> A/fs^2 */
    for (int t = 0; t < MDRL_MAX_TYPES; ++t) {
        const double m = t < p->ntypes ? p->mass[t] : 1.0;
        c->mt_half.cm[t] = (float)(0.5 * p->dt_fs * conv / m);
        c->mt_full.cm[t] = (float)(p->dt_fs * conv / m);
        c->mt_half.mass[t] = c->mt_full.mass[t] = (float)m;
    }
    mdrl_status s = upload_tables(c);
    if (s != MDRL_OK) { mdrl_destroy(c); return s; }
    cudaError_t e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreate(&c->ev0);
    if (e == cudaSuccess) e = cudaEventCreate(&c->ev1);
    if (e == cudaSuccess) e = cudaEventCreate(&c->evf0);
    if (e == cudaSuccess) e = cudaEventCreate(&c->evf1);
    if (e == cudaSuccess) e = cudaMalloc((void **)&c->d_tot, sizeof(DevTotals));
    if (e == cudaSuccess) e = cudaMalloc((void **)&c->d_err, sizeof(unsigned));
    if (e == cudaSuccess) e = cudaMallocHost((void **)&c->h_tot, sizeof(DevTotals));
    if (e == cudaSuccess) e = cudaMallocHost((void **)&c->h_err, sizeof(unsigned));
    /* their device addresses, for the kernel that writes them at the end of a force evaluation */
    if (e == cudaSuccess) e = cudaHostGetDevicePointer((void **)&c->h_tot_dev, c->h_tot, 0);
    if (e == cudaSuccess) e = cudaHostGetDevicePointer((void **)&c->h_err_dev, c->h_err, 0);
    if (e == cudaSuccess) e = cudaMalloc((void **)&c->d_mt, 2 * sizeof(MassTab));
    if (e == cudaSuccess) e = cudaMemcpy(c->d_mt, &c->mt_half, sizeof(MassTab), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(c->d_mt + 1, &c->mt_full, sizeof(MassTab), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, p->device);
    if (e != cudaSuccess) {
        set_error(std::string("context setup: ") + cudaGetErrorString(e));
        mdrl_destroy(c);
        return MDRL_ERR_CUDA;
    }
    *out = c;
    fault_arm_from_env(false);
    return MDRL_OK;
}

static void free_particles(mdrl_ctx *c) {
    dfree(&c->d_ux); dfree(&c->d_uy); dfree(&c->d_uz); dfree(&c->d_uq); dfree(&c->d_ut); dfree(&c->d_inv);
    dfree(&c->d_ox); dfree(&c->d_oy); dfree(&c->d_oz);
    dfree(&c->d_ovx); dfree(&c->d_ovy); dfree(&c->d_ovz); dfree(&c->d_ocnt);
    for (int b = 0; b < 2; ++b) { dfree(&c->d_pos[b]); dfree(&c->d_vel[b]); dfree(&c->d_type[b]); dfree(&c->d_id[b]); }
    dfree(&c->d_cell_of); dfree(&c->d_slot); dfree(&c->d_tmp); dfree(&c->d_sorted); dfree(&c->d_key);
    dfree(&c->d_sortkey);
    dfree(&c->d_F64); dfree(&c->d_F32); dfree(&c->d_cnt);
    dfree(&c->d_Fscr64); dfree(&c->d_Fscr32);
    c->cap = 0;
}

extern "C" mdrl_status mdrl_destroy(mdrl_ctx *c) {
    if (!c) return MDRL_OK;
    cudaSetDevice(c->p.device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    for (int k = 0; k < 2; ++k) {
        if (c->graph_exec[k]) cudaGraphExecDestroy(c->graph_exec[k]);
        if (c->graph[k]) cudaGraphDestroy(c->graph[k]);
    }
    pme_free(c);
    bonded_free(c);
    free_particles(c);
    dfree(&c->d_f2); dfree(&c->d_e2); dfree(&c->d_f4); dfree(&c->d_e4); dfree(&c->d_fr); dfree(&c->d_fp2); dfree(&c->d_fc2);
    dfree(&c->d_pcoef);
    dfree(&c->d_count); dfree(&c->d_start); dfree(&c->d_unit); dfree(&c->d_kepart); dfree(&c->d_work);
    dfree(&c->d_tot); dfree(&c->d_err); dfree(&c->d_mt);
    if (c->h_tot) cudaFreeHost(c->h_tot);
    if (c->h_err) cudaFreeHost(c->h_err);
    dfree(&c->d_pr); dfree(&c->d_pn); dfree(&c->d_pout); dfree(&c->d_ptr); dfree(&c->d_ptn); dfree(&c->d_paux);
    if (c->ev0) cudaEventDestroy(c->ev0);
    if (c->ev1) cudaEventDestroy(c->ev1);
    if (c->evf0) cudaEventDestroy(c->evf0);
    if (c->evf1) cudaEventDestroy(c->evf1);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
    return MDRL_OK;
}

static mdrl_status ensure_cells(mdrl_ctx *c) {
    if (c->ncells) return MDRL_OK;
    MDRL_TRY(check_cells(c));
    c->ncells = c->g.nc[0] * c->g.nc[1] * c->g.nc[2];
    MDRL_TRY(dalloc(&c->d_count, c->ncells));
    MDRL_TRY(dalloc(&c->d_start, c->ncells + 1));
    MDRL_TRY(dalloc(&c->d_unit, (size_t)c->ncells * kHalfShellCells * kMaxItemGroups));
    MDRL_TRY(dalloc(&c->d_work, 1));
    return MDRL_OK;
}

mdrl_status mdrl::ensure_capacity(mdrl_ctx *c, int n) {
    MDRL_TRY(ensure_cells(c));
    if (n <= c->cap) return MDRL_OK;
    free_particles(c);
    const size_t m = (size_t)n;
    MDRL_TRY(dalloc(&c->d_ux, m)); MDRL_TRY(dalloc(&c->d_uy, m)); MDRL_TRY(dalloc(&c->d_uz, m));
    MDRL_TRY(dalloc(&c->d_uq, m)); MDRL_TRY(dalloc(&c->d_ut, m)); MDRL_TRY(dalloc(&c->d_inv, m));
    MDRL_TRY(dalloc(&c->d_ox, m)); MDRL_TRY(dalloc(&c->d_oy, m)); MDRL_TRY(dalloc(&c->d_oz, m));
    MDRL_TRY(dalloc(&c->d_ovx, m)); MDRL_TRY(dalloc(&c->d_ovy, m)); MDRL_TRY(dalloc(&c->d_ovz, m));
    MDRL_TRY(dalloc(&c->d_ocnt, m));
    for (int b = 0; b < 2; ++b) {
        MDRL_TRY(dalloc(&c->d_pos[b], m)); MDRL_TRY(dalloc(&c->d_vel[b], m));
        MDRL_TRY(dalloc(&c->d_type[b], m)); MDRL_TRY(dalloc(&c->d_id[b], m));
    }
    MDRL_TRY(dalloc(&c->d_cell_of, m)); MDRL_TRY(dalloc(&c->d_slot, m));
    MDRL_TRY(dalloc(&c->d_tmp, m)); MDRL_TRY(dalloc(&c->d_sorted, m)); MDRL_TRY(dalloc(&c->d_key, m));
    MDRL_TRY(dalloc(&c->d_sortkey, m));
    if (c->p.accum == MDRL_ACC_FIXED64) { MDRL_TRY(dalloc(&c->d_F64, 3 * m)); }
    else { MDRL_TRY(dalloc(&c->d_F32, 6 * m)); }   /* high and low planes */
    MDRL_TRY(dalloc(&c->d_cnt, m));
    const int nke = (n + 255) / 256;
    MDRL_TRY(dalloc(&c->d_kepart, nke));
    c->kecap = nke;
    c->cap = n;
    c->have_state = false;
    c->graph_n = -1; /* captured graphs hold the old buffer addresses */
    return MDRL_OK;
}

/* ---- kernel dispatch ---------------------------------------------------------------------- */

namespace mdrl {
force_fn pick_force(int order, bool sep, bool extra, int acc, int fw, bool prune, bool exact) {
    if (exact) {
        if (acc == MDRL_ACC_FP32_ATOMIC) return pick_force_set<1, 4, false, kDiffExact>(order, false, extra);
        if (acc == MDRL_ACC_KAHAN) return pick_force_set<2, 4, false, kDiffExact>(order, false, extra);
        if (fw == 8) return prune ? pick_force_set<0, 8, true, kDiffExact>(order, false, extra)
                                  : pick_force_set<0, 8, false, kDiffExact>(order, false, extra);
        return prune ? pick_force_set<0, 4, true, kDiffExact>(order, false, extra)
                     : pick_force_set<0, 4, false, kDiffExact>(order, false, extra);
    }
    if (acc == MDRL_ACC_FP32_ATOMIC) return pick_force_set<1, 4, false, kDiffShift>(order, sep, extra);
    if (acc == MDRL_ACC_KAHAN) return pick_force_set<2, 4, false, kDiffShift>(order, sep, extra);
    if (fw == 8) return prune ? pick_force_set<0, 8, true, kDiffShift>(order, sep, extra)
                              : pick_force_set<0, 8, false, kDiffShift>(order, sep, extra);
    return prune ? pick_force_set<0, 4, true, kDiffShift>(order, sep, extra)
                 : pick_force_set<0, 4, false, kDiffShift>(order, sep, extra);
}

force_fn pick_force_batch(int order, bool sep, bool extra, bool prune) {
    return prune ? pick_batch_set<true>(order, sep, extra) : pick_batch_set<false>(order, sep, extra);
}
}  // namespace mdrl

/* The smem attribute is set once per kernel and device, on the first (uncaptured) launch. */
mdrl_status mdrl::prepare_force_kernel(force_fn fn, int device) {
    static std::mutex mu;
    static std::set<std::pair<const void *, int>> done;
    std::lock_guard<std::mutex> lock(mu);
    const std::pair<const void *, int> key((const void *)fn, device);
    if (!done.count(key)) {
        MDRL_CUDA(cudaFuncSetAttribute((const void *)fn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)force_smem_bytes(MDRL_MAX_TYPES, true, 8)));
        done.insert(key);
    }
    return MDRL_OK;
}

int mdrl::eff_order(const mdrl_ctx *c) { return c->p.eval == MDRL_EVAL_DIRECT ? 0 : c->order; }

/* Result slots of a force launch over `units` units: one per CTA (the warp-item kernel runs
 * steps_per_piece i-tile groups per unit). */
static int force_slots(const mdrl_ctx *c, int units) {
    return c->tile.warps_per_cta == 1 ? units * c->tile.steps_per_piece : units;
}

/* The force launch over units [unit0, unit0 + units) (units < 0: every unit). */
static mdrl_status launch_force_into(mdrl_ctx *c, int n, const float4 *pos, const int *type, bool extra,
                                     unsigned long long *F64, float *F32, int unit0 = 0, int units = -1) {
    if (units < 0) units = c->ncells * kHalfShellCells;
    if (c->tile.warps_per_cta == 1) {
        /* one warp per (unit, i-tile group); fixed point only (set_tile checks) */
        const bool exact = (c->p.flags & MDRL_FLAG_EXACT_DIFF) != 0;
        warp_fn fn = exact ? pick_force_warp_set<0, kDiffExact>(eff_order(c), false, extra)
                           : pick_force_warp_set<0, kDiffShift>(eff_order(c), c->p.arith == MDRL_ARITH_SEPARATE, extra);
        MDRL_TRY(prepare_force_kernel((force_fn)fn, c->p.device));
        const int items = force_slots(c, units);
        const size_t smem = force_warp_smem_bytes(c->p.ntypes, extra);
        /* a persistent grid: the CTAs that fit at once take items from the counter */
        int per_sm = 0;
        MDRL_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, (const void *)fn, 32, smem));
        const int grid = std::min(items, std::max(1, per_sm) * std::max(1, c->num_sms));
        if (items > 0) MDRL_CUDA(cudaMemsetAsync(c->d_work, 0, sizeof(int), c->stream));
        MDRL_CUDA(cudaEventRecord(c->evf0, c->stream));
        if (items > 0)
            fn<<<grid, 32, smem, c->stream>>>(
                pos, type, c->d_start, c->g, table_dev(c), c->d_pcoef, c->p.ntypes, c->ke, n, F64, F32, c->d_cnt,
                c->d_unit, nullptr, nullptr, c->tile.steps_per_piece, c->d_err, unit0, c->d_work, items);
        MDRL_CUDA(cudaGetLastError());
        MDRL_CUDA(cudaEventRecord(c->evf1, c->stream));
        return MDRL_OK;
    }
    const int fw = c->p.accum == MDRL_ACC_FIXED64 ? c->tile.warps_per_cta : kFW;
    const bool prune = c->p.accum == MDRL_ACC_FIXED64 && c->tile.prune_steps;
    force_fn fn = pick_force(eff_order(c), c->p.arith == MDRL_ARITH_SEPARATE, extra, c->p.accum, fw, prune,
                             (c->p.flags & MDRL_FLAG_EXACT_DIFF) != 0);
    const size_t smem = force_smem_bytes(c->p.ntypes, extra, fw);
    MDRL_TRY(prepare_force_kernel(fn, c->p.device));
    MDRL_CUDA(cudaEventRecord(c->evf0, c->stream));
    if (units > 0)
        fn<<<units, fw * 32, smem, c->stream>>>(pos, type, c->d_start, c->g, table_dev(c), c->d_pcoef,
                                                 c->p.ntypes, c->ke, n, F64, F32, c->d_cnt, c->d_unit, nullptr,
                                                 nullptr, tile_word(c->tile.steps_per_piece, c->tile.prune_steps),
                                                 c->d_err, unit0);
    MDRL_CUDA(cudaGetLastError());
    MDRL_CUDA(cudaEventRecord(c->evf1, c->stream));
    return MDRL_OK;
}

static mdrl_status launch_force(mdrl_ctx *c, int n, const float4 *pos, const int *type, bool extra) {
    return launch_force_into(c, n, pos, type, extra, c->d_F64, c->d_F32);
}




/* Bin user-order arrays (already on the device) into the sorted buffers of slot `buf`.  With
 * `spatial` the cells are ordered by Morton key (the force path's order), otherwise by index
 * (the reference's in-cell order). */
/* Bin user-order inputs into cell order (buffer buf).  stage: the inputs may be host memory the
 * device reads directly; the binning pass copies them to the device staging buffers on the way
 * and the gather reads those.  inv: also record each user index's cell-order position. */
static mdrl_status bin_user(mdrl_ctx *c, int n, const float *x, const float *y, const float *z,
                            const float *q, const int *type, int buf, bool spatial, bool stage = false,
                            bool inv = false) {
    MDRL_CUDA(cudaMemsetAsync(c->d_count, 0, sizeof(int) * c->ncells, c->stream));
    MDRL_CUDA(cudaMemsetAsync(c->d_err, 0, sizeof(unsigned), c->stream));
    if (n > 0) {
        k_bin_user<<<nblk(n, 256), 256, 0, c->stream>>>(
            n, x, y, z, c->g, c->d_cell_of, c->d_slot, c->d_count, c->d_err, spatial ? c->d_key : nullptr,
            stage ? q : nullptr, stage ? type : nullptr, stage ? c->d_ux : nullptr, c->d_uy, c->d_uz, c->d_uq,
            c->d_ut);
        if (stage) {
            x = c->d_ux; y = c->d_uy; z = c->d_uz;
            if (q) q = c->d_uq;
            if (type) type = c->d_ut;
        }
    }
    k_scan<<<1, 1024, 0, c->stream>>>(c->ncells, c->d_count, c->d_start, c->d_tot);
    if (n > 0) {
        k_scatter<<<nblk(n, 256), 256, 0, c->stream>>>(n, c->d_cell_of, c->d_slot, c->d_start, c->d_tmp);
        k_cell_sort<<<c->ncells, 128, 0, c->stream>>>(c->d_start, c->d_tmp, c->d_sorted,
                                                       spatial ? c->d_key : nullptr, c->d_sortkey, c->d_err);
        k_gather_user<<<nblk(n, 256), 256, 0, c->stream>>>(n, c->d_sorted, x, y, z, q, type, c->d_pos[buf],
                                                           c->d_type[buf], c->d_id[buf], c->d_F64,
                                                           c->d_F32, c->d_cnt, c->p.ntypes, c->d_err,
                                                           inv ? c->d_inv : nullptr);
    }
    MDRL_CUDA(cudaGetLastError());
    return MDRL_OK;
}

mdrl_status mdrl::device_error_status(unsigned err) {
    if (err & kErrPosition) {
        set_error("positions must be finite and lie in [0, box) on every axis");
        return MDRL_ERR_INVALID_ARG;
    }
    if (err & kErrType) {
        set_error("particle types must lie in [0, ntypes)");
        return MDRL_ERR_INVALID_ARG;
    }
    if (err & kErrCellOverflow) {
        set_error("a cell holds more than 65536 particles (the largest occupancy the in-cell sort and "
                  "the force kernel accept); the units that touch it were skipped");
        return MDRL_ERR_CELL_OVERFLOW;
    }
    if (err & kErrForce) {
        set_error("a force component was NaN or infinite, or (int64 fixed point) reached 5.4e11 "
                  "kcal/mol/A, beyond what the accumulators hold");
        return MDRL_ERR_RANGE;
    }
    return MDRL_OK;
}

mdrl_status mdrl::check_device_errors(mdrl_ctx *c) {
    unsigned err = 0;
    MDRL_CUDA(cudaMemcpy(&err, c->d_err, sizeof(unsigned), cudaMemcpyDeviceToHost));
    return device_error_status(err);
}

static mdrl_status read_stats(mdrl_ctx *c, mdrl_stats *st, float ms) {
    if (!st) return MDRL_OK;
    DevTotals t;
    MDRL_CUDA(cudaMemcpy(&t, c->d_tot, sizeof(t), cudaMemcpyDeviceToHost));
    memset(st, 0, sizeof(*st));
    st->pairs = (int64_t)t.pairs;
    st->below_table = (int64_t)t.below;
    st->max_cell_occupancy = t.max_occ;
    st->ncells = c->ncells;
    st->e_lj = t.e_lj;
    st->e_coul = t.e_coul;
    st->virial = t.virial;
    st->kinetic = t.kinetic;
    st->e_bond = t.e_bond;
    st->e_angle = t.e_angle;
    st->e_dihedral = t.e_dihedral;
    st->device_ms = ms;
    st->pairs_total = (int64_t)t.pairs_total;
    float fms = 0.0f;
    if (cudaEventElapsedTime(&fms, c->evf0, c->evf1) == cudaSuccess) st->force_ms = fms;
    else cudaGetLastError();
    return MDRL_OK;
}

/* The device address of p when the context's device can read and write it in place: page-locked
 * host memory (cudaHostAlloc / cudaHostRegister, mapped), managed memory, or memory of this
 * device; nullptr otherwise (pageable host memory: the caller stages through copies). */
static void *mapped(const mdrl_ctx *c, const void *p) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    if (a.type == cudaMemoryTypeHost || a.type == cudaMemoryTypeManaged) return a.devicePointer;
    if (a.type == cudaMemoryTypeDevice && a.device == c->p.device) return a.devicePointer;
    return nullptr;
}

/* One force evaluation enqueued on the context stream; its last kernel writes the error word and
 * the totals into pinned host memory (copies when there are no particles); force_eval_finish
 * reads them after the one synchronisation of the call. */
static mdrl_status force_eval_enqueue(mdrl_ctx *c, int n, const float *x, const float *y, const float *z,
                                      const float *q, const int *type, float *fx, float *fy, float *fz,
                                      int *counts, bool stage = false) {
    MDRL_TRY(ensure_capacity(c, n));
    MDRL_TRY(bonded_check_atoms(c, n));
    const bool extra = counts != nullptr || (c->p.flags & MDRL_FLAG_ENERGY);
    MDRL_CUDA(cudaMemsetAsync(c->d_tot, 0, sizeof(DevTotals), c->stream));
    MDRL_CUDA(cudaEventRecord(c->ev0, c->stream));
    MDRL_TRY(bin_user(c, n, x, y, z, q, type, 0, true, stage, true));
    MDRL_TRY(launch_force(c, n, c->d_pos[0], c->d_type[0], extra));
    const bool energy = (c->p.flags & MDRL_FLAG_ENERGY) != 0;
    MDRL_TRY(pme_enqueue(c, n, c->d_pos[0], c->d_F64, c->d_F32, energy));
    MDRL_TRY(bonded_enqueue(c, n, c->d_pos[0], c->d_id[0], c->d_F64, c->d_F32, energy));
    k_totals<<<1, 1024, 0, c->stream>>>(force_slots(c, force_items(c->ncells)), c->d_unit, 0, c->d_kepart, c->d_tot,
                                       extra ? 1 : 0);
    if (energy) MDRL_TRY(pme_add_energy(c, n));
    if (energy) MDRL_TRY(bonded_add_energy(c, n));
    if (n > 0)
        k_unsort_inv<<<nblk(n, 256), 256, 0, c->stream>>>(n, c->d_inv, c->d_F64, c->d_F32, c->d_cnt, fx, fy,
                                                          fz, counts, c->d_tot, c->h_tot_dev, c->d_err, c->h_err_dev);
    MDRL_CUDA(cudaGetLastError());
    MDRL_CUDA(cudaEventRecord(c->ev1, c->stream));
    if (n == 0) {
        MDRL_CUDA(cudaMemcpyAsync(c->h_tot, c->d_tot, sizeof(DevTotals), cudaMemcpyDeviceToHost, c->stream));
        MDRL_CUDA(cudaMemcpyAsync(c->h_err, c->d_err, sizeof(unsigned), cudaMemcpyDeviceToHost, c->stream));
    }
    c->have_state = false; /* the sorted buffers now hold this evaluation */
    return MDRL_OK;
}

static mdrl_status force_eval_finish(mdrl_ctx *c, mdrl_stats *st) {
    MDRL_TRY(device_error_status(*c->h_err));
    if (!st) return MDRL_OK;
    const DevTotals &t = *c->h_tot;
    memset(st, 0, sizeof(*st));
    st->pairs = (int64_t)t.pairs;
    st->candidates = -1;
    st->below_table = (int64_t)t.below;
    st->max_cell_occupancy = t.max_occ;
    st->ncells = c->ncells;
    st->e_lj = t.e_lj;
    st->e_coul = t.e_coul;
    st->virial = t.virial;
    st->kinetic = t.kinetic;
    st->e_bond = t.e_bond;
    st->e_angle = t.e_angle;
    st->e_dihedral = t.e_dihedral;
    st->pairs_total = (int64_t)t.pairs_total;
    float ms = 0.0f, fms = 0.0f;
    if (cudaEventElapsedTime(&ms, c->ev0, c->ev1) == cudaSuccess) st->device_ms = ms;
    else cudaGetLastError();
    if (cudaEventElapsedTime(&fms, c->evf0, c->evf1) == cudaSuccess) st->force_ms = fms;
    else cudaGetLastError();
    return MDRL_OK;
}

static mdrl_status force_eval_dev(mdrl_ctx *c, int n, const float *x, const float *y, const float *z,
                                  const float *q, const int *type, float *fx, float *fy, float *fz,
                                  int *counts, mdrl_stats *st) {
    MDRL_TRY(force_eval_enqueue(c, n, x, y, z, q, type, fx, fy, fz, counts));
    MDRL_CUDA(cudaStreamSynchronize(c->stream));
    return force_eval_finish(c, st);
}

extern "C" mdrl_status mdrl_force_eval_device(mdrl_ctx *c, int n, const float *x, const float *y,
                                              const float *z, const float *q, const int *type,
                                              float *fx, float *fy, float *fz, int *counts,
                                              mdrl_stats *st) {
    if (!c || n < 0 || (n > 0 && (!x || !y || !z || !fx || !fy || !fz))) {
        set_error("mdrl_force_eval_device: null or invalid argument");
        return MDRL_ERR_INVALID_ARG;
    }
    MDRL_CUDA(cudaSetDevice(c->p.device));
    return force_eval_dev(c, n, x, y, z, q, type, fx, fy, fz, counts, st);
}

extern "C" mdrl_status mdrl_force_eval(mdrl_ctx *c, int n, const float *x, const float *y,
                                       const float *z, const float *q, const int *type, float *fx,
                                       float *fy, float *fz, int *counts, mdrl_stats *st) {
    if (!c || n < 0 || (n > 0 && (!x || !y || !z || !fx || !fy || !fz))) {
        set_error("mdrl_force_eval: null or invalid argument");
        return MDRL_ERR_INVALID_ARG;
    }
    MDRL_CUDA(cudaSetDevice(c->p.device));
    MDRL_TRY(ensure_capacity(c, n));
    /* Pinned (page-locked) host buffers, or this device's memory: the kernels read the inputs and
     * write the forces in place, coalesced, over the host link; no staging copies. */
    if (n > 0) {
        const void *dx = mapped(c, x), *dy = mapped(c, y), *dz = mapped(c, z);
        void *dfx = mapped(c, fx), *dfy = mapped(c, fy), *dfz = mapped(c, fz);
        const void *dq = q ? mapped(c, q) : nullptr, *dt = type ? mapped(c, type) : nullptr;
        void *dc = counts ? mapped(c, counts) : nullptr;
        if (dx && dy && dz && dfx && dfy && dfz && (!q || dq) && (!type || dt) && (!counts || dc)) {
            MDRL_TRY(force_eval_enqueue(c, n, (const float *)dx, (const float *)dy, (const float *)dz,
                                        (const float *)dq, (const int *)dt, (float *)dfx, (float *)dfy,
                                        (float *)dfz, (int *)dc, true));
            MDRL_CUDA(cudaStreamSynchronize(c->stream));   /* the one synchronisation of the call */
            return force_eval_finish(c, st);
        }
    }
    const size_t fb = sizeof(float) * (size_t)n;
    if (n > 0) {
        MDRL_CUDA(cudaMemcpyAsync(c->d_ux, x, fb, cudaMemcpyHostToDevice, c->stream));
        MDRL_CUDA(cudaMemcpyAsync(c->d_uy, y, fb, cudaMemcpyHostToDevice, c->stream));
        MDRL_CUDA(cudaMemcpyAsync(c->d_uz, z, fb, cudaMemcpyHostToDevice, c->stream));
        if (q) MDRL_CUDA(cudaMemcpyAsync(c->d_uq, q, fb, cudaMemcpyHostToDevice, c->stream));
        if (type) MDRL_CUDA(cudaMemcpyAsync(c->d_ut, type, sizeof(int) * (size_t)n, cudaMemcpyHostToDevice, c->stream));
    }
    MDRL_TRY(force_eval_enqueue(c, n, c->d_ux, c->d_uy, c->d_uz, q ? c->d_uq : nullptr,
                                type ? c->d_ut : nullptr, c->d_ox, c->d_oy, c->d_oz,
                                counts ? c->d_ocnt : nullptr));
    if (n > 0) {
        MDRL_CUDA(cudaMemcpyAsync(fx, c->d_ox, fb, cudaMemcpyDeviceToHost, c->stream));
        MDRL_CUDA(cudaMemcpyAsync(fy, c->d_oy, fb, cudaMemcpyDeviceToHost, c->stream));
        MDRL_CUDA(cudaMemcpyAsync(fz, c->d_oz, fb, cudaMemcpyDeviceToHost, c->stream));
        if (counts) MDRL_CUDA(cudaMemcpyAsync(counts, c->d_ocnt, sizeof(int) * (size_t)n, cudaMemcpyDeviceToHost, c->stream));
    }
    MDRL_CUDA(cudaStreamSynchronize(c->stream));   /* the one synchronisation of the call */
    return force_eval_finish(c, st);
}

/* ---- spatial decomposition ------------------------------------------------------------------ */

/* The cell grid a context builds for these parameters (setup_geometry), without a GPU. */
static void grid_of(const mdrl_params *p, int nc[3], float edge[3]) {
    const float rcf = (float)p->cutoff;
    for (int d = 0; d < 3; ++d) {
        const float L = (float)p->box[d];
        const double ncd = p->ncell[d] > 0 ? (double)p->ncell[d] : std::floor((double)L / (double)rcf);
        nc[d] = ncd > 65536.0 ? 65536 : (int)ncd;
        edge[d] = nc[d] > 0 ? (float)((double)L / (double)nc[d]) : 0.0f;
    }
}

extern "C" mdrl_status mdrl_slab_plan(const mdrl_params *p, int nranks, int rank, mdrl_slab *s) {
    if (!p || !s) { set_error("mdrl_slab_plan: null argument"); return MDRL_ERR_INVALID_ARG; }
    MDRL_TRY(validate_params(p));
    int nc[3];
    float edge[3];
    grid_of(p, nc, edge);
    if (nc[0] < 3 || nc[1] < 3 || nc[2] < 3) {
        set_error("mdrl_slab_plan: the half-shell traversal needs at least 3 cells per axis");
        return MDRL_ERR_RANGE;
    }
    if (nranks < 1 || nranks > nc[0] || rank < 0 || rank >= nranks) {
        set_error("mdrl_slab_plan: need 1 <= nranks <= cell layers along x and 0 <= rank < nranks");
        return MDRL_ERR_INVALID_ARG;
    }
    const int base = nc[0] / nranks, rem = nc[0] % nranks;
    s->nranks = nranks;
    s->rank = rank;
    s->x0 = rank * base + std::min(rank, rem);
    s->x1 = s->x0 + base + (rank < rem ? 1 : 0);
    s->halo_x = s->x1 % nc[0];
    s->import_from = (rank + 1) % nranks;
    s->export_to = (rank + nranks - 1) % nranks;
    for (int d = 0; d < 3; ++d) s->ncell[d] = nc[d];
    return MDRL_OK;
}

extern "C" mdrl_status mdrl_slab_select(const mdrl_params *p, const mdrl_slab *s, int n, const float *x,
                                        int *owned, int *n_owned, int *exported, int *n_exported) {
    if (!p || !s || n < 0 || (n > 0 && !x)) { set_error("mdrl_slab_select: null or invalid argument"); return MDRL_ERR_INVALID_ARG; }
    int nc[3];
    float edge[3];
    grid_of(p, nc, edge);
    if (nc[0] != s->ncell[0] || s->x0 < 0 || s->x1 > nc[0] || s->x0 >= s->x1) {
        set_error("mdrl_slab_select: the slab does not belong to these parameters");
        return MDRL_ERR_INVALID_ARG;
    }
    int no = 0, ne = 0;
    for (int i = 0; i < n; ++i) {
        /* the GPU binning's cell coordinate: floor(x / edge) in FP32, clamped into the grid */
        const float f = std::floor(x[i] / edge[0]);
        const int cx = !(f >= 0.0f) ? 0 : (f >= (float)nc[0] ? nc[0] - 1 : (int)f);
        if (cx < s->x0 || cx >= s->x1) continue;
        if (owned) owned[no] = i;
        ++no;
        if (cx == s->x0 && s->nranks > 1) {
            if (exported) exported[ne] = i;
            ++ne;
        }
    }
    if (n_owned) *n_owned = no;
    if (n_exported) *n_exported = ne;
    return MDRL_OK;
}

extern "C" mdrl_status mdrl_force_eval_fixed(mdrl_ctx *c, int n, const float *x, const float *y, const float *z,
                                             const float *q, const int *type, int hx0, int hx1, int64_t *F,
                                             mdrl_stats *st) {
    if (!c || n < 0 || (n > 0 && (!x || !y || !z || !F))) {
        set_error("mdrl_force_eval_fixed: null or invalid argument");
        return MDRL_ERR_INVALID_ARG;
    }
    if (c->p.accum != MDRL_ACC_FIXED64) {
        set_error("mdrl_force_eval_fixed: needs MDRL_ACC_FIXED64");
        return MDRL_ERR_INVALID_ARG;
    }
    MDRL_CUDA(cudaSetDevice(c->p.device));
    MDRL_TRY(ensure_capacity(c, n));
    if (hx0 < 0 || hx1 > c->g.nc[0] || hx0 > hx1) {
        set_error("mdrl_force_eval_fixed: home layers must satisfy 0 <= home_x0 <= home_x1 <= ncell[0]");
        return MDRL_ERR_INVALID_ARG;
    }
    const size_t fb = sizeof(float) * (size_t)n;
    const void *dx = n ? mapped(c, x) : nullptr, *dy = n ? mapped(c, y) : nullptr, *dz = n ? mapped(c, z) : nullptr;
    const void *dq = (q && n) ? mapped(c, q) : nullptr, *dt = (type && n) ? mapped(c, type) : nullptr;
    void *dF = n ? mapped(c, F) : nullptr;
    const bool direct = n > 0 && dx && dy && dz && (!q || dq) && (!type || dt);
    if (n > 0 && !direct) {
        MDRL_CUDA(cudaMemcpyAsync(c->d_ux, x, fb, cudaMemcpyHostToDevice, c->stream));
        MDRL_CUDA(cudaMemcpyAsync(c->d_uy, y, fb, cudaMemcpyHostToDevice, c->stream));
        MDRL_CUDA(cudaMemcpyAsync(c->d_uz, z, fb, cudaMemcpyHostToDevice, c->stream));
        if (q) MDRL_CUDA(cudaMemcpyAsync(c->d_uq, q, fb, cudaMemcpyHostToDevice, c->stream));
        if (type) MDRL_CUDA(cudaMemcpyAsync(c->d_ut, type, sizeof(int) * (size_t)n, cudaMemcpyHostToDevice, c->stream));
        dx = c->d_ux; dy = c->d_uy; dz = c->d_uz;
        dq = q ? c->d_uq : nullptr;
        dt = type ? c->d_ut : nullptr;
    }
    if (!dF && n > 0 && !c->d_Fscr64) MDRL_TRY(dalloc(&c->d_Fscr64, 3 * (size_t)c->cap));
    long long *Fout = dF ? (long long *)dF : (long long *)c->d_Fscr64;
    MDRL_CUDA(cudaMemsetAsync(c->d_tot, 0, sizeof(DevTotals), c->stream));
    MDRL_CUDA(cudaEventRecord(c->ev0, c->stream));
    MDRL_TRY(bin_user(c, n, (const float *)dx, (const float *)dy, (const float *)dz, (const float *)dq,
                      (const int *)dt, 0, true, direct, true));
    const int per_layer = c->g.nc[1] * c->g.nc[2] * kHalfShellCells;
    const int units = (hx1 - hx0) * per_layer;
    MDRL_TRY(launch_force_into(c, n, c->d_pos[0], c->d_type[0], false, c->d_F64, nullptr, hx0 * per_layer, units));
    k_totals<<<1, 1024, 0, c->stream>>>(force_slots(c, units), c->d_unit, 0, c->d_kepart, c->d_tot, 0);
    if (n > 0) k_unsort_fixed<<<nblk(n, 256), 256, 0, c->stream>>>(n, c->d_inv, c->d_F64, Fout);
    MDRL_CUDA(cudaGetLastError());
    MDRL_CUDA(cudaEventRecord(c->ev1, c->stream));
    if (n > 0 && !dF)
        MDRL_CUDA(cudaMemcpyAsync(F, c->d_Fscr64, 3 * sizeof(long long) * (size_t)n, cudaMemcpyDeviceToHost, c->stream));
    MDRL_CUDA(cudaStreamSynchronize(c->stream));
    MDRL_TRY(check_device_errors(c));
    c->have_state = false;
    float ms = 0.0f;
    if (cudaEventElapsedTime(&ms, c->ev0, c->ev1) != cudaSuccess) cudaGetLastError();
    return read_stats(c, st, ms);
}

extern "C" mdrl_status mdrl_bin(mdrl_ctx *c, int n, const float *x, const float *y, const float *z,
                                int *cell_of, int *cell_count, int *order) {
    if (!c || n < 0 || (n > 0 && (!x || !y || !z))) {
        set_error("mdrl_bin: null or invalid argument");
        return MDRL_ERR_INVALID_ARG;
    }
    MDRL_CUDA(cudaSetDevice(c->p.device));
    MDRL_TRY(ensure_capacity(c, n));
    const size_t fb = sizeof(float) * (size_t)n;
    if (n > 0) {
        MDRL_CUDA(cudaMemcpyAsync(c->d_ux, x, fb, cudaMemcpyHostToDevice, c->stream));
        MDRL_CUDA(cudaMemcpyAsync(c->d_uy, y, fb, cudaMemcpyHostToDevice, c->stream));
        MDRL_CUDA(cudaMemcpyAsync(c->d_uz, z, fb, cudaMemcpyHostToDevice, c->stream));
    }
    MDRL_TRY(bin_user(c, n, c->d_ux, c->d_uy, c->d_uz, nullptr, nullptr, 0, false));
    if (cell_of && n > 0) MDRL_CUDA(cudaMemcpyAsync(cell_of, c->d_cell_of, sizeof(int) * n, cudaMemcpyDeviceToHost, c->stream));
    if (cell_count) MDRL_CUDA(cudaMemcpyAsync(cell_count, c->d_count, sizeof(int) * c->ncells, cudaMemcpyDeviceToHost, c->stream));
    if (order && n > 0) MDRL_CUDA(cudaMemcpyAsync(order, c->d_sorted, sizeof(int) * n, cudaMemcpyDeviceToHost, c->stream));
    MDRL_CUDA(cudaStreamSynchronize(c->stream));
    MDRL_TRY(check_device_errors(c));
    c->have_state = false;
    return MDRL_OK;
}

/* ---- tables ------------------------------------------------------------------------------- */

extern "C" mdrl_status mdrl_set_tables(mdrl_ctx *c, int order, int nseg, int bins, int min_log2,
                                       int nfunc, const float *coef, int flags) {
    if (!c || !coef || order < 1 || order > 3 || nseg < 1 || bins < 16 || bins > 4096 ||
        (bins & (bins - 1)) || (nfunc != 2 && nfunc != 3 && nfunc != 6) ||
        (flags & ~(MDRL_TABLE_RAW | MDRL_TABLE_BIN_LOCAL))) {
        set_error("mdrl_set_tables: invalid argument");
        return MDRL_ERR_INVALID_ARG;
    }
    if ((flags & MDRL_TABLE_BIN_LOCAL) && order < 2) {
        set_error("mdrl_set_tables: the bin-local form is for orders 2 and 3");
        return MDRL_ERR_INVALID_ARG;
    }
    if (min_log2 < -30 || min_log2 > 20 || nseg > 64) {
        set_error("mdrl_set_tables: min_log2 must be in -30..20 and nseg at most 64");
        return MDRL_ERR_INVALID_ARG;
    }
    const double top = std::ldexp(1.0, min_log2 + nseg);
    if (!((double)c->g.rc2 < top)) {
        set_error("mdrl_set_tables: the tables end below rc^2");
        return MDRL_ERR_RANGE;
    }
    MDRL_CUDA(cudaSetDevice(c->p.device));
    const int nidx = nseg * bins, nc = order + 1;
    c->order = order; c->nseg = nseg; c->bins = bins; c->min_log2 = min_log2;
    c->raw = (flags & MDRL_TABLE_RAW) != 0;
    c->local = (flags & MDRL_TABLE_BIN_LOCAL) != 0;
    c->tab.assign((size_t)kNumFunc * nc * nidx, 0.0f);
    memcpy(c->tab.data(), coef, sizeof(float) * (size_t)nfunc * nc * nidx);
    for (int k = 0; k < 2; ++k) {
        if (c->graph_exec[k]) { cudaGraphExecDestroy(c->graph_exec[k]); c->graph_exec[k] = nullptr; }
        if (c->graph[k]) { cudaGraphDestroy(c->graph[k]); c->graph[k] = nullptr; }
    }
    c->graph_n = -1;
    return upload_tables(c);
}

extern "C" mdrl_status mdrl_get_tables(mdrl_ctx *c, int *order, int *nseg, int *bins, int *min_log2,
                                       float *coef) {
    if (!c) { set_error("null context"); return MDRL_ERR_INVALID_ARG; }
    if (order) *order = c->order;
    if (nseg) *nseg = c->nseg;
    if (bins) *bins = c->bins;
    if (min_log2) *min_log2 = c->min_log2;
    if (coef) memcpy(coef, c->tab.data(), sizeof(float) * c->tab.size());
    return MDRL_OK;
}

extern "C" mdrl_status mdrl_get_table_form(mdrl_ctx *c, int *flags) {
    if (!c || !flags) { set_error("mdrl_get_table_form: null argument"); return MDRL_ERR_INVALID_ARG; }
    *flags = (c->raw ? MDRL_TABLE_RAW : 0) | (c->local ? MDRL_TABLE_BIN_LOCAL : 0);
    return MDRL_OK;
}

extern "C" mdrl_status mdrl_get_pair_coefficients(mdrl_ctx *c, float *coef) {
    if (!c || !coef) { set_error("null argument"); return MDRL_ERR_INVALID_ARG; }
    const int T = c->p.ntypes;
    for (int k = 0; k < T * T; ++k) {
        if (c->raw) { coef[4 * k] = 1.0f; coef[4 * k + 1] = -1.0f; coef[4 * k + 2] = 1.0f; coef[4 * k + 3] = -1.0f; }
        else memcpy(coef + 4 * k, c->pcoef.data() + 4 * k, sizeof(float) * 4);
    }
    return MDRL_OK;
}

extern "C" mdrl_status mdrl_set_pair_coefficients(mdrl_ctx *c, const double *coef) {
    if (!c || !coef) { set_error("mdrl_set_pair_coefficients: null argument"); return MDRL_ERR_INVALID_ARG; }
    const int T = c->p.ntypes;
    std::vector<float> pc((size_t)T * T * 4);
    for (size_t k = 0; k < pc.size(); ++k) {
        if (!std::isfinite(coef[k]) || std::fabs(coef[k]) > 3.0e38) {
            set_error("mdrl_set_pair_coefficients: coefficients must be finite FP32 values");
            return MDRL_ERR_INVALID_ARG;
        }
        pc[k] = (float)coef[k];
    }
    MDRL_CUDA(cudaSetDevice(c->p.device));
    if (c->stream) MDRL_CUDA(cudaStreamSynchronize(c->stream));
    c->pcoef = pc;
    c->raw = false;
    /* same size and address: captured step graphs stay valid */
    MDRL_CUDA(cudaMemcpy(c->d_pcoef, pc.data(), sizeof(float) * pc.size(), cudaMemcpyHostToDevice));
    return MDRL_OK;
}

static mdrl_status fit_tables_checked(int order, int nseg, int bins, int min_log2, int samples, float *coef,
                                      bool local, const char *who) {
    if (!coef || order < 1 || order > 3 || nseg < 1 || nseg > 64 || bins < 1 || bins > 4096 ||
        (bins & (bins - 1)) || samples < order + 1 || samples > 1024 || min_log2 < -30 || min_log2 > 20 ||
        (local && order < 2)) {
        set_error(std::string(who) + ": invalid argument");
        return MDRL_ERR_INVALID_ARG;
    }
    std::vector<float> t;
    fit_tables(order, nseg, bins, min_log2, samples, &t, 0.0, local);
    memcpy(coef, t.data(), sizeof(float) * t.size());
    return MDRL_OK;
}

extern "C" mdrl_status mdrl_fit_tables(int order, int nseg, int bins, int min_log2, int samples,
                                       float *coef) {
    return fit_tables_checked(order, nseg, bins, min_log2, samples, coef, false, "mdrl_fit_tables");
}

extern "C" mdrl_status mdrl_fit_tables_bin_local(int order, int nseg, int bins, int min_log2, int samples,
                                                 float *coef) {
    return fit_tables_checked(order, nseg, bins, min_log2, samples, coef, true, "mdrl_fit_tables_bin_local");
}

/* ---- per-pair plugin ---------------------------------------------------------------------- */

typedef void (*pair_fn)(int, const float4 *, const float4 *, const int *, const int *, Geom, TableDev,
                        const float4 *, int, float, float4 *, float2 *, int);

static pair_fn pick_pair(int order, bool sep) {
    switch (order) {
        case 0: return sep ? (pair_fn)k_pair_eval<0, true> : (pair_fn)k_pair_eval<0, false>;
        case 1: return sep ? (pair_fn)k_pair_eval<1, true> : (pair_fn)k_pair_eval<1, false>;
        case 2: return sep ? (pair_fn)k_pair_eval<2, true> : (pair_fn)k_pair_eval<2, false>;
        default: return sep ? (pair_fn)k_pair_eval<3, true> : (pair_fn)k_pair_eval<3, false>;
    }
}

extern "C" mdrl_status mdrl_pair_eval(mdrl_ctx *c, int n, const float *ref, const float *nbr,
                                      const int *tref, const int *tnbr, float *out, float *aux) {
    if (!c || n < 0 || (n > 0 && (!ref || !nbr || !out))) {
        set_error("mdrl_pair_eval: null or invalid argument");
        return MDRL_ERR_INVALID_ARG;
    }
    if (n == 0) return MDRL_OK;
    MDRL_CUDA(cudaSetDevice(c->p.device));
    if (n > c->pcap) {
        MDRL_TRY(dalloc(&c->d_pr, n)); MDRL_TRY(dalloc(&c->d_pn, n)); MDRL_TRY(dalloc(&c->d_pout, n));
        MDRL_TRY(dalloc(&c->d_ptr, n)); MDRL_TRY(dalloc(&c->d_ptn, n)); MDRL_TRY(dalloc(&c->d_paux, n));
        c->pcap = n;
    }
    MDRL_CUDA(cudaMemcpyAsync(c->d_pr, ref, sizeof(float4) * n, cudaMemcpyHostToDevice, c->stream));
    MDRL_CUDA(cudaMemcpyAsync(c->d_pn, nbr, sizeof(float4) * n, cudaMemcpyHostToDevice, c->stream));
    if (tref) MDRL_CUDA(cudaMemcpyAsync(c->d_ptr, tref, sizeof(int) * n, cudaMemcpyHostToDevice, c->stream));
    if (tnbr) MDRL_CUDA(cudaMemcpyAsync(c->d_ptn, tnbr, sizeof(int) * n, cudaMemcpyHostToDevice, c->stream));
    Geom g = c->g;
    if (c->p.flags & MDRL_FLAG_NO_PBC)
        for (int d = 0; d < 3; ++d) { g.L[d] = 0.0f; g.h[d] = 0.0f; }
    pair_fn fn = pick_pair(eff_order(c), c->p.arith == MDRL_ARITH_SEPARATE);
    fn<<<nblk(n, 256), 256, 0, c->stream>>>(n, c->d_pr, c->d_pn, tref ? c->d_ptr : nullptr,
                                            tnbr ? c->d_ptn : nullptr, g, table_dev(c), c->d_pcoef,
                                            c->p.ntypes, c->ke, c->d_pout, aux ? c->d_paux : nullptr,
                                            (c->p.flags & MDRL_FLAG_EXACT_DIFF) ? 1 : 0);
    MDRL_CUDA(cudaGetLastError());
    MDRL_CUDA(cudaMemcpyAsync(out, c->d_pout, sizeof(float4) * n, cudaMemcpyDeviceToHost, c->stream));
    if (aux) MDRL_CUDA(cudaMemcpyAsync(aux, c->d_paux, sizeof(float2) * n, cudaMemcpyDeviceToHost, c->stream));
    MDRL_CUDA(cudaStreamSynchronize(c->stream));
    return MDRL_OK;
}

/* ---- molecular dynamics on device state ---------------------------------------------------- */

extern "C" mdrl_status mdrl_set_state(mdrl_ctx *c, int n, const float *x, const float *y, const float *z,
                                      const float *vx, const float *vy, const float *vz, const float *q,
                                      const int *type) {
    if (!c || n <= 0 || !x || !y || !z || ((vx || vy || vz) && !(vx && vy && vz))) {
        set_error("mdrl_set_state: null or invalid argument");
        return MDRL_ERR_INVALID_ARG;
    }
    MDRL_CUDA(cudaSetDevice(c->p.device));
    MDRL_TRY(ensure_capacity(c, n));
    MDRL_TRY(bonded_check_atoms(c, n));
    const size_t fb = sizeof(float) * (size_t)n;
    MDRL_CUDA(cudaMemcpyAsync(c->d_ux, x, fb, cudaMemcpyHostToDevice, c->stream));
    MDRL_CUDA(cudaMemcpyAsync(c->d_uy, y, fb, cudaMemcpyHostToDevice, c->stream));
    MDRL_CUDA(cudaMemcpyAsync(c->d_uz, z, fb, cudaMemcpyHostToDevice, c->stream));
    if (q) MDRL_CUDA(cudaMemcpyAsync(c->d_uq, q, fb, cudaMemcpyHostToDevice, c->stream));
    if (type) MDRL_CUDA(cudaMemcpyAsync(c->d_ut, type, sizeof(int) * (size_t)n, cudaMemcpyHostToDevice, c->stream));
    if (vx) {
        MDRL_CUDA(cudaMemcpyAsync(c->d_ovx, vx, fb, cudaMemcpyHostToDevice, c->stream));
        MDRL_CUDA(cudaMemcpyAsync(c->d_ovy, vy, fb, cudaMemcpyHostToDevice, c->stream));
        MDRL_CUDA(cudaMemcpyAsync(c->d_ovz, vz, fb, cudaMemcpyHostToDevice, c->stream));
    }
    MDRL_CUDA(cudaMemsetAsync(c->d_tot, 0, sizeof(DevTotals), c->stream));
    c->cur = 0;
    MDRL_TRY(bin_user(c, n, c->d_ux, c->d_uy, c->d_uz, q ? c->d_uq : nullptr, type ? c->d_ut : nullptr, 0, true));
    k_gather_vel<<<nblk(n, 256), 256, 0, c->stream>>>(n, c->d_id[0], vx ? c->d_ovx : nullptr, c->d_ovy,
                                                      c->d_ovz, c->d_vel[0]);
    const bool extra = (c->p.flags & MDRL_FLAG_ENERGY) != 0;
    MDRL_TRY(launch_force(c, n, c->d_pos[0], c->d_type[0], extra));
    MDRL_TRY(pme_enqueue(c, n, c->d_pos[0], c->d_F64, c->d_F32, extra));
    MDRL_TRY(bonded_enqueue(c, n, c->d_pos[0], c->d_id[0], c->d_F64, c->d_F32, extra));
    k_kick<<<nblk(n, 256), 256, 0, c->stream>>>(n, c->d_vel[0], c->d_type[0], c->d_F64, c->d_F32, c->d_mt, 0,
                                                c->d_kepart);
    k_totals<<<1, 1024, 0, c->stream>>>(force_slots(c, force_items(c->ncells)), c->d_unit, nblk(n, 256), c->d_kepart, c->d_tot,
                                       extra ? 1 : 0);
    if (extra) MDRL_TRY(pme_add_energy(c, n));
    if (extra) MDRL_TRY(bonded_add_energy(c, n));
    MDRL_CUDA(cudaGetLastError());
    MDRL_CUDA(cudaStreamSynchronize(c->stream));
    MDRL_TRY(check_device_errors(c));
    c->n = n;
    c->have_state = true;
    return MDRL_OK;
}

/* One step of kernels on the context stream (captured into a graph by mdrl_step). */
static mdrl_status enqueue_step(mdrl_ctx *c, bool extra) {
    const int n = c->n;
    const int a = c->cur, b = 1 - c->cur;
    const bool vv = c->p.integrator == MDRL_INT_VELOCITY_VERLET;
    const MassTab *mt = vv ? c->d_mt : c->d_mt + 1;
    const float dt = (float)c->p.dt_fs;
    MDRL_CUDA(cudaMemsetAsync(c->d_count, 0, sizeof(int) * c->ncells, c->stream));
    k_kick_drift_bin<<<nblk(n, 256), 256, 0, c->stream>>>(n, c->d_pos[a], c->d_vel[a], c->d_type[a], c->d_F64,
                                                          c->d_F32, mt, dt, c->g, c->d_cell_of, c->d_slot,
                                                          c->d_count, c->d_key);
    k_scan<<<1, 1024, 0, c->stream>>>(c->ncells, c->d_count, c->d_start, c->d_tot);
    k_scatter<<<nblk(n, 256), 256, 0, c->stream>>>(n, c->d_cell_of, c->d_slot, c->d_start, c->d_tmp);
    k_cell_sort<<<c->ncells, 128, 0, c->stream>>>(c->d_start, c->d_tmp, c->d_sorted, c->d_key, c->d_sortkey,
                                                   c->d_err);
    k_gather_state<<<nblk(n, 256), 256, 0, c->stream>>>(n, c->d_sorted, c->d_pos[a], c->d_vel[a], c->d_type[a],
                                                        c->d_id[a], c->d_pos[b], c->d_vel[b], c->d_type[b],
                                                        c->d_id[b], c->d_F64, c->d_F32);
    if (extra) MDRL_CUDA(cudaMemsetAsync(c->d_cnt, 0, sizeof(int) * (size_t)n, c->stream));
    MDRL_TRY(launch_force(c, n, c->d_pos[b], c->d_type[b], extra));
    MDRL_TRY(pme_enqueue(c, n, c->d_pos[b], c->d_F64, c->d_F32, extra));
    MDRL_TRY(bonded_enqueue(c, n, c->d_pos[b], c->d_id[b], c->d_F64, c->d_F32, extra));
    /* kinetic energy only when energies are requested */
    if (vv || extra)
        k_kick<<<nblk(n, 256), 256, 0, c->stream>>>(n, c->d_vel[b], c->d_type[b], c->d_F64, c->d_F32, c->d_mt,
                                                    vv ? 1 : 0, extra ? c->d_kepart : nullptr);
    k_totals<<<1, 1024, 0, c->stream>>>(force_slots(c, force_items(c->ncells)), c->d_unit, extra ? nblk(n, 256) : 0,
                                       c->d_kepart, c->d_tot, extra ? 1 : 0);
    if (extra) MDRL_TRY(pme_add_energy(c, n));
    if (extra) MDRL_TRY(bonded_add_energy(c, n));
    MDRL_CUDA(cudaGetLastError());
    return MDRL_OK;
}

extern "C" mdrl_status mdrl_step(mdrl_ctx *c, int nsteps, mdrl_stats *st) {
    if (!c || nsteps < 0) { set_error("mdrl_step: invalid argument"); return MDRL_ERR_INVALID_ARG; }
    if (!c->have_state) { set_error("mdrl_step: call mdrl_set_state first"); return MDRL_ERR_STATE; }
    MDRL_CUDA(cudaSetDevice(c->p.device));
    const bool extra = (c->p.flags & MDRL_FLAG_ENERGY) != 0;
    MDRL_CUDA(cudaMemsetAsync(c->d_tot, 0, offsetof(DevTotals, pairs_total), c->stream));
    MDRL_CUDA(cudaMemsetAsync(&c->d_tot->pairs_total, 0, sizeof(unsigned long long), c->stream));
    MDRL_CUDA(cudaMemsetAsync(c->d_err, 0, sizeof(unsigned), c->stream));
    if (c->graph_n != c->n || c->graph_extra != extra) {
        /* Capture one step per buffer parity (slot 0 -> 1 and slot 1 -> 0). */
        const int saved = c->cur;
        for (int k = 0; k < 2; ++k) {
            if (c->graph_exec[k]) { cudaGraphExecDestroy(c->graph_exec[k]); c->graph_exec[k] = nullptr; }
            if (c->graph[k]) { cudaGraphDestroy(c->graph[k]); c->graph[k] = nullptr; }
            c->cur = k;
            MDRL_CUDA(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
            const mdrl_status s = enqueue_step(c, extra);
            cudaGraph_t g = nullptr;
            const cudaError_t e = cudaStreamEndCapture(c->stream, &g);
            c->cur = saved;
            if (s != MDRL_OK) { if (g) cudaGraphDestroy(g); return s; }
            if (e != cudaSuccess) { set_error(std::string("graph capture: ") + cudaGetErrorString(e)); return MDRL_ERR_CUDA; }
            c->graph[k] = g;
            MDRL_CUDA(cudaGraphInstantiate(&c->graph_exec[k], g, 0));
        }
        c->graph_n = c->n;
        c->graph_extra = extra;
    }
    MDRL_CUDA(cudaEventRecord(c->ev0, c->stream));
    for (int k = 0; k < nsteps; ++k) {
        MDRL_CUDA(cudaGraphLaunch(c->graph_exec[c->cur], c->stream));
        c->cur ^= 1;
    }
    MDRL_CUDA(cudaEventRecord(c->ev1, c->stream));
    MDRL_CUDA(cudaStreamSynchronize(c->stream));
    float ms = 0.0f;
    MDRL_CUDA(cudaEventElapsedTime(&ms, c->ev0, c->ev1));
    MDRL_TRY(read_stats(c, st, ms));
    return check_device_errors(c);
}

extern "C" mdrl_status mdrl_time_force(mdrl_ctx *c, float *ms) {
    if (!c || !ms) { set_error("mdrl_time_force: null argument"); return MDRL_ERR_INVALID_ARG; }
    if (!c->have_state) { set_error("mdrl_time_force: call mdrl_set_state first"); return MDRL_ERR_STATE; }
    MDRL_CUDA(cudaSetDevice(c->p.device));
    const int n = c->n, a = c->cur;
    const bool fp32 = c->p.accum != MDRL_ACC_FIXED64;
    if (fp32 && !c->d_Fscr32) MDRL_TRY(dalloc(&c->d_Fscr32, 6 * (size_t)c->cap));
    if (!fp32 && !c->d_Fscr64) MDRL_TRY(dalloc(&c->d_Fscr64, 3 * (size_t)c->cap));
    if (fp32) MDRL_CUDA(cudaMemsetAsync(c->d_Fscr32, 0, sizeof(float) * 6 * (size_t)n, c->stream));
    else MDRL_CUDA(cudaMemsetAsync(c->d_Fscr64, 0, sizeof(unsigned long long) * 3 * (size_t)n, c->stream));
    MDRL_TRY(launch_force_into(c, n, c->d_pos[a], c->d_type[a], false, c->d_Fscr64, c->d_Fscr32));
    MDRL_CUDA(cudaStreamSynchronize(c->stream));
    MDRL_CUDA(cudaEventElapsedTime(ms, c->evf0, c->evf1));
    return MDRL_OK;
}

extern "C" mdrl_status mdrl_get_state(mdrl_ctx *c, float *x, float *y, float *z, float *vx, float *vy,
                                      float *vz, float *fx, float *fy, float *fz) {
    if (!c) { set_error("null context"); return MDRL_ERR_INVALID_ARG; }
    if (!c->have_state) { set_error("mdrl_get_state: no state"); return MDRL_ERR_STATE; }
    MDRL_CUDA(cudaSetDevice(c->p.device));
    const int n = c->n, a = c->cur;
    k_unsort_state<<<nblk(n, 256), 256, 0, c->stream>>>(n, c->d_id[a], c->d_pos[a], c->d_vel[a], c->d_ux, c->d_uy,
                                                        c->d_uz, c->d_ovx, c->d_ovy, c->d_ovz);
    k_unsort<<<nblk(n, 256), 256, 0, c->stream>>>(n, c->d_id[a], c->d_F64, c->d_F32, c->d_cnt, c->d_ox, c->d_oy,
                                                  c->d_oz, nullptr);
    MDRL_CUDA(cudaGetLastError());
    const size_t fb = sizeof(float) * (size_t)n;
    float *dst[9] = {x, y, z, vx, vy, vz, fx, fy, fz};
    const float *src[9] = {c->d_ux, c->d_uy, c->d_uz, c->d_ovx, c->d_ovy, c->d_ovz, c->d_ox, c->d_oy, c->d_oz};
    for (int k = 0; k < 9; ++k)
        if (dst[k]) MDRL_CUDA(cudaMemcpyAsync(dst[k], src[k], fb, cudaMemcpyDeviceToHost, c->stream));
    MDRL_CUDA(cudaStreamSynchronize(c->stream));
    return MDRL_OK;
}

/* ---- tiles and the autotuner --------------------------------------------------------------- */

static mdrl_status check_tile(const mdrl_tile *t, bool allow8, bool allow_prune, bool allow_warp) {
    if (t && t->warps_per_cta == 1) {
        /* the warp-item kernel: steps_per_piece = i-tile groups per unit; it always prunes */
        if (t->steps_per_piece < 1 || t->steps_per_piece > kMaxItemGroups || t->prune_steps != 1) {
            set_error("tile: one warp per item takes 1..4 i-tile groups (steps_per_piece) and prune_steps 1");
            return MDRL_ERR_INVALID_ARG;
        }
        if (!allow_warp) {
            set_error("tile: one warp per item needs MDRL_ACC_FIXED64");
            return MDRL_ERR_INVALID_ARG;
        }
        return MDRL_OK;
    }
    if (!t || (t->warps_per_cta != 4 && t->warps_per_cta != 8) || t->steps_per_piece < 1 ||
        t->steps_per_piece > 32 || (t->prune_steps != 0 && t->prune_steps != 1)) {
        set_error("tile: warps_per_cta must be 1, 4 or 8, steps_per_piece in 1..32, prune_steps 0 or 1");
        return MDRL_ERR_INVALID_ARG;
    }
    if (t->warps_per_cta == 8 && !allow8) {
        set_error("tile: 8 warps per CTA needs MDRL_ACC_FIXED64 (and no batch)");
        return MDRL_ERR_INVALID_ARG;
    }
    if (t->prune_steps && !allow_prune) {
        set_error("tile: pruning needs MDRL_ACC_FIXED64");
        return MDRL_ERR_INVALID_ARG;
    }
    return MDRL_OK;
}

static void drop_graphs(mdrl_ctx *c) {
    for (int k = 0; k < 2; ++k) {
        if (c->graph_exec[k]) { cudaGraphExecDestroy(c->graph_exec[k]); c->graph_exec[k] = nullptr; }
        if (c->graph[k]) { cudaGraphDestroy(c->graph[k]); c->graph[k] = nullptr; }
    }
    c->graph_n = -1;
}

namespace mdrl {
mdrl_status set_tile(mdrl_ctx *c, const mdrl_tile *t, bool allow8, bool allow_warp) {
    MDRL_TRY(check_tile(t, allow8, c->p.accum == MDRL_ACC_FIXED64, allow_warp));
    if (t->warps_per_cta != c->tile.warps_per_cta || t->steps_per_piece != c->tile.steps_per_piece ||
        t->prune_steps != c->tile.prune_steps) {
        MDRL_CUDA(cudaSetDevice(c->p.device));
        if (c->stream) MDRL_CUDA(cudaStreamSynchronize(c->stream));
        drop_graphs(c);
        c->tile = *t;
    }
    return MDRL_OK;
}

/* The process-wide tuning cache, optionally backed by the file named by MDRL_TUNE_CACHE. */
static std::mutex g_tune_mu;
static std::map<std::string, mdrl_tile> g_tune;
static bool g_tune_loaded = false;

static void tune_load_locked() {
    if (g_tune_loaded) return;
    g_tune_loaded = true;
    const char *path = getenv("MDRL_TUNE_CACHE");
    if (!path || !*path) return;
    std::ifstream in(path);
    std::string key;
    int w, s, pr;
    float ms;
    while (in >> key >> w >> s >> pr >> ms)
        if (((w == 4 || w == 8) && s >= 1 && s <= 32 && (pr == 0 || pr == 1)) ||
            (w == 1 && s >= 1 && s <= kMaxItemGroups && pr == 1))
            g_tune[key] = mdrl_tile{w, s, pr};
}

static void tune_store_locked(const std::string &key, const mdrl_tile &t, float ms) {
    g_tune[key] = t;
    const char *path = getenv("MDRL_TUNE_CACHE");
    if (!path || !*path) return;
    std::ofstream out(path, std::ios::app);
    out << key << ' ' << t.warps_per_cta << ' ' << t.steps_per_piece << ' ' << t.prune_steps << ' ' << ms << '\n';
}

bool tune_lookup(const std::string &key, mdrl_tile *t) {
    std::lock_guard<std::mutex> lock(g_tune_mu);
    tune_load_locked();
    auto it = g_tune.find(key);
    if (it == g_tune.end()) return false;
    *t = it->second;
    return true;
}

void tune_store(const std::string &key, const mdrl_tile &t, float ms) {
    std::lock_guard<std::mutex> lock(g_tune_mu);
    tune_load_locked();
    tune_store_locked(key, t, ms);
}

std::string tune_key_common(const mdrl_ctx *c) {
    char buf[160];
    snprintf(buf, sizeof buf, "t%d-o%d-b%d-a%d-c%d-q%d-e%d", c->p.ntypes, eff_order(c), c->bins, c->p.arith,
             c->p.accum, c->ke != 0.0f ? 1 : 0, c->p.eval);
    return buf;
}
}  // namespace mdrl

static const int kTuneSpp[] = {3, 4, 6, 8, 12};

extern "C" mdrl_status mdrl_set_tile(mdrl_ctx *c, const mdrl_tile *t) {
    if (!c || !t) { set_error("mdrl_set_tile: null argument"); return MDRL_ERR_INVALID_ARG; }
    return set_tile(c, t, c->p.accum == MDRL_ACC_FIXED64, c->p.accum == MDRL_ACC_FIXED64);
}

extern "C" mdrl_status mdrl_get_tile(mdrl_ctx *c, mdrl_tile *t) {
    if (!c || !t) { set_error("mdrl_get_tile: null argument"); return MDRL_ERR_INVALID_ARG; }
    *t = c->tile;
    return MDRL_OK;
}

extern "C" mdrl_status mdrl_autotune(mdrl_ctx *c, int flags, mdrl_tile *best, float *best_ms, float *default_ms) {
    if (!c) { set_error("mdrl_autotune: null context"); return MDRL_ERR_INVALID_ARG; }
    if (!c->have_state) { set_error("mdrl_autotune: call mdrl_set_state first"); return MDRL_ERR_STATE; }
    MDRL_CUDA(cudaSetDevice(c->p.device));
    char buf[96];
    const int ppc8 = (int)std::lround(8.0 * c->n / std::max(1, c->ncells));
    snprintf(buf, sizeof buf, "ctx-%dx%dx%d-p%d-", c->g.nc[0], c->g.nc[1], c->g.nc[2], ppc8);
    const std::string key = std::string(buf) + tune_key_common(c);
    auto time_tile = [&](const mdrl_tile &t, float *ms) -> mdrl_status {
        MDRL_TRY(set_tile(c, &t, true, true));
        float v[5];
        for (int r = 0; r < 5; ++r) MDRL_TRY(mdrl_time_force(c, &v[r]));
        std::sort(v, v + 5);
        *ms = v[2];
        return MDRL_OK;
    };
    const mdrl_tile def = {kFW, kStepsPerPiece, 0};
    mdrl_tile pick = def;
    float pick_ms = 0.0f, def_ms = 0.0f;
    const bool cached = !(flags & MDRL_TUNE_RETIME) && tune_lookup(key, &pick);
    if (cached) {
        MDRL_TRY(time_tile(pick, &pick_ms));
        if (default_ms) MDRL_TRY(time_tile(def, &def_ms));
    } else {
        pick_ms = 3.0e38f;
        const int nfw = c->p.accum == MDRL_ACC_FIXED64 ? 2 : 1;
        for (int a = 0; a < nfw; ++a)
            for (int spp : kTuneSpp)
                for (int pr = 0; pr < nfw; ++pr) {   /* pruning exists with fixed point only */
                    const mdrl_tile t = {a == 0 ? 4 : 8, spp, pr};
                    float ms;
                    MDRL_TRY(time_tile(t, &ms));
                    if (t.warps_per_cta == def.warps_per_cta && t.steps_per_piece == def.steps_per_piece &&
                        t.prune_steps == def.prune_steps)
                        def_ms = ms;
                    if (ms < pick_ms) { pick_ms = ms; pick = t; }
                }
        if (c->p.accum == MDRL_ACC_FIXED64)
            for (int grp = 1; grp <= 3; ++grp) {   /* one warp per (unit, i-tile group) */
                const mdrl_tile t = {1, grp, 1};
                float ms;
                MDRL_TRY(time_tile(t, &ms));
                if (ms < pick_ms) { pick_ms = ms; pick = t; }
            }
        tune_store(key, pick, pick_ms);
    }
    MDRL_TRY(set_tile(c, &pick, true, true));
    if (best) *best = pick;
    if (best_ms) *best_ms = pick_ms;
    if (default_ms) *default_ms = def_ms;
    return MDRL_OK;
}

/* ---- long-range electrostatics ------------------------------------------------------------- */

extern "C" mdrl_status mdrl_set_pme(mdrl_ctx *c, const mdrl_pme_params *p) {
    if (!c) { set_error("mdrl_set_pme: null context"); return MDRL_ERR_INVALID_ARG; }
    MDRL_CUDA(cudaSetDevice(c->p.device));
    if (c->stream) MDRL_CUDA(cudaStreamSynchronize(c->stream));
    drop_graphs(c);
    double beta = 0.0;
    if (p) {
        MDRL_TRY(pme_setup(c, p));
        mdrl_pme_params r;
        mdrl_get_pme(c, &r, nullptr);
        beta = r.beta;
    } else {
        pme_free(c);
    }
    /* the Coulomb slots: Ewald real-space pair with PME, plain r^-3 / r^-1 without */
    c->raw = false;
    c->local = c->order >= 2;
    fit_tables(c->order, c->nseg, c->bins, c->min_log2, 8, &c->tab, beta, c->local);
    return upload_tables(c);
}
