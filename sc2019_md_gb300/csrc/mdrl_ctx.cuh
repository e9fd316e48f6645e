/*
 * mdrl_ctx.cuh — the context structure and host helpers shared by mdrl.cu (single system) and
 * mdrl_batch.cu (batched replicas).
 */
#pragma once

#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "mdrl_internal.h"
#include "mdrl_force.cuh"

using mdrl::set_error;

namespace mdrl {
struct PmeState;
struct BondedState;
}

#define MDRL_CUDA(call)                                                                   \
    do {                                                                                  \
        if (mdrl::fault_hit(#call)) {                                                     \
            set_error(std::string(#call) + ": injected failure (MDRL_FAULT)");           \
            return MDRL_ERR_CUDA;                                                         \
        }                                                                                 \
        cudaError_t e_ = (call);                                                          \
        if (e_ != cudaSuccess) {                                                          \
            set_error(std::string(#call) + ": " + cudaGetErrorString(e_));                \
            return MDRL_ERR_CUDA;                                                         \
        }                                                                                 \
    } while (0)

#define MDRL_TRY(expr)                         \
    do {                                       \
        mdrl_status s_ = (expr);               \
        if (s_ != MDRL_OK) return s_;          \
    } while (0)

template <class T>
inline mdrl_status dalloc(T **p, size_t count) {
    if (*p) { cudaFree(*p); *p = nullptr; }
    if (count == 0) return MDRL_OK;
    MDRL_CUDA(cudaMalloc((void **)p, sizeof(T) * count));
    return MDRL_OK;
}

template <class T>
inline void dfree(T **p) {
    if (*p) { cudaFree(*p); *p = nullptr; }
}

struct mdrl_ctx {
    typedef mdrl::Geom Geom;
    typedef mdrl::MassTab MassTab;
    typedef mdrl::UnitOut UnitOut;
    typedef mdrl::DevTotals DevTotals;
    mdrl_params p;
    Geom g;
    int ncells = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    cudaEvent_t evf0 = nullptr, evf1 = nullptr; /* around the force kernel */

    /* tables */
    int order = 1, nseg = 0, bins = 256, min_log2 = -2;
    bool raw = false;
    bool local = false;          /* coefficients in u = r2 - bin start (MDRL_TABLE_BIN_LOCAL) */
    std::vector<float> tab;      /* canonical [6][order+1][nseg*bins] */
    std::vector<float> pcoef;    /* [T*T*4] */
    float ke = 0.0f;
    float2 *d_f2 = nullptr, *d_e2 = nullptr;
    float4 *d_f4 = nullptr, *d_e4 = nullptr, *d_fp2 = nullptr;
    float *d_fc2 = nullptr;
    float4 *d_fr = nullptr;      /* order 1: force functions packed per index (32 B) */
    float4 *d_pcoef = nullptr;
    MassTab mt_half, mt_full;
    MassTab *d_mt = nullptr;     /* device copies: [0] half kick, [1] full kick */

    /* particle buffers */
    int cap = 0, n = 0;
    float *d_ux = nullptr, *d_uy = nullptr, *d_uz = nullptr, *d_uq = nullptr;
    int *d_ut = nullptr;
    int *d_inv = nullptr;   /* cell-order position of each user index (force evaluations) */
    float *d_ox = nullptr, *d_oy = nullptr, *d_oz = nullptr; /* user-order outputs */
    float *d_ovx = nullptr, *d_ovy = nullptr, *d_ovz = nullptr;
    int *d_ocnt = nullptr;
    float4 *d_pos[2] = {nullptr, nullptr}, *d_vel[2] = {nullptr, nullptr};
    int *d_type[2] = {nullptr, nullptr}, *d_id[2] = {nullptr, nullptr};
    int cur = 0;
    int *d_cell_of = nullptr, *d_slot = nullptr, *d_tmp = nullptr, *d_sorted = nullptr;
    int *d_count = nullptr, *d_start = nullptr;
    int *d_work = nullptr;      /* the persistent warp kernel's item counter */
    unsigned *d_key = nullptr;   /* in-cell sort key (Morton code inside the cell) */
    unsigned long long *d_sortkey = nullptr;   /* sorted chunks of cells above kSortSmall */
    unsigned long long *d_F64 = nullptr;
    float *d_F32 = nullptr;
    unsigned long long *d_Fscr64 = nullptr; /* scratch accumulators for mdrl_time_force */
    float *d_Fscr32 = nullptr;
    int *d_cnt = nullptr;
    UnitOut *d_unit = nullptr;
    double *d_kepart = nullptr;
    int kecap = 0;
    DevTotals *d_tot = nullptr;
    DevTotals *h_tot = nullptr;  /* pinned host copies, read back with the results of a call */
    unsigned *h_err = nullptr;
    DevTotals *h_tot_dev = nullptr;  /* the same two, as device addresses */
    unsigned *h_err_dev = nullptr;
    unsigned *d_err = nullptr;
    int num_sms = 0;

    /* pair-eval staging */
    int pcap = 0;
    float4 *d_pr = nullptr, *d_pn = nullptr, *d_pout = nullptr;
    int *d_ptr = nullptr, *d_ptn = nullptr;
    float2 *d_paux = nullptr;

    /* state */
    bool have_state = false;
    cudaGraph_t graph[2] = {nullptr, nullptr};          /* one step from buffer slot k to 1-k */
    cudaGraphExec_t graph_exec[2] = {nullptr, nullptr};
    int graph_n = -1;
    bool graph_extra = false;

    /* long-range electrostatics (mdrl_set_pme), null when off */
    mdrl::PmeState *pme = nullptr;
    mdrl::BondedState *bonded = nullptr;   /* bonded terms (mdrl_set_bonded), or none */

    /* force-kernel tile (mdrl_set_tile / mdrl_autotune) */
    mdrl_tile tile = {mdrl::kFW, mdrl::kStepsPerPiece, 0};
};

namespace mdrl {
mdrl_status ensure_capacity(mdrl_ctx *c, int n);
TableDev table_dev(const mdrl_ctx *c);
int eff_order(const mdrl_ctx *c);
mdrl_status check_device_errors(mdrl_ctx *c);

/* Raise the dynamic shared-memory limit of a force kernel once per kernel and device. */
mdrl_status prepare_force_kernel(force_fn fn, int device);
inline int nblk(int n, int b) { return (n + b - 1) / b; }
/* PME (mdrl_pme.cu): setup, teardown, the reciprocal part of a force evaluation, its energies. */
mdrl_status pme_setup(mdrl_ctx *c, const mdrl_pme_params *p);
void pme_free(mdrl_ctx *c);
mdrl_status pme_enqueue(mdrl_ctx *c, int n, const float4 *pos, unsigned long long *F64, float *F32, bool energy);
mdrl_status pme_add_energy(mdrl_ctx *c, int n);
/* Bonded terms (mdrl_bonded.cu): forces into the accumulators of cell-order buffer pos / pid
 * (after the pair kernel), energies into the totals (after k_totals). */
mdrl_status bonded_enqueue(mdrl_ctx *c, int n, const float4 *pos, const int *pid, unsigned long long *F64,
                           float *F32, bool energy);
mdrl_status bonded_add_energy(mdrl_ctx *c, int n);
mdrl_status bonded_check_atoms(const mdrl_ctx *c, int n);
void bonded_free(mdrl_ctx *c);
mdrl_status upload_tables(mdrl_ctx *c);
/* Tiles: change (re-capturing graphs), and the autotuner's process-wide cache. */
/* allow8: 8-warp CTAs and pruning (fixed point, one system); allow_warp: one warp per item
 * (fixed point) */
mdrl_status set_tile(mdrl_ctx *c, const mdrl_tile *t, bool allow8, bool allow_warp);
bool tune_lookup(const std::string &key, mdrl_tile *t);
void tune_store(const std::string &key, const mdrl_tile &t, float ms);
std::string tune_key_common(const mdrl_ctx *c);
}  // namespace mdrl
