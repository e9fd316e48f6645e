/*
 * mdrl_batch.cu — batched independent replicas.
 *
 * A batch holds any number of periodic systems of different sizes and box shapes that share the
 * force field (types, cutoff, tables, integrator).  Their particles are concatenated: replica r
 * owns [p_off_r, p_off_r + n_r) of the user arrays and, after every binning, of the cell-sorted
 * arrays too (global cell ids are replica-major, so the scan over all cells keeps each replica's
 * particles together).  A step is one launch per kernel for the whole batch, captured in a CUDA
 * graph: kick + drift + bin (per-particle replica geometry), scan, scatter, in-cell sort, gather,
 * one force launch over a work list, second kick, totals.
 *
 * Force work list.  A replica with at least 3 cells of edge >= rc per axis contributes its
 * ncells x 14 half-shell units (the single-system kernel with its per-unit periodic shift, the
 * replica's geometry and cell offset).  One with fewer cells but every edge above 2 rc contributes every pair of its
 * cells (a <= b) within reach, evaluated by the same tiled Newton-3 code with the per-pair
 * minimum image.  One with an edge of at most 2 rc (always above rc) contributes blocks of 128
 * particles that sum every periodic image within rc.  Items are ordered by estimated cost,
 * largest first, so the block scheduler (the dynamic work queue of the launch) starts the long
 * ones early.
 *
 * Accumulation is int64 fixed point only: the all-pairs blocks store complete per-particle
 * forces and the half-shell units add theirs with integer atomics, both exact.
 */
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <numeric>
#include <string>
#include <vector>

#include "mdrl_ctx.cuh"
#include "mdrl_force_warp.cuh"

using namespace mdrl;

namespace {

struct RepTotals {
    double e_lj, e_coul, virial, kinetic;
    unsigned long long pairs, below;
};

/* Cell of each user-order particle in its replica's grid, with the arrival slot. */
__global__ void k_bbin_user(int n, const float *__restrict__ x, const float *__restrict__ y,
                            const float *__restrict__ z, const int *__restrict__ rep_of,
                            const BatchRep *__restrict__ reps, int *__restrict__ cell_of,
                            int *__restrict__ slot, int *__restrict__ count, unsigned *__restrict__ err,
                            unsigned *__restrict__ key) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const BatchRep &rp = reps[rep_of[i]];
    const Geom g = rp.g;
    const float px = x[i], py = y[i], pz = z[i];
    if (!in_box(g, px, py, pz)) atomicOr(err, kErrPosition);
    const int c = cell_of_pos(g, px, py, pz);
    key[i] = cell_morton(g, px, py, pz, c);
    const int gc = rp.cell_off + c;
    cell_of[i] = gc;
    slot[i] = cell_slot(count, gc);
}

/* v += F * cm[type], x += v * dt, wrap into the replica's box, bin. */
__global__ void k_bkick_drift_bin(int n, float4 *__restrict__ pos, float4 *__restrict__ vel,
                                  const int *__restrict__ ptype, const unsigned long long *__restrict__ F64,
                                  const MassTab *__restrict__ mt, float dt, const int *__restrict__ rep_of,
                                  const BatchRep *__restrict__ reps, int *__restrict__ cell_of,
                                  int *__restrict__ slot, int *__restrict__ count, unsigned *__restrict__ key) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const BatchRep &rp = reps[rep_of[k]];
    const Geom g = rp.g;
    const float cm = mt->cm[ptype[k]];
    float4 v = vel[k];
    float4 p = pos[k];
    v.x = __fmaf_rn(from_fixed(F64[k]), cm, v.x);
    v.y = __fmaf_rn(from_fixed(F64[(size_t)n + k]), cm, v.y);
    v.z = __fmaf_rn(from_fixed(F64[2 * (size_t)n + k]), cm, v.z);
    p.x = wrap_pos(__fmaf_rn(v.x, dt, p.x), g.L[0]);
    p.y = wrap_pos(__fmaf_rn(v.y, dt, p.y), g.L[1]);
    p.z = wrap_pos(__fmaf_rn(v.z, dt, p.z), g.L[2]);
    vel[k] = v;
    pos[k] = p;
    const int c = cell_of_pos(g, p.x, p.y, p.z);
    key[k] = cell_morton(g, p.x, p.y, p.z, c);
    const int gc = rp.cell_off + c;
    cell_of[k] = gc;
    slot[k] = cell_slot(count, gc);
}

/* Per-replica totals of the last force evaluation (its items, in item order) and, when vel is
 * given, its kinetic energy (particles in cell order); one CTA per replica, fixed order. */
/* With a one-warp-per-item tile the slots are laid out as [the other items' CTAs][G slots per
 * half-shell item]; item_begin2 / rep_items2 then list a replica's half-shell items (positions in
 * that list), whose G slots follow slot0 (nullptr: a single list). */
__global__ void __launch_bounds__(128) k_rep_totals(const int *__restrict__ item_begin,
                                                    const int *__restrict__ rep_items,
                                                    const int *__restrict__ item_begin2,
                                                    const int *__restrict__ rep_items2, int slot0, int G,
                                                    const UnitOut *__restrict__ uout,
                                                    const BatchRep *__restrict__ reps,
                                                    const float4 *__restrict__ vel,
                                                    const int *__restrict__ ptype, const MassTab *__restrict__ mt,
                                                    RepTotals *__restrict__ out) {
    __shared__ double s_d[128][4];
    __shared__ unsigned long long s_u[128][2];
    const int r = blockIdx.x, t = threadIdx.x;
    double a = 0, b = 0, c = 0, k = 0;
    unsigned long long p = 0, q = 0;
    for (int e = item_begin[r] + t; e < item_begin[r + 1]; e += 128) {
        const UnitOut u = uout[rep_items[e]];
        a += u.e_lj; b += u.e_coul; c += u.virial;
        p += u.pairs; q += u.below;
    }
    if (item_begin2)
        for (int e = G * item_begin2[r] + t; e < G * item_begin2[r + 1]; e += 128) {
            const UnitOut u = uout[slot0 + G * rep_items2[e / G] + e % G];
            a += u.e_lj; b += u.e_coul; c += u.virial;
            p += u.pairs; q += u.below;
        }
    if (vel) {
        const BatchRep &rp = reps[r];
        for (int e = t; e < rp.n; e += 128) {
            const float4 v = vel[rp.p_off + e];
            const float m = mt->mass[ptype[rp.p_off + e]];
            k += (double)(0.5f * m * (v.x * v.x + v.y * v.y + v.z * v.z) * (1.0f / 4.184e-4f));
        }
    }
    s_d[t][0] = a; s_d[t][1] = b; s_d[t][2] = c; s_d[t][3] = k;
    s_u[t][0] = p; s_u[t][1] = q;
    __syncthreads();
    for (int off = 64; off > 0; off >>= 1) {
        if (t < off) {
            for (int m = 0; m < 4; ++m) s_d[t][m] += s_d[t + off][m];
            s_u[t][0] += s_u[t + off][0];
            s_u[t][1] += s_u[t + off][1];
        }
        __syncthreads();
    }
    if (t == 0) {
        RepTotals o;
        o.e_lj = s_d[0][0]; o.e_coul = s_d[0][1]; o.virial = s_d[0][2]; o.kinetic = s_d[0][3];
        o.pairs = s_u[0][0]; o.below = s_u[0][1];
        out[r] = o;
    }
}

}  // namespace

struct mdrl_batch {
    mdrl_ctx *c = nullptr;   /* force field, tables, stream, events and the particle buffers */
    int nrep = 0, ntot = 0, ncells = 0, nitems = 0;
    std::vector<BatchRep> reps;
    std::vector<BatchItem> items;
    std::vector<int> item_begin, rep_items;
    BatchRep *d_reps = nullptr;
    BatchItem *d_items = nullptr;
    int *d_rep_of = nullptr, *d_item_begin = nullptr, *d_rep_items = nullptr;
    /* the same work split for one-warp-per-item tiles: the warp kernel's list (n_cp explicit cell
     * pairs, then n_hs half-shell units) and the all-image blocks (the CTA kernel), each in cost
     * order, with per-replica lists */
    int n_hs = 0, n_cp = 0, n_ot = 0;
    BatchItem *d_items_hs = nullptr, *d_items_ot = nullptr;
    int *d_begin_hs = nullptr, *d_list_hs = nullptr, *d_begin_ot = nullptr, *d_list_ot = nullptr;
    RepTotals *d_reptot = nullptr;
    bool have_eval = false;  /* the unit outputs hold a force evaluation */
};

/* Replica geometry: cells of edge >= rc (at least one per axis); the path follows from them. */
static mdrl_status replica_geometry(const mdrl_params &p, const mdrl_replica &r, int index, BatchRep *out) {
    char buf[256];
    const float rcf = (float)p.cutoff;
    BatchRep b;
    memset(&b, 0, sizeof(b));
    b.g.rc2 = rcf * rcf;
    bool cells3 = true, min_image = true;
    for (int d = 0; d < 3; ++d) {
        const double Ld = r.box[d];
        const float L = (float)Ld;
        if (!(Ld > 0.0) || !std::isfinite(Ld) || !(L > rcf)) {
            snprintf(buf, sizeof buf, "replica %d: box edge %d (%.6f) must be finite and exceed the cutoff %.6f",
                     index, d, Ld, (double)rcf);
            set_error(buf);
            return MDRL_ERR_RANGE;
        }
        int nc = (int)std::floor((double)L / (double)rcf);
        float edge = (float)((double)L / (double)nc);
        while (nc > 1 && edge < rcf) { --nc; edge = (float)((double)L / (double)nc); }
        b.g.L[d] = L;
        b.g.h[d] = 0.5f * L;
        b.g.nc[d] = nc;
        b.g.edge[d] = edge;
        if (nc < 3) cells3 = false;
        /* the one-wrap image is the only candidate within rc when the edge exceeds 2 rc (with a
         * margin far above FP32 rounding of the difference and its wrap) */
        if (!((double)L >= 2.0 * (double)rcf * (1.0 + 1.0 / 1024.0))) min_image = false;
    }
    b.path = cells3 ? kPathHalfShell : (min_image ? kPathMinImage : kPathAllImages);
    if (r.n < 1) {
        snprintf(buf, sizeof buf, "replica %d: needs at least one particle", index);
        set_error(buf);
        return MDRL_ERR_INVALID_ARG;
    }
    b.n = r.n;
    *out = b;
    return MDRL_OK;
}

extern "C" mdrl_status mdrl_batch_destroy(mdrl_batch *b) {
    if (!b) return MDRL_OK;
    if (b->c) {
        cudaSetDevice(b->c->p.device);
        if (b->c->stream) cudaStreamSynchronize(b->c->stream);
    }
    dfree(&b->d_reps); dfree(&b->d_items); dfree(&b->d_rep_of); dfree(&b->d_item_begin);
    dfree(&b->d_rep_items); dfree(&b->d_reptot);
    dfree(&b->d_items_hs); dfree(&b->d_items_ot); dfree(&b->d_begin_hs); dfree(&b->d_list_hs);
    dfree(&b->d_begin_ot); dfree(&b->d_list_ot);
    if (b->c) mdrl_destroy(b->c);
    delete b;
    return MDRL_OK;
}

extern "C" mdrl_status mdrl_batch_create(const mdrl_params *p, int nrep, const mdrl_replica *reps,
                                         mdrl_batch **out) {
    if (!p || !reps || !out || nrep < 1) { set_error("mdrl_batch_create: null or invalid argument"); return MDRL_ERR_INVALID_ARG; }
    *out = nullptr;
    if (p->accum != MDRL_ACC_FIXED64) {
        set_error("mdrl_batch_create: batched replicas accumulate in int64 fixed point (MDRL_ACC_FIXED64)");
        return MDRL_ERR_INVALID_ARG;
    }
    if (p->flags & MDRL_FLAG_NO_PBC) {
        set_error("mdrl_batch_create: replicas are periodic (MDRL_FLAG_NO_PBC is not supported)");
        return MDRL_ERR_INVALID_ARG;
    }
    if (p->flags & MDRL_FLAG_EXACT_DIFF) {
        set_error("mdrl_batch_create: MDRL_FLAG_EXACT_DIFF is for single systems (the small-box replica "
                  "paths use the reference's difference rule)");
        return MDRL_ERR_INVALID_ARG;
    }
    std::vector<BatchRep> hrep(nrep);
    long long ntot = 0, ncells = 0;
    for (int r = 0; r < nrep; ++r) {
        MDRL_TRY(replica_geometry(*p, reps[r], r, &hrep[r]));
        hrep[r].p_off = (int)ntot;
        hrep[r].cell_off = (int)ncells;
        ntot += reps[r].n;
        ncells += (long long)hrep[r].g.nc[0] * hrep[r].g.nc[1] * hrep[r].g.nc[2];
        if (ntot > (1LL << 28) || ncells > (1LL << 24)) {
            set_error("mdrl_batch_create: too many particles or cells in the batch");
            return MDRL_ERR_RANGE;
        }
    }
    /* work list, with an estimated cost per item (candidate pairs) */
    std::vector<BatchItem> items;
    std::vector<double> cost;
    for (int r = 0; r < nrep; ++r) {
        const BatchRep &b = hrep[r];
        const int nc = b.g.nc[0] * b.g.nc[1] * b.g.nc[2];
        const double ppc = (double)b.n / nc;
        if (b.path == kPathHalfShell) {
            for (int u = 0; u < nc * kHalfShellCells; ++u) {
                items.push_back({r, u});
                cost.push_back((u % kHalfShellCells) == 0 ? 0.5 * ppc * ppc : ppc * ppc);
            }
        } else if (b.path == kPathMinImage) {
            /* every pair of cells a <= b whose minimum-image gap is within rc */
            const double rc = (double)(float)p->cutoff;
            for (int a = 0; a < nc; ++a)
                for (int c = a; c < nc; ++c) {
                    const int ia[3] = {a / (b.g.nc[1] * b.g.nc[2]), (a / b.g.nc[2]) % b.g.nc[1], a % b.g.nc[2]};
                    const int ic[3] = {c / (b.g.nc[1] * b.g.nc[2]), (c / b.g.nc[2]) % b.g.nc[1], c % b.g.nc[2]};
                    double gap2 = 0.0;
                    for (int d = 0; d < 3; ++d) {
                        const int da = std::abs(ia[d] - ic[d]);
                        const int dm = std::min(da, b.g.nc[d] - da);
                        const double gd = std::max(0, dm - 1) * (double)b.g.edge[d];
                        gap2 += gd * gd;
                    }
                    if (gap2 > rc * rc * (1.0 + 1e-6)) continue;
                    items.push_back({r, a * nc + c});
                    cost.push_back(a == c ? 0.5 * ppc * ppc : ppc * ppc);
                }
        } else {
            for (int b0 = 0; b0 < b.n; b0 += kBatchFT) {
                items.push_back({r, b0});
                cost.push_back((double)std::min(kBatchFT, b.n - b0) * b.n * 2.0);
            }
        }
    }
    if (items.size() > (size_t)2147483647) { set_error("mdrl_batch_create: work list too long"); return MDRL_ERR_RANGE; }
    std::vector<int> perm(items.size());
    std::iota(perm.begin(), perm.end(), 0);
    std::stable_sort(perm.begin(), perm.end(), [&](int a, int b) { return cost[a] > cost[b]; });
    mdrl_batch *bt = new mdrl_batch();
    bt->nrep = nrep;
    bt->ntot = (int)ntot;
    bt->ncells = (int)ncells;
    bt->nitems = (int)items.size();
    bt->reps = hrep;
    bt->items.resize(items.size());
    for (size_t k = 0; k < perm.size(); ++k) bt->items[k] = items[perm[k]];
    bt->item_begin.assign(nrep + 1, 0);
    for (const BatchItem &it : bt->items) bt->item_begin[it.rep + 1]++;
    for (int r = 0; r < nrep; ++r) bt->item_begin[r + 1] += bt->item_begin[r];
    bt->rep_items.assign(bt->items.size(), 0);
    {
        std::vector<int> fill(bt->item_begin.begin(), bt->item_begin.end() - 1);
        for (int k = 0; k < bt->nitems; ++k) bt->rep_items[fill[bt->items[k].rep]++] = k;
    }
    /* the split for one-warp-per-item tiles (cost order kept within each list) */
    std::vector<BatchItem> items_hs, items_cp, items_ot;
    for (const BatchItem &it : bt->items) {
        const int path = hrep[it.rep].path;
        (path == kPathHalfShell ? items_hs : (path == kPathMinImage ? items_cp : items_ot)).push_back(it);
    }
    bt->n_hs = (int)items_hs.size();
    bt->n_cp = (int)items_cp.size();
    bt->n_ot = (int)items_ot.size();
    items_hs.insert(items_hs.begin(), items_cp.begin(), items_cp.end());   /* the warp list: pairs, then units */
    auto rep_lists = [&](const std::vector<BatchItem> &v, std::vector<int> &begin, std::vector<int> &list) {
        begin.assign(nrep + 1, 0);
        for (const BatchItem &it : v) begin[it.rep + 1]++;
        for (int r = 0; r < nrep; ++r) begin[r + 1] += begin[r];
        list.assign(v.size(), 0);
        std::vector<int> fill(begin.begin(), begin.end() - 1);
        for (size_t k = 0; k < v.size(); ++k) list[fill[v[k].rep]++] = (int)k;
    };
    std::vector<int> begin_hs, list_hs, begin_ot, list_ot;
    rep_lists(items_hs, begin_hs, list_hs);
    rep_lists(items_ot, begin_ot, list_ot);
    /* the context carries the force field; its own box is the first replica's (never used) */
    mdrl_params pc = *p;
    for (int d = 0; d < 3; ++d) { pc.box[d] = reps[0].box[d]; pc.ncell[d] = 0; }
    mdrl_status s = mdrl_create(&pc, &bt->c);
    if (s != MDRL_OK) { delete bt; return s; }
    mdrl_ctx *c = bt->c;
    auto fail = [&](mdrl_status st) { mdrl_batch_destroy(bt); return st; };
    /* the context's cell buffers sized for the whole batch (ensure_capacity keeps them) */
    c->ncells = bt->ncells;
    if ((s = dalloc(&c->d_count, (size_t)bt->ncells)) != MDRL_OK) return fail(s);
    if ((s = dalloc(&c->d_start, (size_t)bt->ncells + 1)) != MDRL_OK) return fail(s);
    if ((s = dalloc(&c->d_unit, std::max((size_t)bt->nitems,
                                         (size_t)bt->n_ot + ((size_t)bt->n_cp + bt->n_hs) * kMaxItemGroups))) != MDRL_OK)
        return fail(s);
    if ((s = ensure_capacity(c, bt->ntot)) != MDRL_OK) return fail(s);
    std::vector<int> rep_of(bt->ntot);
    for (int r = 0; r < nrep; ++r)
        std::fill(rep_of.begin() + hrep[r].p_off, rep_of.begin() + hrep[r].p_off + hrep[r].n, r);
    if ((s = dalloc(&bt->d_reps, (size_t)nrep)) != MDRL_OK) return fail(s);
    if ((s = dalloc(&bt->d_items, (size_t)bt->nitems)) != MDRL_OK) return fail(s);
    if ((s = dalloc(&bt->d_rep_of, (size_t)bt->ntot)) != MDRL_OK) return fail(s);
    if ((s = dalloc(&bt->d_item_begin, (size_t)nrep + 1)) != MDRL_OK) return fail(s);
    if ((s = dalloc(&bt->d_rep_items, (size_t)bt->nitems)) != MDRL_OK) return fail(s);
    if ((s = dalloc(&bt->d_reptot, (size_t)nrep)) != MDRL_OK) return fail(s);
    if ((s = dalloc(&bt->d_items_hs, std::max<size_t>(1, items_hs.size()))) != MDRL_OK) return fail(s);
    if ((s = dalloc(&bt->d_items_ot, std::max<size_t>(1, items_ot.size()))) != MDRL_OK) return fail(s);
    if ((s = dalloc(&bt->d_begin_hs, (size_t)nrep + 1)) != MDRL_OK) return fail(s);
    if ((s = dalloc(&bt->d_begin_ot, (size_t)nrep + 1)) != MDRL_OK) return fail(s);
    if ((s = dalloc(&bt->d_list_hs, std::max<size_t>(1, list_hs.size()))) != MDRL_OK) return fail(s);
    if ((s = dalloc(&bt->d_list_ot, std::max<size_t>(1, list_ot.size()))) != MDRL_OK) return fail(s);
    cudaError_t e = cudaMemcpy(bt->d_reps, bt->reps.data(), sizeof(BatchRep) * nrep, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(bt->d_items, bt->items.data(), sizeof(BatchItem) * bt->nitems, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(bt->d_rep_of, rep_of.data(), sizeof(int) * bt->ntot, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(bt->d_item_begin, bt->item_begin.data(), sizeof(int) * (nrep + 1), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(bt->d_rep_items, bt->rep_items.data(), sizeof(int) * bt->nitems, cudaMemcpyHostToDevice);
    if (e == cudaSuccess && !items_hs.empty())
        e = cudaMemcpy(bt->d_items_hs, items_hs.data(), sizeof(BatchItem) * items_hs.size(), cudaMemcpyHostToDevice);
    if (e == cudaSuccess && bt->n_ot) e = cudaMemcpy(bt->d_items_ot, items_ot.data(), sizeof(BatchItem) * bt->n_ot, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(bt->d_begin_hs, begin_hs.data(), sizeof(int) * (nrep + 1), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(bt->d_begin_ot, begin_ot.data(), sizeof(int) * (nrep + 1), cudaMemcpyHostToDevice);
    if (e == cudaSuccess && !list_hs.empty())
        e = cudaMemcpy(bt->d_list_hs, list_hs.data(), sizeof(int) * list_hs.size(), cudaMemcpyHostToDevice);
    if (e == cudaSuccess && bt->n_ot) e = cudaMemcpy(bt->d_list_ot, list_ot.data(), sizeof(int) * bt->n_ot, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        set_error(std::string("mdrl_batch_create: ") + cudaGetErrorString(e));
        return fail(MDRL_ERR_CUDA);
    }
    *out = bt;
    return MDRL_OK;
}

/* Result slots of a batch force launch (one per CTA). */
static int batch_slots(const mdrl_batch *b) {
    return b->c->tile.warps_per_cta == 1 ? b->n_ot + (b->n_cp + b->n_hs) * b->c->tile.steps_per_piece : b->nitems;
}

static mdrl_status batch_launch_force(mdrl_batch *b, const float4 *pos, const int *type, bool extra,
                                      unsigned long long *F64) {
    mdrl_ctx *c = b->c;
    if (c->tile.warps_per_cta == 1) {
        /* the replicas with an edge of at most 2 rc in the CTA kernel (every periodic image,
         * default tile), then one warp per (item, i-tile group): the explicit cell pairs of the
         * other small replicas (per-pair wrap), then the half-shell units */
        const bool sep = c->p.arith == MDRL_ARITH_SEPARATE;
        force_fn fo = pick_force_batch(eff_order(c), sep, extra, false);
        warp_fn fp = pick_force_warp_batch(eff_order(c), sep, extra, true);
        warp_fn fw = pick_force_warp_batch(eff_order(c), sep, extra, false);
        MDRL_TRY(prepare_force_kernel(fo, c->p.device));
        MDRL_TRY(prepare_force_kernel((force_fn)fp, c->p.device));
        MDRL_TRY(prepare_force_kernel((force_fn)fw, c->p.device));
        const int G = c->tile.steps_per_piece;
        const size_t wsm = force_warp_smem_bytes(c->p.ntypes, extra);
        MDRL_CUDA(cudaEventRecord(c->evf0, c->stream));
        if (b->n_ot)
            fo<<<b->n_ot, kBatchFT, force_smem_bytes(c->p.ntypes, extra, kBatchFT / 32), c->stream>>>(
                pos, type, c->d_start, c->g, table_dev(c), c->d_pcoef, c->p.ntypes, c->ke, b->ntot, F64, nullptr,
                c->d_cnt, c->d_unit, b->d_items_ot, b->d_reps, tile_word(kStepsPerPiece, 0), c->d_err, 0);
        if (b->n_cp)
            fp<<<b->n_cp * G, 32, wsm, c->stream>>>(
                pos, type, c->d_start, c->g, table_dev(c), c->d_pcoef, c->p.ntypes, c->ke, b->ntot, F64, nullptr,
                c->d_cnt, c->d_unit + b->n_ot, b->d_items_hs, b->d_reps, G, c->d_err, 0, nullptr, 0);
        if (b->n_hs)
            fw<<<b->n_hs * G, 32, wsm, c->stream>>>(
                pos, type, c->d_start, c->g, table_dev(c), c->d_pcoef, c->p.ntypes, c->ke, b->ntot, F64, nullptr,
                c->d_cnt, c->d_unit + b->n_ot + (size_t)b->n_cp * G, b->d_items_hs + b->n_cp, b->d_reps, G, c->d_err, 0,
                nullptr, 0);
        MDRL_CUDA(cudaGetLastError());
        MDRL_CUDA(cudaEventRecord(c->evf1, c->stream));
        return MDRL_OK;
    }
    force_fn fn = pick_force_batch(eff_order(c), c->p.arith == MDRL_ARITH_SEPARATE, extra, c->tile.prune_steps != 0);
    MDRL_TRY(prepare_force_kernel(fn, c->p.device));
    const size_t smem = force_smem_bytes(c->p.ntypes, extra, kBatchFT / 32);
    MDRL_CUDA(cudaEventRecord(c->evf0, c->stream));
    fn<<<b->nitems, kBatchFT, smem, c->stream>>>(pos, type, c->d_start, c->g, table_dev(c), c->d_pcoef,
                                                  c->p.ntypes, c->ke, b->ntot, F64, nullptr, c->d_cnt, c->d_unit,
                                                  b->d_items, b->d_reps, tile_word(c->tile.steps_per_piece, c->tile.prune_steps), c->d_err, 0);
    MDRL_CUDA(cudaGetLastError());
    MDRL_CUDA(cudaEventRecord(c->evf1, c->stream));
    return MDRL_OK;
}

/* Bin the user-order arrays already on the device into slot `buf` and clear the accumulators. */
static mdrl_status batch_bin_user(mdrl_batch *b, const float *q, const int *type, int buf) {
    mdrl_ctx *c = b->c;
    const int n = b->ntot;
    MDRL_CUDA(cudaMemsetAsync(c->d_count, 0, sizeof(int) * (size_t)b->ncells, c->stream));
    MDRL_CUDA(cudaMemsetAsync(c->d_err, 0, sizeof(unsigned), c->stream));
    k_bbin_user<<<nblk(n, 256), 256, 0, c->stream>>>(n, c->d_ux, c->d_uy, c->d_uz, b->d_rep_of, b->d_reps,
                                                     c->d_cell_of, c->d_slot, c->d_count, c->d_err, c->d_key);
    k_scan<<<1, 1024, 0, c->stream>>>(b->ncells, c->d_count, c->d_start, c->d_tot);
    k_scatter<<<nblk(n, 256), 256, 0, c->stream>>>(n, c->d_cell_of, c->d_slot, c->d_start, c->d_tmp);
    k_cell_sort<<<b->ncells, 128, 0, c->stream>>>(c->d_start, c->d_tmp, c->d_sorted, c->d_key, c->d_sortkey,
                                                   c->d_err);
    k_gather_user<<<nblk(n, 256), 256, 0, c->stream>>>(n, c->d_sorted, c->d_ux, c->d_uy, c->d_uz, q, type,
                                                       c->d_pos[buf], c->d_type[buf], c->d_id[buf], c->d_F64,
                                                       nullptr, c->d_cnt, c->p.ntypes, c->d_err);
    MDRL_CUDA(cudaGetLastError());
    return MDRL_OK;
}

static mdrl_status upload_user(mdrl_batch *b, const float *x, const float *y, const float *z,
                               const float *q, const int *type) {
    mdrl_ctx *c = b->c;
    const size_t fb = sizeof(float) * (size_t)b->ntot;
    MDRL_CUDA(cudaMemcpyAsync(c->d_ux, x, fb, cudaMemcpyHostToDevice, c->stream));
    MDRL_CUDA(cudaMemcpyAsync(c->d_uy, y, fb, cudaMemcpyHostToDevice, c->stream));
    MDRL_CUDA(cudaMemcpyAsync(c->d_uz, z, fb, cudaMemcpyHostToDevice, c->stream));
    if (q) MDRL_CUDA(cudaMemcpyAsync(c->d_uq, q, fb, cudaMemcpyHostToDevice, c->stream));
    if (type) MDRL_CUDA(cudaMemcpyAsync(c->d_ut, type, sizeof(int) * (size_t)b->ntot, cudaMemcpyHostToDevice, c->stream));
    return MDRL_OK;
}

static mdrl_status batch_read_totals(mdrl_batch *b, mdrl_stats *st, float ms) {
    if (!st) return MDRL_OK;
    mdrl_ctx *c = b->c;
    DevTotals t;
    MDRL_CUDA(cudaMemcpy(&t, c->d_tot, sizeof(t), cudaMemcpyDeviceToHost));
    memset(st, 0, sizeof(*st));
    st->pairs = (int64_t)t.pairs;
    st->candidates = -1;
    st->below_table = (int64_t)t.below;
    st->max_cell_occupancy = t.max_occ;
    st->ncells = b->ncells;
    st->e_lj = t.e_lj;
    st->e_coul = t.e_coul;
    st->virial = t.virial;
    st->kinetic = t.kinetic;
    st->device_ms = ms;
    st->pairs_total = (int64_t)t.pairs_total;
    float fms = 0.0f;
    if (cudaEventElapsedTime(&fms, c->evf0, c->evf1) == cudaSuccess) st->force_ms = fms;
    else cudaGetLastError();
    return MDRL_OK;
}

extern "C" mdrl_status mdrl_batch_force_eval(mdrl_batch *b, const float *x, const float *y, const float *z,
                                             const float *q, const int *type, float *fx, float *fy,
                                             float *fz, int *counts, mdrl_stats *st) {
    if (!b || !x || !y || !z || !fx || !fy || !fz) {
        set_error("mdrl_batch_force_eval: null argument");
        return MDRL_ERR_INVALID_ARG;
    }
    mdrl_ctx *c = b->c;
    MDRL_CUDA(cudaSetDevice(c->p.device));
    const int n = b->ntot;
    const bool extra = counts != nullptr || (c->p.flags & MDRL_FLAG_ENERGY);
    MDRL_TRY(upload_user(b, x, y, z, q, type));
    MDRL_CUDA(cudaMemsetAsync(c->d_tot, 0, sizeof(DevTotals), c->stream));
    MDRL_CUDA(cudaEventRecord(c->ev0, c->stream));
    MDRL_TRY(batch_bin_user(b, q ? c->d_uq : nullptr, type ? c->d_ut : nullptr, 0));
    MDRL_TRY(batch_launch_force(b, c->d_pos[0], c->d_type[0], extra, c->d_F64));
    k_totals<<<1, 1024, 0, c->stream>>>(batch_slots(b), c->d_unit, 0, c->d_kepart, c->d_tot, extra ? 1 : 0);
    k_unsort<<<nblk(n, 256), 256, 0, c->stream>>>(n, c->d_id[0], c->d_F64, nullptr, c->d_cnt, c->d_ox, c->d_oy,
                                                  c->d_oz, counts ? c->d_ocnt : nullptr);
    MDRL_CUDA(cudaGetLastError());
    MDRL_CUDA(cudaEventRecord(c->ev1, c->stream));
    const size_t fb = sizeof(float) * (size_t)n;
    MDRL_CUDA(cudaMemcpyAsync(fx, c->d_ox, fb, cudaMemcpyDeviceToHost, c->stream));
    MDRL_CUDA(cudaMemcpyAsync(fy, c->d_oy, fb, cudaMemcpyDeviceToHost, c->stream));
    MDRL_CUDA(cudaMemcpyAsync(fz, c->d_oz, fb, cudaMemcpyDeviceToHost, c->stream));
    if (counts) MDRL_CUDA(cudaMemcpyAsync(counts, c->d_ocnt, sizeof(int) * (size_t)n, cudaMemcpyDeviceToHost, c->stream));
    MDRL_CUDA(cudaStreamSynchronize(c->stream));
    float ms = 0.0f;
    MDRL_CUDA(cudaEventElapsedTime(&ms, c->ev0, c->ev1));
    MDRL_TRY(check_device_errors(c));
    c->have_state = false;
    b->have_eval = true;
    return batch_read_totals(b, st, ms);
}

extern "C" mdrl_status mdrl_batch_set_state(mdrl_batch *b, const float *x, const float *y, const float *z,
                                            const float *vx, const float *vy, const float *vz,
                                            const float *q, const int *type) {
    if (!b || !x || !y || !z || ((vx || vy || vz) && !(vx && vy && vz))) {
        set_error("mdrl_batch_set_state: null or invalid argument");
        return MDRL_ERR_INVALID_ARG;
    }
    mdrl_ctx *c = b->c;
    MDRL_CUDA(cudaSetDevice(c->p.device));
    const int n = b->ntot;
    const size_t fb = sizeof(float) * (size_t)n;
    MDRL_TRY(upload_user(b, x, y, z, q, type));
    if (vx) {
        MDRL_CUDA(cudaMemcpyAsync(c->d_ovx, vx, fb, cudaMemcpyHostToDevice, c->stream));
        MDRL_CUDA(cudaMemcpyAsync(c->d_ovy, vy, fb, cudaMemcpyHostToDevice, c->stream));
        MDRL_CUDA(cudaMemcpyAsync(c->d_ovz, vz, fb, cudaMemcpyHostToDevice, c->stream));
    }
    MDRL_CUDA(cudaMemsetAsync(c->d_tot, 0, sizeof(DevTotals), c->stream));
    c->cur = 0;
    MDRL_TRY(batch_bin_user(b, q ? c->d_uq : nullptr, type ? c->d_ut : nullptr, 0));
    k_gather_vel<<<nblk(n, 256), 256, 0, c->stream>>>(n, c->d_id[0], vx ? c->d_ovx : nullptr, c->d_ovy, c->d_ovz,
                                                      c->d_vel[0]);
    const bool extra = (c->p.flags & MDRL_FLAG_ENERGY) != 0;
    MDRL_TRY(batch_launch_force(b, c->d_pos[0], c->d_type[0], extra, c->d_F64));
    k_kick<<<nblk(n, 256), 256, 0, c->stream>>>(n, c->d_vel[0], c->d_type[0], c->d_F64, nullptr, c->d_mt, 0,
                                                c->d_kepart);
    k_totals<<<1, 1024, 0, c->stream>>>(batch_slots(b), c->d_unit, nblk(n, 256), c->d_kepart, c->d_tot, extra ? 1 : 0);
    MDRL_CUDA(cudaGetLastError());
    MDRL_CUDA(cudaStreamSynchronize(c->stream));
    MDRL_TRY(check_device_errors(c));
    c->n = n;
    c->have_state = true;
    b->have_eval = true;
    return MDRL_OK;
}

static mdrl_status batch_enqueue_step(mdrl_batch *b, bool extra) {
    mdrl_ctx *c = b->c;
    const int n = b->ntot;
    const int a = c->cur, d = 1 - c->cur;
    const bool vv = c->p.integrator == MDRL_INT_VELOCITY_VERLET;
    const MassTab *mt = vv ? c->d_mt : c->d_mt + 1;
    const float dt = (float)c->p.dt_fs;
    MDRL_CUDA(cudaMemsetAsync(c->d_count, 0, sizeof(int) * (size_t)b->ncells, c->stream));
    k_bkick_drift_bin<<<nblk(n, 256), 256, 0, c->stream>>>(n, c->d_pos[a], c->d_vel[a], c->d_type[a], c->d_F64, mt,
                                                           dt, b->d_rep_of, b->d_reps, c->d_cell_of, c->d_slot,
                                                           c->d_count, c->d_key);
    k_scan<<<1, 1024, 0, c->stream>>>(b->ncells, c->d_count, c->d_start, c->d_tot);
    k_scatter<<<nblk(n, 256), 256, 0, c->stream>>>(n, c->d_cell_of, c->d_slot, c->d_start, c->d_tmp);
    k_cell_sort<<<b->ncells, 128, 0, c->stream>>>(c->d_start, c->d_tmp, c->d_sorted, c->d_key, c->d_sortkey,
                                                   c->d_err);
    k_gather_state<<<nblk(n, 256), 256, 0, c->stream>>>(n, c->d_sorted, c->d_pos[a], c->d_vel[a], c->d_type[a],
                                                        c->d_id[a], c->d_pos[d], c->d_vel[d], c->d_type[d],
                                                        c->d_id[d], c->d_F64, nullptr);
    if (extra) MDRL_CUDA(cudaMemsetAsync(c->d_cnt, 0, sizeof(int) * (size_t)n, c->stream));
    MDRL_TRY(batch_launch_force(b, c->d_pos[d], c->d_type[d], extra, c->d_F64));
    if (vv || extra)
        k_kick<<<nblk(n, 256), 256, 0, c->stream>>>(n, c->d_vel[d], c->d_type[d], c->d_F64, nullptr, c->d_mt,
                                                    vv ? 1 : 0, extra ? c->d_kepart : nullptr);
    k_totals<<<1, 1024, 0, c->stream>>>(batch_slots(b), c->d_unit, extra ? nblk(n, 256) : 0, c->d_kepart, c->d_tot,
                                       extra ? 1 : 0);
    MDRL_CUDA(cudaGetLastError());
    return MDRL_OK;
}

extern "C" mdrl_status mdrl_batch_step(mdrl_batch *b, int nsteps, mdrl_stats *st) {
    if (!b || nsteps < 0) { set_error("mdrl_batch_step: invalid argument"); return MDRL_ERR_INVALID_ARG; }
    mdrl_ctx *c = b->c;
    if (!c->have_state) { set_error("mdrl_batch_step: call mdrl_batch_set_state first"); return MDRL_ERR_STATE; }
    MDRL_CUDA(cudaSetDevice(c->p.device));
    const bool extra = (c->p.flags & MDRL_FLAG_ENERGY) != 0;
    MDRL_CUDA(cudaMemsetAsync(c->d_tot, 0, offsetof(DevTotals, pairs_total), c->stream));
    MDRL_CUDA(cudaMemsetAsync(&c->d_tot->pairs_total, 0, sizeof(unsigned long long), c->stream));
    MDRL_CUDA(cudaMemsetAsync(c->d_err, 0, sizeof(unsigned), c->stream));
    if (c->graph_n != b->ntot || c->graph_extra != extra) {
        const int saved = c->cur;
        for (int k = 0; k < 2; ++k) {
            if (c->graph_exec[k]) { cudaGraphExecDestroy(c->graph_exec[k]); c->graph_exec[k] = nullptr; }
            if (c->graph[k]) { cudaGraphDestroy(c->graph[k]); c->graph[k] = nullptr; }
            c->cur = k;
            MDRL_CUDA(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
            const mdrl_status s = batch_enqueue_step(b, extra);
            cudaGraph_t g = nullptr;
            const cudaError_t e = cudaStreamEndCapture(c->stream, &g);
            c->cur = saved;
            if (s != MDRL_OK) { if (g) cudaGraphDestroy(g); return s; }
            if (e != cudaSuccess) { set_error(std::string("graph capture: ") + cudaGetErrorString(e)); return MDRL_ERR_CUDA; }
            c->graph[k] = g;
            MDRL_CUDA(cudaGraphInstantiate(&c->graph_exec[k], g, 0));
        }
        c->graph_n = b->ntot;
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
    MDRL_TRY(batch_read_totals(b, st, ms));
    return check_device_errors(c);
}

extern "C" mdrl_status mdrl_batch_get_state(mdrl_batch *b, float *x, float *y, float *z, float *vx, float *vy,
                                            float *vz, float *fx, float *fy, float *fz) {
    if (!b) { set_error("null batch"); return MDRL_ERR_INVALID_ARG; }
    mdrl_ctx *c = b->c;
    if (!c->have_state) { set_error("mdrl_batch_get_state: no state"); return MDRL_ERR_STATE; }
    MDRL_CUDA(cudaSetDevice(c->p.device));
    const int n = b->ntot, a = c->cur;
    k_unsort_state<<<nblk(n, 256), 256, 0, c->stream>>>(n, c->d_id[a], c->d_pos[a], c->d_vel[a], c->d_ux, c->d_uy,
                                                        c->d_uz, c->d_ovx, c->d_ovy, c->d_ovz);
    k_unsort<<<nblk(n, 256), 256, 0, c->stream>>>(n, c->d_id[a], c->d_F64, nullptr, c->d_cnt, c->d_ox, c->d_oy,
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

extern "C" mdrl_status mdrl_batch_replica_stats(mdrl_batch *b, mdrl_stats *out) {
    if (!b || !out) { set_error("mdrl_batch_replica_stats: null argument"); return MDRL_ERR_INVALID_ARG; }
    if (!b->have_eval) { set_error("mdrl_batch_replica_stats: no force evaluation yet"); return MDRL_ERR_STATE; }
    mdrl_ctx *c = b->c;
    MDRL_CUDA(cudaSetDevice(c->p.device));
    const int a = c->cur;
    const bool kin = c->have_state;
    const bool warp = c->tile.warps_per_cta == 1;
    k_rep_totals<<<b->nrep, 128, 0, c->stream>>>(warp ? b->d_begin_ot : b->d_item_begin, warp ? b->d_list_ot : b->d_rep_items,
                                                 warp ? b->d_begin_hs : nullptr, warp ? b->d_list_hs : nullptr, b->n_ot,
                                                 warp ? c->tile.steps_per_piece : 1, c->d_unit, b->d_reps,
                                                 kin ? c->d_vel[a] : nullptr, c->d_type[a], c->d_mt,
                                                 b->d_reptot);
    MDRL_CUDA(cudaGetLastError());
    std::vector<RepTotals> h(b->nrep);
    MDRL_CUDA(cudaMemcpyAsync(h.data(), b->d_reptot, sizeof(RepTotals) * b->nrep, cudaMemcpyDeviceToHost, c->stream));
    MDRL_CUDA(cudaStreamSynchronize(c->stream));
    for (int r = 0; r < b->nrep; ++r) {
        mdrl_stats &s = out[r];
        memset(&s, 0, sizeof(s));
        s.pairs = (int64_t)h[r].pairs;
        s.candidates = -1;
        s.below_table = (int64_t)h[r].below;
        s.ncells = b->reps[r].g.nc[0] * b->reps[r].g.nc[1] * b->reps[r].g.nc[2];
        s.e_lj = h[r].e_lj;
        s.e_coul = h[r].e_coul;
        s.virial = h[r].virial;
        s.kinetic = h[r].kinetic;
    }
    return MDRL_OK;
}

extern "C" mdrl_status mdrl_batch_layout(mdrl_batch *b, int *path, int *ncell, int *items, int *total_items) {
    if (!b) { set_error("null batch"); return MDRL_ERR_INVALID_ARG; }
    for (int r = 0; r < b->nrep; ++r) {
        if (path) path[r] = b->reps[r].path;
        if (ncell) for (int d = 0; d < 3; ++d) ncell[3 * r + d] = b->reps[r].g.nc[d];
        if (items) items[r] = b->item_begin[r + 1] - b->item_begin[r];
    }
    if (total_items) *total_items = b->nitems;
    return MDRL_OK;
}

extern "C" mdrl_status mdrl_batch_time_force(mdrl_batch *b, float *ms) {
    if (!b || !ms) { set_error("mdrl_batch_time_force: null argument"); return MDRL_ERR_INVALID_ARG; }
    mdrl_ctx *c = b->c;
    if (!c->have_state) { set_error("mdrl_batch_time_force: call mdrl_batch_set_state first"); return MDRL_ERR_STATE; }
    MDRL_CUDA(cudaSetDevice(c->p.device));
    const int a = c->cur;
    if (!c->d_Fscr64) MDRL_TRY(dalloc(&c->d_Fscr64, 3 * (size_t)c->cap));
    MDRL_CUDA(cudaMemsetAsync(c->d_Fscr64, 0, sizeof(unsigned long long) * 3 * (size_t)b->ntot, c->stream));
    MDRL_TRY(batch_launch_force(b, c->d_pos[a], c->d_type[a], false, c->d_Fscr64));
    MDRL_CUDA(cudaStreamSynchronize(c->stream));
    MDRL_CUDA(cudaEventElapsedTime(ms, c->evf0, c->evf1));
    return MDRL_OK;
}

extern "C" mdrl_status mdrl_batch_set_tile(mdrl_batch *b, const mdrl_tile *t) {
    if (!b || !t) { set_error("mdrl_batch_set_tile: null argument"); return MDRL_ERR_INVALID_ARG; }
    const mdrl_tile before = b->c->tile;
    MDRL_TRY(set_tile(b->c, t, false, true));
    /* another tile lays the result slots out differently: the last evaluation's no longer apply */
    if (before.warps_per_cta != t->warps_per_cta || before.steps_per_piece != t->steps_per_piece ||
        before.prune_steps != t->prune_steps)
        b->have_eval = false;
    return MDRL_OK;
}

extern "C" mdrl_status mdrl_batch_autotune(mdrl_batch *b, int flags, mdrl_tile *best, float *best_ms,
                                           float *default_ms) {
    if (!b) { set_error("mdrl_batch_autotune: null batch"); return MDRL_ERR_INVALID_ARG; }
    mdrl_ctx *c = b->c;
    if (!c->have_state) { set_error("mdrl_batch_autotune: call mdrl_batch_set_state first"); return MDRL_ERR_STATE; }
    MDRL_CUDA(cudaSetDevice(c->p.device));
    char buf[96];
    snprintf(buf, sizeof buf, "batch-r%d-n%d-c%d-i%d-", b->nrep, b->ntot, b->ncells, b->nitems);
    const std::string key = std::string(buf) + tune_key_common(c);
    auto time_tile = [&](const mdrl_tile &t, float *ms) -> mdrl_status {
        MDRL_TRY(set_tile(c, &t, false, true));
        float v[5];
        for (int r = 0; r < 5; ++r) MDRL_TRY(mdrl_batch_time_force(b, &v[r]));
        std::sort(v, v + 5);
        *ms = v[2];
        return MDRL_OK;
    };
    const mdrl_tile def = {kBatchFT / 32, kStepsPerPiece, 0};
    mdrl_tile pick = def;
    float pick_ms = 0.0f, def_ms = 0.0f;
    const bool cached = !(flags & MDRL_TUNE_RETIME) && tune_lookup(key, &pick) &&
                        (pick.warps_per_cta == 4 || pick.warps_per_cta == 1);
    if (cached) {
        MDRL_TRY(time_tile(pick, &pick_ms));
        if (default_ms) MDRL_TRY(time_tile(def, &def_ms));
    } else {
        pick_ms = 3.0e38f;
        for (int spp : {3, 4, 6, 8, 12})
            for (int pr = 0; pr < 2; ++pr) {
                const mdrl_tile t = {kBatchFT / 32, spp, pr};
                float ms;
                MDRL_TRY(time_tile(t, &ms));
                if (spp == def.steps_per_piece && pr == def.prune_steps) def_ms = ms;
                if (ms < pick_ms) { pick_ms = ms; pick = t; }
            }
        for (int grp = 1; grp <= 3; ++grp) {     /* one warp per (half-shell unit, i-tile group) */
            const mdrl_tile t = {1, grp, 1};
            float ms;
            MDRL_TRY(time_tile(t, &ms));
            if (ms < pick_ms) { pick_ms = ms; pick = t; }
        }
        tune_store(key, pick, pick_ms);
    }
    MDRL_TRY(set_tile(c, &pick, false, true));
    b->have_eval = false;   /* the timings overwrote the result slots */
    if (best) *best = pick;
    if (best_ms) *best_ms = pick_ms;
    if (default_ms) *default_ms = def_ms;
    return MDRL_OK;
}

extern "C" mdrl_status mdrl_batch_set_pair_coefficients(mdrl_batch *b, const double *coef) {
    if (!b) { set_error("mdrl_batch_set_pair_coefficients: null batch"); return MDRL_ERR_INVALID_ARG; }
    return mdrl_set_pair_coefficients(b->c, coef);
}
