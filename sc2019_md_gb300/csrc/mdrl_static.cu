/*
 * mdrl_static.cu — mdrl_force_eval_static: one force evaluation that allocates no memory.
 *
 * Who needs it: code that must not call cudaMalloc — a caller that runs under a memory pool or
 * allocator it does not own (a framework whose caching allocator has reserved the device, a
 * plugin host that forbids device allocations), a caller inside a latency-critical loop that
 * cannot afford an allocation on first use, or a tool that must leave the device's allocation
 * state exactly as it found it.  mdrl_force_eval needs a context (mdrl_create), and a context
 * allocates its buffers; this entry point needs none.
 *
 * How: all scratch of the path — cell counts and starts, the in-cell order and its keys, the
 * cell-sorted copy of the particles, the int64 force accumulators, the per-unit reduction slots
 * and the tables — lives in one file-scope static __device__ array of kStaticBytes (16 MiB),
 * which every GPU that loads the library holds until the process exits.  The caller passes
 * device pointers to its inputs and outputs and a stream.
 *
 * Limits: n <= 131,072 particles, <= 4,096 cells, nseg * bins <= 16,384 table entries, int64
 * fixed-point accumulation only; larger requests are rejected with MDRL_ERR_RANGE and a message.
 *
 * Set-up: every call looks up the device address of the array in the current CUDA context with
 * cudaGetSymbolAddress (a __device__ array has one copy per context, so an address cached from
 * another context, or from before a cudaDeviceReset, would be stale).  Tables are fitted on the
 * host and copied into the array when the table parameters change or the array belongs to a
 * context (unique context ID) or address other than the one the copy went to; the first call in
 * a context therefore copies tables, so make it before any stream capture.  The call runs on the
 * current device, which must be p->device.
 *
 * Sharing: every call uses the same array, which keeps the previous call's contents; the call
 * clears what must start at zero.  Two calls whose work overlaps on the GPU (different streams,
 * or threads without ordering) race on the array: serialise them.
 */
#include <cuda.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "mdrl_force.cuh"

namespace mdrl {

constexpr int kStaticMaxN = 131072;
constexpr int kStaticMaxCells = 4096;
constexpr int kStaticMaxTable = 16384;
constexpr size_t kStaticBytes = size_t(16) << 20;
constexpr int kStaticMaxDevices = 64;

static __device__ __align__(256) unsigned char g_static_scratch[kStaticBytes];

namespace {

constexpr size_t align256(size_t v) { return (v + 255) & ~size_t(255); }

/* Byte offsets of the sub-buffers inside the array. */
struct Layout {
    size_t err, tot, count, start, unit, cell_of, slot, tmp, sorted, key, sortkey, pos, type, id, F64, tabf,
        tabe, tabr, pcoef, end;
};

constexpr Layout make_layout() {
    Layout l{};
    size_t o = 0;
    l.err = o;     o = align256(o + sizeof(unsigned));
    l.tot = o;     o = align256(o + sizeof(DevTotals));
    l.count = o;   o = align256(o + sizeof(int) * kStaticMaxCells);
    l.start = o;   o = align256(o + sizeof(int) * (kStaticMaxCells + 1));
    l.unit = o;    o = align256(o + sizeof(UnitOut) * kHalfShellCells * kStaticMaxCells);
    l.cell_of = o; o = align256(o + sizeof(int) * kStaticMaxN);
    l.slot = o;    o = align256(o + sizeof(int) * kStaticMaxN);
    l.tmp = o;     o = align256(o + sizeof(int) * kStaticMaxN);
    l.sorted = o;  o = align256(o + sizeof(int) * kStaticMaxN);
    l.key = o;     o = align256(o + sizeof(unsigned) * kStaticMaxN);
    l.sortkey = o; o = align256(o + sizeof(unsigned long long) * kStaticMaxN);
    l.pos = o;     o = align256(o + sizeof(float4) * kStaticMaxN);
    l.type = o;    o = align256(o + sizeof(int) * kStaticMaxN);
    l.id = o;      o = align256(o + sizeof(int) * kStaticMaxN);
    l.F64 = o;     o = align256(o + sizeof(unsigned long long) * 3 * kStaticMaxN);
    l.tabf = o;    o = align256(o + sizeof(float4) * 3 * kStaticMaxTable);
    l.tabe = o;    o = align256(o + sizeof(float4) * 3 * kStaticMaxTable);
    l.tabr = o;    o = align256(o + sizeof(float4) * 2 * kStaticMaxTable);
    l.pcoef = o;   o = align256(o + sizeof(float4) * MDRL_MAX_TYPES * MDRL_MAX_TYPES);
    l.end = o;
    return l;
}

constexpr Layout kLayout = make_layout();
static_assert(kLayout.end <= kStaticBytes, "static scratch layout exceeds the array");

/* Which tables the array holds on one device: valid only for the context (unique ID) and
 * array address they were copied to. */
struct DeviceSlot {
    unsigned long long ctx_id = 0;   /* 0: unknown context, never matches */
    unsigned char *base = nullptr;   /* device address of g_static_scratch the tables went to */
    bool have_tables = false;
    int order = 0, nseg = 0, bins = 0, min_log2 = 0, ntypes = 0;
    double sigma[MDRL_MAX_TYPES] = {}, epsilon[MDRL_MAX_TYPES] = {};
};

std::mutex g_mu;
DeviceSlot g_slots[kStaticMaxDevices];

/* The unique ID of the current CUDA context (cuCtxGetCurrent + cuCtxGetId through the runtime's
 * driver entry points, so the library needs no link-time dependency on the driver library), or
 * 0 when it cannot be obtained, in which case the tables are copied on every call. */
typedef CUresult (*ctx_get_current_fn)(CUcontext *);
typedef CUresult (*ctx_get_id_fn)(CUcontext, unsigned long long *);

unsigned long long current_context_id() {
    static ctx_get_current_fn get_current = nullptr;
    static ctx_get_id_fn get_id = nullptr;
    static bool looked_up = false;
    if (!looked_up) {
        looked_up = true;
        cudaDriverEntryPointQueryResult q1, q2;
        void *f1 = nullptr, *f2 = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 12000, cudaEnableDefault, &q1) == cudaSuccess &&
            q1 == cudaDriverEntryPointSuccess &&
            cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000, cudaEnableDefault, &q2) == cudaSuccess &&
            q2 == cudaDriverEntryPointSuccess) {
            get_current = (ctx_get_current_fn)f1;
            get_id = (ctx_get_id_fn)f2;
        } else {
            cudaGetLastError();
        }
    }
    if (!get_current || !get_id) return 0;
    CUcontext ctx = nullptr;
    unsigned long long id = 0;
    if (get_current(&ctx) != CUDA_SUCCESS || !ctx || get_id(ctx, &id) != CUDA_SUCCESS) return 0;
    return id;
}

mdrl_status fail(mdrl_status s, const std::string &msg) {
    set_error("mdrl_force_eval_static: " + msg);
    return s;
}

#define ST_CUDA(call)                                                                             \
    do {                                                                                          \
        if (fault_hit(#call)) return fail(MDRL_ERR_CUDA, std::string(#call) + ": injected failure (MDRL_FAULT)"); \
        cudaError_t e_ = (call);                                                                  \
        if (e_ != cudaSuccess) return fail(MDRL_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

int seg_count(float rc2, int min_log2) {
    int e;
    std::frexp(rc2, &e);
    return (e - 1) - min_log2 + 1;
}

}  // namespace
}  // namespace mdrl

using namespace mdrl;

extern "C" mdrl_status mdrl_force_eval_static(const mdrl_params *p, int n, const float *x, const float *y,
                                              const float *z, const float *q, const int *type, float *fx,
                                              float *fy, float *fz, int64_t *pairs_out, void *stream_ptr) {
    if (!p || n < 0 || (n > 0 && (!x || !y || !z || !fx || !fy || !fz)))
        return fail(MDRL_ERR_INVALID_ARG, "null or invalid argument");
    fault_arm_from_env(false);
    if (n > kStaticMaxN)
        return fail(MDRL_ERR_RANGE, "n = " + std::to_string(n) + " exceeds the static scratch limit of " +
                                        std::to_string(kStaticMaxN) + " particles");
    if (p->accum != MDRL_ACC_FIXED64)
        return fail(MDRL_ERR_INVALID_ARG, "only int64 fixed-point accumulation (MDRL_ACC_FIXED64) is supported");
    /* the checks mdrl_create makes (box, cutoff, types, table parameters incl. the first segment's
     * exponent, modes, coulomb_k) */
    if (validate_params(p) != MDRL_OK) return fail(MDRL_ERR_INVALID_ARG, mdrl_last_error());

    /* geometry, as mdrl_create sets it up */
    Geom g;
    const float rcf = (float)p->cutoff;
    g.rc2 = rcf * rcf;
    long long ncells = 1;
    for (int d = 0; d < 3; ++d) {
        if (!(p->box[d] > 0.0)) return fail(MDRL_ERR_INVALID_ARG, "box edges must be positive");
        const float L = (float)p->box[d];
        const double ncd = p->ncell[d] > 0 ? (double)p->ncell[d] : std::floor((double)L / (double)rcf);
        if (ncd > (double)kStaticMaxCells)
            return fail(MDRL_ERR_RANGE, "axis " + std::to_string(d) + ": more cells than the static scratch holds");
        const int nc = (int)ncd;
        g.L[d] = L;
        g.h[d] = 0.5f * L;
        g.nc[d] = nc;
        g.edge[d] = nc > 0 ? (float)((double)L / (double)nc) : 0.0f;
        if (nc < 3 || (double)g.edge[d] < (double)rcf)
            return fail(MDRL_ERR_RANGE, "each axis needs at least 3 cells of edge >= rc");
        ncells *= nc;
    }
    if (ncells > kStaticMaxCells)
        return fail(MDRL_ERR_RANGE, std::to_string(ncells) + " cells exceed the static scratch limit of " +
                                        std::to_string(kStaticMaxCells));
    const int order = p->table_order, bins = p->table_bins, m0 = p->table_min_log2;
    const int nseg = seg_count(g.rc2, m0);
    if (nseg < 1) return fail(MDRL_ERR_RANGE, "cutoff lies below the first table segment");
    const long long nidx64 = (long long)nseg * bins;   /* 64-bit: no overflow before the check */
    if (nidx64 > kStaticMaxTable)
        return fail(MDRL_ERR_RANGE, std::to_string(nidx64) + " table entries exceed the static scratch limit of " +
                                        std::to_string(kStaticMaxTable));
    const int nidx = (int)nidx64;

    int dev = 0;
    ST_CUDA(cudaGetDevice(&dev));
    if (dev != p->device)
        return fail(MDRL_ERR_INVALID_ARG, "p->device (" + std::to_string(p->device) +
                                              ") is not the current device (" + std::to_string(dev) + ")");
    if (dev < 0 || dev >= kStaticMaxDevices) return fail(MDRL_ERR_RANGE, "device ordinal too large");
    cudaStream_t st = (cudaStream_t)stream_ptr;

    std::lock_guard<std::mutex> lock(g_mu);
    DeviceSlot &slot = g_slots[dev];
    /* the array's address in the current context, looked up on every call */
    void *ptr = nullptr;
    ST_CUDA(cudaGetSymbolAddress(&ptr, g_static_scratch));
    unsigned char *b = (unsigned char *)ptr;
    const unsigned long long ctx_id = current_context_id();
    unsigned *d_err = (unsigned *)(b + kLayout.err);
    DevTotals *d_tot = (DevTotals *)(b + kLayout.tot);
    int *d_count = (int *)(b + kLayout.count);
    int *d_start = (int *)(b + kLayout.start);
    UnitOut *d_unit = (UnitOut *)(b + kLayout.unit);
    int *d_cell_of = (int *)(b + kLayout.cell_of);
    int *d_slot = (int *)(b + kLayout.slot);
    int *d_tmp = (int *)(b + kLayout.tmp);
    int *d_sorted = (int *)(b + kLayout.sorted);
    unsigned *d_key = (unsigned *)(b + kLayout.key);
    unsigned long long *d_sortkey = (unsigned long long *)(b + kLayout.sortkey);
    float4 *d_pos = (float4 *)(b + kLayout.pos);
    int *d_type = (int *)(b + kLayout.type);
    int *d_id = (int *)(b + kLayout.id);
    unsigned long long *d_F64 = (unsigned long long *)(b + kLayout.F64);
    float4 *d_pcoef = (float4 *)(b + kLayout.pcoef);

    /* tables and multipliers: refit and copy in when they differ from what the array holds */
    bool same = slot.have_tables && ctx_id != 0 && slot.ctx_id == ctx_id && slot.base == b &&
                slot.order == order && slot.nseg == nseg && slot.bins == bins && slot.min_log2 == m0 &&
                slot.ntypes == p->ntypes;
    for (int t = 0; same && t < p->ntypes; ++t)
        same = slot.sigma[t] == p->sigma[t] && slot.epsilon[t] == p->epsilon[t];
    if (!same) {
        /* the copies below overwrite the array: it holds no valid tables until they complete */
        slot.have_tables = false;
        std::vector<float> tab;
        fit_tables(order, nseg, bins, m0, 8, &tab, 0.0, order >= 2);
        std::vector<float> pc;
        mix_pair_coefficients(*p, &pc, nullptr);
        const int nc = order + 1;
        auto coef = [&](int f, int k, int i) { return tab[((size_t)f * nc + k) * nidx + i]; };
        if (order == 1) {
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
            ST_CUDA(cudaMemcpyAsync(b + kLayout.tabr, fr.data(), sizeof(float4) * fr.size(), cudaMemcpyHostToDevice, st));
            ST_CUDA(cudaMemcpyAsync(b + kLayout.tabf, f2.data(), sizeof(float2) * f2.size(), cudaMemcpyHostToDevice, st));
            ST_CUDA(cudaMemcpyAsync(b + kLayout.tabe, e2.data(), sizeof(float2) * e2.size(), cudaMemcpyHostToDevice, st));
        } else {
            std::vector<float4> f4((size_t)3 * nidx), e4((size_t)3 * nidx);
            for (int i = 0; i < nidx; ++i)
                for (int f = 0; f < 3; ++f) {
                    float a[4] = {0, 0, 0, 0}, e[4] = {0, 0, 0, 0};
                    for (int k = 0; k < nc; ++k) { a[k] = coef(f, k, i); e[k] = coef(3 + f, k, i); }
                    f4[(size_t)3 * i + f] = make_float4(a[0], a[1], a[2], a[3]);
                    e4[(size_t)3 * i + f] = make_float4(e[0], e[1], e[2], e[3]);
                }
            ST_CUDA(cudaMemcpyAsync(b + kLayout.tabf, f4.data(), sizeof(float4) * f4.size(), cudaMemcpyHostToDevice, st));
            ST_CUDA(cudaMemcpyAsync(b + kLayout.tabe, e4.data(), sizeof(float4) * e4.size(), cudaMemcpyHostToDevice, st));
        }
        const int T = p->ntypes;
        std::vector<float4> pc4((size_t)T * T);
        for (int k = 0; k < T * T; ++k) pc4[k] = make_float4(pc[4 * k], pc[4 * k + 1], pc[4 * k + 2], pc[4 * k + 3]);
        ST_CUDA(cudaMemcpyAsync(d_pcoef, pc4.data(), sizeof(float4) * pc4.size(), cudaMemcpyHostToDevice, st));
        ST_CUDA(cudaStreamSynchronize(st)); /* the host vectors go out of scope */
        slot.have_tables = true;
        slot.ctx_id = ctx_id;
        slot.base = b;
        slot.order = order; slot.nseg = nseg; slot.bins = bins; slot.min_log2 = m0; slot.ntypes = T;
        for (int t = 0; t < T; ++t) { slot.sigma[t] = p->sigma[t]; slot.epsilon[t] = p->epsilon[t]; }
    }
    TableDev tab;
    tab.f2 = (const float2 *)(b + kLayout.tabf); tab.e2 = (const float2 *)(b + kLayout.tabe);
    tab.f4 = (const float4 *)(b + kLayout.tabf); tab.e4 = (const float4 *)(b + kLayout.tabe);
    tab.fr = (const float4 *)(b + kLayout.tabr);
    tab.fp2 = nullptr;   /* the packed order-2 rows are read by the one-warp-per-item kernel only */
    tab.fc2 = nullptr;
    tab.order = order; tab.nseg = nseg; tab.bins = bins;
    int lb = 0;
    while ((1 << lb) < bins) ++lb;
    tab.lb = lb; tab.min_log2 = m0; tab.r2min = std::ldexp(1.0f, m0);
    tab.local = order >= 2 ? 1 : 0;   /* as a context fits them */

    /* state that must start at zero; the previous call's contents are otherwise left in place */
    const int nc = (int)ncells;
    ST_CUDA(cudaMemsetAsync(d_err, 0, sizeof(unsigned), st));
    ST_CUDA(cudaMemsetAsync(d_tot, 0, sizeof(DevTotals), st));
    ST_CUDA(cudaMemsetAsync(d_count, 0, sizeof(int) * nc, st));
    const int blk = 256, grid = (n + blk - 1) / blk;
    if (n > 0) k_bin_user<<<grid, blk, 0, st>>>(n, x, y, z, g, d_cell_of, d_slot, d_count, d_err, d_key);
    k_scan<<<1, 1024, 0, st>>>(nc, d_count, d_start, d_tot);
    if (n > 0) {
        k_scatter<<<grid, blk, 0, st>>>(n, d_cell_of, d_slot, d_start, d_tmp);
        k_cell_sort<<<nc, 128, 0, st>>>(d_start, d_tmp, d_sorted, d_key, d_sortkey, d_err);
        k_gather_user<<<grid, blk, 0, st>>>(n, d_sorted, x, y, z, q, type, d_pos, d_type, d_id, d_F64, nullptr,
                                            nullptr, p->ntypes, d_err);
    }
    const int ord = p->eval == MDRL_EVAL_DIRECT ? 0 : order;
    force_fn fn = pick_force(ord, p->arith == MDRL_ARITH_SEPARATE, false, MDRL_ACC_FIXED64, kFW, false,
                             (p->flags & MDRL_FLAG_EXACT_DIFF) != 0);
    const size_t smem = force_smem_bytes(p->ntypes, false);
    ST_CUDA(cudaFuncSetAttribute((const void *)fn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)force_smem_bytes(MDRL_MAX_TYPES, true, 8)));
    fn<<<nc * kHalfShellCells, kFT, smem, st>>>(d_pos, d_type, d_start, g, tab, d_pcoef, p->ntypes,
                                                (float)p->coulomb_k, n, d_F64, nullptr, nullptr, d_unit, nullptr,
                                                nullptr, tile_word(kStepsPerPiece, 0), d_err, 0);
    k_totals<<<1, 1024, 0, st>>>(force_items(nc), d_unit, 0, nullptr, d_tot, 0);
    if (n > 0)
        k_unsort<<<grid, blk, 0, st>>>(n, d_id, d_F64, nullptr, nullptr, fx, fy, fz, nullptr);
    ST_CUDA(cudaGetLastError());
    unsigned err = 0;
    DevTotals tot;
    ST_CUDA(cudaMemcpyAsync(&err, d_err, sizeof(unsigned), cudaMemcpyDeviceToHost, st));
    ST_CUDA(cudaMemcpyAsync(&tot, d_tot, sizeof(DevTotals), cudaMemcpyDeviceToHost, st));
    ST_CUDA(cudaStreamSynchronize(st));
    const mdrl_status es = device_error_status(err);
    if (es != MDRL_OK) return fail(es, mdrl_last_error());
    if (pairs_out) *pairs_out = (int64_t)tot.pairs;
    return MDRL_OK;
}
