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
 * Set-up: the first call on a device (with that device current) looks up the device address of
 * the array with cudaGetSymbolAddress; make that first call before any stream capture.  Tables
 * are fitted on the host and copied into the array when the table parameters change.
 *
 * Sharing: every call uses the same array, which keeps the previous call's contents; the call
 * clears what must start at zero.  Two calls whose work overlaps on the GPU (different streams,
 * or threads without ordering) race on the array: serialise them.
 */
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
    size_t err, tot, count, start, unit, cell_of, slot, tmp, sorted, key, pos, type, id, F64, tabf,
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

/* What the array currently holds on one device. */
struct DeviceSlot {
    unsigned char *base = nullptr;   /* device address of g_static_scratch */
    bool have_tables = false;
    int order = 0, nseg = 0, bins = 0, min_log2 = 0, ntypes = 0;
    double sigma[MDRL_MAX_TYPES] = {}, epsilon[MDRL_MAX_TYPES] = {};
};

std::mutex g_mu;
DeviceSlot g_slots[kStaticMaxDevices];

mdrl_status fail(mdrl_status s, const std::string &msg) {
    set_error("mdrl_force_eval_static: " + msg);
    return s;
}

#define ST_CUDA(call)                                                                             \
    do {                                                                                          \
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
    if (n > kStaticMaxN)
        return fail(MDRL_ERR_RANGE, "n = " + std::to_string(n) + " exceeds the static scratch limit of " +
                                        std::to_string(kStaticMaxN) + " particles");
    if (p->accum != MDRL_ACC_FIXED64)
        return fail(MDRL_ERR_INVALID_ARG, "only int64 fixed-point accumulation (MDRL_ACC_FIXED64) is supported");
    if (p->ntypes < 1 || p->ntypes > MDRL_MAX_TYPES || p->table_order < 1 || p->table_order > 3 ||
        p->table_bins < 16 || p->table_bins > 4096 || (p->table_bins & (p->table_bins - 1)) ||
        !(p->cutoff > 0.0) || (p->eval != MDRL_EVAL_TABLE && p->eval != MDRL_EVAL_DIRECT) ||
        (p->arith != MDRL_ARITH_FMA && p->arith != MDRL_ARITH_SEPARATE))
        return fail(MDRL_ERR_INVALID_ARG, "invalid parameters");
    for (int t = 0; t < p->ntypes; ++t)
        if (!(p->sigma[t] > 0) || !(p->epsilon[t] >= 0)) return fail(MDRL_ERR_INVALID_ARG, "invalid type parameters");

    /* geometry, as mdrl_create sets it up */
    Geom g;
    const float rcf = (float)p->cutoff;
    g.rc2 = rcf * rcf;
    long long ncells = 1;
    for (int d = 0; d < 3; ++d) {
        if (!(p->box[d] > 0.0)) return fail(MDRL_ERR_INVALID_ARG, "box edges must be positive");
        const float L = (float)p->box[d];
        const int nc = p->ncell[d] > 0 ? p->ncell[d] : (int)std::floor((double)L / (double)rcf);
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
    const int nidx = nseg * bins;
    if (nidx > kStaticMaxTable)
        return fail(MDRL_ERR_RANGE, std::to_string(nidx) + " table entries exceed the static scratch limit of " +
                                        std::to_string(kStaticMaxTable));

    int dev = 0;
    ST_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kStaticMaxDevices) return fail(MDRL_ERR_RANGE, "device ordinal too large");
    cudaStream_t st = (cudaStream_t)stream_ptr;

    std::lock_guard<std::mutex> lock(g_mu);
    DeviceSlot &slot = g_slots[dev];
    if (!slot.base) {
        void *ptr = nullptr;
        ST_CUDA(cudaGetSymbolAddress(&ptr, g_static_scratch));
        slot.base = (unsigned char *)ptr;
    }
    unsigned char *b = slot.base;
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
    float4 *d_pos = (float4 *)(b + kLayout.pos);
    int *d_type = (int *)(b + kLayout.type);
    int *d_id = (int *)(b + kLayout.id);
    unsigned long long *d_F64 = (unsigned long long *)(b + kLayout.F64);
    float4 *d_pcoef = (float4 *)(b + kLayout.pcoef);

    /* tables and multipliers: refit and copy in when they differ from what the array holds */
    bool same = slot.have_tables && slot.order == order && slot.nseg == nseg && slot.bins == bins &&
                slot.min_log2 == m0 && slot.ntypes == p->ntypes;
    for (int t = 0; same && t < p->ntypes; ++t)
        same = slot.sigma[t] == p->sigma[t] && slot.epsilon[t] == p->epsilon[t];
    if (!same) {
        std::vector<float> tab;
        fit_tables(order, nseg, bins, m0, 8, &tab);
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
        slot.order = order; slot.nseg = nseg; slot.bins = bins; slot.min_log2 = m0; slot.ntypes = T;
        for (int t = 0; t < T; ++t) { slot.sigma[t] = p->sigma[t]; slot.epsilon[t] = p->epsilon[t]; }
    }
    TableDev tab;
    tab.f2 = (const float2 *)(b + kLayout.tabf); tab.e2 = (const float2 *)(b + kLayout.tabe);
    tab.f4 = (const float4 *)(b + kLayout.tabf); tab.e4 = (const float4 *)(b + kLayout.tabe);
    tab.fr = (const float4 *)(b + kLayout.tabr);
    tab.order = order; tab.nseg = nseg; tab.bins = bins;
    int lb = 0;
    while ((1 << lb) < bins) ++lb;
    tab.lb = lb; tab.min_log2 = m0; tab.r2min = std::ldexp(1.0f, m0);

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
        k_cell_sort<<<nc, 128, 0, st>>>(d_start, d_tmp, d_sorted, d_key);
        k_gather_user<<<grid, blk, 0, st>>>(n, d_sorted, x, y, z, q, type, d_pos, d_type, d_id, d_F64, nullptr,
                                            nullptr, p->ntypes, d_err);
    }
    const int ord = p->eval == MDRL_EVAL_DIRECT ? 0 : order;
    force_fn fn = pick_force(ord, p->arith == MDRL_ARITH_SEPARATE, false, MDRL_ACC_FIXED64);
    const size_t smem = force_smem_bytes(p->ntypes, false);
    ST_CUDA(cudaFuncSetAttribute((const void *)fn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)force_smem_bytes(MDRL_MAX_TYPES, true, 8)));
    fn<<<nc * kHalfShellCells, kFT, smem, st>>>(d_pos, d_type, d_start, g, tab, d_pcoef, p->ntypes,
                                                (float)p->coulomb_k, n, d_F64, nullptr, nullptr, d_unit, nullptr,
                                                nullptr, tile_word(kStepsPerPiece, 0));
    k_totals<<<1, 1024, 0, st>>>(force_items(nc), d_unit, 0, nullptr, d_tot, 0);
    if (n > 0)
        k_unsort<<<grid, blk, 0, st>>>(n, d_id, d_F64, nullptr, nullptr, fx, fy, fz, nullptr);
    ST_CUDA(cudaGetLastError());
    unsigned err = 0;
    DevTotals tot;
    ST_CUDA(cudaMemcpyAsync(&err, d_err, sizeof(unsigned), cudaMemcpyDeviceToHost, st));
    ST_CUDA(cudaMemcpyAsync(&tot, d_tot, sizeof(DevTotals), cudaMemcpyDeviceToHost, st));
    ST_CUDA(cudaStreamSynchronize(st));
    if (err & kErrPosition) return fail(MDRL_ERR_INVALID_ARG, "positions must be finite and lie in [0, box)");
    if (err & kErrType) return fail(MDRL_ERR_INVALID_ARG, "particle types must lie in [0, ntypes)");
    if (pairs_out) *pairs_out = (int64_t)tot.pairs;
    return MDRL_OK;
}
