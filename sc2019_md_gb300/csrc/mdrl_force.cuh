/*
 * mdrl_force.cuh — the half-shell pair-force kernel (sm_103a).
 *
 * One CTA of 4 warps per unit = (home cell h, half-shell neighbour f), f = 0..13 in the
 * reference's filter order (SC/Particle_Pair_Gen_HalfShell.v:14-24).  The CTA stages h's and
 * the neighbour's particles (256 at a time) in shared memory.  The (i, j) square is cut into
 * pieces of 32 i-particles x (8 * kStepsPerPiece) j-particles, dealt round-robin to the warps.
 * Staging uses cp.async: positions (float4) and types go from global to shared memory directly.
 *
 * Inside a piece, lane = row * 8 + col (4 rows x 8 columns): the lane keeps the 8 i-particles
 * i = row + 4k (k < 8) in registers, and in each step takes j = 8 * step + col.  A step
 * evaluates 8 candidates per lane; the j force of the step is summed in registers, reduced over
 * the 4 rows with two shuffles per component and added to the warp's private shared-memory
 * accumulator; the i forces stay in registers for the whole piece and are reduce-scattered over
 * the 8 columns at its end (after which each lane owns one i's complete partial sum).  When the
 * unit is done the 4 warp accumulators are summed in warp order and added to global memory with
 * one atomic per particle and component (int64 fixed point 2^-24: exact, so the result does not
 * depend on the order in which CTAs finish).
 *
 * Periodic wrap.  The reference applies one wrap per pair (d > L/2 -> d - L, d < -L/2 -> d + L;
 * SC/r2_compute_with_pbc.v:81-127).  A unit instead adds a precomputed -L, 0 or +L to
 * fl(xi - xj) per axis, by whether the neighbour cell lies across the box boundary: the same two
 * roundings.  With at least 3 cells of edge e >= rc per axis (L = n e) the two rules agree on
 * every pair that can pass the filter: where they differ, the unit's rule leaves |d| above 1.5 e
 * or the reference's leaves it above e (adjacent cells are less than 2 e apart, cells across the
 * boundary more than e), both above rc; so the accepted pairs and their d are bit-identical
 * (checked exhaustively on 3-cell systems with particles on cell and box faces).  WRAP = true
 * keeps the per-pair rule for explicit cell pairs of small boxes (batches).
 *
 * Within a cell the particles are in Morton order of their position inside the cell, so the 4 i
 * x 8 j candidates of one warp instruction are spatially coherent: for ~70 % of them no lane
 * passes the filter and the warp skips the force path; the busy ones carry ~14 accepted lanes.
 *
 * Table address.  r2e = max(r2, 2^min_log2); (bits(r2e) >> (23 - log2 bins)) - ((127 +
 * min_log2) << log2 bins) is segment * bins + bin, the address the RTL forms from the exponent
 * and the top mantissa bits (SC/RL_LJ_Evaluate_Pairs_1st_Order.v:179-193).  Accepted pairs have
 * r2 <= rc2, and the host guarantees the tables extend past rc2.
 */
#pragma once

#include <type_traits>

#include "mdrl_kernels.cuh"

namespace mdrl {

#ifndef MDRL_FORCE_WARPS
#define MDRL_FORCE_WARPS 4
#endif
#ifndef MDRL_STEPS_PER_PIECE
#define MDRL_STEPS_PER_PIECE 6
#endif
#ifndef MDRL_FORCE_CTAS_PER_SM
#define MDRL_FORCE_CTAS_PER_SM (16 / MDRL_FORCE_WARPS)
#endif
constexpr int kFW = MDRL_FORCE_WARPS;  /* default warps per force CTA (tiles may use 8) */
constexpr int kFT = kFW * 32;
constexpr int kStepsPerPiece = MDRL_STEPS_PER_PIECE;   /* default j-steps (of 8 particles) per piece */
/* The tile word a force launch takes: steps per piece in bits 0-7 (pruning is a template
 * parameter of the kernel; bit 8 records it). */
inline int tile_word(int steps_per_piece, int prune) { return (steps_per_piece & 0xff) | ((prune ? 1 : 0) << 8); }
constexpr int kFCtas = MDRL_FORCE_CTAS_PER_SM;         /* resident CTAs per SM the registers allow */
constexpr int kBatchFT = 128;          /* threads of a batched-replica CTA (4 warps) */

struct BatchRep;
struct BatchItem;
typedef void (*force_fn)(const float4 *, const int *, const int *, Geom, TableDev, const float4 *,
                         int, float, int, unsigned long long *, float *, int *, UnitOut *,
                         const BatchItem *, const BatchRep *, int, unsigned *, int);

/* Work items (one per unit): the result slots k_totals sums. */
inline int force_items(int ncells) { return ncells * kHalfShellCells; }

/* fw: warps per CTA (8 only with int64 fixed point); prune: survivor lists (fixed point only);
 * exact: the exact-difference rule (fused arithmetic only) */
force_fn pick_force(int order, bool sep, bool extra, int acc, int fw = kFW, bool prune = false,
                    bool exact = false);
/* the batched-replica instantiation (int64 fixed point, difference rule per item) */
force_fn pick_force_batch(int order, bool sep, bool extra, bool prune);

inline size_t force_smem_bytes(int ntypes, bool extra, int fw = kFW) {
    return sizeof(float4) * (2 * kChunk + ntypes * ntypes) + sizeof(int) * 2 * kChunk +
           sizeof(float) * fw * 6 * kChunk + (extra ? sizeof(int) * fw * 2 * kChunk : 0);
}

/* The pair functions of an accepted pair at r2e = max(r2, 2^min_log2).  Order 1 reads one
 * 32-byte row {c0_14, c1_14, c0_8, c1_8}{c0_3, c1_3, 0, 0}; orders 2-3 read float4 rows. */
template <int ORDER, bool SEP, bool ENERGY>
__device__ __forceinline__ void pair_functions_fast(const TableDev &t, float r2, bool coul, float &v14,
                                                    float &v8, float &v3, float &v12, float &v6, float &v1) {
    if (ORDER == 0) {
        int below;
        pair_functions<0, SEP, ENERGY>(t, r2, coul, v14, v8, v3, v12, v6, v1, below);
        return;
    }
    const float r2e = fmaxf(r2, t.r2min);
    const int idx = (int)(__float_as_uint(r2e) >> (23 - t.lb)) - ((127 + t.min_log2) << t.lb);
    if (ORDER == 1) {
        const float4 a = __ldg(t.fr + 2 * idx);
        v14 = madd<SEP>(a.y, r2e, a.x);
        v8 = madd<SEP>(a.w, r2e, a.z);
        v3 = 0.0f;
        if (coul) { const float4 c = __ldg(t.fr + 2 * idx + 1); v3 = madd<SEP>(c.y, r2e, c.x); }
        if (ENERGY) {
            const float2 d = __ldg(t.e2 + 3 * idx), e = __ldg(t.e2 + 3 * idx + 1);
            v12 = madd<SEP>(d.y, r2e, d.x);
            v6 = madd<SEP>(e.y, r2e, e.x);
            v1 = 0.0f;
            if (coul) { const float2 gg = __ldg(t.e2 + 3 * idx + 2); v1 = madd<SEP>(gg.y, r2e, gg.x); }
        }
    } else {
        const float x = table_variable(t, r2e);
        v14 = poly4<ORDER, SEP>(__ldg(t.f4 + 3 * idx), x);
        v8 = poly4<ORDER, SEP>(__ldg(t.f4 + 3 * idx + 1), x);
        v3 = coul ? poly4<ORDER, SEP>(__ldg(t.f4 + 3 * idx + 2), x) : 0.0f;
        if (ENERGY) {
            v12 = poly4<ORDER, SEP>(__ldg(t.e4 + 3 * idx), x);
            v6 = poly4<ORDER, SEP>(__ldg(t.e4 + 3 * idx + 1), x);
            v1 = coul ? poly4<ORDER, SEP>(__ldg(t.e4 + 3 * idx + 2), x) : 0.0f;
        }
    }
}

/* Pair difference rules of a unit (the first two give the reference's d for every pair that can
 * pass the filter; see the header):
 *   kDiffShift  fl(fl(xi - xj) + s)        (the unit's -L/0/+L shift: half-shell units)
 *   kDiffWrap   the one-wrap rule per pair (explicit cell pairs of small boxes in batches)
 *   kDiffExact  fl(xi' - xj'): the exact minimum-image difference rounded once
 *               (MDRL_FLAG_EXACT_DIFF).  The unit's shift is taken off the far (high) coordinate
 *               when the cells are staged: across the +L face the home cell is the last one, so
 *               xi' = xi - L (exact: xi >= 2L/3 with at least 3 cells, Sterbenz); across the -L
 *               face the neighbour is the last cell and xj' = xj - L.  The reference's rule
 *               rounds fl(xi - xj) of two far-apart coordinates first, an absolute error up to
 *               ulp(L)/2 that r^-14 amplifies 14-fold in a close pair's force. */
enum : int { kDiffShift = 1, kDiffWrap = 2, kDiffExact = 3 };

template <int MODE>
__device__ __forceinline__ float pair_diff(float a, float b, float L, float h, float s) {
    const float d = __fsub_rn(a, b);
    if (MODE == kDiffExact) return d;
    return MODE == kDiffWrap ? wrap_d(d, L, h) : __fadd_rn(d, s);
}

/* Asynchronous global -> shared copies (cp.async): a staged particle goes to shared memory
 * without a round trip through registers, and the copies run while the CTA clears its
 * accumulators.  cp.async.wait_all is a hardware wait for the thread's own copies (no polling);
 * the barrier after it makes every thread's copies visible. */
__device__ __forceinline__ void cp_async16(void *smem, const void *gmem) {
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 16;" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async4(void *smem, const void *gmem) {
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

/* Sum of v over the 8 column lanes, scattered: on return lane col holds, in v[0..2], the sums of
 * the input v[3*col .. 3*col+2] (each input v has 24 entries). */
__device__ __forceinline__ void reduce_scatter24(float (&v)[24], int col) {
    const bool b4 = col & 4, b2 = col & 2, b1 = col & 1;
#pragma unroll
    for (int t = 0; t < 12; ++t) {
        const float send = b4 ? v[t] : v[12 + t];
        const float keep = b4 ? v[12 + t] : v[t];
        v[t] = keep + __shfl_xor_sync(0xffffffffu, send, 4);
    }
#pragma unroll
    for (int t = 0; t < 6; ++t) {
        const float send = b2 ? v[t] : v[6 + t];
        const float keep = b2 ? v[6 + t] : v[t];
        v[t] = keep + __shfl_xor_sync(0xffffffffu, send, 2);
    }
#pragma unroll
    for (int t = 0; t < 3; ++t) {
        const float send = b1 ? v[t] : v[3 + t];
        const float keep = b1 ? v[3 + t] : v[t];
        v[t] = keep + __shfl_xor_sync(0xffffffffu, send, 1);
    }
}

__device__ __forceinline__ int reduce_scatter8i(int (&v)[8], int col) {
    const bool b4 = col & 4, b2 = col & 2, b1 = col & 1;
#pragma unroll
    for (int t = 0; t < 4; ++t) {
        const int send = b4 ? v[t] : v[4 + t];
        const int keep = b4 ? v[4 + t] : v[t];
        v[t] = keep + __shfl_xor_sync(0xffffffffu, send, 4);
    }
#pragma unroll
    for (int t = 0; t < 2; ++t) {
        const int send = b2 ? v[t] : v[2 + t];
        const int keep = b2 ? v[2 + t] : v[t];
        v[t] = keep + __shfl_xor_sync(0xffffffffu, send, 2);
    }
    const int send = b1 ? v[0] : v[1];
    const int keep = b1 ? v[1] : v[0];
    return keep + __shfl_xor_sync(0xffffffffu, send, 1);
}

/* Compensated FP32 accumulation: add v to the high plane with an atomic that returns the old
 * value, recompute the rounded sum and add its exact rounding error (Knuth's TwoSum) to the low
 * plane.  high + low then carries the global sum to ~FP32^2 relative error. */
__device__ __forceinline__ void kahan_add(float *hi, float *lo, float v) {
    const float old = atomicAdd(hi, v);
    const float s = __fadd_rn(old, v);
    const float bb = __fsub_rn(s, old);
    const float e = __fadd_rn(__fsub_rn(old, __fsub_rn(s, bb)), __fsub_rn(v, bb));
    if (e != 0.0f) atomicAdd(lo, e);
}

/* Add one particle's force (fx, fy, fz) to the accumulators of mode ACC.  A sum the mode cannot
 * hold (NaN or infinite; with fixed point also |F| >= kFixMax) raises kErrForce in *err. */
template <int ACC>
__device__ __forceinline__ void flush_force(unsigned long long *F64, float *F32, int n, int g, float fx,
                                            float fy, float fz, unsigned *err) {
    if (ACC == 0) check_force(err, fx, fy, fz);
    else if (!(isfinite(fx) && isfinite(fy) && isfinite(fz)) && err) atomicOr(err, kErrForce);
    if (ACC == 1) {
        atomicAdd(F32 + g, fx);
        atomicAdd(F32 + n + g, fy);
        atomicAdd(F32 + 2 * n + g, fz);
    } else if (ACC == 2) {
        kahan_add(F32 + g, F32 + 3 * (size_t)n + g, fx);
        kahan_add(F32 + n + g, F32 + 4 * (size_t)n + g, fy);
        kahan_add(F32 + 2 * n + g, F32 + 5 * (size_t)n + g, fz);
    } else {
        atomicAdd(F64 + g, to_fixed(fx));
        atomicAdd(F64 + n + g, to_fixed(fy));
        atomicAdd(F64 + 2 * n + g, to_fixed(fz));
    }
}

/* ---- batched replicas ----------------------------------------------------------------------
 * One launch covers every replica of a batch; a work item is one of
 *   (replica, half-shell unit)  at least 3 cells of edge >= rc per axis: the path below with the
 *                               replica's geometry and cell offset (per-unit shift);
 *   (replica, cell pair a <= b) every edge above 2 rc but fewer cells: the same tiled Newton-3
 *                               path over an explicit pair of cells, per-pair minimum image;
 *   (replica, 128 particles)    an edge of at most 2 rc (always above rc): every periodic image
 *                               within rc, all_images_body. */
enum : int { kPathHalfShell = 0, kPathMinImage = 1, kPathAllImages = 2 };

struct BatchRep {
    Geom g;
    int cell_off;    /* first global cell of the replica */
    int p_off, n;    /* its particles: [p_off, p_off + n) of the cell-sorted arrays */
    int path;        /* kPath* */
};

struct BatchItem {
    int rep;
    int unit;        /* half-shell unit, or first particle (relative) of an all-pairs block */
};

/* Forces of a replica with a box edge of at most 2 rc (always above rc), where more than one
 * periodic image of a pair can lie within rc.  Per axis the candidates are fl(xi - xj),
 * fl(. - L), fl(. + L) with fl(d*d) <= rc2 (a necessary condition for r2 <= rc2, since r2 >=
 * each rounded square); every combination with 0 < r2 <= rc2 is a pair, and at most two
 * candidates pass per axis because the edge exceeds rc.  Thread t owns particle i = b0 + t and
 * sums f_ij over every j != i and image, each ordered pair evaluated from i's side
 * (QQ = (ke*qi)*qj), so the particle's force is complete and is stored without atomics;
 * energies and the virial carry a factor 1/2, and pairs count j > i. */
template <int ORDER, bool SEP, bool EXTRA, int FW>
__device__ __forceinline__ void all_images_body(const float4 *__restrict__ pos, const int *__restrict__ ptype,
                                                   const BatchRep &rp, int b0, TableDev tab,
                                                   const float4 *sCoef, int ntypes, float ke, int ntot,
                                                   unsigned long long *__restrict__ F64,
                                                   int *__restrict__ counts, float4 *sJp, int *sJt,
                                                   float &acc_elj, float &acc_ec, float &acc_vir,
                                                   unsigned &acc_pairs, unsigned &acc_below, unsigned *err) {
    const Geom &g = rp.g;
    const int tid = threadIdx.x;
    const int i = b0 + tid;
    const bool have = i < rp.n;
    float4 pi = make_float4(0.f, 0.f, 0.f, 0.f);
    int ti = 0;
    if (have) { pi = pos[rp.p_off + i]; ti = ptype[rp.p_off + i] * ntypes; }
    const float qi = __fmul_rn(ke, pi.w);
    const bool coul = ke != 0.0f;
    float fx = 0.f, fy = 0.f, fz = 0.f;
    int cnt = 0;
    auto eval = [&](float dx, float dy, float dz, float r2, float qj, int tj, bool upper) {
        float v14, v8, v3, v12, v6, v1;
        pair_functions_fast<ORDER, SEP, EXTRA>(tab, r2, coul, v14, v8, v3, v12, v6, v1);
        const float4 pc = sCoef[ti + tj];
        const float qq = __fmul_rn(qi, qj);
        const float fs = combine_force<SEP>(pc, qq, coul, v14, v8, v3);
        fx += __fmul_rn(fs, dx); fy += __fmul_rn(fs, dy); fz += __fmul_rn(fs, dz);
        if (upper) ++acc_pairs;
        if (EXTRA) {
            ++cnt;
            if (upper) acc_below += (ORDER > 0 && r2 < tab.r2min) ? 1u : 0u;
            acc_elj += 0.5f * combine_elj<SEP>(pc, v12, v6);
            if (coul) acc_ec += 0.5f * __fmul_rn(qq, v1);
            acc_vir += 0.5f * __fmul_rn(fs, r2);
        }
    };
    for (int j0 = 0; j0 < rp.n; j0 += (FW * 32)) {
        const int nj = min((FW * 32), rp.n - j0);
        __syncthreads();
        if (tid < nj) { sJp[tid] = pos[rp.p_off + j0 + tid]; sJt[tid] = ptype[rp.p_off + j0 + tid]; }
        __syncthreads();
        if (!have) continue;
        for (int jj = 0; jj < nj; ++jj) {
            const int j = j0 + jj;
            if (j == i) continue;
            const float4 pj = sJp[jj];
            float c[3][2];
            int nc[3];
            const float d0[3] = {__fsub_rn(pi.x, pj.x), __fsub_rn(pi.y, pj.y), __fsub_rn(pi.z, pj.z)};
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                const float cand[3] = {d0[a], __fsub_rn(d0[a], g.L[a]), __fadd_rn(d0[a], g.L[a])};
                int k = 0;
                c[a][0] = c[a][1] = 0.0f;
#pragma unroll
                for (int m = 0; m < 3; ++m)
                    if (__fmul_rn(cand[m], cand[m]) <= g.rc2 && k < 2) {
                        if (k == 0) c[a][0] = cand[m]; else c[a][1] = cand[m];
                        ++k;
                    }
                nc[a] = k;
            }
            for (int ax = 0; ax < nc[0]; ++ax)
                for (int ay = 0; ay < nc[1]; ++ay)
                    for (int az = 0; az < nc[2]; ++az) {
                        const float dx = ax ? c[0][1] : c[0][0];
                        const float dy = ay ? c[1][1] : c[1][0];
                        const float dz = az ? c[2][1] : c[2][0];
                        const float r2 = __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
                        if (r2 > 0.0f && r2 <= g.rc2) eval(dx, dy, dz, r2, pj.w, sJt[jj], j > i);
                    }
        }
    }
    if (have) {
        const size_t gi = (size_t)rp.p_off + i;
        check_force(err, fx, fy, fz);
        F64[gi] = to_fixed(fx);
        F64[(size_t)ntot + gi] = to_fixed(fy);
        F64[2 * (size_t)ntot + gi] = to_fixed(fz);
        if (EXTRA) counts[gi] = cnt;
    }
}

/* One unit: home-cell particles [hs, hs + ni_all) against neighbour-cell particles
 * [cs, cs + nj_all) (the same cell when self), with the pair-difference rule MODE (kDiff*); writes the unit's totals to uout[blockIdx.x]. */
template <int ORDER, bool SEP, bool EXTRA, int ACC, int MODE, int FW, bool PRUNE>
__device__ __forceinline__ void force_unit(const float4 *__restrict__ pos, const int *__restrict__ ptype,
                                           int hs, int ni_all, int cs, int nj_all, bool self, const Geom &g,
                                           float sx, float sy, float sz, const TableDev &tab,
                                           const float4 *__restrict__ pcoef, int ntypes, float ke, int n,
                                           unsigned long long *__restrict__ F64, float *__restrict__ F32,
                                           int *__restrict__ counts, UnitOut *__restrict__ uout, float4 *sIp,
                                           float4 *sJp, float4 *sCoef, int *sIt, int *sJt, float *sF, int *sC,
                                           double (*s_red)[3], unsigned long long (*s_cnt)[2], int tilecfg,
                                           unsigned *err) {
    const int spp = tilecfg & 0xff;               /* j-steps per piece */
    constexpr bool prune = PRUNE;                 /* survivor lists (below) */
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int row = lane >> 3, col = lane & 7;
    const bool coul = ke != 0.0f;
    const float far = 1.0e18f;   /* padding lanes: finite, so r2 ~ 3e36 > rc2 */
    float *wFi = sF + warp * 6 * kChunk;
    float *wFj = wFi + 3 * kChunk;
    int *wCi = sC + warp * 2 * kChunk;
    int *wCj = wCi + kChunk;

    /* Survivor lists (when the tile asks for pruning).  The boxes of each group of 4 i-particles
     * (the 4 rows of one register slot k: i = 32 ti + 4 k + row) are tested against the box of each
     * 8-j step; a (32-i tile, step) pair survives when any of its 8 groups comes within rc, and
     * carries the 8-bit mask of those groups, so the step loop skips the dead slots (a
     * warp-uniform bit test).  A lower bound on every pair's r2 from the two boxes decides; the
     * half widths carry a margin of 2^-20 x the largest box edge, above the rounding of the box
     * centres, widths and gaps and of the pair differences, so a dropped slot holds no pair that
     * passes the filter. */
    __shared__ float4 s_gb[2][kChunk / 4];
    __shared__ float4 s_sb[2][kChunk / 8];
    __shared__ unsigned char s_km[kChunk / 32][kChunk / 8];
    __shared__ int s_nsurv[kChunk / 32];
    __shared__ unsigned char s_list[kChunk / 32][kChunk / 8];
    __shared__ unsigned char s_klist[kChunk / 32][kChunk / 8];
    const float margin = 9.5367431640625e-07f * fmaxf(g.L[0], fmaxf(g.L[1], g.L[2]));

    for (int t = tid; t < ntypes * ntypes; t += (FW * 32)) sCoef[t] = pcoef[t];

    float acc_elj = 0.0f, acc_ec = 0.0f, acc_vir = 0.0f;
    unsigned acc_pairs = 0, acc_below = 0;

    for (int i0 = 0; i0 < ni_all; i0 += kChunk) {
        for (int j0 = self ? i0 : 0; j0 < nj_all; j0 += kChunk) {
            const int ni = min(kChunk, ni_all - i0), nj = min(kChunk, nj_all - j0);
            const bool diag = self && (i0 == j0);
            __syncthreads();
            /* stage both cells' positions (16 B) and types (4 B) with cp.async */
            for (int t = tid; t < ni; t += (FW * 32)) {
                cp_async16(sIp + t, pos + hs + i0 + t);
                cp_async4(sIt + t, ptype + hs + i0 + t);
            }
            for (int t = tid; t < nj; t += (FW * 32)) {
                cp_async16(sJp + t, pos + cs + j0 + t);
                cp_async4(sJt + t, ptype + cs + j0 + t);
            }
            /* sF and sC start 16-byte aligned (after 16 (2 kChunk + T^2) + 8 kChunk bytes) */
            for (int t = tid; t < FW * 6 * kChunk / 4; t += (FW * 32))
                reinterpret_cast<float4 *>(sF)[t] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            if (EXTRA)
                for (int t = tid; t < FW * 2 * kChunk / 4; t += (FW * 32))
                    reinterpret_cast<int4 *>(sC)[t] = make_int4(0, 0, 0, 0);
            cp_async_wait_all();
            if (MODE == kDiffExact && (sx != 0.0f || sy != 0.0f || sz != 0.0f)) {
                /* take the box edge off the high side's coordinates (exact); each thread shifts
                 * the elements it copied, which its own wait has completed */
                const float ix = sx < 0.0f ? sx : 0.0f, iy = sy < 0.0f ? sy : 0.0f, iz = sz < 0.0f ? sz : 0.0f;
                const float jx = sx > 0.0f ? sx : 0.0f, jy = sy > 0.0f ? sy : 0.0f, jz = sz > 0.0f ? sz : 0.0f;
                for (int t = tid; t < ni; t += (FW * 32)) {
                    float4 pp = sIp[t];
                    pp.x = __fadd_rn(pp.x, ix); pp.y = __fadd_rn(pp.y, iy); pp.z = __fadd_rn(pp.z, iz);
                    sIp[t] = pp;
                }
                for (int t = tid; t < nj; t += (FW * 32)) {
                    float4 pp = sJp[t];
                    pp.x = __fsub_rn(pp.x, jx); pp.y = __fsub_rn(pp.y, jy); pp.z = __fsub_rn(pp.z, jz);
                    sJp[t] = pp;
                }
            }
            __syncthreads();

            const int nti = (ni + 31) >> 5;
            const int S = (nj + 7) >> 3;                         /* j-steps of 8 */
            if constexpr (PRUNE) {
            /* boxes: each group of 4 i (4 lanes of a warp, one group per register slot), and a
             * thread each step.  A group with no particle keeps an empty box (lower > upper), whose
             * test below fails. */
            for (int ti = warp; ti < nti; ti += FW) {
                const int il = ti * 32 + lane;
                float lx = 3.0e38f, ly = 3.0e38f, lz = 3.0e38f, ux = -3.0e38f, uy = -3.0e38f, uz = -3.0e38f;
                if (il < ni) {
                    const float4 pp = sIp[il];
                    lx = ux = pp.x; ly = uy = pp.y; lz = uz = pp.z;
                }
#pragma unroll
                for (int o = 1; o < 4; o <<= 1) {
                    lx = fminf(lx, __shfl_xor_sync(0xffffffffu, lx, o));
                    ly = fminf(ly, __shfl_xor_sync(0xffffffffu, ly, o));
                    lz = fminf(lz, __shfl_xor_sync(0xffffffffu, lz, o));
                    ux = fmaxf(ux, __shfl_xor_sync(0xffffffffu, ux, o));
                    uy = fmaxf(uy, __shfl_xor_sync(0xffffffffu, uy, o));
                    uz = fmaxf(uz, __shfl_xor_sync(0xffffffffu, uz, o));
                }
                if ((lane & 3) == 0) {
                    const int gi = ti * 8 + (lane >> 2);
                    if (lx <= ux) {
                        /* the unit's shift folds into the centre: d = xi - xj + s */
                        const bool sh = MODE == kDiffShift;
                        s_gb[0][gi] = make_float4(0.5f * (lx + ux) + (sh ? sx : 0.0f), 0.5f * (ly + uy) + (sh ? sy : 0.0f),
                                                  0.5f * (lz + uz) + (sh ? sz : 0.0f), 0.0f);
                        s_gb[1][gi] = make_float4(0.5f * (ux - lx) + margin, 0.5f * (uy - ly) + margin,
                                                  0.5f * (uz - lz) + margin, 0.0f);
                    } else {
                        s_gb[0][gi] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
                        s_gb[1][gi] = make_float4(-1.0f, 0.0f, 0.0f, 0.0f);   /* empty: never kept */
                    }
                }
            }
            for (int st = tid; st < S; st += FW * 32) {
                float lx = 3.0e38f, ly = 3.0e38f, lz = 3.0e38f, ux = -3.0e38f, uy = -3.0e38f, uz = -3.0e38f;
                for (int u = 0; u < 8 && 8 * st + u < nj; ++u) {
                    const float4 pp = sJp[8 * st + u];
                    lx = fminf(lx, pp.x); ly = fminf(ly, pp.y); lz = fminf(lz, pp.z);
                    ux = fmaxf(ux, pp.x); uy = fmaxf(uy, pp.y); uz = fmaxf(uz, pp.z);
                }
                s_sb[0][st] = make_float4(0.5f * (lx + ux), 0.5f * (ly + uy), 0.5f * (lz + uz), 0.0f);
                s_sb[1][st] = make_float4(0.5f * (ux - lx), 0.5f * (uy - ly), 0.5f * (uz - lz), 0.0f);
            }
            __syncthreads();
            /* live-group mask of pair q = ti * S + st (steps before 4 ti are the diagonal's lower half) */
            for (int q = tid; q < nti * S; q += FW * 32) {
                const int ti = q / S, st = q - ti * S;
                unsigned km = 0;
                if (!diag || st >= 4 * ti) {
                    const float4 jc = s_sb[0][st], jh = s_sb[1][st];
#pragma unroll
                    for (int k = 0; k < 8; ++k) {
                        const float4 tc = s_gb[0][ti * 8 + k], th = s_gb[1][ti * 8 + k];
                        float ex = tc.x - jc.x, ey = tc.y - jc.y, ez = tc.z - jc.z;
                        if (MODE == kDiffWrap) {
                            ex = wrap_d(ex, g.L[0], g.h[0]); ey = wrap_d(ey, g.L[1], g.h[1]); ez = wrap_d(ez, g.L[2], g.h[2]);
                        }
                        const float gx = fmaxf(fabsf(ex) - (th.x + jh.x), 0.0f);
                        const float gy = fmaxf(fabsf(ey) - (th.y + jh.y), 0.0f);
                        const float gz = fmaxf(fabsf(ez) - (th.z + jh.z), 0.0f);
                        if (th.x >= 0.0f && gx * gx + gy * gy + gz * gz <= g.rc2) km |= 1u << k;
                    }
                }
                s_km[ti][st] = (unsigned char)km;
            }
            __syncthreads();
            for (int ti = tid; ti < nti; ti += FW * 32) {
                int c = 0;
                for (int st = 0; st < S; ++st) {
                    const unsigned char km = s_km[ti][st];
                    if (km) { s_list[ti][c] = (unsigned char)st; s_klist[ti][c] = km; ++c; }
                }
                s_nsurv[ti] = c;
            }
            __syncthreads();
            }
            /* pieces: runs of spp steps of one tile -- its surviving steps, or without pruning the
             * steps [first, S) with first = 4 ti on the diagonal */
            int npieces = 0;
            for (int ti = 0; ti < nti; ++ti)
                npieces += ((prune ? s_nsurv[ti] : S - (diag ? 4 * ti : 0)) + spp - 1) / spp;
            for (int p = warp; p < npieces; p += FW) {
                int ti = 0, r = p, nst = 0;
                for (;; ++ti) {
                    nst = prune ? s_nsurv[ti] : S - (diag ? 4 * ti : 0);
                    const int cnt = (nst + spp - 1) / spp;
                    if (r < cnt) break;
                    r -= cnt;
                }
                const int base = prune ? 0 : (diag ? 4 * ti : 0);
                const int k0 = r * spp;
                const int k1 = min(nst, k0 + spp);
                float xi[8], yi[8], zi[8], qi[8];
                int tti[8];
#pragma unroll
                for (int k = 0; k < 8; ++k) {
                    const int il = ti * 32 + row + 4 * k;
                    if (il < ni) {
                        const float4 pp = sIp[il];
                        xi[k] = pp.x; yi[k] = pp.y; zi[k] = pp.z;
                        qi[k] = __fmul_rn(ke, pp.w);
                        tti[k] = sIt[il] * ntypes;
                    } else {
                        xi[k] = far; yi[k] = far; zi[k] = far; qi[k] = 0.0f; tti[k] = 0;
                    }
                }
                float fi[24];
#pragma unroll
                for (int t = 0; t < 24; ++t) fi[t] = 0.0f;
                int ci[8] = {0, 0, 0, 0, 0, 0, 0, 0};
                bool piece_hit = false;   /* this lane accepted a pair in the piece */
                for (int kk = k0; kk < k1; ++kk) {
                    const int jl = (prune ? (int)s_list[ti][kk] : base + kk) * 8 + col;
                    const unsigned live = prune ? (unsigned)s_klist[ti][kk] : 0xffu;   /* warp-uniform */
                    float xj = -far, yj = -far, zj = -far, qj = 0.0f;
                    int ttj = 0;
                    if (jl < nj) {
                        const float4 pp = sJp[jl];
                        xj = pp.x; yj = pp.y; zj = pp.z; qj = pp.w;
                        ttj = sJt[jl];
                    }
                    float fjx = 0.f, fjy = 0.f, fjz = 0.f;
                    int cj = 0;
                    bool hit = false;     /* this lane accepted a pair in the step */
#pragma unroll
                    for (int k = 0; k < 8; ++k) {
                        if (prune && !((live >> k) & 1u)) continue;
                        const float dx = pair_diff<MODE>(xi[k], xj, g.L[0], g.h[0], sx);
                        const float dy = pair_diff<MODE>(yi[k], yj, g.L[1], g.h[1], sy);
                        const float dz = pair_diff<MODE>(zi[k], zj, g.L[2], g.h[2], sz);
                        const float r2 = __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)),
                                                   __fmul_rn(dz, dz));
                        bool ok = (r2 > 0.0f) && (r2 <= g.rc2);
                        if (diag) ok = ok && (ti * 32 + row + 4 * k < jl);
                        if (ok) {
                            float v14, v8, v3, v12, v6, v1;
                            pair_functions_fast<ORDER, SEP, EXTRA>(tab, r2, coul, v14, v8, v3, v12, v6, v1);
                            const float4 pc = sCoef[tti[k] + ttj];
                            const float qq = __fmul_rn(qi[k], qj);
                            const float fs = combine_force<SEP>(pc, qq, coul, v14, v8, v3);
                            const float fx = __fmul_rn(fs, dx), fy = __fmul_rn(fs, dy), fz = __fmul_rn(fs, dz);
                            fi[3 * k] += fx; fi[3 * k + 1] += fy; fi[3 * k + 2] += fz;
                            fjx -= fx; fjy -= fy; fjz -= fz;
                            hit = true;
                            ++acc_pairs;
                            if (EXTRA) {
                                ++ci[k];
                                ++cj;
                                acc_below += (ORDER > 0 && r2 < tab.r2min) ? 1u : 0u;
                                acc_elj += combine_elj<SEP>(pc, v12, v6);
                                if (coul) acc_ec += __fmul_rn(qq, v1);
                                acc_vir += __fmul_rn(fs, r2);
                            }
                        }
                    }
                    /* a step in which no lane accepted a pair adds nothing: without pruning, skip
                     * its reduction (with pruning nearly every surviving step has a pair, and the
                     * vote costs more than it saves) */
                    if (PRUNE || __any_sync(0xffffffffu, hit)) {
                        piece_hit = piece_hit || hit;
#pragma unroll
                        for (int o = 8; o < 32; o <<= 1) {
                            fjx += __shfl_xor_sync(0xffffffffu, fjx, o);
                            fjy += __shfl_xor_sync(0xffffffffu, fjy, o);
                            fjz += __shfl_xor_sync(0xffffffffu, fjz, o);
                            if (EXTRA) cj += __shfl_xor_sync(0xffffffffu, cj, o);
                        }
                        if (row == 0 && jl < nj) {
                            wFj[jl] += fjx;
                            wFj[kChunk + jl] += fjy;
                            wFj[2 * kChunk + jl] += fjz;
                            if (EXTRA) wCj[jl] += cj;
                        }
                    }
                }
                if (PRUNE || __any_sync(0xffffffffu, piece_hit)) {
                    reduce_scatter24(fi, col);
                    int cnt_i = 0;
                    if (EXTRA) cnt_i = reduce_scatter8i(ci, col);
                    const int il = ti * 32 + row + 4 * col;
                    if (il < ni) {
                        wFi[il] += fi[0];
                        wFi[kChunk + il] += fi[1];
                        wFi[2 * kChunk + il] += fi[2];
                        if (EXTRA) wCi[il] += cnt_i;
                    }
                }
            }
            __syncthreads();
            /* sum the warp accumulators in warp order; one atomic per particle and component */
            for (int t = tid; t < ni; t += (FW * 32)) {
                float v0 = 0.f, v1 = 0.f, v2 = 0.f;
                int cc = 0;
#pragma unroll
                for (int w = 0; w < FW; ++w) {
                    const float *a = sF + w * 6 * kChunk;
                    v0 += a[t]; v1 += a[kChunk + t]; v2 += a[2 * kChunk + t];
                    if (diag) { v0 += a[3 * kChunk + t]; v1 += a[4 * kChunk + t]; v2 += a[5 * kChunk + t]; }
                    if (EXTRA) cc += sC[w * 2 * kChunk + t] + (diag ? sC[w * 2 * kChunk + kChunk + t] : 0);
                }
                flush_force<ACC>(F64, F32, n, hs + i0 + t, v0, v1, v2, err);
                if (EXTRA && cc) atomicAdd(counts + hs + i0 + t, cc);
            }
            if (!diag) {
                for (int t = tid; t < nj; t += (FW * 32)) {
                    float v0 = 0.f, v1 = 0.f, v2 = 0.f;
                    int cc = 0;
#pragma unroll
                    for (int w = 0; w < FW; ++w) {
                        const float *a = sF + w * 6 * kChunk + 3 * kChunk;
                        v0 += a[t]; v1 += a[kChunk + t]; v2 += a[2 * kChunk + t];
                        if (EXTRA) cc += sC[w * 2 * kChunk + kChunk + t];
                    }
                    flush_force<ACC>(F64, F32, n, cs + j0 + t, v0, v1, v2, err);
                    if (EXTRA && cc) atomicAdd(counts + cs + j0 + t, cc);
                }
            }
        }
    }

    double e1 = acc_elj, e2 = acc_ec, e3 = acc_vir;
    unsigned long long c1 = acc_pairs, c2 = acc_below;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        c1 += __shfl_xor_sync(0xffffffffu, c1, o);
        if (EXTRA) {
            e1 += __shfl_xor_sync(0xffffffffu, e1, o);
            e2 += __shfl_xor_sync(0xffffffffu, e2, o);
            e3 += __shfl_xor_sync(0xffffffffu, e3, o);
            c2 += __shfl_xor_sync(0xffffffffu, c2, o);
        }
    }
    if (lane == 0) {
        s_red[warp][0] = e1; s_red[warp][1] = e2; s_red[warp][2] = e3;
        s_cnt[warp][0] = c1; s_cnt[warp][1] = c2;
    }
    __syncthreads();
    if (tid == 0) {
        UnitOut u;
        u.e_lj = u.e_coul = u.virial = 0.0;
        u.pairs = u.below = 0ull;
        for (int w = 0; w < FW; ++w) {
            u.e_lj += s_red[w][0]; u.e_coul += s_red[w][1]; u.virial += s_red[w][2];
            u.pairs += s_cnt[w][0]; u.below += s_cnt[w][1];
        }
        uout[blockIdx.x] = u;
    }
}

/* DIFF: the difference rule of half-shell units (kDiffShift, or kDiffExact for
 * MDRL_FLAG_EXACT_DIFF); batches pick the per-pair wrap for explicit cell pairs per item. */
template <int ORDER, bool SEP, bool EXTRA, int ACC, int DIFF, bool BATCH = false, int FW = kFW, bool PRUNE = false>
__global__ void __launch_bounds__(FW * 32, (FW == kFW ? kFCtas : 16 / FW))
k_force(const float4 *__restrict__ pos, const int *__restrict__ ptype,
        const int *__restrict__ cstart, Geom gparam, TableDev tab, const float4 *__restrict__ pcoef,
        int ntypes, float ke, int n, unsigned long long *__restrict__ F64,
        float *__restrict__ F32, int *__restrict__ counts, UnitOut *__restrict__ uout,
        const BatchItem *__restrict__ items, const BatchRep *__restrict__ reps, int tilecfg,
        unsigned *__restrict__ err, int unit0) {
    extern __shared__ float4 smem[];
    float4 *sIp = smem;
    float4 *sJp = sIp + kChunk;
    float4 *sCoef = sJp + kChunk;
    int *sIt = reinterpret_cast<int *>(sCoef + ntypes * ntypes);
    int *sJt = sIt + kChunk;
    float *sF = reinterpret_cast<float *>(sJt + kChunk);             /* [FW][2][3][kChunk] */
    int *sC = reinterpret_cast<int *>(sF + FW * 6 * kChunk);       /* [FW][2][kChunk] */
    __shared__ double s_red[FW][3];
    __shared__ unsigned long long s_cnt[FW][2];

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    int unit = blockIdx.x + unit0, coff = 0;   /* unit0: first unit of a restricted home range */
    bool cell_pair = false, use_wrap = false;
    Geom gb;
    if (BATCH) {
        const BatchItem it = items[blockIdx.x];
        const BatchRep rp = reps[it.rep];
        if (rp.path == kPathAllImages) {
            for (int t = tid; t < ntypes * ntypes; t += (FW * 32)) sCoef[t] = pcoef[t];
            float e1 = 0.f, e2 = 0.f, e3 = 0.f;
            unsigned c1 = 0, c2 = 0;
            all_images_body<ORDER, SEP, EXTRA, FW>(pos, ptype, rp, it.unit, tab, sCoef, ntypes, ke, n, F64, counts,
                                                  sJp, sJt, e1, e2, e3, c1, c2, err);
            double d1 = e1, d2 = e2, d3 = e3;
            unsigned long long u1 = c1, u2 = c2;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                u1 += __shfl_xor_sync(0xffffffffu, u1, o);
                if (EXTRA) {
                    d1 += __shfl_xor_sync(0xffffffffu, d1, o);
                    d2 += __shfl_xor_sync(0xffffffffu, d2, o);
                    d3 += __shfl_xor_sync(0xffffffffu, d3, o);
                    u2 += __shfl_xor_sync(0xffffffffu, u2, o);
                }
            }
            if (lane == 0) {
                s_red[warp][0] = d1; s_red[warp][1] = d2; s_red[warp][2] = d3;
                s_cnt[warp][0] = u1; s_cnt[warp][1] = u2;
            }
            __syncthreads();
            if (tid == 0) {
                UnitOut u;
                u.e_lj = u.e_coul = u.virial = 0.0;
                u.pairs = u.below = 0ull;
                for (int w = 0; w < FW; ++w) {
                    u.e_lj += s_red[w][0]; u.e_coul += s_red[w][1]; u.virial += s_red[w][2];
                    u.pairs += s_cnt[w][0]; u.below += s_cnt[w][1];
                }
                uout[blockIdx.x] = u;
            }
            return;
        }
        gb = rp.g;
        unit = it.unit;
        coff = rp.cell_off;
        cell_pair = rp.path == kPathMinImage;
        /* half-shell items take the per-unit shift (exact for every pair that can pass the
         * filter, see the header); explicit cell pairs wrap per pair */
        use_wrap = cell_pair;
    }
    const Geom &g = BATCH ? gb : gparam;
    int h, c;
    bool self;
    float sx = 0.0f, sy = 0.0f, sz = 0.0f;
    if (BATCH && cell_pair) {
        /* an explicit pair of the replica's cells, every pair with the per-pair minimum image */
        const int nct = g.nc[0] * g.nc[1] * g.nc[2];
        h = unit / nct;
        c = unit - h * nct;
        self = h == c;
    } else {
        h = unit / kHalfShellCells;
        const int f = unit - h * kHalfShellCells;
        const int nyz = g.nc[1] * g.nc[2];
        const int hx = h / nyz, hy = (h / g.nc[2]) % g.nc[1], hz = h % g.nc[2];
        int cx = hx + c_halfshell[f][0], cy = hy + c_halfshell[f][1], cz = hz + c_halfshell[f][2];
        /* neighbour across the +L face: its particles sit at x + L, so d = xi - xj - L */
        sx = cx >= g.nc[0] ? -g.L[0] : (cx < 0 ? g.L[0] : 0.0f);
        sy = cy >= g.nc[1] ? -g.L[1] : (cy < 0 ? g.L[1] : 0.0f);
        sz = cz >= g.nc[2] ? -g.L[2] : (cz < 0 ? g.L[2] : 0.0f);
        cx = cx < 0 ? cx + g.nc[0] : (cx >= g.nc[0] ? cx - g.nc[0] : cx);
        cy = cy < 0 ? cy + g.nc[1] : (cy >= g.nc[1] ? cy - g.nc[1] : cy);
        cz = cz < 0 ? cz + g.nc[2] : (cz >= g.nc[2] ? cz - g.nc[2] : cz);
        c = (cx * g.nc[1] + cy) * g.nc[2] + cz;
        self = (f == 0);
    }
    const int hs = cstart[coff + h], ni_all = cstart[coff + h + 1] - hs;
    const int cs = cstart[coff + c], nj_all = cstart[coff + c + 1] - cs;
    if (ni_all > kMaxCellOcc || nj_all > kMaxCellOcc) {
        /* an overflowing cell (reported by the in-cell sort): skip the unit, bounded time */
        if (tid == 0) {
            UnitOut u;
            u.e_lj = u.e_coul = u.virial = 0.0;
            u.pairs = u.below = 0ull;
            uout[blockIdx.x] = u;
        }
        return;
    }
#define MDRL_UNIT_ARGS pos, ptype, hs, ni_all, cs, nj_all, self, g, sx, sy, sz, tab, pcoef, ntypes, ke, n, F64, F32, \
                       counts, uout, sIp, sJp, sCoef, sIt, sJt, sF, sC, s_red, s_cnt, tilecfg, err
    /* one unit body per kernel where the rule is fixed (a second body cost more in instruction
     * fetch than a skipped add saves); the batch picks per item */
    if (BATCH && use_wrap)
        force_unit<ORDER, SEP, EXTRA, ACC, kDiffWrap, FW, PRUNE>(MDRL_UNIT_ARGS);
    else
        force_unit<ORDER, SEP, EXTRA, ACC, DIFF, FW, PRUNE>(MDRL_UNIT_ARGS);
#undef MDRL_UNIT_ARGS
}

/* ---- instantiation sets ----------------------------------------------------------------------
 * Each set is instantiated explicitly in one translation unit (mdrl_force_*.cu), so the sets
 * compile in parallel; everywhere else the declarations below keep them from being instantiated. */
/* One set: every order x extra (x arithmetic mode for the reference's difference rule; the exact
 * rule is instantiated with fused arithmetic only). */
template <int ACC, int FW, bool PRUNE, int DIFF>
force_fn pick_force_set(int order, bool sep, bool extra) {
    auto w = [&](auto ord, auto sp, auto ex) -> force_fn {
        constexpr int O = decltype(ord)::value;
        constexpr bool S = decltype(sp)::value, E = decltype(ex)::value;
        return (force_fn)k_force<O, S, E, ACC, DIFF, false, FW, PRUNE>;
    };
    auto se = [&](auto ord) -> force_fn {
        using T = std::true_type;
        using F = std::false_type;
        if (DIFF == kDiffShift && sep) return extra ? w(ord, T{}, T{}) : w(ord, T{}, F{});
        return extra ? w(ord, F{}, T{}) : w(ord, F{}, F{});
    };
    switch (order) {
        case 0: return se(std::integral_constant<int, 0>{});
        case 1: return se(std::integral_constant<int, 1>{});
        case 2: return se(std::integral_constant<int, 2>{});
        default: return se(std::integral_constant<int, 3>{});
    }
}

template <bool PRUNE>
force_fn pick_batch_set(int order, bool sep, bool extra) {
    auto w = [&](auto ord, auto sp, auto ex) -> force_fn {
        constexpr int O = decltype(ord)::value;
        constexpr bool S = decltype(sp)::value, E = decltype(ex)::value;
        return (force_fn)k_force<O, S, E, 0, kDiffShift, true, kBatchFT / 32, PRUNE>;
    };
    auto se = [&](auto ord) -> force_fn {
        using T = std::true_type;
        using F = std::false_type;
        if (sep) return extra ? w(ord, T{}, T{}) : w(ord, T{}, F{});
        return extra ? w(ord, F{}, T{}) : w(ord, F{}, F{});
    };
    switch (order) {
        case 0: return se(std::integral_constant<int, 0>{});
        case 1: return se(std::integral_constant<int, 1>{});
        case 2: return se(std::integral_constant<int, 2>{});
        default: return se(std::integral_constant<int, 3>{});
    }
}

extern template force_fn pick_force_set<0, 4, false, kDiffShift>(int, bool, bool);
extern template force_fn pick_force_set<0, 4, true, kDiffShift>(int, bool, bool);
extern template force_fn pick_force_set<0, 8, false, kDiffShift>(int, bool, bool);
extern template force_fn pick_force_set<0, 8, true, kDiffShift>(int, bool, bool);
extern template force_fn pick_force_set<1, 4, false, kDiffShift>(int, bool, bool);
extern template force_fn pick_force_set<2, 4, false, kDiffShift>(int, bool, bool);
extern template force_fn pick_force_set<0, 4, false, kDiffExact>(int, bool, bool);
extern template force_fn pick_force_set<0, 4, true, kDiffExact>(int, bool, bool);
extern template force_fn pick_force_set<0, 8, false, kDiffExact>(int, bool, bool);
extern template force_fn pick_force_set<0, 8, true, kDiffExact>(int, bool, bool);
extern template force_fn pick_force_set<1, 4, false, kDiffExact>(int, bool, bool);
extern template force_fn pick_force_set<2, 4, false, kDiffExact>(int, bool, bool);
extern template force_fn pick_batch_set<false>(int, bool, bool);
extern template force_fn pick_batch_set<true>(int, bool, bool);

}  // namespace mdrl
