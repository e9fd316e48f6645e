/*
 * mdrl_force_warp.cuh — the half-shell pair-force kernel with one warp per work item (sm_103a).
 *
 * Work item = (unit, i-tile group): a unit is (home cell h, half-shell neighbour f) as in
 * mdrl_force.cuh (the reference's pair set, SC/Particle_Pair_Gen_HalfShell.v:14-24); the home
 * cell's particles are cut into i-tiles of 32, and group g of G takes tiles g, g + G, g + 2G, ...
 * Each CTA is a single warp and owns its item alone: there is no staging into shared memory and
 * no barrier.  The warp
 *   1. computes the bounding box of each 8-particle j-step of the neighbour cell (one lane per
 *      step, straight from the cell-sorted positions in global memory, L1-resident);
 *   2. per i-tile: loads the tile's 32 i-particles into registers (lane = row * 8 + col holds
 *      i = row + 4k, k < 8, as in mdrl_force.cuh), boxes its eight 4-particle groups, tests every
 *      (group, step) pair with the same exact lower bound as the per-unit pre-pass of
 *      mdrl_force.cuh, and compacts the steps with a live group into a list (ballot + popc);
 *   3. runs the surviving steps: j = 8 * step + col is read from global memory, the 8 register
 *      slots whose group is live are filtered (0 < r2 <= rc2) and the accepted pairs evaluated
 *      with the same arithmetic as mdrl_force.cuh; the step's j forces are summed over the 4 rows
 *      (xor shuffles leave the sum on every row) and rows 0..2 add component x, y, z to the
 *      warp's j accumulator in shared memory, so one instruction covers the 24 values;
 *   4. reduce-scatters the i forces over the 8 columns at the end of the tile and adds them to the
 *      global accumulators (one atomic per particle and component), and at the end of the item
 *      adds the j accumulator (only particles that received a pair).
 * Deterministic: every FP32 partial sum has a fixed order (steps in list order, rows in a fixed
 * xor tree), the item decomposition does not depend on scheduling, and the int64 fixed-point
 * global sums are exact.
 *
 * Items are taken face-class first (self, the 3 face neighbours, 6 edges, 4 corners), so the
 * small corner units finish the launch.  For one system the grid is persistent: as many 32-thread
 * CTAs as fit on the GPU at once, each taking the next item from a counter (an atomic per item)
 * until none is left, so no slot waits for the block scheduler between items.  In a batch the
 * items are the half-shell units of the replicas with at least 3 cells per axis, from the batch's
 * cost-ordered list.
 *
 * L1 footprint.  The force table and the cells' particles are read through L1, which shares its
 * 256 KB with the shared memory of the 16 resident CTAs, so each CTA keeps only what it must in
 * shared memory (force multipliers as float2; energy multipliers and partner counts only in
 * energy launches) and order-2 rows are read from a packed 36-byte copy of the table: on the
 * 1M-atom system (16 types) this raised the L1 hit rate from 66 % to 91 %.
 */
#pragma once

#include "mdrl_force.cuh"

namespace mdrl {

constexpr int kWarpJChunk = 256;              /* j particles per chunk: 32 steps of 8 */
constexpr int kWarpJStride = kWarpJChunk + 8; /* row stride of the j accumulator (no bank conflicts) */
constexpr int kMaxItemGroups = 4;             /* i-tile groups per unit */

/* Half-shell offsets in launch order: self, faces, edges, corners (indices into c_halfshell). */
__constant__ int c_unit_order[kHalfShellCells] = {0, 1, 3, 9, 2, 4, 6, 8, 10, 12, 5, 7, 11, 13};

/* pair_functions_fast with the order-2 force coefficients read from the packed rows (36 bytes per
 * index instead of 48: a smaller L1 footprint); the same values and arithmetic. */
template <int ORDER, bool SEP, bool ENERGY>
__device__ __forceinline__ void pair_functions_packed(const TableDev &t, float r2, bool coul, float &v14,
                                                      float &v8, float &v3, float &v12, float &v6, float &v1) {
    if (ORDER != 2) {
        pair_functions_fast<ORDER, SEP, ENERGY>(t, r2, coul, v14, v8, v3, v12, v6, v1);
        return;
    }
    const float r2e = fmaxf(r2, t.r2min);
    const int idx = (int)(__float_as_uint(r2e) >> (23 - t.lb)) - ((127 + t.min_log2) << t.lb);
    const float x = table_variable(t, r2e);
    const float4 a = __ldg(t.fp2 + 2 * idx), b = __ldg(t.fp2 + 2 * idx + 1);
    v14 = madd<SEP>(madd<SEP>(a.z, x, a.y), x, a.x);
    v8 = madd<SEP>(madd<SEP>(b.y, x, b.x), x, a.w);
    v3 = coul ? madd<SEP>(madd<SEP>(__ldg(t.fc2 + idx), x, b.w), x, b.z) : 0.0f;
    if (ENERGY) {
        v12 = poly4<ORDER, SEP>(__ldg(t.e4 + 3 * idx), x);
        v6 = poly4<ORDER, SEP>(__ldg(t.e4 + 3 * idx + 1), x);
        v1 = coul ? poly4<ORDER, SEP>(__ldg(t.e4 + 3 * idx + 2), x) : 0.0f;
    }
}

/* Shared memory of one item's warp: (A14, B8) per type pair, and (A12, B6) with energies; the
 * step and group boxes; the j accumulator (and partner counts with EXTRA); the step list. */
inline size_t force_warp_smem_bytes(int ntypes, bool extra) {
    const size_t t2 = (size_t)((ntypes * ntypes + 1) & ~1);
    return sizeof(float2) * t2 * (extra ? 2 : 1) + sizeof(float4) * (2 * 32 + 2 * 8) +
           sizeof(float) * 3 * kWarpJStride + (extra ? sizeof(int) * kWarpJChunk : 0) + sizeof(unsigned) * 32;
}

/* The warp kernel's launch signature: force_fn plus the persistent grid's item counter (zero at
 * launch) and item count (work == nullptr: one item per CTA, blockIdx.x). */
typedef void (*warp_fn)(const float4 *, const int *, const int *, Geom, TableDev, const float4 *, int, float,
                        int, unsigned long long *, float *, int *, UnitOut *, const BatchItem *,
                        const BatchRep *, int, unsigned *, int, int *, int);

/* BATCH: the items are the half-shell units of a batch's replicas, items[b / G] (replica geometry
 * and cell offset from reps); otherwise every unit of one system, in launch order. */
template <int ORDER, bool SEP, bool EXTRA, int ACC, int MODE, bool BATCH = false>
__global__ void __launch_bounds__(32, 16)
k_force_warp(const float4 *__restrict__ pos, const int *__restrict__ ptype, const int *__restrict__ cstart,
             Geom gparam, TableDev tab, const float4 *__restrict__ pcoef, int ntypes, float ke, int n,
             unsigned long long *__restrict__ F64, float *__restrict__ F32, int *__restrict__ counts,
             UnitOut *__restrict__ uout, const BatchItem *__restrict__ items, const BatchRep *__restrict__ reps,
             int tilecfg, unsigned *__restrict__ err, int unit0, int *__restrict__ work, int nitems) {
    constexpr int nst = kWarpJChunk / 8;                        /* steps per chunk */
    const int t2 = (ntypes * ntypes + 1) & ~1;
    extern __shared__ float4 wsm[];
    float2 *sCoefF = reinterpret_cast<float2 *>(wsm);           /* (A14, B8) [T^2] */
    float2 *sCoefE = sCoefF + t2;                               /* (A12, B6) [T^2], EXTRA only */
    float4 *sSB = reinterpret_cast<float4 *>(sCoefE + (EXTRA ? t2 : 0));   /* step boxes: [2][nst] centre, half */
    float4 *sGB = sSB + 2 * nst;                                /* group boxes of the tile: [2][8] */
    float *sFj = reinterpret_cast<float *>(sGB + 2 * 8);        /* [3][kWarpJStride] */
    int *sCj = reinterpret_cast<int *>(sFj + 3 * kWarpJStride); /* [kWarpJChunk], EXTRA only */
    unsigned *sList = reinterpret_cast<unsigned *>(sCj + (EXTRA ? kWarpJChunk : 0));   /* [32] */

    const int lane = threadIdx.x, row = lane >> 3, col = lane & 7;
    const int G = tilecfg & 0xff;
    const bool coul = ke != 0.0f;
    const float far = 1.0e18f;

    /* item -> (home cell, half-shell neighbour, group).  One system: unit class position first,
     * then home cell, then group; unit0 is the first unit (home-major) of a restricted launch,
     * whose home cells are whole.  Batch: the listed unit of a replica, its cells from coff on;
     * with the per-pair wrap (MODE kDiffWrap) the unit is an explicit pair of the replica's cells
     * (a * cells + b, a <= b) of a box whose edges all exceed 2 rc. */
    constexpr bool kCellPair = BATCH && MODE == kDiffWrap;
    const int total = work ? nitems : (int)gridDim.x;
    int bfirst = blockIdx.x;
    if (work) {
        int t0 = 0;
        if (lane == 0) t0 = atomicAdd(work, 1);
        bfirst = __shfl_sync(0xffffffffu, t0, 0);
    }
    for (int b = bfirst; b < total;) {   /* one item per pass; one pass without a counter */
    int f = 0, h, grp, coff = 0, cpair = 0;
    Geom g;
    if (BATCH) {
        const BatchItem it = items[b / G];
        const BatchRep rp = reps[it.rep];
        g = rp.g;
        coff = rp.cell_off;
        grp = b - (b / G) * G;
        if (kCellPair) {
            const int nct = g.nc[0] * g.nc[1] * g.nc[2];
            h = it.unit / nct;
            cpair = it.unit - h * nct;
        } else {
            h = it.unit / kHalfShellCells;
            f = it.unit - h * kHalfShellCells;
        }
    } else {
        g = gparam;
        const int nh = total / (kHalfShellCells * G);
        const int fpos = b / (nh * G);
        const int rem = b - fpos * nh * G;
        const int hh = rem / G;
        grp = rem - hh * G;
        f = c_unit_order[fpos];
        h = unit0 / kHalfShellCells + hh;
    }

    const int nyz = g.nc[1] * g.nc[2];
    const int hx = h / nyz, hy = (h / g.nc[2]) % g.nc[1], hz = h % g.nc[2];
    int cx = hx + c_halfshell[f][0], cy = hy + c_halfshell[f][1], cz = hz + c_halfshell[f][2];
    /* the unit's periodic shift (none for explicit cell pairs, which wrap per pair) */
    const float sx = kCellPair ? 0.0f : (cx >= g.nc[0] ? -g.L[0] : (cx < 0 ? g.L[0] : 0.0f));
    const float sy = kCellPair ? 0.0f : (cy >= g.nc[1] ? -g.L[1] : (cy < 0 ? g.L[1] : 0.0f));
    const float sz = kCellPair ? 0.0f : (cz >= g.nc[2] ? -g.L[2] : (cz < 0 ? g.L[2] : 0.0f));
    cx = cx < 0 ? cx + g.nc[0] : (cx >= g.nc[0] ? cx - g.nc[0] : cx);
    cy = cy < 0 ? cy + g.nc[1] : (cy >= g.nc[1] ? cy - g.nc[1] : cy);
    cz = cz < 0 ? cz + g.nc[2] : (cz >= g.nc[2] ? cz - g.nc[2] : cz);
    const int c = kCellPair ? cpair : (cx * g.nc[1] + cy) * g.nc[2] + cz;
    const bool self = kCellPair ? (h == cpair) : (f == 0);
    const int hs = cstart[coff + h], ni_all = cstart[coff + h + 1] - hs;
    const int cs = cstart[coff + c], nj_all = cstart[coff + c + 1] - cs;

    float acc_elj = 0.0f, acc_ec = 0.0f, acc_vir = 0.0f;
    unsigned acc_pairs = 0, acc_below = 0;

    /* an overflowing cell (reported by the in-cell sort) skips the unit: bounded time */
    const bool skip = ni_all > kMaxCellOcc || nj_all > kMaxCellOcc || grp * 32 >= ni_all;
    /* exact rule: the box edge comes off the high side's coordinates (see pair_diff) */
    const float ix = (MODE == kDiffExact && sx < 0.0f) ? sx : 0.0f, iy = (MODE == kDiffExact && sy < 0.0f) ? sy : 0.0f,
                iz = (MODE == kDiffExact && sz < 0.0f) ? sz : 0.0f;
    const float jx = (MODE == kDiffExact && sx > 0.0f) ? sx : 0.0f, jy = (MODE == kDiffExact && sy > 0.0f) ? sy : 0.0f,
                jz = (MODE == kDiffExact && sz > 0.0f) ? sz : 0.0f;
    const float margin = 9.5367431640625e-07f * fmaxf(g.L[0], fmaxf(g.L[1], g.L[2]));

    if (!skip) {
        for (int t = lane; t < ntypes * ntypes; t += 32) {
            const float4 c4 = pcoef[t];
            sCoefF[t] = make_float2(c4.x, c4.y);
            if (EXTRA) sCoefE[t] = make_float2(c4.z, c4.w);
        }

        for (int j0 = 0; j0 < nj_all; j0 += kWarpJChunk) {
            const int nj = min(kWarpJChunk, nj_all - j0);
            const int S = (nj + 7) >> 3;
            if (self && j0 + nj <= grp * 32) continue;   /* every j below every i of the item */
            /* clear the j accumulator; box this lane's j-step */
            for (int t = lane; t < 3 * kWarpJStride; t += 32) sFj[t] = 0.0f;
            if (EXTRA)
                for (int t = lane; t < kWarpJChunk; t += 32) sCj[t] = 0;
            if (lane < S) {
                float lx = 3.0e38f, ly = 3.0e38f, lz = 3.0e38f, ux = -3.0e38f, uy = -3.0e38f, uz = -3.0e38f;
                for (int u = 0; u < 8 && 8 * lane + u < nj; ++u) {
                    float4 pp = __ldg(pos + cs + j0 + 8 * lane + u);
                    if (MODE == kDiffExact) { pp.x = __fsub_rn(pp.x, jx); pp.y = __fsub_rn(pp.y, jy); pp.z = __fsub_rn(pp.z, jz); }
                    lx = fminf(lx, pp.x); ly = fminf(ly, pp.y); lz = fminf(lz, pp.z);
                    ux = fmaxf(ux, pp.x); uy = fmaxf(uy, pp.y); uz = fmaxf(uz, pp.z);
                }
                sSB[lane] = make_float4(0.5f * (lx + ux), 0.5f * (ly + uy), 0.5f * (lz + uz), 0.0f);
                sSB[nst + lane] = make_float4(0.5f * (ux - lx), 0.5f * (uy - ly), 0.5f * (uz - lz), 0.0f);
            }
            __syncwarp();

            for (int ti = grp; ti * 32 < ni_all; ti += G) {
                const int i0 = ti * 32;
                if (self && j0 + nj <= i0) break;          /* later tiles are further past the chunk */
                /* the tile's 8 groups of 4 (i = i0 + 4k + row): boxes from global memory */
                if (lane < 8) {
                    float lx = 3.0e38f, ly = 3.0e38f, lz = 3.0e38f, ux = -3.0e38f, uy = -3.0e38f, uz = -3.0e38f;
                    for (int r = 0; r < 4; ++r) {
                        const int il = i0 + 4 * lane + r;
                        if (il < ni_all) {
                            float4 pp = __ldg(pos + hs + il);
                            if (MODE == kDiffExact) { pp.x = __fadd_rn(pp.x, ix); pp.y = __fadd_rn(pp.y, iy); pp.z = __fadd_rn(pp.z, iz); }
                            lx = fminf(lx, pp.x); ly = fminf(ly, pp.y); lz = fminf(lz, pp.z);
                            ux = fmaxf(ux, pp.x); uy = fmaxf(uy, pp.y); uz = fmaxf(uz, pp.z);
                        }
                    }
                    if (lx <= ux) {
                        const bool sh = MODE == kDiffShift;   /* the unit's shift folds into the centre */
                        sGB[lane] = make_float4(0.5f * (lx + ux) + (sh ? sx : 0.0f), 0.5f * (ly + uy) + (sh ? sy : 0.0f),
                                                0.5f * (lz + uz) + (sh ? sz : 0.0f), 0.0f);
                        sGB[8 + lane] = make_float4(0.5f * (ux - lx) + margin, 0.5f * (uy - ly) + margin,
                                                    0.5f * (uz - lz) + margin, 0.0f);
                    } else {
                        sGB[lane] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
                        sGB[8 + lane] = make_float4(-1.0f, 0.0f, 0.0f, 0.0f);   /* empty: never live */
                    }
                }
                __syncwarp();
                /* live-group mask of this lane's step; steps wholly below the tile on the diagonal
                 * of the self unit hold no pair i < j */
                unsigned km = 0;
                if (lane < S && !(self && j0 + 8 * lane + 7 <= i0)) {
                    const float4 jc = sSB[lane], jh = sSB[nst + lane];
#pragma unroll
                    for (int k = 0; k < 8; ++k) {
                        const float4 tc = sGB[k], th = sGB[8 + k];
                        float ex = tc.x - jc.x, ey = tc.y - jc.y, ez = tc.z - jc.z;
                        if (MODE == kDiffWrap) {   /* the centres' minimum image */
                            ex = wrap_d(ex, g.L[0], g.h[0]); ey = wrap_d(ey, g.L[1], g.h[1]); ez = wrap_d(ez, g.L[2], g.h[2]);
                        }
                        const float gx = fmaxf(fabsf(ex) - (th.x + jh.x), 0.0f);
                        const float gy = fmaxf(fabsf(ey) - (th.y + jh.y), 0.0f);
                        const float gz = fmaxf(fabsf(ez) - (th.z + jh.z), 0.0f);
                        if (th.x >= 0.0f && gx * gx + gy * gy + gz * gz <= g.rc2) km |= 1u << k;
                    }
                }
                const unsigned ball = __ballot_sync(0xffffffffu, km != 0);
                if (km) sList[__popc(ball & ((1u << lane) - 1u))] = (unsigned)lane | (km << 8);
                const int nsurv = __popc(ball);
                __syncwarp();

                float xi[8], yi[8], zi[8], qi[8];
                int tti[8];
#pragma unroll
                for (int k = 0; k < 8; ++k) {
                    const int il = i0 + row + 4 * k;
                    if (il < ni_all) {
                        float4 pp = __ldg(pos + hs + il);
                        if (MODE == kDiffExact) { pp.x = __fadd_rn(pp.x, ix); pp.y = __fadd_rn(pp.y, iy); pp.z = __fadd_rn(pp.z, iz); }
                        xi[k] = pp.x; yi[k] = pp.y; zi[k] = pp.z;
                        qi[k] = __fmul_rn(ke, pp.w);
                        tti[k] = __ldg(ptype + hs + il) * ntypes;
                    } else {
                        xi[k] = far; yi[k] = far; zi[k] = far; qi[k] = 0.0f; tti[k] = 0;
                    }
                }
                float fi[24];
#pragma unroll
                for (int t = 0; t < 24; ++t) fi[t] = 0.0f;
                int ci[8] = {0, 0, 0, 0, 0, 0, 0, 0};

                for (int p = 0; p < nsurv; ++p) {
                    const unsigned e = sList[p];
                    const int st = (int)(e & 31u);
                    const unsigned live = e >> 8;                       /* warp-uniform */
                    const int jl = 8 * st + col;                        /* in the chunk */
                    const int jidx = j0 + jl;                           /* in the cell */
                    /* diagonal steps of the self unit need i < j per candidate */
                    const int jthr = (self && j0 + 8 * st < i0 + 32) ? jidx : 0x7fffffff;
                    float xj = -far, yj = -far, zj = -far, qj = 0.0f;
                    int ttj = 0;
                    if (jl < nj) {
                        float4 pp = __ldg(pos + cs + jidx);
                        if (MODE == kDiffExact) { pp.x = __fsub_rn(pp.x, jx); pp.y = __fsub_rn(pp.y, jy); pp.z = __fsub_rn(pp.z, jz); }
                        xj = pp.x; yj = pp.y; zj = pp.z; qj = pp.w;
                        ttj = __ldg(ptype + cs + jidx);
                    }
                    float fjx = 0.f, fjy = 0.f, fjz = 0.f;
                    int cj = 0;
#pragma unroll
                    for (int k = 0; k < 8; ++k) {
                        if (!((live >> k) & 1u)) continue;
                        const float dx = pair_diff<MODE>(xi[k], xj, g.L[0], g.h[0], sx);
                        const float dy = pair_diff<MODE>(yi[k], yj, g.L[1], g.h[1], sy);
                        const float dz = pair_diff<MODE>(zi[k], zj, g.L[2], g.h[2], sz);
                        const float r2 = __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
                        const bool ok = (r2 > 0.0f) && (r2 <= g.rc2) && (i0 + row + 4 * k < jthr);
                        if (ok) {
                            float v14, v8, v3, v12, v6, v1;
                            pair_functions_packed<ORDER, SEP, EXTRA>(tab, r2, coul, v14, v8, v3, v12, v6, v1);
                            const float2 pf = sCoefF[tti[k] + ttj];
                            const float4 pc = make_float4(pf.x, pf.y, 0.0f, 0.0f);
                            const float qq = __fmul_rn(qi[k], qj);
                            const float fs = combine_force<SEP>(pc, qq, coul, v14, v8, v3);
                            const float fx = __fmul_rn(fs, dx), fy = __fmul_rn(fs, dy), fz = __fmul_rn(fs, dz);
                            fi[3 * k] += fx; fi[3 * k + 1] += fy; fi[3 * k + 2] += fz;
                            fjx -= fx; fjy -= fy; fjz -= fz;
                            ++acc_pairs;
                            if (EXTRA) {
                                ++ci[k];
                                ++cj;
                                acc_below += (ORDER > 0 && r2 < tab.r2min) ? 1u : 0u;
                                const float2 pe = sCoefE[tti[k] + ttj];
                                acc_elj += combine_elj<SEP>(make_float4(0.0f, 0.0f, pe.x, pe.y), v12, v6);
                                if (coul) acc_ec += __fmul_rn(qq, v1);
                                acc_vir += __fmul_rn(fs, r2);
                            }
                        }
                    }
                    /* sum over the 4 rows: every row ends with the step's sums */
#pragma unroll
                    for (int o = 8; o < 32; o <<= 1) {
                        fjx += __shfl_xor_sync(0xffffffffu, fjx, o);
                        fjy += __shfl_xor_sync(0xffffffffu, fjy, o);
                        fjz += __shfl_xor_sync(0xffffffffu, fjz, o);
                        if (EXTRA) cj += __shfl_xor_sync(0xffffffffu, cj, o);
                    }
                    if (jl < nj) {
                        if (row < 3) sFj[row * kWarpJStride + jl] += row == 0 ? fjx : (row == 1 ? fjy : fjz);
                        else if (EXTRA) sCj[jl] += cj;
                    }
                }
                /* i forces: reduce-scatter over the columns, lane owns i = i0 + row + 4 col */
                reduce_scatter24(fi, col);
                int cnt_i = 0;
                if (EXTRA) cnt_i = reduce_scatter8i(ci, col);
                const int il = i0 + row + 4 * col;
                if (il < ni_all && nsurv > 0) {
                    flush_force<ACC>(F64, F32, n, hs + il, fi[0], fi[1], fi[2], err);
                    if (EXTRA && cnt_i) atomicAdd(counts + hs + il, cnt_i);
                }
                __syncwarp();
            }
            __syncwarp();
            /* j forces of the chunk: one atomic per particle and component that received a pair */
            for (int t = lane; t < nj; t += 32) {
                const float v0 = sFj[t], v1 = sFj[kWarpJStride + t], v2 = sFj[2 * kWarpJStride + t];
                if (v0 != 0.0f || v1 != 0.0f || v2 != 0.0f || !(v0 == v0 && v1 == v1 && v2 == v2))
                    flush_force<ACC>(F64, F32, n, cs + j0 + t, v0, v1, v2, err);
                if (EXTRA && sCj[t]) atomicAdd(counts + cs + j0 + t, sCj[t]);
            }
            __syncwarp();
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
        UnitOut u;
        u.e_lj = e1; u.e_coul = e2; u.virial = e3;
        u.pairs = c1; u.below = c2;
        uout[b] = u;
    }
    if (!work) break;
    __syncwarp();   /* this item's shared-memory reads are done before the next item writes */
    int t1 = 0;
    if (lane == 0) t1 = atomicAdd(work, 1);
    b = __shfl_sync(0xffffffffu, t1, 0);
    }
}

/* One set: every order x extra (x arithmetic mode for the reference's difference rule; the exact
 * rule is instantiated with fused arithmetic only). */
template <int ACC, int DIFF>
warp_fn pick_force_warp_set(int order, bool sep, bool extra) {
    auto w = [&](auto ord, auto sp, auto ex) -> warp_fn {
        constexpr int O = decltype(ord)::value;
        constexpr bool S = decltype(sp)::value, E = decltype(ex)::value;
        return k_force_warp<O, S, E, ACC, DIFF>;
    };
    auto se = [&](auto ord) -> warp_fn {
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

/* the batched-replica sets: half-shell replicas (per-unit shift), and explicit cell pairs of
 * replicas with fewer than 3 cells per axis but every edge above 2 rc (per-pair wrap) */
warp_fn pick_force_warp_batch(int order, bool sep, bool extra, bool cell_pairs);

extern template warp_fn pick_force_warp_set<0, kDiffShift>(int, bool, bool);
extern template warp_fn pick_force_warp_set<0, kDiffExact>(int, bool, bool);

}  // namespace mdrl
