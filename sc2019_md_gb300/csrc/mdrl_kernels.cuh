/*
 * mdrl_kernels.cuh — sm_103a kernels of the range-limited force path.
 *
 * Data layout in HBM (all particle arrays are in cell-sorted order after binning):
 *   pos   float4[n]  (x, y, z, q)        one 16-byte coalesced load per particle
 *   type  int[n]
 *   F     3 x int64[n] (SoA, 2^-24 kcal/mol/A fixed point) or 3 x float[n] (FP32-atomic mode)
 *   cell_start int[ncells + 1]           cell c holds sorted particles [start[c], start[c+1])
 *
 * Pair datapath, per candidate (the reference RTL order, SC/r2_compute_with_pbc.v:81-127,
 * SC/Filter_Logic.v:234, SC/RL_LJ_Evaluate_Pairs_1st_Order.v:179-193,409-468,
 * SC/RL_Evaluate_Pairs_1st_Order.v:325-395):
 *   d = x_ref - x_nbr, one conditional +-L wrap per axis;
 *   r2 = (dx*dx + dy*dy) + dz*dz, each operation rounded (the pair list is bit-identical to an
 *        all-pairs FP32 evaluation of the same positions);
 *   keep when 0 < r2 <= rc2;
 *   table index = (exponent(r2) - 127 - min_log2) * bins + top mantissa bits;
 *   v_k = c1*r2 + c0 (or Horner for orders 2-3), fscal = ((QQ*v3) + B*v8) + A*v14,
 *   f = fscal * d, added to i and subtracted from j (Newton's third law).
 */
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "mdrl_internal.h"

namespace mdrl {

/* Tables packed for the kernels: for order 1, per table index three float2 {c0, c1} (force:
 * r^-14, r^-8, r^-3; energy: r^-12, r^-6, r^-1); for orders 2-3, three float4 {c0..c3}.
 * Polynomial form: monomial in r2 (the reference's form: c0 + c1 r2 + ...), or, when `local`
 * is set (orders 2-3), in the bin-local variable u = r2 - b0, b0 the start of r2's bin.  u is
 * exact in FP32 (r2 and b0 share a binade and b0 <= r2 < 2 b0), so the local form carries no
 * cancellation between large monomial terms. */
struct TableDev {
    const float2 *f2, *e2;
    const float4 *f4, *e4;
    const float4 *fr;   /* order 1, force functions packed per index in one 32-byte sector:
                           {c0_14, c1_14, c0_8, c1_8}, {c0_3, c1_3, 0, 0} */
    const float4 *fp2;  /* order 2, the force functions' 9 coefficients without padding: per index
                           {c0_14, c1_14, c2_14, c0_8}, {c1_8, c2_8, c0_3, c1_3} ... */
    const float *fc2;   /* ... and c2_3 */
    int order, nseg, bins, lb, min_log2;
    float r2min;
    int local;          /* orders 2-3: coefficients in u = r2 - bin start */
};

/* The polynomial variable of an in-table r2e: r2e itself, or r2e minus its bin's start (the r2
 * bit pattern with the mantissa bits below the bin index cleared). */
__device__ __forceinline__ float table_variable(const TableDev &t, float r2e) {
    if (!t.local) return r2e;
    const float b0 = __uint_as_float(__float_as_uint(r2e) & ~((1u << (23 - t.lb)) - 1u));
    return __fsub_rn(r2e, b0);
}

/* The 14 cells of the half shell in the reference's filter order (mdrl_internal.h). */
__constant__ int c_halfshell[kHalfShellCells][3] = MDRL_HALFSHELL_OFFSETS;

/* Error bits raised by kernels and read by the host after a call.  kErrForce: a force sum that
 * the accumulators cannot hold -- NaN or infinite, or (int64 fixed point) a magnitude at or above
 * kFixMax, which the conversion would saturate. */
enum : unsigned { kErrPosition = 1u, kErrType = 2u, kErrForce = 4u, kErrCellOverflow = 8u };

/* Cell occupancy: cells up to kSortSmall particles are ordered in one shared-memory pass; larger
 * ones in sorted chunks of kSortSmall merged by binary search; above kMaxCellOcc a cell raises
 * kErrCellOverflow (MDRL_ERR_CELL_OVERFLOW), keeps its arrival order, and the force kernel skips
 * the units that touch it, so a pathological input costs bounded time. */
constexpr int kSortSmall = 1024;
constexpr int kMaxCellOcc = 65536;

/* The largest force (kcal/mol/A) a 2^-24 fixed-point component holds without saturating: the
 * conversion clamps at 9e18 units. */
constexpr float kFixMax = 9.0e18f / 16777216.0f;

/* Per-type mass factors, kept in device memory and read through a pointer (a by-value kernel
 * parameter indexed by a particle's type would be copied to local memory in every thread). */
struct MassTab {
    float cm[MDRL_MAX_TYPES];   /* velocity increment per unit force for the kick */
    float mass[MDRL_MAX_TYPES]; /* amu, for the kinetic energy */
};

__device__ __forceinline__ float wrap_d(float d, float L, float h) {
    return d > h ? __fsub_rn(d, L) : (d < -h ? __fadd_rn(d, L) : d);
}

/* The exact-difference rule per pair (MDRL_FLAG_EXACT_DIFF): the wrap direction from fl(xi - xj)
 * as above, then the box edge comes off the high coordinate (exact for coordinates in [0, L):
 * the one wrapped lies above L/2) and the difference is rounded once. */
__device__ __forceinline__ float wrap_exact(float xi, float xj, float L, float h) {
    const float d = __fsub_rn(xi, xj);
    if (d > h) return __fsub_rn(__fsub_rn(xi, L), xj);
    if (d < -h) return __fsub_rn(xi, __fsub_rn(xj, L));
    return d;
}

template <bool SEP>
__device__ __forceinline__ float madd(float a, float b, float c) {
    return SEP ? __fadd_rn(__fmul_rn(a, b), c) : __fmaf_rn(a, b, c);
}

__device__ __forceinline__ int table_index(const TableDev &t, float r2, float &r2e, int &below) {
    const unsigned b = __float_as_uint(r2);
    int seg = (int)(b >> 23) - 127 - t.min_log2;
    int bin = (int)((b >> (23 - t.lb)) & (unsigned)(t.bins - 1));
    r2e = r2;
    below = 0;
    if (seg < 0) {
        seg = 0; bin = 0; r2e = t.r2min; below = 1;
    } else if (seg >= t.nseg) {
        seg = t.nseg - 1; bin = t.bins - 1;
    }
    return seg * t.bins + bin;
}

template <int ORDER, bool SEP>
__device__ __forceinline__ float poly4(float4 c, float x) {
    float v = (ORDER >= 3) ? c.w : c.z;
    if (ORDER >= 3) v = madd<SEP>(v, x, c.z);
    v = madd<SEP>(v, x, c.y);
    return madd<SEP>(v, x, c.x);
}

/* The pair functions v14, v8, v3 (and v12, v6, v1 when ENERGY) at r2. */
template <int ORDER, bool SEP, bool ENERGY>
__device__ __forceinline__ void pair_functions(const TableDev &t, float r2, bool coul, float &v14,
                                               float &v8, float &v3, float &v12, float &v6,
                                               float &v1, int &below) {
    if (ORDER == 0) {
        const float i2 = __fdiv_rn(1.0f, r2);
        const float i4 = __fmul_rn(i2, i2), i6 = __fmul_rn(i4, i2), i8 = __fmul_rn(i4, i4);
        const float i12 = __fmul_rn(i6, i6), i14 = __fmul_rn(i12, i2);
        const float i1 = __fsqrt_rn(i2), i3 = __fmul_rn(i2, i1);
        v14 = i14; v8 = i8; v3 = i3; v12 = i12; v6 = i6; v1 = i1;
        below = 0;
        return;
    }
    float r2e;
    const int idx = table_index(t, r2, r2e, below);
    if (ORDER == 1) {
        const float2 a = __ldg(t.f2 + 3 * idx), b = __ldg(t.f2 + 3 * idx + 1);
        v14 = madd<SEP>(a.y, r2e, a.x);
        v8 = madd<SEP>(b.y, r2e, b.x);
        v3 = 0.0f;
        if (coul) { const float2 c = __ldg(t.f2 + 3 * idx + 2); v3 = madd<SEP>(c.y, r2e, c.x); }
        if (ENERGY) {
            const float2 d = __ldg(t.e2 + 3 * idx), e = __ldg(t.e2 + 3 * idx + 1);
            v12 = madd<SEP>(d.y, r2e, d.x);
            v6 = madd<SEP>(e.y, r2e, e.x);
            v1 = 0.0f;
            if (coul) { const float2 g = __ldg(t.e2 + 3 * idx + 2); v1 = madd<SEP>(g.y, r2e, g.x); }
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

/* fscal = ((QQ*v3) + B*v8) + A*v14 ; energies el = Be*v6 + Ae*v12, ec = QQ*v1. */
template <bool SEP>
__device__ __forceinline__ float combine_force(float4 pc, float qq, bool coul, float v14, float v8,
                                               float v3) {
    if (SEP) {
        float fs = __fmul_rn(pc.y, v8);
        if (coul) fs = __fadd_rn(__fmul_rn(qq, v3), fs);
        return __fadd_rn(fs, __fmul_rn(pc.x, v14));
    }
    const float fs = __fmaf_rn(pc.y, v8, coul ? __fmul_rn(qq, v3) : 0.0f);
    return __fmaf_rn(pc.x, v14, fs);
}

template <bool SEP>
__device__ __forceinline__ float combine_elj(float4 pc, float v12, float v6) {
    return SEP ? __fadd_rn(__fmul_rn(pc.w, v6), __fmul_rn(pc.z, v12))
               : __fmaf_rn(pc.z, v12, __fmul_rn(pc.w, v6));
}

/* 2^-24 fixed point.  NaN converts to 0 and magnitudes beyond kFixMax saturate; callers report
 * both through force_ok / kErrForce rather than let them pass silently. */
__device__ __forceinline__ unsigned long long to_fixed(float v) {
    float s = v * kFixScale;
    if (!(s == s)) s = 0.0f;
    s = fminf(fmaxf(s, -9.0e18f), 9.0e18f);
    return (unsigned long long)__float2ll_rn(s);
}

/* True when every component is finite and below kFixMax in magnitude (NaN fails the compare). */
__device__ __forceinline__ bool force_ok(float fx, float fy, float fz) {
    return fabsf(fx) < kFixMax && fabsf(fy) < kFixMax && fabsf(fz) < kFixMax;
}

/* Raise kErrForce when a force sum cannot be represented (one atomic per offending thread). */
__device__ __forceinline__ void check_force(unsigned *err, float fx, float fy, float fz) {
    if (!force_ok(fx, fy, fz) && err) atomicOr(err, kErrForce);
}

__device__ __forceinline__ float from_fixed(unsigned long long v) {
    return __ll2float_rn((long long)v) * kFixInv;
}

/* ------------------------------------------------------------------------------------------ */
/* Binning: cell = floor(pos / edge) (MS/GenInputCellList_LJArgon.m:98-112), stable within the
 * cell (input order, :114-121).  count -> scan -> scatter -> per-cell rank sort.              */

__device__ __forceinline__ int cell_coord(float v, float edge, int n) {
    const float f = floorf(__fdiv_rn(v, edge));
    if (!(f >= 0.0f)) return 0;
    if (f >= (float)n) return n - 1;
    return (int)f;
}

__device__ __forceinline__ int cell_of_pos(const Geom &g, float x, float y, float z) {
    const int cx = cell_coord(x, g.edge[0], g.nc[0]);
    const int cy = cell_coord(y, g.edge[1], g.nc[1]);
    const int cz = cell_coord(z, g.edge[2], g.nc[2]);
    return (cx * g.nc[1] + cy) * g.nc[2] + cz;
}

/* 30-bit Morton code of a position inside its cell (10 bits per axis): the in-cell sort key of
 * the force path.  Only an ordering, so its rounding does not matter; ties break on the index. */
__device__ __forceinline__ unsigned spread10(unsigned v) {
    v &= 0x3ffu;
    v = (v | (v << 16)) & 0x030000ffu;
    v = (v | (v << 8)) & 0x0300f00fu;
    v = (v | (v << 4)) & 0x030c30c3u;
    v = (v | (v << 2)) & 0x09249249u;
    return v;
}

__device__ __forceinline__ unsigned cell_morton(const Geom &g, float x, float y, float z, int c) {
    const int cz = c % g.nc[2], cy = (c / g.nc[2]) % g.nc[1], cx = c / (g.nc[1] * g.nc[2]);
    const float p[3] = {x, y, z};
    const int cc[3] = {cx, cy, cz};
    unsigned q[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        /* an ordering only: the fast reciprocal (deterministic) is as good as an IEEE division */
        const float loc = (p[d] - (float)cc[d] * g.edge[d]) * __fdividef(1024.0f, g.edge[d]);
        q[d] = (unsigned)min(1023, max(0, (int)loc));
    }
    return (spread10(q[0]) << 2) | (spread10(q[1]) << 1) | spread10(q[2]);
}

__device__ __forceinline__ bool in_box(const Geom &g, float x, float y, float z) {
    return x >= 0.0f && x < g.L[0] && y >= 0.0f && y < g.L[1] && z >= 0.0f && z < g.L[2];
}

/* Arrival slot of a particle in cell c: lanes of a warp that share c take consecutive slots with
 * one atomic per distinct cell (cell-sorted particles mostly share cells within a warp). */
__device__ __forceinline__ int cell_slot(int *count, int c) {
    const unsigned active = __activemask();
    const unsigned peers = __match_any_sync(active, c);
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(peers) - 1;
    const int rank = __popc(peers & ((1u << lane) - 1u));
    int base = 0;
    if (lane == leader) base = atomicAdd(count + c, __popc(peers));
    base = __shfl_sync(peers, base, leader);
    return base + rank;
}

/* Cell of each user-order particle, with its arrival slot in the cell.  With ux non-null the
 * user arrays (which may be pinned host memory read over the host link) are also copied, in
 * coalesced order, to device staging ux, uy, uz, uq (q given), ut (type given), so that the
 * gather that follows reads device memory. */
static __global__ void k_bin_user(int n, const float *__restrict__ x, const float *__restrict__ y,
                           const float *__restrict__ z, Geom g, int *__restrict__ cell_of,
                           int *__restrict__ slot, int *__restrict__ count,
                           unsigned *__restrict__ err, unsigned *__restrict__ key,
                           const float *__restrict__ q = nullptr, const int *__restrict__ type = nullptr,
                           float *__restrict__ ux = nullptr, float *__restrict__ uy = nullptr,
                           float *__restrict__ uz = nullptr, float *__restrict__ uq = nullptr,
                           int *__restrict__ ut = nullptr) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float px = x[i], py = y[i], pz = z[i];
    if (ux) {
        ux[i] = px; uy[i] = py; uz[i] = pz;
        if (q) uq[i] = q[i];
        if (type) ut[i] = type[i];
    }
    if (!in_box(g, px, py, pz)) atomicOr(err, kErrPosition);
    const int c = cell_of_pos(g, px, py, pz);
    cell_of[i] = c;
    if (key) key[i] = cell_morton(g, px, py, pz, c);
    slot[i] = cell_slot(count, c);
}

/* Exclusive scan of the cell counts (one CTA), plus the largest occupancy. */
static __global__ void __launch_bounds__(1024) k_scan(int ncells, const int *__restrict__ count,
                                               int *__restrict__ start, DevTotals *tot) {
    __shared__ int s_sum[1024];
    __shared__ int s_max[1024];
    const int t = threadIdx.x;
    const int per = (ncells + 1023) / 1024;
    const int b = t * per, e = min(ncells, b + per);
    int sum = 0, mx = 0;
    for (int k = b; k < e; ++k) { const int c = count[k]; sum += c; mx = max(mx, c); }
    s_sum[t] = sum;
    s_max[t] = mx;
    __syncthreads();
    for (int off = 1; off < 1024; off <<= 1) {
        const int v = (t >= off) ? s_sum[t - off] : 0;
        const int m = (t >= off) ? s_max[t - off] : 0;
        __syncthreads();
        s_sum[t] += v;
        s_max[t] = max(s_max[t], m);
        __syncthreads();
    }
    int run = s_sum[t] - sum;
    for (int k = b; k < e; ++k) { start[k] = run; run += count[k]; }
    if (t == 1023) { start[ncells] = s_sum[1023]; tot->max_occ = s_max[1023]; }
}

static __global__ void k_scatter(int n, const int *__restrict__ cell_of, const int *__restrict__ slot,
                          const int *__restrict__ start, int *__restrict__ tmp) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    tmp[start[cell_of[i]] + slot[i]] = i;
}

/* Order each cell's particles: by index (the reference's in-cell order, input order), or, when
 * key is given, by (key, index).  The rank of an element is the number of smaller ones (the
 * (key, index) pairs are distinct).  scratch[n] (64-bit) holds the sorted chunks of cells above
 * kSortSmall. */
static __global__ void __launch_bounds__(128) k_cell_sort(const int *__restrict__ start,
                                                          const int *__restrict__ tmp,
                                                          int *__restrict__ sorted,
                                                          const unsigned *__restrict__ key,
                                                          unsigned long long *__restrict__ scratch,
                                                          unsigned *__restrict__ err) {
    __shared__ __align__(16) unsigned long long s_k[kSortSmall];
    const int c = blockIdx.x;
    const int s = start[c], m = start[c + 1] - s;
    if (m == 0) return;
    if (m > kMaxCellOcc) {
        if (threadIdx.x == 0) atomicOr(err, kErrCellOverflow);
        for (int e = threadIdx.x; e < m; e += blockDim.x) sorted[s + e] = tmp[s + e];
        return;
    }
    if (m <= kSortSmall) {
        for (int e = threadIdx.x; e < m; e += blockDim.x) {
            const int id = tmp[s + e];
            s_k[e] = ((unsigned long long)(key ? key[id] : 0u) << 32) | (unsigned)id;
        }
        if ((m & 1) && threadIdx.x == 0) s_k[m] = ~0ull;     /* pad to an even count: never smaller */
        __syncthreads();
        const int m2 = (m + 1) >> 1;
        const ulonglong2 *s_k2 = reinterpret_cast<const ulonglong2 *>(s_k);
        for (int e = threadIdx.x; e < m; e += blockDim.x) {
            const unsigned long long me = s_k[e];
            /* rank = number of smaller keys; two keys per shared load, four independent counters */
            int r0 = 0, r1 = 0, r2 = 0, r3 = 0;
            int q = 0;
            for (; q + 1 < m2; q += 2) {
                const ulonglong2 a = s_k2[q], b = s_k2[q + 1];
                r0 += a.x < me; r1 += a.y < me; r2 += b.x < me; r3 += b.y < me;
            }
            if (q < m2) { const ulonglong2 a = s_k2[q]; r0 += a.x < me; r1 += a.y < me; }
            sorted[s + r0 + r1 + r2 + r3] = (int)(me & 0xffffffffu);
        }
        return;
    }
    /* large cell: sort each chunk of kSortSmall in shared memory (rank count) into scratch ... */
    for (int c0 = 0; c0 < m; c0 += kSortSmall) {
        const int mc = min(kSortSmall, m - c0);
        __syncthreads();
        for (int e = threadIdx.x; e < mc; e += blockDim.x) {
            const int id = tmp[s + c0 + e];
            s_k[e] = ((unsigned long long)(key ? key[id] : 0u) << 32) | (unsigned)id;
        }
        __syncthreads();
        for (int e = threadIdx.x; e < mc; e += blockDim.x) {
            const unsigned long long me = s_k[e];
            int r = 0;
            for (int q = 0; q < mc; ++q) r += s_k[q] < me;
            scratch[s + c0 + r] = me;
        }
    }
    __syncthreads();   /* the block's global writes are visible to the block after the barrier */
    /* ... then an element's rank = its rank in its chunk + the keys below it in every other chunk
     * (binary search: O(m log kSortSmall / kSortSmall) per element) */
    for (int e = threadIdx.x; e < m; e += blockDim.x) {
        const unsigned long long me = scratch[s + e];
        const int ce = e / kSortSmall;
        int r = e - ce * kSortSmall;
        for (int c0 = 0, cc = 0; c0 < m; c0 += kSortSmall, ++cc) {
            if (cc == ce) continue;
            const unsigned long long *a = scratch + s + c0;
            int lo = 0, hi = min(kSortSmall, m - c0);   /* first index with a[idx] >= me */
            while (lo < hi) {
                const int mid = (lo + hi) >> 1;
                if (a[mid] < me) lo = mid + 1; else hi = mid;
            }
            r += lo;
        }
        sorted[s + r] = (int)(me & 0xffffffffu);
    }
}

/* Gather user-order inputs into cell order and clear the force accumulators. */
static __global__ void k_gather_user(int n, const int *__restrict__ sorted, const float *__restrict__ x,
                              const float *__restrict__ y, const float *__restrict__ z,
                              const float *__restrict__ q, const int *__restrict__ type,
                              float4 *__restrict__ pos, int *__restrict__ ptype,
                              int *__restrict__ pid, unsigned long long *__restrict__ F64,
                              float *__restrict__ F32, int *__restrict__ counts, int ntypes,
                              unsigned *__restrict__ err, int *__restrict__ inv = nullptr) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const int id = sorted[k];
    if (inv) inv[id] = k;
    pos[k] = make_float4(x[id], y[id], z[id], q ? q[id] : 0.0f);
    int t = type ? type[id] : 0;
    if (t < 0 || t >= ntypes) { atomicOr(err, kErrType); t = 0; }
    ptype[k] = t;
    pid[k] = id;
    if (F64) { F64[k] = 0ull; F64[n + k] = 0ull; F64[2 * n + k] = 0ull; }
    if (F32) {
#pragma unroll
        for (int d = 0; d < 6; ++d) F32[(size_t)d * n + k] = 0.0f;   /* hi planes 0-2, lo planes 3-5 */
    }
    if (counts) counts[k] = 0;
}

/* Totals over units and kinetic-energy partials, in a fixed order (one CTA of 1024 threads:
 * strided partial sums, then warp shuffles and a final warp; the same order every call).  GB300
 * runs FP64 at a small fraction of its FP32 rate, so the FP64 energy sums run only when energies
 * were computed. */
static __global__ void __launch_bounds__(1024) k_totals(int nunits, const UnitOut *__restrict__ uout,
                                                        int nke, const double *__restrict__ kepart,
                                                        DevTotals *tot, int with_energy) {
    __shared__ double s_d[32][4];
    __shared__ unsigned long long s_u[32][2];
    const int t = threadIdx.x, lane = t & 31, w = t >> 5;
    double a = 0, b = 0, c = 0, k = 0;
    unsigned long long p = 0, q = 0;
    /* unrolled so that the loads of several slots are in flight at once (the sums keep their order) */
#pragma unroll 8
    for (int u = t; u < nunits; u += 1024) {
        p += uout[u].pairs;
        if (with_energy) {
            a += uout[u].e_lj; b += uout[u].e_coul; c += uout[u].virial;
            q += uout[u].below;
        }
    }
#pragma unroll 8
    for (int u = t; u < nke; u += 1024) k += kepart[u];
    const bool fp = with_energy || nke > 0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        p += __shfl_xor_sync(0xffffffffu, p, o);
        q += __shfl_xor_sync(0xffffffffu, q, o);
        if (fp) {
            a += __shfl_xor_sync(0xffffffffu, a, o);
            b += __shfl_xor_sync(0xffffffffu, b, o);
            c += __shfl_xor_sync(0xffffffffu, c, o);
            k += __shfl_xor_sync(0xffffffffu, k, o);
        }
    }
    if (lane == 0) { s_d[w][0] = a; s_d[w][1] = b; s_d[w][2] = c; s_d[w][3] = k; s_u[w][0] = p; s_u[w][1] = q; }
    __syncthreads();
    if (w != 0) return;
    a = s_d[lane][0]; b = s_d[lane][1]; c = s_d[lane][2]; k = s_d[lane][3];
    p = s_u[lane][0]; q = s_u[lane][1];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        p += __shfl_xor_sync(0xffffffffu, p, o);
        q += __shfl_xor_sync(0xffffffffu, q, o);
        if (fp) {
            a += __shfl_xor_sync(0xffffffffu, a, o);
            b += __shfl_xor_sync(0xffffffffu, b, o);
            c += __shfl_xor_sync(0xffffffffu, c, o);
            k += __shfl_xor_sync(0xffffffffu, k, o);
        }
    }
    if (lane == 0) {
        tot->e_lj = a; tot->e_coul = b; tot->virial = c;
        tot->e_bond = tot->e_angle = tot->e_dihedral = 0.0;   /* the bonded kernel adds its own */
        if (nke > 0) tot->kinetic = k;
        tot->pairs = p; tot->below = q;
        tot->pairs_total += p;
    }
}

/* Sorted forces back to user order as float (and counts). */
static __global__ void k_unsort(int n, const int *__restrict__ pid, const unsigned long long *__restrict__ F64,
                         const float *__restrict__ F32, const int *__restrict__ cnt_s,
                         float *__restrict__ fx, float *__restrict__ fy, float *__restrict__ fz,
                         int *__restrict__ cnt_u) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const int id = pid[k];
    if (F64) {
        fx[id] = from_fixed(F64[k]); fy[id] = from_fixed(F64[n + k]); fz[id] = from_fixed(F64[2 * n + k]);
    } else {
        fx[id] = F32[k] + F32[3 * (size_t)n + k];
        fy[id] = F32[n + k] + F32[4 * (size_t)n + k];
        fz[id] = F32[2 * n + k] + F32[5 * (size_t)n + k];
    }
    if (cnt_u) cnt_u[id] = cnt_s[k];
}

/* The same in user order (inv = cell-order position of each user index): the writes are
 * coalesced, so fx, fy, fz, cnt_u may be pinned host memory written over the host link. */
static __global__ void k_unsort_inv(int n, const int *__restrict__ inv, const unsigned long long *__restrict__ F64,
                                    const float *__restrict__ F32, const int *__restrict__ cnt_s,
                                    float *__restrict__ fx, float *__restrict__ fy, float *__restrict__ fz,
                                    int *__restrict__ cnt_u, const DevTotals *__restrict__ tot_d = nullptr,
                                    DevTotals *tot_h = nullptr, const unsigned *__restrict__ err_d = nullptr,
                                    unsigned *err_h = nullptr) {
    const int id = blockIdx.x * blockDim.x + threadIdx.x;
    /* the call's last kernel also hands the totals and the error word to pinned (mapped) host
     * memory: both are final here (stream order), and the call needs no copies after it */
    if (id == 0 && tot_h) { *tot_h = *tot_d; *err_h = *err_d; }
    if (id >= n) return;
    const int k = inv[id];
    if (F64) {
        fx[id] = from_fixed(F64[k]); fy[id] = from_fixed(F64[n + k]); fz[id] = from_fixed(F64[2 * n + k]);
    } else {
        fx[id] = F32[k] + F32[3 * (size_t)n + k];
        fy[id] = F32[n + k] + F32[4 * (size_t)n + k];
        fz[id] = F32[2 * n + k] + F32[5 * (size_t)n + k];
    }
    if (cnt_u) cnt_u[id] = cnt_s[k];
}

/* The raw int64 accumulators in user order (x, y, z planes of n), for partial evaluations that
 * are summed exactly (spatial decomposition). */
static __global__ void k_unsort_fixed(int n, const int *__restrict__ inv, const unsigned long long *__restrict__ F64,
                                      long long *__restrict__ out) {
    const int id = blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= n) return;
    const int k = inv[id];
    out[id] = (long long)F64[k];
    out[(size_t)n + id] = (long long)F64[(size_t)n + k];
    out[2 * (size_t)n + id] = (long long)F64[2 * (size_t)n + k];
}

/* ------------------------------------------------------------------------------------------ */
/* Motion update on cell-sorted state.                                                         */

__device__ __forceinline__ float wrap_pos(float x, float L) {
    if (x < 0.0f) x = __fadd_rn(x, L);
    else if (x >= L) x = __fsub_rn(x, L);
    if (!(x >= 0.0f && x < L)) {
        x = __fsub_rn(x, __fmul_rn(L, floorf(__fdiv_rn(x, L))));
        if (!(x >= 0.0f && x < L)) x = 0.0f;
    }
    return x;
}

__device__ __forceinline__ float force_of(const unsigned long long *F64, const float *F32, int n,
                                          int k, int d) {
    /* FP32 accumulation keeps a high and a low (compensation) plane; the low one is zero in
     * the plain FP32-atomic mode */
    return F64 ? from_fixed(F64[(size_t)d * n + k]) : F32[(size_t)d * n + k] + F32[(size_t)(d + 3) * n + k];
}

/* v += F * cm[type] (half or full kick), x += v * dt, wrap, and bin the new position. */
static __global__ void k_kick_drift_bin(int n, float4 *__restrict__ pos, float4 *__restrict__ vel,
                                 const int *__restrict__ ptype,
                                 const unsigned long long *__restrict__ F64,
                                 const float *__restrict__ F32, const MassTab *__restrict__ mt, float dt, Geom g,
                                 int *__restrict__ cell_of, int *__restrict__ slot,
                                 int *__restrict__ count, unsigned *__restrict__ key) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const float cm = mt->cm[ptype[k]];
    float4 v = vel[k];
    float4 p = pos[k];
    v.x = __fmaf_rn(force_of(F64, F32, n, k, 0), cm, v.x);
    v.y = __fmaf_rn(force_of(F64, F32, n, k, 1), cm, v.y);
    v.z = __fmaf_rn(force_of(F64, F32, n, k, 2), cm, v.z);
    p.x = wrap_pos(__fmaf_rn(v.x, dt, p.x), g.L[0]);
    p.y = wrap_pos(__fmaf_rn(v.y, dt, p.y), g.L[1]);
    p.z = wrap_pos(__fmaf_rn(v.z, dt, p.z), g.L[2]);
    vel[k] = v;
    pos[k] = p;
    const int c = cell_of_pos(g, p.x, p.y, p.z);
    cell_of[k] = c;
    key[k] = cell_morton(g, p.x, p.y, p.z, c);
    slot[k] = cell_slot(count, c);
}

/* Reorder the state into the new cell order and clear the force accumulators. */
static __global__ void k_gather_state(int n, const int *__restrict__ sorted,
                               const float4 *__restrict__ pos0, const float4 *__restrict__ vel0,
                               const int *__restrict__ type0, const int *__restrict__ id0,
                               float4 *__restrict__ pos1, float4 *__restrict__ vel1,
                               int *__restrict__ type1, int *__restrict__ id1,
                               unsigned long long *__restrict__ F64, float *__restrict__ F32) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const int o = sorted[k];
    pos1[k] = pos0[o];
    vel1[k] = vel0[o];
    type1[k] = type0[o];
    id1[k] = id0[o];
    if (F64) { F64[k] = 0ull; F64[n + k] = 0ull; F64[2 * n + k] = 0ull; }
    if (F32) {
#pragma unroll
        for (int d = 0; d < 6; ++d) F32[(size_t)d * n + k] = 0.0f;   /* hi planes 0-2, lo planes 3-5 */
    }
}

/* Second half kick (velocity Verlet) and, when asked, per-block kinetic-energy partials
 * (FP32 per particle and within the block, in a fixed order; FP64 across blocks). */
static __global__ void __launch_bounds__(256) k_kick(int n, float4 *__restrict__ vel, const int *__restrict__ ptype,
                                                     const unsigned long long *__restrict__ F64,
                                                     const float *__restrict__ F32, const MassTab *__restrict__ mt, int do_kick,
                                                     double *__restrict__ kepart) {
    __shared__ float s_k[8];
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    float ke = 0.0f;
    if (k < n) {
        const int t = ptype[k];
        float4 v = vel[k];
        if (do_kick) {
            const float cm = mt->cm[t];
            v.x = __fmaf_rn(force_of(F64, F32, n, k, 0), cm, v.x);
            v.y = __fmaf_rn(force_of(F64, F32, n, k, 1), cm, v.y);
            v.z = __fmaf_rn(force_of(F64, F32, n, k, 2), cm, v.z);
            vel[k] = v;
        }
        /* 1/2 m v^2 in kcal/mol with v in A/fs and m in amu: divide by 4.184e-4. */
        if (kepart) ke = 0.5f * mt->mass[t] * (v.x * v.x + v.y * v.y + v.z * v.z) * (1.0f / 4.184e-4f);
    }
    if (!kepart) return;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) ke += __shfl_xor_sync(0xffffffffu, ke, o);
    if ((threadIdx.x & 31) == 0) s_k[threadIdx.x >> 5] = ke;
    __syncthreads();
    if (threadIdx.x == 0) {
        double b = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) b += s_k[w];
        kepart[blockIdx.x] = b;
    }
}

/* Sorted state back to user order. */
static __global__ void k_unsort_state(int n, const int *__restrict__ pid, const float4 *__restrict__ pos,
                               const float4 *__restrict__ vel, float *__restrict__ x,
                               float *__restrict__ y, float *__restrict__ z, float *__restrict__ vx,
                               float *__restrict__ vy, float *__restrict__ vz) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const int id = pid[k];
    const float4 p = pos[k], v = vel[k];
    x[id] = p.x; y[id] = p.y; z[id] = p.z;
    vx[id] = v.x; vy[id] = v.y; vz[id] = v.z;
}

/* Gather user-order velocities into cell order (set_state). */
static __global__ void k_gather_vel(int n, const int *__restrict__ pid, const float *__restrict__ vx,
                             const float *__restrict__ vy, const float *__restrict__ vz,
                             float4 *__restrict__ vel) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const int id = pid[k];
    vel[k] = vx ? make_float4(vx[id], vy[id], vz[id], 0.0f) : make_float4(0.f, 0.f, 0.f, 0.f);
}

/* ------------------------------------------------------------------------------------------ */
/* Per-pair evaluation: the drop-in for the OpenCL library function RL_LJ_Evaluation.          */

template <int ORDER, bool SEP>
static __global__ void k_pair_eval(int n, const float4 *__restrict__ ref, const float4 *__restrict__ nbr,
                            const int *__restrict__ tref, const int *__restrict__ tnbr, Geom g,
                            TableDev tab, const float4 *__restrict__ pcoef, int ntypes, float ke,
                            float4 *__restrict__ out, float2 *__restrict__ aux, int exact) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const float4 a = ref[k], b = nbr[k];
    const int ta = tref ? tref[k] : 0, tb = tnbr ? tnbr[k] : 0;
    float dx, dy, dz;
    if (exact) {
        dx = wrap_exact(a.x, b.x, g.L[0], g.h[0]);
        dy = wrap_exact(a.y, b.y, g.L[1], g.h[1]);
        dz = wrap_exact(a.z, b.z, g.L[2], g.h[2]);
    } else {
        dx = wrap_d(__fsub_rn(a.x, b.x), g.L[0], g.h[0]);
        dy = wrap_d(__fsub_rn(a.y, b.y), g.L[1], g.h[1]);
        dz = wrap_d(__fsub_rn(a.z, b.z), g.L[2], g.h[2]);
    }
    const float r2 = __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
    float4 o = make_float4(0.f, 0.f, 0.f, 0.f);
    float fs = 0.0f;
    if (r2 > 0.0f && r2 <= g.rc2) {
        const bool coul = ke != 0.0f;
        float v14, v8, v3, v12, v6, v1;
        int below;
        pair_functions<ORDER, SEP, false>(tab, r2, coul, v14, v8, v3, v12, v6, v1, below);
        const float4 pc = pcoef[ta * ntypes + tb];
        const float qq = __fmul_rn(__fmul_rn(ke, a.w), b.w);
        fs = combine_force<SEP>(pc, qq, coul, v14, v8, v3);
        o = make_float4(__fmul_rn(fs, dx), __fmul_rn(fs, dy), __fmul_rn(fs, dz), 0.0f);
    }
    out[k] = o;
    if (aux) aux[k] = make_float2(r2, fs);
}

}  // namespace mdrl
