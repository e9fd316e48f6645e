/*
 * oracle.cpp — CPU restatement of the reference's range-limited force path.
 *
 * TEST INFRASTRUCTURE ONLY (see oracle.h): the checker for tests/, __graft_entry__.smoke() and
 * the timed CPU baseline of bench.py.  Compiled with -ffp-contract=off so every float expression
 * rounds once per operation, exactly as written, on x86-64 and on aarch64 alike.
 */
#include "oracle.h"

#include <math.h>

#include <cmath>
#include <stdlib.h>
#include <string.h>

#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

inline uint32_t f2u(float f) { uint32_t u; memcpy(&u, &f, 4); return u; }

/* The 14 cells a home cell pairs with, in the reference's filter order
 * (MS/FullScale_Simulation_LJArgon.m:11-19 and :381-749; SC/Particle_Pair_Gen_HalfShell.v:14-24):
 * F0 222 (home), F1 223, F2 231 232, F3 233 311, F4 312 313, F5 321 322, F6 323 331, F7 332 333,
 * where digit 2 is the home coordinate and 1/3 are -1/+1. */
const int kHalfShell[14][3] = {
    {0, 0, 0},  {0, 0, 1},  {0, 1, -1}, {0, 1, 0},  {0, 1, 1},  {1, -1, -1}, {1, -1, 0},
    {1, -1, 1}, {1, 0, -1}, {1, 0, 0},  {1, 0, 1},  {1, 1, -1}, {1, 1, 0},   {1, 1, 1}};

/* One conditional +-L wrap of a coordinate difference (SC/r2_compute_with_pbc.v:81-127).
 * Returns the wrapped difference and reports which way it wrapped. */
inline float wrap1(float d, float L, int *dir) {
    *dir = 0;
    if (L <= 0.0f) return d;
    const float h = 0.5f * L;
    if (d > h) { *dir = -1; return d - L; }
    if (d < -h) { *dir = 1; return d + L; }
    return d;
}

inline float mul(float a, float b) { return a * b; }
inline float add(float a, float b) { return a + b; }

/* Start of table bin idx: 2^(min_log2 + seg) * (1 + bin / bins), exact in FP32 and FP64. */
inline double bin_start(const orc_sys *s, int idx) {
    const int seg = idx / s->bins, bin = idx - seg * s->bins;
    return ldexp(1.0 + (double)bin / s->bins, s->min_log2 + seg);
}

/* Polynomial c_order*x^order + ... + c0 by Horner's rule, one coefficient plane per power;
 * x = r2 (monomial tables) or u = r2 - bin start (bin-local tables; exact in FP32, r2 lying in
 * the bin). */
inline float poly32(const orc_sys *s, int f, int idx, float r2) {
    const int nidx = s->nseg * s->bins;
    const float *t = s->tab + (size_t)f * (s->order + 1) * nidx;
    const float x = s->local ? r2 - (float)bin_start(s, idx) : r2;
    float v = t[(size_t)s->order * nidx + idx];
    for (int k = s->order - 1; k >= 0; --k) {
        const float c = t[(size_t)k * nidx + idx];
        v = s->arith ? add(mul(v, x), c) : fmaf(v, x, c);
    }
    return v;
}

inline double poly64(const orc_sys *s, int f, int idx, double r2) {
    const int nidx = s->nseg * s->bins;
    const float *t = s->tab + (size_t)f * (s->order + 1) * nidx;
    const double x = s->local ? r2 - bin_start(s, idx) : r2;
    double v = t[(size_t)s->order * nidx + idx];
    for (int k = s->order - 1; k >= 0; --k) v = v * x + (double)t[(size_t)k * nidx + idx];
    return v;
}

inline int ilog2(int v) { int l = 0; while ((1 << l) < v) ++l; return l; }

/* Table address from the r2 bit pattern (SC/RL_LJ_Evaluate_Pairs_1st_Order.v:179-193):
 * segment = exponent field - 127 - min_log2, bin = the top log2(bins) mantissa bits.
 * Below the first segment the pair is evaluated at the first table point and flagged; above
 * the last it uses the last bin (host validation keeps rc2 inside the table). */
inline int table_index(const orc_sys *s, float r2, float *r2e, int *below) {
    const uint32_t b = f2u(r2);
    const int lb = ilog2(s->bins);
    int seg = (int)(b >> 23) - 127 - s->min_log2;
    int bin = (int)((b >> (23 - lb)) & (uint32_t)(s->bins - 1));
    *r2e = r2;
    *below = 0;
    if (seg < 0) {
        seg = 0; bin = 0; *r2e = ldexpf(1.0f, s->min_log2); *below = 1;
    } else if (seg >= s->nseg) {
        seg = s->nseg - 1; bin = s->bins - 1;
    }
    return seg * s->bins + bin;
}

struct PairOut { float fx, fy, fz, fs, r2, elj, ec; int below; int dir[3]; float dx, dy, dz; };

/* The per-pair FP32 datapath.  Operation order (the reference RTL's):
 *   d = ref - nbr, wrap; r2 = (dx*dx + dy*dy) + dz*dz; keep when 0 < r2 <= rc2;
 *   v_k = poly_k(r2) (tables) or the direct powers of 1/r2;
 *   fscal = ((QQ*v3) + B*v8) + A*v14, QQ = (ke*qi)*qj;  f = fscal * d.
 * In fused mode each "x*y + z" above is one fmaf. */
inline int pair32_at(const orc_sys *s, float qi, int ti, float qj, int tj, PairOut *o);

/* The exact-difference rule: the wrap direction as wrap1 decides it, then the box edge comes off
 * the high coordinate (xi - L when xi is the high one, xj - L otherwise; exact for coordinates in
 * [0, L)) and the difference is rounded once. */
inline float wrap_exact(float xi, float xj, float L, int *dir) {
    float d = wrap1(xi - xj, L, dir);
    if (*dir < 0) d = (xi - L) - xj;
    else if (*dir > 0) d = xi - (xj - L);
    return d;
}

inline int pair32(const orc_sys *s, float xi, float yi, float zi, float qi, int ti, float xj,
                  float yj, float zj, float qj, int tj, PairOut *o) {
    if (s->exact) {
        o->dx = wrap_exact(xi, xj, s->box[0], &o->dir[0]);
        o->dy = wrap_exact(yi, yj, s->box[1], &o->dir[1]);
        o->dz = wrap_exact(zi, zj, s->box[2], &o->dir[2]);
    } else {
        o->dx = wrap1(xi - xj, s->box[0], &o->dir[0]);
        o->dy = wrap1(yi - yj, s->box[1], &o->dir[1]);
        o->dz = wrap1(zi - zj, s->box[2], &o->dir[2]);
    }
    return pair32_at(s, qi, ti, qj, tj, o);
}

/* The datapath from r2 on, for the difference already in o->dx, o->dy, o->dz. */
inline int pair32_at(const orc_sys *s, float qi, int ti, float qj, int tj, PairOut *o) {
    const float r2 = add(add(mul(o->dx, o->dx), mul(o->dy, o->dy)), mul(o->dz, o->dz));
    o->r2 = r2;
    o->fx = o->fy = o->fz = o->fs = o->elj = o->ec = 0.0f;
    o->below = 0;
    if (!(r2 > 0.0f && r2 <= s->rc2)) return 0;

    float v14, v8, v3 = 0.0f, v12, v6, v1 = 0.0f;
    if (s->eval == 0) {
        float r2e;
        const int idx = table_index(s, r2, &r2e, &o->below);
        v14 = poly32(s, ORC_F14, idx, r2e);
        v8 = poly32(s, ORC_F8, idx, r2e);
        v12 = poly32(s, ORC_F12, idx, r2e);
        v6 = poly32(s, ORC_F6, idx, r2e);
        if (s->ke != 0.0f) {
            v3 = poly32(s, ORC_F3, idx, r2e);
            v1 = poly32(s, ORC_F1, idx, r2e);
        }
    } else {
        const float i2 = 1.0f / r2;
        const float i4 = i2 * i2, i6 = i4 * i2, i8 = i4 * i4, i12 = i6 * i6, i14 = i12 * i2;
        const float i1 = sqrtf(i2), i3 = i2 * i1;
        v14 = i14; v8 = i8; v12 = i12; v6 = i6; v3 = i3; v1 = i1;
    }
    const float *pc = s->pcoef + 4 * (ti * s->ntypes + tj);
    const float A = pc[0], B = pc[1], Ae = pc[2], Be = pc[3];
    float fs, el, ec = 0.0f;
    if (s->arith) {
        fs = mul(B, v8);
        if (s->ke != 0.0f) fs = add(mul(mul(s->ke, qi), qj) * v3, fs);
        fs = add(fs, mul(A, v14));
        el = add(mul(Be, v6), mul(Ae, v12));
        if (s->ke != 0.0f) ec = mul(mul(mul(s->ke, qi), qj), v1);
    } else {
        const float qq = (s->ke != 0.0f) ? mul(mul(s->ke, qi), qj) : 0.0f;
        fs = fmaf(B, v8, (s->ke != 0.0f) ? mul(qq, v3) : 0.0f);
        fs = fmaf(A, v14, fs);
        el = fmaf(Ae, v12, mul(Be, v6));
        ec = mul(qq, v1);
    }
    o->fs = fs;
    o->fx = mul(fs, o->dx);
    o->fy = mul(fs, o->dy);
    o->fz = mul(fs, o->dz);
    o->elj = el;
    o->ec = ec;
    return 1;
}

struct Cells {
    std::vector<int> cell_of, start, order;
    int nc[3] = {0, 0, 0};
    int maxocc = 0;
};

void build_cells(const orc_sys *s, Cells *c) {
    c->nc[0] = s->ncell[0]; c->nc[1] = s->ncell[1]; c->nc[2] = s->ncell[2];
    const int ncells = c->nc[0] * c->nc[1] * c->nc[2];
    c->cell_of.resize(s->n);
    c->start.resize(ncells + 1);
    c->order.resize(s->n);
    c->maxocc = orc_bin(s->n, s->x, s->y, s->z, s->box, s->ncell, c->cell_of.data(),
                        c->start.data(), c->order.data());
}

inline int wrapc(int v, int n) { return v < 0 ? v + n : (v >= n ? v - n : v); }

/* Visit every unique candidate pair of the half-shell traversal (the home cell's own pairs once,
 * with i before j in cell order), calling fn(i, j) with original particle ids. */
template <class Fn>
void for_each_candidate(const orc_sys *s, const Cells &c, int hbegin, int hend, Fn fn) {
    const int nx = c.nc[0], ny = c.nc[1], nz = c.nc[2];
    for (int h = hbegin; h < hend; ++h) {
        const int hx = h / (ny * nz), hy = (h / nz) % ny, hz = h % nz;
        for (int f = 0; f < 14; ++f) {
            const int cx = wrapc(hx + kHalfShell[f][0], nx);
            const int cy = wrapc(hy + kHalfShell[f][1], ny);
            const int cz = wrapc(hz + kHalfShell[f][2], nz);
            const int cn = (cx * ny + cy) * nz + cz;
            for (int a = c.start[h]; a < c.start[h + 1]; ++a) {
                const int jb = (f == 0) ? a + 1 : c.start[cn];
                for (int b = jb; b < c.start[cn + 1]; ++b) fn(c.order[a], c.order[b]);
            }
        }
    }
}

int check_sys(const orc_sys *s) {
    if (!s || s->n < 0) return -1;
    if (s->n > 0 && (!s->x || !s->y || !s->z || !s->type)) return -1;
    if (s->ncell[0] < 1 || s->ncell[1] < 1 || s->ncell[2] < 1) return -1;
    if (s->eval == 0 && (!s->tab || s->bins < 1 || s->nseg < 1 || s->order < 1)) return -1;
    return 0;
}

inline float qof(const orc_sys *s, int i) { return s->q ? s->q[i] : 0.0f; }

}  // namespace

extern "C" {

int orc_bin(int n, const float *x, const float *y, const float *z, const float box[3],
            const int ncell[3], int *cell_of, int *cell_start, int *order) {
    /* cell = floor(pos / edge) in FP32, 0-based; the reference's 1-based
     * "floor(pos/rc)+1, pos==0 -> 1" (MS/GenInputCellList_LJArgon.m:98-112) is the same cell.
     * Particles are appended to their cell in input order (:114-121). */
    const int nx = ncell[0], ny = ncell[1], nz = ncell[2];
    const int ncells = nx * ny * nz;
    float edge[3];
    for (int d = 0; d < 3; ++d) edge[d] = (float)((double)box[d] / (double)ncell[d]);
    std::vector<int> count(ncells, 0);
    const float *p[3] = {x, y, z};
    for (int i = 0; i < n; ++i) {
        int c[3];
        for (int d = 0; d < 3; ++d) {
            const float v = floorf(p[d][i] / edge[d]);
            int cv;
            if (!(v >= 0.0f)) cv = 0;                       /* negative or NaN -> first cell */
            else if (v >= (float)ncell[d]) cv = ncell[d] - 1; /* past the end -> last cell */
            else cv = (int)v;
            c[d] = cv;
        }
        cell_of[i] = (c[0] * ny + c[1]) * nz + c[2];
        count[cell_of[i]]++;
    }
    int maxocc = 0;
    cell_start[0] = 0;
    for (int k = 0; k < ncells; ++k) {
        cell_start[k + 1] = cell_start[k] + count[k];
        if (count[k] > maxocc) maxocc = count[k];
    }
    std::vector<int> fill(cell_start, cell_start + ncells);
    for (int i = 0; i < n; ++i) order[fill[cell_of[i]]++] = i;
    return maxocc;
}

int orc_pair_f32(const orc_sys *s, float xi, float yi, float zi, float qi, int ti, float xj,
                 float yj, float zj, float qj, int tj, float *out) {
    PairOut o;
    const int ok = pair32(s, xi, yi, zi, qi, ti, xj, yj, zj, qj, tj, &o);
    out[0] = o.fx; out[1] = o.fy; out[2] = o.fz; out[3] = o.fs;
    out[4] = o.r2; out[5] = o.elj; out[6] = o.ec; out[7] = (float)o.below;
    return ok;
}

int orc_force_cells(const orc_sys *s, double *F, double *Fabs, int *counts, orc_stats *st) {
    if (check_sys(s)) return -1;
    Cells c;
    build_cells(s, &c);
    const int n = s->n;
    if (F) memset(F, 0, sizeof(double) * 3 * n);
    if (Fabs) memset(Fabs, 0, sizeof(double) * 3 * n);
    if (counts) memset(counts, 0, sizeof(int) * n);
    orc_stats acc;
    memset(&acc, 0, sizeof(acc));
    const int ncells = c.nc[0] * c.nc[1] * c.nc[2];
    for_each_candidate(s, c, 0, ncells, [&](int i, int j) {
        PairOut o;
        acc.candidates++;
        if (!pair32(s, s->x[i], s->y[i], s->z[i], qof(s, i), s->type[i], s->x[j], s->y[j],
                    s->z[j], qof(s, j), s->type[j], &o))
            return;
        acc.pairs++;
        acc.below_table += o.below;
        acc.e_lj += o.elj;
        acc.e_coul += o.ec;
        acc.virial += (double)o.fs * (double)o.r2;
        if (F) {
            F[3 * i] += o.fx; F[3 * i + 1] += o.fy; F[3 * i + 2] += o.fz;
            F[3 * j] -= o.fx; F[3 * j + 1] -= o.fy; F[3 * j + 2] -= o.fz;
        }
        if (Fabs) {
            const double ax = fabs(o.fx), ay = fabs(o.fy), az = fabs(o.fz);
            Fabs[3 * i] += ax; Fabs[3 * i + 1] += ay; Fabs[3 * i + 2] += az;
            Fabs[3 * j] += ax; Fabs[3 * j + 1] += ay; Fabs[3 * j + 2] += az;
        }
        if (counts) { counts[i]++; counts[j]++; }
    });
    if (st) *st = acc;
    return c.maxocc;
}

int64_t orc_force_cells_fixed(const orc_sys *s, int hbegin, int hend, int64_t *F) {
    if (check_sys(s)) return -1;
    Cells c;
    build_cells(s, &c);
    const int n = s->n;
    memset(F, 0, sizeof(int64_t) * 3 * n);
    const int ncells = c.nc[0] * c.nc[1] * c.nc[2];
    if (hbegin < 0) hbegin = 0;
    if (hend < 0 || hend > ncells) hend = ncells;
    int64_t pairs = 0;
    /* each pair's FP32 force as 2^-24 fixed point (round to nearest), summed in int64: the sum of
     * any partition of the pairs over ranks is the same integer */
    auto fix = [](float v) { return (int64_t)llrint((double)v * 16777216.0); };
    for_each_candidate(s, c, hbegin, hend, [&](int i, int j) {
        PairOut o;
        if (!pair32(s, s->x[i], s->y[i], s->z[i], qof(s, i), s->type[i], s->x[j], s->y[j],
                    s->z[j], qof(s, j), s->type[j], &o))
            return;
        ++pairs;
        const int64_t fx = fix(o.fx), fy = fix(o.fy), fz = fix(o.fz);
        F[3 * i] += fx; F[3 * i + 1] += fy; F[3 * i + 2] += fz;
        F[3 * j] -= fx; F[3 * j + 1] -= fy; F[3 * j + 2] -= fz;
    });
    return pairs;
}

int orc_force_direct64(const orc_sys *s, double *F, orc_stats *st) {
    if (check_sys(s) || !s->pcoef64) return -1;
    Cells c;
    build_cells(s, &c);
    const int n = s->n;
    memset(F, 0, sizeof(double) * 3 * n);
    orc_stats acc;
    memset(&acc, 0, sizeof(acc));
    const int ncells = c.nc[0] * c.nc[1] * c.nc[2];
    for_each_candidate(s, c, 0, ncells, [&](int i, int j) {
        PairOut o;
        acc.candidates++;
        if (!pair32(s, s->x[i], s->y[i], s->z[i], qof(s, i), s->type[i], s->x[j], s->y[j],
                    s->z[j], qof(s, j), s->type[j], &o))
            return;
        acc.pairs++;
        /* exact differences, wrapped the way the FP32 pair was */
        const double dx = (double)s->x[i] - (double)s->x[j] + o.dir[0] * (double)s->box[0];
        const double dy = (double)s->y[i] - (double)s->y[j] + o.dir[1] * (double)s->box[1];
        const double dz = (double)s->z[i] - (double)s->z[j] + o.dir[2] * (double)s->box[2];
        const double r2 = dx * dx + dy * dy + dz * dz;
        const double i2 = 1.0 / r2, i4 = i2 * i2, i6 = i4 * i2, i8 = i4 * i4;
        const double i12 = i6 * i6, i14 = i12 * i2, i1 = sqrt(i2), i3 = i2 * i1;
        const double *pc = s->pcoef64 + 4 * (s->type[i] * s->ntypes + s->type[j]);
        const double qq = s->ke64 * (double)qof(s, i) * (double)qof(s, j);
        const double fs = (qq * i3 + pc[1] * i8) + pc[0] * i14;
        acc.e_lj += pc[3] * i6 + pc[2] * i12;
        acc.e_coul += qq * i1;
        acc.virial += fs * r2;
        F[3 * i] += fs * dx; F[3 * i + 1] += fs * dy; F[3 * i + 2] += fs * dz;
        F[3 * j] -= fs * dx; F[3 * j + 1] -= fs * dy; F[3 * j + 2] -= fs * dz;
    });
    if (st) *st = acc;
    return c.maxocc;
}

int orc_force_split64(const orc_sys *s, int f32_diff, int tables, double *F, orc_stats *st) {
    if (check_sys(s) || !s->pcoef64 || (tables && s->eval != 0)) return -1;
    Cells c;
    build_cells(s, &c);
    const int n = s->n;
    memset(F, 0, sizeof(double) * 3 * n);
    orc_stats acc;
    memset(&acc, 0, sizeof(acc));
    const int ncells = c.nc[0] * c.nc[1] * c.nc[2];
    for_each_candidate(s, c, 0, ncells, [&](int i, int j) {
        PairOut o;
        acc.candidates++;
        if (!pair32(s, s->x[i], s->y[i], s->z[i], qof(s, i), s->type[i], s->x[j], s->y[j],
                    s->z[j], qof(s, j), s->type[j], &o))
            return;
        acc.pairs++;
        double dx, dy, dz;
        if (f32_diff == 1) {
            dx = o.dx; dy = o.dy; dz = o.dz;   /* the datapath's rounded fl(fl(xi - xj) +- L) */
        } else {
            dx = (double)s->x[i] - (double)s->x[j] + o.dir[0] * (double)s->box[0];
            dy = (double)s->y[i] - (double)s->y[j] + o.dir[1] * (double)s->box[1];
            dz = (double)s->z[i] - (double)s->z[j] + o.dir[2] * (double)s->box[2];
            if (f32_diff == 2) {   /* the exact minimum-image difference rounded once */
                dx = (float)dx; dy = (float)dy; dz = (float)dz;
            }
        }
        double r2 = dx * dx + dy * dy + dz * dz;
        const double *pc = s->pcoef64 + 4 * (s->type[i] * s->ntypes + s->type[j]);
        const double qq = s->ke64 * (double)qof(s, i) * (double)qof(s, j);
        double fs;
        if (tables) {
            float r2e;
            int below;
            const int idx = table_index(s, o.r2, &r2e, &below);
            if (below) r2 = r2e;
            fs = pc[1] * poly64(s, ORC_F8, idx, r2) + pc[0] * poly64(s, ORC_F14, idx, r2);
            if (s->ke != 0.0f) fs += qq * poly64(s, ORC_F3, idx, r2);
        } else {
            const double i2 = 1.0 / r2, i4 = i2 * i2, i8 = i4 * i4, i14 = i8 * i4 * i2;
            fs = (qq * i2 * sqrt(i2) + pc[1] * i8) + pc[0] * i14;
        }
        F[3 * i] += fs * dx; F[3 * i + 1] += fs * dy; F[3 * i + 2] += fs * dz;
        F[3 * j] -= fs * dx; F[3 * j + 1] -= fs * dy; F[3 * j + 2] -= fs * dz;
    });
    if (st) *st = acc;
    return c.maxocc;
}

int orc_force_tables64(const orc_sys *s, double *F, orc_stats *st) {
    if (check_sys(s) || !s->pcoef64 || s->eval != 0) return -1;
    Cells c;
    build_cells(s, &c);
    const int n = s->n;
    memset(F, 0, sizeof(double) * 3 * n);
    orc_stats acc;
    memset(&acc, 0, sizeof(acc));
    const int ncells = c.nc[0] * c.nc[1] * c.nc[2];
    for_each_candidate(s, c, 0, ncells, [&](int i, int j) {
        PairOut o;
        acc.candidates++;
        if (!pair32(s, s->x[i], s->y[i], s->z[i], qof(s, i), s->type[i], s->x[j], s->y[j],
                    s->z[j], qof(s, j), s->type[j], &o))
            return;
        acc.pairs++;
        const double dx = (double)s->x[i] - (double)s->x[j] + o.dir[0] * (double)s->box[0];
        const double dy = (double)s->y[i] - (double)s->y[j] + o.dir[1] * (double)s->box[1];
        const double dz = (double)s->z[i] - (double)s->z[j] + o.dir[2] * (double)s->box[2];
        double r2 = dx * dx + dy * dy + dz * dz;
        float r2e;
        int below;
        const int idx = table_index(s, o.r2, &r2e, &below);
        if (below) r2 = r2e;
        const double *pc = s->pcoef64 + 4 * (s->type[i] * s->ntypes + s->type[j]);
        const double qq = s->ke64 * (double)qof(s, i) * (double)qof(s, j);
        double fs = pc[1] * poly64(s, ORC_F8, idx, r2) + pc[0] * poly64(s, ORC_F14, idx, r2);
        double el = pc[3] * poly64(s, ORC_F6, idx, r2) + pc[2] * poly64(s, ORC_F12, idx, r2);
        double ec = 0.0;
        if (s->ke != 0.0f) {
            fs += qq * poly64(s, ORC_F3, idx, r2);
            ec = qq * poly64(s, ORC_F1, idx, r2);
        }
        acc.e_lj += el;
        acc.e_coul += ec;
        acc.virial += fs * r2;
        F[3 * i] += fs * dx; F[3 * i + 1] += fs * dy; F[3 * i + 2] += fs * dz;
        F[3 * j] -= fs * dx; F[3 * j + 1] -= fs * dy; F[3 * j + 2] -= fs * dz;
    });
    if (st) *st = acc;
    return c.maxocc;
}

int64_t orc_force_cells_mt(const orc_sys *s, int nthreads, int hbegin, int hend, float *F) {
    if (check_sys(s)) return -1;
    Cells c;
    build_cells(s, &c);
    const int n = s->n;
    const int ncells = c.nc[0] * c.nc[1] * c.nc[2];
    if (hend < 0 || hend > ncells) hend = ncells;
    if (hbegin < 0) hbegin = 0;
#ifdef _OPENMP
    if (nthreads <= 0) nthreads = omp_get_max_threads();
#else
    nthreads = 1;
#endif
    std::vector<float> part((size_t)nthreads * 3 * n, 0.0f);
    int64_t pairs = 0;
#ifdef _OPENMP
#pragma omp parallel num_threads(nthreads) reduction(+ : pairs)
#endif
    {
#ifdef _OPENMP
        const int t = omp_get_thread_num();
#else
        const int t = 0;
#endif
        float *Ft = part.data() + (size_t)t * 3 * n;
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 1)
#endif
        for (int h = hbegin; h < hend; ++h) {
            for_each_candidate(s, c, h, h + 1, [&](int i, int j) {
                PairOut o;
                if (!pair32(s, s->x[i], s->y[i], s->z[i], qof(s, i), s->type[i], s->x[j],
                            s->y[j], s->z[j], qof(s, j), s->type[j], &o))
                    return;
                pairs++;
                Ft[3 * i] += o.fx; Ft[3 * i + 1] += o.fy; Ft[3 * i + 2] += o.fz;
                Ft[3 * j] -= o.fx; Ft[3 * j + 1] -= o.fy; Ft[3 * j + 2] -= o.fz;
            });
        }
    }
#ifdef _OPENMP
#pragma omp parallel for num_threads(nthreads) schedule(static)
#endif
    for (int k = 0; k < 3 * n; ++k) {
        float v = 0.0f;
        for (int t = 0; t < nthreads; ++t) v += part[(size_t)t * 3 * n + k];
        F[k] = v;
    }
    return pairs;
}

int64_t orc_force_allpairs_mt(const orc_sys *s, int nthreads, float *F) {
    if (!s || s->n < 0) return -1;
    const int n = s->n;
#ifdef _OPENMP
    if (nthreads <= 0) nthreads = omp_get_max_threads();
#endif
    int64_t pairs = 0;
#ifdef _OPENMP
#pragma omp parallel for num_threads(nthreads) schedule(dynamic, 16) reduction(+ : pairs)
#endif
    for (int i = 0; i < n; ++i) {
        float fx = 0.0f, fy = 0.0f, fz = 0.0f;
        for (int j = 0; j < n; ++j) {
            PairOut o;
            if (!pair32(s, s->x[i], s->y[i], s->z[i], qof(s, i), s->type[i], s->x[j], s->y[j],
                        s->z[j], qof(s, j), s->type[j], &o))
                continue;
            pairs++;
            fx += o.fx; fy += o.fy; fz += o.fz;
        }
        F[3 * i] = fx; F[3 * i + 1] = fy; F[3 * i + 2] = fz;
    }
    return pairs;
}

int64_t orc_force_allimage(const orc_sys *s, double *F, double *F32sum, double *Fabs, int *counts,
                           orc_stats *st) {
    if (!s || s->n < 0 || (s->n > 0 && (!s->x || !s->y || !s->z || !s->type))) return -1;
    if (s->eval == 0 && (!s->tab || !s->pcoef64)) return -1;
    const int n = s->n;
    if (F) memset(F, 0, sizeof(double) * 3 * n);
    if (F32sum) memset(F32sum, 0, sizeof(double) * 3 * n);
    if (Fabs) memset(Fabs, 0, sizeof(double) * 3 * n);
    if (counts) memset(counts, 0, sizeof(int) * n);
    orc_stats acc;
    memset(&acc, 0, sizeof(acc));
    const float *p[3] = {s->x, s->y, s->z};
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j) {
            if (j == i) continue;
            float cand[3][3];
            int nc[3];
            double shift[3][3];
            for (int a = 0; a < 3; ++a) {
                const float d0 = p[a][i] - p[a][j];
                const float L = s->box[a];
                const float c3[3] = {d0, d0 - L, d0 + L};
                const double sh[3] = {0.0, -(double)L, (double)L};
                nc[a] = 0;
                for (int m = 0; m < 3; ++m)
                    if (c3[m] * c3[m] <= s->rc2) { cand[a][nc[a]] = c3[m]; shift[a][nc[a]] = sh[m]; ++nc[a]; }
            }
            for (int ax = 0; ax < nc[0]; ++ax)
                for (int ay = 0; ay < nc[1]; ++ay)
                    for (int az = 0; az < nc[2]; ++az) {
                        PairOut o;
                        o.dx = cand[0][ax]; o.dy = cand[1][ay]; o.dz = cand[2][az];
                        if (j > i) acc.candidates++;
                        /* the FP32 datapath of the ordered pair (i's side: QQ = (ke*qi)*qj) */
                        if (!pair32_at(s, qof(s, i), s->type[i], qof(s, j), s->type[j], &o)) continue;
                        if (counts) counts[i]++;
                        if (F32sum) { F32sum[3 * i] += o.fx; F32sum[3 * i + 1] += o.fy; F32sum[3 * i + 2] += o.fz; }
                        if (Fabs) {
                            Fabs[3 * i] += fabs(o.fx); Fabs[3 * i + 1] += fabs(o.fy); Fabs[3 * i + 2] += fabs(o.fz);
                        }
                        if (j < i) continue;
                        acc.pairs++;
                        acc.below_table += o.below;
                        /* FP64 evaluation of the unordered pair at the exact difference */
                        const double ex = (double)s->x[i] - (double)s->x[j] + shift[0][ax];
                        const double ey = (double)s->y[i] - (double)s->y[j] + shift[1][ay];
                        const double ez = (double)s->z[i] - (double)s->z[j] + shift[2][az];
                        double e2 = ex * ex + ey * ey + ez * ez;
                        const double *pc = s->pcoef64 + 4 * (s->type[i] * s->ntypes + s->type[j]);
                        const double qq = s->ke64 * (double)qof(s, i) * (double)qof(s, j);
                        double fs, el, ec = 0.0;
                        if (s->eval == 0) {
                            float r2e;
                            int below;
                            const int idx = table_index(s, o.r2, &r2e, &below);
                            if (below) e2 = r2e;
                            fs = pc[1] * poly64(s, ORC_F8, idx, e2) + pc[0] * poly64(s, ORC_F14, idx, e2);
                            el = pc[3] * poly64(s, ORC_F6, idx, e2) + pc[2] * poly64(s, ORC_F12, idx, e2);
                            if (s->ke != 0.0f) {
                                fs += qq * poly64(s, ORC_F3, idx, e2);
                                ec = qq * poly64(s, ORC_F1, idx, e2);
                            }
                        } else {
                            const double i2 = 1.0 / e2, i4 = i2 * i2, i6 = i4 * i2, i8 = i4 * i4;
                            const double i12 = i6 * i6, i14 = i12 * i2, i1 = sqrt(i2), i3 = i2 * i1;
                            fs = (qq * i3 + pc[1] * i8) + pc[0] * i14;
                            el = pc[3] * i6 + pc[2] * i12;
                            ec = qq * i1;
                        }
                        acc.e_lj += el;
                        acc.e_coul += ec;
                        acc.virial += fs * e2;
                        if (F) {
                            F[3 * i] += fs * ex; F[3 * i + 1] += fs * ey; F[3 * i + 2] += fs * ez;
                            F[3 * j] -= fs * ex; F[3 * j + 1] -= fs * ey; F[3 * j + 2] -= fs * ez;
                        }
                    }
        }
    if (st) *st = acc;
    return acc.pairs;
}

int orc_ewald64(const orc_sys *s, double beta, int nmax, double *F, double *energy) {
    if (!s || s->n < 0 || !s->q || beta <= 0.0 || nmax < 1) return -1;
    const int n = s->n;
    const double ke = s->ke64;
    const double L[3] = {s->box[0], s->box[1], s->box[2]};
    const double V = L[0] * L[1] * L[2];
    const double rc2 = s->rc2;
    const double PI = 3.14159265358979323846;
    if (F) memset(F, 0, sizeof(double) * 3 * n);
    double e_real = 0.0, e_rec = 0.0, qsum = 0.0, q2sum = 0.0;
    std::vector<double> P(3 * (size_t)n), Q(n);
    for (int i = 0; i < n; ++i) {
        P[3 * i] = s->x[i]; P[3 * i + 1] = s->y[i]; P[3 * i + 2] = s->z[i];
        Q[i] = s->q[i];
        qsum += Q[i];
        q2sum += Q[i] * Q[i];
    }
    /* real space */
    for (int i = 0; i < n; ++i)
        for (int j = i + 1; j < n; ++j) {
            double d[3], r2 = 0.0;
            for (int a = 0; a < 3; ++a) {
                d[a] = P[3 * i + a] - P[3 * j + a];
                d[a] -= L[a] * std::floor(d[a] / L[a] + 0.5);
                r2 += d[a] * d[a];
            }
            if (!(r2 > 0.0 && r2 <= rc2)) continue;
            const double r = std::sqrt(r2);
            const double qq = ke * Q[i] * Q[j];
            e_real += qq * std::erfc(beta * r) / r;
            if (F) {
                const double fs = qq * (std::erfc(beta * r) / r + 2.0 * beta / std::sqrt(PI) * std::exp(-beta * beta * r2)) / r2;
                for (int a = 0; a < 3; ++a) { F[3 * i + a] += fs * d[a]; F[3 * j + a] -= fs * d[a]; }
            }
        }
    /* reciprocal space over the half space of n (n and -n contribute alike) */
    const int w = 2 * nmax + 1;
    std::vector<double> cr[3], ci[3];   /* cos / sin(2 pi k x_j / L) for k = -nmax..nmax */
    for (int a = 0; a < 3; ++a) {
        cr[a].resize((size_t)n * w);
        ci[a].resize((size_t)n * w);
        for (int j = 0; j < n; ++j)
            for (int k = -nmax; k <= nmax; ++k) {
                const double t = 2.0 * PI * k * P[3 * j + a] / L[a];
                cr[a][(size_t)j * w + k + nmax] = std::cos(t);
                ci[a][(size_t)j * w + k + nmax] = std::sin(t);
            }
    }
    std::vector<double> er(n), ei(n);
    for (int n1 = 0; n1 <= nmax; ++n1)
        for (int n2 = -nmax; n2 <= nmax; ++n2)
            for (int n3 = -nmax; n3 <= nmax; ++n3) {
                if (n1 == 0 && (n2 < 0 || (n2 == 0 && n3 <= 0))) continue;   /* half space, no m = 0 */
                const double m[3] = {n1 / L[0], n2 / L[1], n3 / L[2]};
                const double m2 = m[0] * m[0] + m[1] * m[1] + m[2] * m[2];
                const double g = std::exp(-PI * PI * m2 / (beta * beta)) / m2;
                if (g < 1e-300) continue;
                double sr = 0.0, si = 0.0;
                for (int j = 0; j < n; ++j) {
                    const size_t o = (size_t)j * w;
                    /* e = e1 e2 e3 */
                    const double ar = cr[0][o + n1 + nmax], ai = ci[0][o + n1 + nmax];
                    const double br = cr[1][o + n2 + nmax], bi = ci[1][o + n2 + nmax];
                    const double cr3 = cr[2][o + n3 + nmax], ci3 = ci[2][o + n3 + nmax];
                    const double abr = ar * br - ai * bi, abi = ar * bi + ai * br;
                    er[j] = abr * cr3 - abi * ci3;
                    ei[j] = abr * ci3 + abi * cr3;
                    sr += Q[j] * er[j];
                    si += Q[j] * ei[j];
                }
                e_rec += 2.0 * g * (sr * sr + si * si);
                if (F) {
                    /* F_j = (2 ke q_j / V) sum_m g m Im[conj(S) e_j], both half spaces */
                    const double c = 2.0 * 2.0 * ke / V * g;
                    for (int j = 0; j < n; ++j) {
                        const double im = sr * ei[j] - si * er[j];
                        for (int a = 0; a < 3; ++a) F[3 * j + a] += c * Q[j] * m[a] * im;
                    }
                }
            }
    e_rec *= ke / (2.0 * PI * V);
    if (energy) {
        energy[0] = e_real;
        energy[1] = e_rec;
        energy[2] = -ke * beta / std::sqrt(PI) * q2sum;
        energy[3] = -ke * PI * qsum * qsum / (2.0 * V * beta * beta);
    }
    return 0;
}

/* SC/C_Model_ForceEval/MD_Evaluation_Model.cpp, restated.  Line numbers refer to that file.
 * Every float expression keeps the reference's types: pow(float,int) is evaluated in double and
 * stored to float (:19-20, :105-108), "0.5 * MASS * (...)" is a double product (:144), and the
 * "+-0.5" of the minimum-image rounding is a double (:82-97). */
int orc_cmodel_run(int n, int iters, float box, float cutoff, float *pos, float *vel,
                   float *energy, int *counts) {
    const float EPS = 1.995996 * 1.995996;               /* :17 */
    const float SIGMA = 0.1675 * 2;                      /* :18 */
    const float SIGMA_12 = pow((double)SIGMA, 12.0);     /* :19 */
    const float SIGMA_6 = pow((double)SIGMA, 6.0);       /* :20 */
    const float Ar_weight = 39.95f, Nav = 6.022e23f;     /* :15-16 */
    const float MASS = Ar_weight / Nav / 1000;           /* :21 */
    const float DT = 2E-15;                              /* :22 */
    const float CUTOFF_RADIUS_2 = cutoff * cutoff;       /* :24 */
    const float bx = box, by = box, bz = box;            /* :26-28 */
    std::vector<float> F(3 * (size_t)n);
    for (int it = 0; it < iters; ++it) {                 /* :57 */
        float System_Energy = 0;
        float System_Kinetic_Energy = 0;
        for (int i = 0; i < n; ++i) {                    /* :63 */
            float Evdw_acc = 0, Fx_acc = 0, Fy_acc = 0, Fz_acc = 0;
            const float rx = pos[3 * i], ry = pos[3 * i + 1], rz = pos[3 * i + 2];
            int nb = 0;
            for (int j = 0; j < n; ++j) {                /* :72 */
                float dx = rx - pos[3 * j];
                float dy = ry - pos[3 * j + 1];
                float dz = rz - pos[3 * j + 2];
                if (dx >= 0) dx -= bx * (int)((double)(dx / bx) + 0.5);   /* :81-86 */
                else dx -= bx * (int)((double)(dx / bx) - 0.5);
                if (dy >= 0) dy -= by * (int)((double)(dy / by) + 0.5);
                else dy -= by * (int)((double)(dy / by) - 0.5);
                if (dz >= 0) dz -= bz * (int)((double)(dz / bz) + 0.5);
                else dz -= bz * (int)((double)(dz / bz) - 0.5);
                const float r2 = dx * dx + dy * dy + dz * dz;            /* :99 */
                if (r2 > 0 && r2 <= CUTOFF_RADIUS_2) {                    /* :101 */
                    nb++;
                    const float inv_r2 = 1 / r2;
                    const float inv_r8 = pow((double)inv_r2, 4.0);
                    const float inv_r14 = pow((double)inv_r2, 7.0);
                    const float inv_r6 = pow((double)inv_r2, 3.0);
                    const float inv_r12 = pow((double)inv_r2, 6.0);
                    const float vdw12 = 4 * EPS * SIGMA_12 * inv_r12;
                    const float vdw6 = 4 * EPS * SIGMA_6 * inv_r6;
                    const float vdw14 = 48 * EPS * SIGMA_12 * inv_r14;
                    const float vdw8 = 24 * EPS * SIGMA_6 * inv_r8;
                    const float Fvdw = vdw14 - vdw8;
                    const float Evdw = vdw12 - vdw6;
                    Fx_acc += Fvdw * dx;
                    Fy_acc += Fvdw * dy;
                    Fz_acc += Fvdw * dz;
                    Evdw_acc += Evdw;
                }
            }
            if (counts) counts[i] = nb;
            F[3 * i] = Fx_acc; F[3 * i + 1] = Fy_acc; F[3 * i + 2] = Fz_acc;
            const float ax = Fx_acc / MASS, ay = Fy_acc / MASS, az = Fz_acc / MASS;  /* :133-135 */
            float vx = vel[3 * i], vy = vel[3 * i + 1], vz = vel[3 * i + 2];
            vx += ax * DT; vy += ay * DT; vz += az * DT;                            /* :140-142 */
            const float Ek = 0.5 * (double)MASS * (double)(vx * vx + vy * vy + vz * vz); /* :144 */
            vel[3 * i] = vx; vel[3 * i + 1] = vy; vel[3 * i + 2] = vz;
            System_Energy += Evdw_acc;
            System_Kinetic_Energy += Ek;
        }
        System_Energy = (double)System_Energy * 0.5;                                /* :157 */
        energy[2 * it] = System_Energy;
        energy[2 * it + 1] = System_Kinetic_Energy;
        for (int i = 0; i < n; ++i) {                                               /* :164 */
            float px = pos[3 * i], py = pos[3 * i + 1], pz = pos[3 * i + 2];
            px += vel[3 * i] * DT; py += vel[3 * i + 1] * DT; pz += vel[3 * i + 2] * DT;
            if (px < 0) px += bx; else if (px >= bx) px -= bx;                      /* :177-197 */
            if (py < 0) py += by; else if (py >= by) py -= by;
            if (pz < 0) pz += bz; else if (pz >= bz) pz -= bz;
            pos[3 * i] = px; pos[3 * i + 1] = py; pos[3 * i + 2] = pz;
        }
    }
    return 1;
}

}  /* extern "C" */
