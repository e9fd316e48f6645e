/*
 * oracle.h — CPU restatement of the reference's range-limited (RL) force path.
 *
 * TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and bench.py's
 * cpu_baseline / reference arm may load this library, and only as the checker or as
 * the timed CPU baseline.  The product library (libmdrl) never links or calls it.
 *
 * What each entry point restates (paths relative to the reference project):
 *   orc_bin            MS/GenInputCellList_LJArgon.m:87-135, MS/FullScale_Simulation_LJArgon.m:211-244
 *   orc_pair_f32       SC/r2_compute_with_pbc.v:81-127 (d = ref - nbr, one +-L wrap),
 *                      SC/Filter_Logic.v:234 / C model MD_Evaluation_Model.cpp:101 (0 < r2 <= rc2),
 *                      SC/RL_LJ_Evaluate_Pairs_1st_Order.v:171-193,409-468 (bit-indexed table,
 *                      c1*r2 + c0, components), SC/RL_Evaluate_Pairs_1st_Order.v:325-395
 *                      (F = (QQ*r3 + B*r8) + A*r14)
 *   orc_force_cells    half-shell cell traversal of MS/FullScale_Simulation_LJArgon.m:369-965
 *                      (home cell + 13 neighbours, Newton's third law to the neighbour)
 *   orc_force_direct64 FP64 direct LJ + Coulomb on the same pair set (the FP64 oracle)
 *   orc_force_tables64 FP64 evaluation of the same table polynomials (isolates FP32 error)
 *   orc_force_allimage every periodic image within rc of every pair, for boxes whose edge lies in
 *                      (rc, 3 rc) where the half shell does not apply (no counterpart in the
 *                      reference, which requires 3 cells per axis; the pair datapath is
 *                      orc_pair_f32's, the forces the FP64 table evaluation of orc_force_tables64)
 *   orc_ewald64        FP64 Ewald sum of the point charges (real space erfc within rc, reciprocal
 *                      space as a direct sum over wave vectors, self and background terms): the
 *                      checker of the long-range (PME) path; no counterpart in the reference, whose
 *                      RL path truncates Coulomb at rc (its Long_Range/ RTL is a partial PME)
 *   orc_cmodel_run     SC/C_Model_ForceEval/MD_Evaluation_Model.cpp:57-203, expression by expression
 *   orc_bonded64       (bonded.cpp) FP64 bond / angle + Urey-Bradley / dihedral terms as stated in
 *                      Bonded/calc_bond_v2.v, calc_angle_v2.v, calcTorsion_v2.v (parity unpinned:
 *                      the reference has no bonded golden values; checked by properties)
 *
 * Parity is pinned by the reference's own fixtures (tests/golden/, see make_golden.py) and by
 * the unmodified reference C model built under oracle/_ref (see build_ref.sh).
 */
#ifndef MDRL_ORACLE_H
#define MDRL_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Table functions, in the order of the coefficient planes of orc_sys.tab. */
enum { ORC_F14 = 0, ORC_F8 = 1, ORC_F3 = 2, ORC_F12 = 3, ORC_F6 = 4, ORC_F1 = 5, ORC_NFUNC = 6 };

typedef struct {
    int n;
    const float *x, *y, *z, *q;
    const int *type;
    float box[3];        /* periodic box edge; a pair difference wraps once when |d| > box/2 */
    int ncell[3];        /* cells per dimension (edge = box/ncell) */
    float rc2;           /* cutoff squared; a pair is kept when 0 < r2 <= rc2 */
    int ntypes;
    const float *pcoef;  /* [ntypes*ntypes*4]: A14, B8, A12, B6 (B terms carry the minus sign) */
    float ke;            /* Coulomb constant; 0 disables the r^-3 / r^-1 terms */
    int eval;            /* 0: tables, 1: direct FP32 powers */
    int arith;           /* 0: fused multiply-add, 1: separately rounded mul and add */
    int order, nseg, bins, min_log2;
    const float *tab;    /* [ORC_NFUNC][order+1][nseg*bins] */
    const double *pcoef64; /* [ntypes*ntypes*4] FP64 mixing coefficients for orc_force_direct64 */
    double ke64;
    int local;           /* tables: 0 monomial in r2, 1 coefficients of u = r2 - bin start */
    int exact;           /* differences: 0 the reference's fl(fl(xi - xj) -+ L), 1 the exact
                            minimum-image difference rounded once (edge off the high coordinate) */
} orc_sys;

typedef struct {
    int64_t pairs;        /* unique pairs with 0 < r2 <= rc2 */
    int64_t candidates;   /* pairs whose r2 was tested */
    int64_t below_table;  /* pairs with r2 below the first table segment (evaluated clamped) */
    double e_lj, e_coul;  /* potential energy, each pair once */
    double virial;        /* sum over pairs of fscal * r2 */
} orc_stats;

/* Binning.  cell_of[i] = (cx*ny + cy)*nz + cz with c = floor(x / (box/ncell)) clamped into
 * range; cell_start has ncells+1 entries; order[k] lists particle ids cell by cell, each cell in
 * input order (a stable counting sort).  Returns the largest cell occupancy. */
int orc_bin(int n, const float *x, const float *y, const float *z, const float box[3],
            const int ncell[3], int *cell_of, int *cell_start, int *order);

/* One pair, FP32.  Returns 1 when the pair passes the cutoff filter.  out[0..7] =
 * {fx, fy, fz, fscal, r2, e_lj, e_coul, below_table}; the force terms are zero for rejected
 * pairs, r2 is always written. */
int orc_pair_f32(const orc_sys *s, float xi, float yi, float zi, float qi, int ti,
                 float xj, float yj, float zj, float qj, int tj, float *out);

/* Half-shell cell-list force.  F[3n] (double) is the exact-order-free sum of the FP32 per-pair
 * forces; Fabs[3n] the sum of their magnitudes (for rounding bounds); counts[n] the number of
 * partners of each particle.  Any output pointer may be NULL. */
int orc_force_cells(const orc_sys *s, double *F, double *Fabs, int *counts, orc_stats *st);

/* Same pair set, FP64 physics: A/r^14 + B/r^8 + ke*qi*qj/r^3 with exact differences. */
int orc_force_direct64(const orc_sys *s, double *F, orc_stats *st);

/* The half-shell traversal restricted to home cells [hbegin, hend) (hend < 0: all), each pair's
 * FP32 force rounded to 2^-24 fixed point and summed in int64 into F[3n] (x, y, z interleaved):
 * the checker of the spatial decomposition, whose ranks' partial sums must add up to the
 * single-domain result exactly.  Returns the pair count. */
int64_t orc_force_cells_fixed(const orc_sys *s, int hbegin, int hend, int64_t *F);

/* Same pair set, FP64 evaluation of the FP32 table polynomials (index from the FP32 r2). */
int orc_force_tables64(const orc_sys *s, double *F, orc_stats *st);

/* The pieces of the force error, for its decomposition: the same accepted pairs with FP64
 * arithmetic throughout, the differences exact (f32_diff = 0) or the FP32 datapath's rounded
 * d = fl(fl(xi - xj) +- L) (f32_diff = 1), and the pair functions as direct FP64 powers
 * (tables = 0) or the FP32 tables evaluated in FP64 (tables = 1, as orc_force_tables64). */
int orc_force_split64(const orc_sys *s, int f32_diff, int tables, double *F, orc_stats *st);

/* Multi-threaded FP32 half-shell force (the timed CPU baseline) over home cells
 * [hbegin, hend) (hend < 0: all).  F[3n] float.  Returns the number of pairs evaluated. */
int64_t orc_force_cells_mt(const orc_sys *s, int nthreads, int hbegin, int hend, float *F);

/* All-pairs FP32 direct force (the C model's O(N^2) loop generalised to types and charges),
 * multi-threaded over i.  F[3n] float.  Returns the number of (ordered) pairs in cutoff. */
int64_t orc_force_allpairs_mt(const orc_sys *s, int nthreads, float *F);

/* All-image pairs: per axis the candidates fl(xi - xj), fl(. - L), fl(. + L) with
 * fl(d*d) <= rc2; every combination with 0 < r2 <= rc2 (r2 = (dx*dx + dy*dy) + dz*dz in FP32,
 * rounded per operation) is one pair.  Every ordered pair (i, j != i) runs the FP32 datapath from
 * i's side (QQ = (ke*qi)*qj): F32sum[3i..] sums those FP32 forces in FP64 and Fabs their
 * magnitudes, counts[i] the partners.  F is the FP64 table evaluation at the exact difference of
 * each unordered pair (Newton's third law).  Any output may be NULL.  Returns the number of
 * unordered pairs, -1 on error. */
int64_t orc_force_allimage(const orc_sys *s, double *F, double *F32sum, double *Fabs, int *counts,
                           orc_stats *st);

/* Ewald sum in FP64 of the charges s->q at s->x/y/z in the periodic box s->box (tin-foil
 * boundary), prefactor ke = s->ke64:
 *   real       ke sum_{i<j, |r_ij| <= rc} qi qj erfc(beta r)/r   (minimum image; rc^2 = s->rc2 <= (L/2)^2)
 *   reciprocal ke / (2 pi V) sum_{m != 0, |n_a| <= nmax} exp(-pi^2 m^2 / beta^2) / m^2 |S(m)|^2,
 *              m = (n1/L1, n2/L2, n3/L3), S(m) = sum_j q_j exp(2 pi i m . r_j)
 *   self       -ke beta / sqrt(pi) sum q^2
 *   background -ke pi Q^2 / (2 V beta^2)   (Q = sum q; zero for a neutral system)
 * F (n*3, optional) receives the forces of the real and reciprocal parts; energy[4] the four terms.
 * Returns 0, or -1 on bad input. */
int orc_ewald64(const orc_sys *s, double beta, int nmax, double *F, double *energy);

/* The reference C model, restated: n particles (positions pos[3n], velocities vel[3n], both
 * updated in place), iters iterations, box edge and cutoff as given (the reference uses 24 and
 * 8).  energy[2*iters] receives the printed System_Energy and System_Kinetic_Energy of each
 * iteration; counts[n] (optional) the partner count of each particle in the last iteration. */
int orc_cmodel_run(int n, int iters, float box, float cutoff, float *pos, float *vel,
                   float *energy, int *counts);

/* Bonded terms (bonded.cpp).  Parameters per term: bond {k, r0} (E = k (r - r0)^2); angle
 * {k_theta, theta0, k_ub, s0} (E = k_theta (theta - theta0)^2 + k_ub (d13 - s0)^2, atoms i-j-l
 * with j the vertex); dihedral {k, n, delta} (E = k (1 + cos(n phi + delta)) for n > 0,
 * k (phi - delta)^2 wrapped into [-pi, pi] for n = 0).  Units kcal/mol, Angstrom, radian. */
typedef struct {
    int nb;
    const int *bond_atoms;     /* [2 nb] */
    const double *bond_par;    /* [2 nb] */
    int na;
    const int *angle_atoms;    /* [3 na] */
    const double *angle_par;   /* [4 na] */
    int nd;
    const int *dih_atoms;      /* [4 nd] */
    const double *dih_par;     /* [3 nd] */
} orc_bonded;

/* FP64 bonded forces F[3n] (overwritten) and energies E[3] = {bonds, angles, dihedrals}; box
 * edges > 0 wrap each difference once.  Returns 0, or < 0 on bad arguments / atom indices. */
int orc_bonded64(int n, const double *x, const double *y, const double *z, const double box[3],
                 const orc_bonded *b, double *F, double *E);

#ifdef __cplusplus
}
#endif
#endif
