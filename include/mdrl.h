/*
 * mdrl.h — C ABI of libmdrl, a GB300 (sm_103a) implementation of the range-limited (RL)
 * non-bonded force path of the SC2019-MD design: cell-list binning, half-shell pair generation
 * (home cell + 13 neighbour cells), the 0 < r2 <= rc2 filter, LJ r^-14 / r^-8 plus Coulomb r^-3
 * from interpolation tables indexed by the r2 bit pattern, Newton's-third-law force accumulation
 * in deterministic int64 fixed point, and the motion update.
 *
 * Plain C: pointers, sizes and status codes only.  Every call returns an mdrl_status; the text
 * of the last error on the calling thread is available from mdrl_last_error().  No call exits the
 * process or throws across the ABI.
 *
 * Threading: one context per host thread.  Calls on one context are serialised by the caller;
 * distinct contexts may be used concurrently from different threads (each owns its own CUDA
 * stream and device buffers).
 *
 * Reference interfaces replaced (paths within the reference project):
 *   int MD_Evaluation_Model()                 Range_Limited/C_Model_ForceEval/MD_Evaluation_Model.h:1
 *                                             (.cpp:9-205)  -> MD_Evaluation_Model() below
 *   float4 RL_LJ_Evaluation(int2, float4, float4)
 *                                             Range_Limited_demo/SourceCode/OpenCL_HDL_Lib/
 *                                             RL_LJ_Evaluation.h:1 (.xml:5-45)  -> mdrl_pair_eval
 *   the RL force path of the MATLAB golden model
 *                                             MatlabScripts/FullScale_Simulation_LJArgon.m:356-1164
 *                                             -> mdrl_force_eval / mdrl_step
 */
#ifndef MDRL_H
#define MDRL_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MDRL_MAX_TYPES 16

typedef enum {
    MDRL_OK = 0,
    MDRL_ERR_INVALID_ARG = 1,   /* a parameter or input failed validation */
    MDRL_ERR_CELL_OVERFLOW = 2, /* a cell holds more particles than the kernels can stage */
    MDRL_ERR_RANGE = 3,         /* rc > L/2, fewer than 3 cells per dimension, table range */
    MDRL_ERR_CUDA = 4,          /* a CUDA runtime call failed */
    MDRL_ERR_TIMEOUT = 5,       /* a bounded device-side wait gave up */
    MDRL_ERR_STATE = 6          /* call order: e.g. mdrl_step before mdrl_set_state */
} mdrl_status;

/* Force accumulation. */
enum {
    MDRL_ACC_FIXED64 = 0,   /* FP32 partial sums in a fixed traversal order, int64 2^-24 atomics:
                               bit-reproducible run to run */
    MDRL_ACC_FP32_ATOMIC = 1, /* FP32 atomics ("plain"): order-dependent rounding */
    MDRL_ACC_KAHAN = 2      /* FP32 partial sums in a fixed order, then a compensated FP32 global
                               sum (high + low planes, TwoSum error of every atomic) */
};

/* Per-pair arithmetic. */
enum {
    MDRL_ARITH_FMA = 0,      /* c1*r2 + c0 and the force combination as fused multiply-adds */
    MDRL_ARITH_SEPARATE = 1  /* every multiply and add rounded separately, as the reference's
                                golden vectors (MATLAB polyval in single precision) */
};

/* Pair function evaluation. */
enum {
    MDRL_EVAL_TABLE = 0,  /* polynomial tables indexed by the r2 bit pattern */
    MDRL_EVAL_DIRECT = 1  /* FP32 powers of 1/r2 */
};

/* Motion update. */
enum {
    MDRL_INT_VELOCITY_VERLET = 0, /* kick(dt/2) drift(dt) rebin force kick(dt/2) */
    MDRL_INT_EULER = 1            /* v += a dt; x += v dt (the reference's symplectic Euler,
                                     MD_Evaluation_Model.cpp:133-150,164-202) */
};

/* Flags. */
#define MDRL_FLAG_ENERGY 0x1u      /* evaluate LJ / Coulomb energy and the virial every step */
#define MDRL_FLAG_PAIR_COUNTS 0x2u /* count partners per particle (pair-list parity) */
#define MDRL_FLAG_NO_PBC 0x4u      /* no periodic wrap of pair differences (mdrl_pair_eval) */
/* Pair differences as the exact minimum-image difference rounded once: the box edge is taken off
 * the coordinate on the far (high) side first, which is exact, so a pair across the boundary
 * keeps FP32 relative precision in d.  Without the flag the reference's datapath is used,
 * d = fl(fl(xi - xj) -+ L) (SC/r2_compute_with_pbc.v:81-127; MD_Evaluation_Model.cpp:77-99),
 * whose first rounding is an absolute error up to ulp(L)/2; its pair list is the reference's
 * bit for bit.  The two rules give the same pair set except for pairs within a few ulps of rc.
 * Fused arithmetic (MDRL_ARITH_FMA) only; single-system contexts and mdrl_force_eval_static. */
#define MDRL_FLAG_EXACT_DIFF 0x8u

typedef struct {
    double box[3];         /* periodic box edges, Angstrom; positions live in [0, box) */
    double cutoff;         /* rc, Angstrom; pairs with 0 < r2 <= rc^2 interact */
    int ncell[3];          /* cells per dimension; 0 = floor(box / cutoff) */
    int ntypes;            /* 1..MDRL_MAX_TYPES */
    double sigma[MDRL_MAX_TYPES];   /* Angstrom */
    double epsilon[MDRL_MAX_TYPES]; /* kcal/mol */
    double mass[MDRL_MAX_TYPES];    /* amu */
    double coulomb_k;      /* kcal*Angstrom/(mol*e^2); 0 = LJ only */
    int table_order;       /* 1..3 (polynomial order of each bin) */
    int table_bins;        /* bins per power-of-two segment: power of two, 16..4096 */
    int table_min_log2;    /* the first segment starts at r2 = 2^table_min_log2 */
    int eval;              /* MDRL_EVAL_* */
    int arith;             /* MDRL_ARITH_* */
    int accum;             /* MDRL_ACC_* */
    int integrator;        /* MDRL_INT_* */
    double dt_fs;          /* time step, fs */
    uint32_t flags;        /* MDRL_FLAG_* */
    int device;            /* CUDA device ordinal */
} mdrl_params;

typedef struct {
    int64_t pairs;          /* unique pairs with 0 < r2 <= rc2 in the last force evaluation */
    int64_t candidates;     /* candidate pairs tested by the half-shell traversal */
    int64_t below_table;    /* pairs evaluated at the first table point (r2 below the table) */
    int max_cell_occupancy;
    int ncells;
    double e_lj, e_coul;    /* kcal/mol (MDRL_FLAG_ENERGY) */
    double virial;          /* sum over pairs of fscal*r2, kcal/mol (MDRL_FLAG_ENERGY) */
    double kinetic;         /* kcal/mol, after the last step */
    double device_ms;       /* device time of the last call, CUDA events */
    int64_t pairs_total;    /* pairs summed over every force evaluation of the last call */
    double force_ms;        /* device time of the last half-shell force kernel, CUDA events */
    double e_bond, e_angle, e_dihedral; /* bonded-term energies, kcal/mol (MDRL_FLAG_ENERGY) */
} mdrl_stats;

typedef struct mdrl_ctx mdrl_ctx;

/* Tile of the half-shell force kernel.  Either the CTA kernel: warps per CTA (4, or 8 with
 * MDRL_ACC_FIXED64 outside a batch), j-steps of 8 particles per work piece (1..32), and whether a
 * unit first drops the (32-i, 8-j) blocks whose bounding boxes are beyond rc (exact; pays with
 * many particles per cell or cells well above rc).  Or, with warps_per_cta = 1 (MDRL_ACC_FIXED64,
 * also in batches), one warp per work item: steps_per_piece (1..4) is then the number of i-tile
 * groups each unit is split into, and prune_steps must be 1 (the kernel always prunes).
 * Default {4, 6, 0}; mdrl_autotune picks among both kinds. */
typedef struct {
    int warps_per_cta;
    int steps_per_piece;
    int prune_steps;
} mdrl_tile;

/* Library identity and the last error text of the calling thread ("" when none). */
const char *mdrl_version(void);
const char *mdrl_last_error(void);

/* The 14 half-shell cell offsets the force kernel traverses, offsets[14*3] = (dx, dy, dz), in the
 * reference's filter order (home cell first); host only. */
void mdrl_halfshell_offsets(int *offsets);

/* Fill *p with defaults: 1 type of argon (sigma 3.4, epsilon 0.238, 39.95 amu), rc 8.5,
 * first-order 256-bin tables from 2^-2, FMA arithmetic, fixed-point accumulation,
 * velocity Verlet at 2 fs, device 0. */
void mdrl_default_params(mdrl_params *p);

/* Fit the unit-prefactor tables on the host in FP64 (no GPU needed): coef receives 6 functions
 * (r^-14, r^-8, r^-3, r^-12, r^-6, r^-1 as powers of r2) x (order+1) planes x nseg*bins, plane k
 * holding the coefficient of r2^k of each bin's least-squares polynomial through `samples`
 * equally spaced points (the reference uses 8). */
mdrl_status mdrl_fit_tables(int order, int nseg, int bins, int min_log2, int samples, float *coef);

/* Table polynomial forms (mdrl_set_tables' flags, mdrl_get_table_form). */
#define MDRL_TABLE_RAW 0x1        /* the coefficients carry their physical prefactors */
#define MDRL_TABLE_BIN_LOCAL 0x2  /* plane k holds the coefficient of u^k, u = r2 - (start of r2's
                                     bin); orders 2-3.  u is exact in FP32, so the polynomial has
                                     no cancellation between large monomial terms.  The library
                                     fits its own order-2 and order-3 tables in this form. */

/* The same fit in the bin-local form (MDRL_TABLE_BIN_LOCAL): plane k holds the coefficient of
 * u^k.  No counterpart in the reference, whose tables are monomial in r2. */
mdrl_status mdrl_fit_tables_bin_local(int order, int nseg, int bins, int min_log2, int samples, float *coef);

/* Create / destroy a context.  Validates the parameters, builds the FP64-fitted tables and
 * uploads them; device buffers for particles are sized on first use. */
mdrl_status mdrl_create(const mdrl_params *p, mdrl_ctx **out);
mdrl_status mdrl_destroy(mdrl_ctx *ctx);

/* Replace the generated tables, e.g. with the reference's ROM images.  coef holds nfunc
 * functions (2: r^-14, r^-8; 3: + r^-3; 6: + r^-12, r^-6, r^-1), each as (order+1) planes of
 * nseg*bins coefficients, plane k holding the coefficient of r2^k.  flags (MDRL_TABLE_*):
 * MDRL_TABLE_RAW (the value 1 of the earlier raw_coefficients argument) when the tables already
 * carry their physical prefactors (as the reference's do) -- the per-type multipliers become
 * A = 1, B = -1, ke*qi*qj unchanged; MDRL_TABLE_BIN_LOCAL when the planes are coefficients of
 * u = r2 - bin start (orders 2-3 only). */
mdrl_status mdrl_set_tables(mdrl_ctx *ctx, int order, int nseg, int bins, int min_log2, int nfunc,
                            const float *coef, int flags);

/* The MDRL_TABLE_* flags of the tables in use. */
mdrl_status mdrl_get_table_form(mdrl_ctx *ctx, int *flags);

/* Read back the tables in use (same layout as mdrl_set_tables with nfunc = 6; the form from
 * mdrl_get_table_form).  Pass coef = NULL to query the sizes. */
mdrl_status mdrl_get_tables(mdrl_ctx *ctx, int *order, int *nseg, int *bins, int *min_log2,
                            float *coef);

/* Read back the per-type-pair multipliers in use: [ntypes*ntypes*4] = A14, B8, A12, B6 with the
 * B terms negative (A14 = 48*eps*sig^12, B8 = -24*eps*sig^6, A12 = 4*eps*sig^12,
 * B6 = -4*eps*sig^6, Lorentz-Berthelot mixing). */
mdrl_status mdrl_get_pair_coefficients(mdrl_ctx *ctx, float *coef);

/* Replace the per-type-pair multipliers (no counterpart in the reference, whose single LJ type
 * is baked into its tables): coef[ntypes*ntypes*4] = A14, B8, A12, B6 in FP64 (stored as FP32),
 * e.g. from an Amber topology's E = A/r^12 - B/r^6: A14 = 12A, B8 = -6B, A12 = A, B6 = -B.
 * The matrix should be symmetric for Newton's third law to hold. */
mdrl_status mdrl_set_pair_coefficients(mdrl_ctx *ctx, const double *coef);

/* Bonded terms, evaluated after the pair forces of every mdrl_force_eval / mdrl_set_state /
 * mdrl_step and added to the same accumulators (replaces the reference's bonded engine,
 * Bonded/Bonded_Top.v:57-396, whose forces its summation logic adds to the range-limited ones;
 * per-term units Bonded/calc_bond_v2.v:16-127, calc_angle_v2.v:10-311, calcTorsion_v2.v:1-443,
 * which take their parameters from the term packets documented at Bonded_Top.v:30-44).  Atoms are
 * user indices.  Per term:
 *   bond      atoms {i, j},       params {k, r0}:                E = k (r - r0)^2
 *   angle     atoms {i, j, l},    params {k_theta, theta0, k_ub, s0} (j the vertex):
 *             E = k_theta (theta - theta0)^2 + k_ub (|r_il| - s0)^2 (k_ub = 0: no Urey-Bradley)
 *   dihedral  atoms {i, j, k, l}, params {k, n, delta}, n an integer in [0, 12]:
 *             E = k (1 + cos(n phi + delta)) for n > 0, k (phi - delta)^2 (wrapped) for n = 0;
 *             phi is the IUPAC dihedral (trans = pi); several terms may share atoms.
 * Units kcal/mol, Angstrom, radian; vectors take the one-wrap periodic rule (box edge taken off
 * the far coordinate first).  Terms are evaluated in FP32, a bond's stretch r - r0 from a
 * compensated r^2 - r0^2 so that stiff bonds at their rest length keep FP32 relative precision.
 * There are no non-bonded exclusions (the reference has none): bonded atoms also interact
 * through the pair path.  Zero counts remove the terms.  Not available for replica batches. */
mdrl_status mdrl_set_bonded(mdrl_ctx *ctx, int nbonds, const int *bond_atoms, const double *bond_params,
                            int nangles, const int *angle_atoms, const double *angle_params,
                            int ndihedrals, const int *dihedral_atoms, const double *dihedral_params);
mdrl_status mdrl_get_bonded_counts(mdrl_ctx *ctx, int *nbonds, int *nangles, int *ndihedrals);
/* Device time (ms, CUDA events) of one bonded-term launch on the current state, into scratch
 * accumulators (the state is unchanged); 0 work without terms.  Needs mdrl_set_state. */
mdrl_status mdrl_time_bonded(mdrl_ctx *ctx, float *ms);

/* Cell-list binning only (host arrays).  cell_of[n]: cell of each particle,
 * (cx*ny + cy)*nz + cz with c = floor(x / (box/ncell)); cell_count[ncells]; order[n]: particle
 * ids cell by cell, each cell in input order.  Any output may be NULL. */
mdrl_status mdrl_bin(mdrl_ctx *ctx, int n, const float *x, const float *y, const float *z,
                     int *cell_of, int *cell_count, int *order);

/* One force evaluation on host arrays (copies in, evaluates, copies out).  q may be NULL
 * (neutral), type may be NULL (all type 0).  counts[n] (optional) receives each particle's
 * partner count; it requires no flag.  stats may be NULL. */
mdrl_status mdrl_force_eval(mdrl_ctx *ctx, int n, const float *x, const float *y, const float *z,
                            const float *q, const int *type, float *fx, float *fy, float *fz,
                            int *counts, mdrl_stats *stats);

/* The same on device arrays, enqueued on the context's stream and synchronised before return. */
mdrl_status mdrl_force_eval_device(mdrl_ctx *ctx, int n, const float *x, const float *y,
                                   const float *z, const float *q, const int *type, float *fx,
                                   float *fy, float *fz, int *counts, mdrl_stats *stats);

/* Per-pair evaluation, the drop-in for RL_LJ_Evaluation(particle_id, reference_pos,
 * neighbor_pos): for each k < n, ref[4k..4k+3] = (x, y, z, q) and nbr likewise; out[4k..4k+3] =
 * (Fx, Fy, Fz, 0), zero when the pair fails the filter.  type_ref / type_nbr may be NULL (type
 * 0).  aux (optional) [2n] receives (r2, fscal) for every pair.  Host arrays. */
mdrl_status mdrl_pair_eval(mdrl_ctx *ctx, int n, const float *ref, const float *nbr,
                           const int *type_ref, const int *type_nbr, float *out, float *aux);

/* Molecular dynamics on device-resident state.  set_state copies n particles in (velocities
 * may be NULL: zero); step advances nsteps with the configured integrator, rebinning every
 * step; get_state copies positions, velocities and the last forces out in the original particle
 * order (any pointer may be NULL). */
mdrl_status mdrl_set_state(mdrl_ctx *ctx, int n, const float *x, const float *y, const float *z,
                           const float *vx, const float *vy, const float *vz, const float *q,
                           const int *type);
mdrl_status mdrl_step(mdrl_ctx *ctx, int nsteps, mdrl_stats *stats);
mdrl_status mdrl_get_state(mdrl_ctx *ctx, float *x, float *y, float *z, float *vx, float *vy,
                           float *vz, float *fx, float *fy, float *fz);

/* Timing: launch the half-shell force kernel once on the current device state (after
 * mdrl_set_state / mdrl_step) into a scratch accumulator, bracketed by CUDA events on the
 * context's stream; *ms receives the kernel's device time.  The state is not modified. */
mdrl_status mdrl_time_force(mdrl_ctx *ctx, float *ms);

/* ---- spatial decomposition of one system over ranks (slabs of cells along x) ---------------
 * The partition the reference's strong-scaling model describes (MatlabScripts/
 * SC19_MD_Strong_Scale_Performance.m:130-212): each rank owns a slab of whole cell layers along x;
 * the half shell reaches one layer in +x only, so before the force pass a rank imports the first
 * cell layer of the next rank's slab (positions, charges, types: the halo), evaluates every unit
 * whose home cell lies in its slab -- halo particles receive their Newton-3 partial forces -- and
 * returns the halo's int64 forces to their owner, which adds them (exact integer sums: the
 * decomposed forces equal the single-domain ones bit for bit when each cell keeps its particles
 * in the same relative order).  Host-side planning only; the exchange is the caller's (NCCL,
 * MPI, ...).  No counterpart in the reference's code, which runs on one FPGA. */
typedef struct {
    int nranks, rank;
    int x0, x1;        /* owned cell layers [x0, x1) along x */
    int halo_x;        /* the imported layer: x1 modulo the layer count (the next rank's x0) */
    int import_from;   /* rank owning halo_x: halo positions come from it, its forces go back */
    int export_to;     /* rank that imports this rank's first layer x0 */
    int ncell[3];      /* the cell grid of the whole box (as a context builds it) */
} mdrl_slab;

/* The slab of `rank` among `nranks` (layers split as evenly as possible, every rank at least one;
 * nranks must not exceed the layer count).  Host only. */
mdrl_status mdrl_slab_plan(const mdrl_params *p, int nranks, int rank, mdrl_slab *slab);

/* Which particles (host arrays, any number) this rank owns (cell layer in [x0, x1)) and which of
 * them it exports (layer x0); the cell of a particle is the one the GPU binning assigns.  owned
 * and exported receive indices into x in increasing order; either may be NULL.  Host only. */
mdrl_status mdrl_slab_select(const mdrl_params *p, const mdrl_slab *slab, int n, const float *x,
                             int *owned, int *n_owned, int *exported, int *n_exported);

/* One force evaluation (host or device arrays as mdrl_force_eval) of the units whose home cell
 * lies in layers [home_x0, home_x1) (0 and ncell[0]: all), with the forces returned as the raw
 * int64 accumulators (units of 2^-24 kcal/mol/A, F[3n]: x, y and z planes) so that partial
 * results of several evaluations sum exactly.  MDRL_ACC_FIXED64 only. */
mdrl_status mdrl_force_eval_fixed(mdrl_ctx *ctx, int n, const float *x, const float *y, const float *z,
                                  const float *q, const int *type, int home_x0, int home_x1,
                                  int64_t *F, mdrl_stats *stats);

/* One force evaluation that allocates no memory; it has no counterpart in the reference.
 * For callers that cannot call cudaMalloc (a device owned by another allocator or memory pool,
 * a plugin host that forbids allocations, a loop that cannot pay for a first-use allocation):
 * no context is needed, and all scratch (cell lists, sorted particles, int64 accumulators,
 * reduction slots, tables) lives in one 16 MiB static device array that every GPU loading the
 * library holds until the process exits.  x, y, z, q, type and fx, fy, fz are DEVICE pointers
 * (q and type may be NULL); stream is a cudaStream_t (NULL = the legacy default stream); the
 * call synchronises that stream.  *pairs_out (optional) receives the number of pairs.
 * Limits: n <= 131072, <= 4096 cells, nseg * bins <= 16384, MDRL_ACC_FIXED64 only; beyond them
 * the call returns MDRL_ERR_RANGE.  The call runs on the current device, which must be
 * p->device (else MDRL_ERR_INVALID_ARG).  Every call looks up the array's address in the current
 * CUDA context; the first call in a context (and any call whose table parameters differ from the
 * previous call's) copies the tables in with synchronous host copies, so make it before any stream
 * capture.  All calls share the array and it keeps the last call's contents: calls whose GPU work
 * overlaps race and must be serialised by the caller. */
mdrl_status mdrl_force_eval_static(const mdrl_params *p, int n, const float *x, const float *y,
                                   const float *z, const float *q, const int *type, float *fx,
                                   float *fy, float *fz, int64_t *pairs_out, void *stream);

/* ---- batched independent replicas --------------------------------------------------------
 * No counterpart in the reference (whose path is one system at a time).  A batch holds nrep
 * periodic systems that share the force field of the params (types, cutoff, tables, arithmetic,
 * integrator, dt, flags; box and ncell are per replica); every call covers all of them with one
 * launch per kernel, and mdrl_batch_step replays a captured CUDA graph per step.
 * Arrays are the replicas' particles concatenated in replica order (replica r owns
 * [sum_{s<r} n_s, sum_{s<=r} n_s)), positions in [0, box_r).
 * Replica paths: with at least 3 cells of edge >= rc per axis the half-shell traversal (forces,
 * pair lists and trajectories equal to a single-system context's); with fewer (each box edge
 * must still exceed rc) an all-pairs evaluation, by the one-wrap minimum image when every edge
 * exceeds 2 rc, otherwise over every periodic image within rc.  MDRL_ACC_FIXED64 only. */
typedef struct mdrl_batch mdrl_batch;

typedef struct {
    int n;            /* particles (>= 1) */
    double box[3];    /* periodic box edges, each > cutoff */
} mdrl_replica;

enum { MDRL_PATH_HALF_SHELL = 0, MDRL_PATH_MIN_IMAGE = 1, MDRL_PATH_ALL_IMAGES = 2 };

mdrl_status mdrl_batch_create(const mdrl_params *p, int nrep, const mdrl_replica *reps,
                              mdrl_batch **out);
mdrl_status mdrl_batch_destroy(mdrl_batch *batch);
/* Per replica (arrays of nrep, any may be NULL): the path, cells per axis [3*nrep], and work
 * items of the force launch; *total_items the launch's grid. */
mdrl_status mdrl_batch_layout(mdrl_batch *batch, int *path, int *ncell, int *items, int *total_items);
/* One force evaluation of every replica on host arrays (see mdrl_force_eval). */
mdrl_status mdrl_batch_force_eval(mdrl_batch *batch, const float *x, const float *y, const float *z,
                                  const float *q, const int *type, float *fx, float *fy, float *fz,
                                  int *counts, mdrl_stats *stats);
/* Device-resident MD of every replica (see mdrl_set_state / mdrl_step / mdrl_get_state). */
mdrl_status mdrl_batch_set_state(mdrl_batch *batch, const float *x, const float *y, const float *z,
                                 const float *vx, const float *vy, const float *vz, const float *q,
                                 const int *type);
mdrl_status mdrl_batch_step(mdrl_batch *batch, int nsteps, mdrl_stats *stats);
mdrl_status mdrl_batch_get_state(mdrl_batch *batch, float *x, float *y, float *z, float *vx,
                                 float *vy, float *vz, float *fx, float *fy, float *fz);
/* Per-replica totals (out[nrep]) of the last force evaluation: pairs, below_table, ncells and,
 * with MDRL_FLAG_ENERGY, e_lj, e_coul, virial; kinetic from the current velocities. */
mdrl_status mdrl_batch_replica_stats(mdrl_batch *batch, mdrl_stats *out);
/* Device time of one force launch over the whole batch (see mdrl_time_force). */
mdrl_status mdrl_batch_time_force(mdrl_batch *batch, float *ms);
/* See mdrl_set_pair_coefficients. */
mdrl_status mdrl_batch_set_pair_coefficients(mdrl_batch *batch, const double *coef);

/* ---- long-range electrostatics (smooth particle-mesh Ewald) -------------------------------
 * No counterpart on the reference's RL path, which truncates Coulomb at rc (its Long_Range/ RTL
 * is a partial PME: B-spline coefficients on a 4x4x4 patch, a 16^3 grid, FFT cores).  With PME
 * on, the Coulomb table slots hold the Ewald real-space pair erfc(beta r)/r (the tables are
 * refitted), and every force evaluation, step and energy adds the reciprocal-space part
 * (B-spline charge spreading into an int64 fixed-point grid, 3-D FFTs, the influence function,
 * force gather into the same accumulators) plus the self and neutralising-background energies.
 * e_coul then holds the full Ewald energy; the virial covers the real-space pairs only.
 * Single-system contexts only. */
typedef struct {
    double beta;        /* Ewald splitting (1/A); 0: the beta with erfc(beta rc) = tolerance */
    double tolerance;   /* default 1e-5 */
    double spacing;     /* target grid spacing (A) for axes whose grid is 0; default 1.0 */
    int grid[3];        /* FFT points per axis; 0: from spacing, rounded up to 2^a 3^b 5^c 7^d */
    int order;          /* B-spline order, 4 or 6; default 4 */
} mdrl_pme_params;

void mdrl_default_pme_params(mdrl_pme_params *p);
/* p = NULL switches PME off (and refits the plain Coulomb tables). */
mdrl_status mdrl_set_pme(mdrl_ctx *ctx, const mdrl_pme_params *p);
/* The resolved parameters (beta, grid) and whether PME is on. */
mdrl_status mdrl_get_pme(mdrl_ctx *ctx, mdrl_pme_params *p, int *enabled);

/* ---- tiles and the autotuner ---------------------------------------------------------------
 * No counterpart in the reference.  mdrl_autotune times the force kernel (mdrl_time_force's
 * launch, median of 5) for every candidate tile on the context's current state (call it after
 * mdrl_set_state), keeps the fastest and returns it with its time and the default tile's time.
 * Candidates: warps per CTA {4, 8} (8 with MDRL_ACC_FIXED64 only) x steps per piece
 * {3, 4, 6, 8, 12} x pruning {off, on}.  Results are cached per process under a key of the cell grid, mean cell
 * occupancy (to 1/8), types, table order and bins, arithmetic, accumulation and Coulomb on/off;
 * a cached key is reused without timing unless flags has MDRL_TUNE_RETIME.  When the environment
 * variable MDRL_TUNE_CACHE names a file, results are appended to it and read back by later
 * processes.  The tile is part of the captured step graph, which is re-captured after a change. */
#define MDRL_TUNE_RETIME 1
mdrl_status mdrl_set_tile(mdrl_ctx *ctx, const mdrl_tile *tile);
mdrl_status mdrl_get_tile(mdrl_ctx *ctx, mdrl_tile *tile);
mdrl_status mdrl_autotune(mdrl_ctx *ctx, int flags, mdrl_tile *best, float *best_ms, float *default_ms);
/* The same for a batch (4 warps per CTA; steps per piece and pruning tuned), after
 * mdrl_batch_set_state. */
mdrl_status mdrl_batch_set_tile(mdrl_batch *batch, const mdrl_tile *tile);
mdrl_status mdrl_batch_autotune(mdrl_batch *batch, int flags, mdrl_tile *best, float *best_ms,
                                float *default_ms);

/* Drop-in for the reference C model's entry point.  Reads the argon PDB named by the
 * environment variable MDRL_INPUT (N from MDRL_N, default 500; iterations from MDRL_ITERS,
 * default 100), runs the reference's all-pairs direct FP32 force and symplectic-Euler update on
 * the GPU with the reference's constants and rounding, and prints
 * "Iteration %d, System energy is %f, Kinetic Energy is %f" per iteration to stdout.
 * Returns 1 on success and 0 on error (text in mdrl_last_error()). */
int MD_Evaluation_Model(void);

/* The same run with explicit arguments and no file or stdout: pos[3n] and vel[3n] are updated
 * in place, energy[2*iters] receives (System_Energy, System_Kinetic_Energy) per iteration,
 * counts[n] (optional) the partner counts of the last iteration. */
mdrl_status mdrl_cmodel_run(int n, int iters, float box, float cutoff, float *pos, float *vel,
                            float *energy, int *counts);

#ifdef __cplusplus
}
#endif
#endif /* MDRL_H */
