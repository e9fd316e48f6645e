/*
 * mdrl_internal.h — declarations shared by the libmdrl translation units.
 */
#ifndef MDRL_INTERNAL_H
#define MDRL_INTERNAL_H

#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/mdrl.h"

namespace mdrl {

/* Table functions, in the order of the canonical coefficient planes. */
enum { kF14 = 0, kF8 = 1, kF3 = 2, kF12 = 3, kF6 = 4, kF1 = 5, kNumFunc = 6 };

/* Force CTA geometry: 8 warps; a warp evaluates a 32 x 32 (i, j) piece as 8 rows x 4 columns
 * of lanes, each lane holding 4 i particles. */
constexpr int kWarps = 8;
constexpr int kThreads = kWarps * 32;
constexpr int kChunk = 256;       /* particles of one cell staged in shared memory at a time */
constexpr int kHalfShellCells = 14;

/* The 14 cells a home cell pairs with, as (dx, dy, dz) cell offsets, in the reference's filter
 * order (SC/Particle_Pair_Gen_HalfShell.v:14-24; MatlabScripts/FullScale_Simulation_LJArgon.m
 * :381-749): in the reference's digits (2 = home, 1/3 = -1/+1) 222, 223, 231, 232, 233, 311, 312,
 * 313, 321, 322, 323, 331, 332, 333; its 8 filters take 222 | 223 | 231 232 | 233 311 |
 * 312 313 | 321 322 | 323 331 | 332 333.  The kernels' constant table is initialised from this. */
#define MDRL_HALFSHELL_OFFSETS                                                                   \
    {{0, 0, 0},  {0, 0, 1},  {0, 1, -1}, {0, 1, 0},  {0, 1, 1},  {1, -1, -1}, {1, -1, 0},         \
     {1, -1, 1}, {1, 0, -1}, {1, 0, 0},  {1, 0, 1},  {1, 1, -1}, {1, 1, 0},   {1, 1, 1}}

/* Fixed-point force scale: 2^24 units per kcal/mol/Angstrom. */
constexpr float kFixScale = 16777216.0f;
constexpr float kFixInv = 5.9604644775390625e-8f;

/* Periodic geometry passed by value to kernels. */
struct Geom {
    float L[3];      /* box edges (0 = no wrap) */
    float h[3];      /* L / 2 */
    float edge[3];   /* cell edges */
    int nc[3];       /* cells per dimension */
    float rc2;
};

/* Per-unit reduction slots written by the force kernel (one unit = home cell x neighbour). */
struct UnitOut {
    double e_lj, e_coul, virial;
    unsigned long long pairs, below;
};

/* Device-side totals. */
struct DevTotals {
    double e_lj, e_coul, virial, kinetic;
    unsigned long long pairs, below, pairs_total;
    int max_occ;
    int pad;
    double e_bond, e_angle, e_dihedral;   /* bonded terms (zero without them) */
};

/* beta > 0: the Coulomb slots hold the Ewald real-space pair (erfc-screened) instead of r^-3, r^-1;
 * local: coefficients of u = r2 - bin start (MDRL_TABLE_BIN_LOCAL) instead of powers of r2 */
void fit_tables(int order, int nseg, int bins, int min_log2, int samples, std::vector<float> *out,
                double beta = 0.0, bool local = false);
void mix_pair_coefficients(const mdrl_params &p, std::vector<float> *pc, std::vector<double> *pc64);

void set_error(const std::string &msg);

/* Host validation of a parameter block (box, cutoff, types, tables, modes, time step); sets the
 * error text and returns INVALID_ARG on the first failure. */
mdrl_status validate_params(const mdrl_params *p);

/* Host-side fault injection for tests of the error paths (no GPU fault is involved).  The
 * environment variable MDRL_FAULT = "[create:]<call>[@k]" is read by mdrl_create (and by
 * mdrl_force_eval_static): the k-th (default first) CUDA runtime call whose source text starts
 * with <call> (e.g. "cudaMemcpyAsync", "cudaGraphLaunch") is not made, and the library reports it
 * as failed with an error text that says "injected".  Without "create:" the count starts when
 * mdrl_create returns, so the fault lands in a later entry point; with it, inside mdrl_create.
 * One fault per arming; an empty or absent variable disarms. */
void fault_arm_from_env(bool at_create);
bool fault_hit(const char *call_text);

/* The status (and error text) for the kernels' error word; MDRL_OK when it is zero. */
mdrl_status device_error_status(unsigned err);

}  // namespace mdrl

#endif
