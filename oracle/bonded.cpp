/*
 * bonded.cpp — FP64 restatement of the bonded terms (bond, angle with Urey-Bradley, dihedral).
 *
 * TEST INFRASTRUCTURE ONLY (see oracle.h): the checker of libmdrl's bonded kernel.
 *
 * The reference evaluates bonded terms in its own engine (Bonded/Bonded_Top.v), whose units
 * state the ProtoMol (CHARMM-style) algorithm in their comments and then implement parts of it
 * with constants baked in: Bonded/calc_bond_v2.v:40-95 (harmonic bond, F1 = -(dU/dr / r) r12,
 * F2 = -F1), Bonded/calc_angle_v2.v:55-290 (harmonic angle theta = atan2(|r12 x r32|, r12.r32),
 * dtheta1 = (r12^ cos - r32^) / (sin d12), plus a Urey-Bradley 1-3 spring) and
 * Bonded/calcTorsion_v2.v:70-285 (phi = -atan2(c.b, a.b) from the plane normals
 * a = r12 x r23, b = r23 x r34, c = r23 x a; k (1 + cos(n phi + delta)) for n > 0, k (phi -
 * delta)^2 with the difference wrapped into [-pi, pi] for n = 0).  No golden values exist for
 * these units, so this restatement follows the stated algorithm and is checked by properties
 * (finite differences of the energy, zero net force and torque, closed-form cases).
 *
 * The dihedral gradient is Blondel & Karplus, J. Comput. Chem. 17 (1996) 1132: with F = r1 - r2,
 * G = r2 - r3, H = r4 - r3, A = F x G, B = H x G, their phi (cos = A.B / |A||B|, sin =
 * (B x A).G / |A||B||G|) equals ProtoMol's -atan2(c.b, a.b), and
 *   dphi/dr1 = -|G|/A^2 A,  dphi/dr4 = |G|/B^2 B,
 *   dphi/dr2 = |G|/A^2 A + (F.G)/(A^2 |G|) A - (H.G)/(B^2 |G|) B,
 *   dphi/dr3 = -|G|/B^2 B - (F.G)/(A^2 |G|) A + (H.G)/(B^2 |G|) B.
 *
 * Vectors between bonded atoms take the one-wrap periodic rule per axis when box[d] > 0 (the
 * reference's bonded engine uses raw differences; the two agree whenever a term does not straddle
 * the box boundary).  Degenerate geometry (a zero bond length, an angle of 0 or pi, collinear
 * dihedral atoms) contributes no force, as in the GPU kernel.
 */
#include "oracle.h"

#include <math.h>

namespace {

struct V3 {
    double x, y, z;
};
inline V3 operator-(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 operator+(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V3 operator*(double s, V3 a) { return {s * a.x, s * a.y, s * a.z}; }
inline double dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline V3 cross(V3 a, V3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }

inline double wrap1(double d, double L) {
    if (L <= 0.0) return d;
    if (d > 0.5 * L) return d - L;
    if (d < -0.5 * L) return d + L;
    return d;
}

struct Ctx {
    const double *x, *y, *z;
    double L[3];
    double *F;
    V3 diff(int i, int j) const {
        return {wrap1(x[i] - x[j], L[0]), wrap1(y[i] - y[j], L[1]), wrap1(z[i] - z[j], L[2])};
    }
    void add(int i, V3 f) const {
        F[3 * i] += f.x;
        F[3 * i + 1] += f.y;
        F[3 * i + 2] += f.z;
    }
};

constexpr double kPi = 3.14159265358979323846;

}  // namespace

extern "C" int orc_bonded64(int n, const double *x, const double *y, const double *z, const double box[3],
                            const orc_bonded *b, double *F, double *E) {
    if (n < 0 || !b || !F || !E || (n > 0 && (!x || !y || !z))) return -1;
    Ctx c{x, y, z, {box ? box[0] : 0.0, box ? box[1] : 0.0, box ? box[2] : 0.0}, F};
    for (int k = 0; k < 3 * n; ++k) F[k] = 0.0;
    E[0] = E[1] = E[2] = 0.0;
    auto ok = [n](int a) { return a >= 0 && a < n; };

    for (int t = 0; t < b->nb; ++t) {
        const int i = b->bond_atoms[2 * t], j = b->bond_atoms[2 * t + 1];
        if (!ok(i) || !ok(j)) return -2;
        const double k = b->bond_par[2 * t], r0 = b->bond_par[2 * t + 1];
        const V3 r = c.diff(i, j);
        const double d = sqrt(dot(r, r));
        E[0] += k * (d - r0) * (d - r0);
        if (d > 0.0) {
            const V3 fi = (-2.0 * k * (d - r0) / d) * r;
            c.add(i, fi);
            c.add(j, -1.0 * fi);
        }
    }

    for (int t = 0; t < b->na; ++t) {
        const int i = b->angle_atoms[3 * t], j = b->angle_atoms[3 * t + 1], l = b->angle_atoms[3 * t + 2];
        if (!ok(i) || !ok(j) || !ok(l)) return -2;
        const double kt = b->angle_par[4 * t], t0 = b->angle_par[4 * t + 1];
        const double kub = b->angle_par[4 * t + 2], s0 = b->angle_par[4 * t + 3];
        const V3 r12 = c.diff(i, j), r32 = c.diff(l, j);
        const V3 r13 = r12 - r32;
        const double d12 = sqrt(dot(r12, r12)), d32 = sqrt(dot(r32, r32)), d13 = sqrt(dot(r13, r13));
        const V3 cr = cross(r12, r32);
        const double crn = sqrt(dot(cr, cr)), dt = dot(r12, r32);
        const double theta = atan2(crn, dt);
        E[1] += kt * (theta - t0) * (theta - t0) + kub * (d13 - s0) * (d13 - s0);
        V3 f1{0, 0, 0}, f3{0, 0, 0};
        if (d12 > 0.0 && d32 > 0.0) {
            const double sn = crn / (d12 * d32), cs = dt / (d12 * d32);
            if (sn > 1e-6) {
                const double dpot = 2.0 * kt * (theta - t0);
                const V3 u12 = (1.0 / d12) * r12, u32 = (1.0 / d32) * r32;
                f1 = (-dpot / (sn * d12)) * (cs * u12 - u32);
                f3 = (-dpot / (sn * d32)) * (cs * u32 - u12);
            }
        }
        if (kub != 0.0 && d13 > 0.0) {
            const V3 ub = (2.0 * kub * (d13 - s0) / d13) * r13;
            f1 = f1 - ub;
            f3 = f3 + ub;
        }
        c.add(i, f1);
        c.add(l, f3);
        c.add(j, -1.0 * (f1 + f3));
    }

    for (int t = 0; t < b->nd; ++t) {
        const int a1 = b->dih_atoms[4 * t], a2 = b->dih_atoms[4 * t + 1];
        const int a3 = b->dih_atoms[4 * t + 2], a4 = b->dih_atoms[4 * t + 3];
        if (!ok(a1) || !ok(a2) || !ok(a3) || !ok(a4)) return -2;
        const double k = b->dih_par[3 * t], per = b->dih_par[3 * t + 1], delta = b->dih_par[3 * t + 2];
        const V3 Fv = c.diff(a1, a2), G = c.diff(a2, a3), H = c.diff(a4, a3);
        const V3 A = cross(Fv, G), B = cross(H, G);
        const double A2 = dot(A, A), B2 = dot(B, B), Gn = sqrt(dot(G, G));
        if (!(A2 > 1e-12) || !(B2 > 1e-12) || !(Gn > 1e-6)) continue;
        const double ab = sqrt(A2 * B2);
        const double cosp = dot(A, B) / ab, sinp = dot(cross(B, A), G) / (ab * Gn);
        const double phi = atan2(sinp, cosp);
        double dpot;
        if (per > 0.0) {
            E[2] += k * (1.0 + cos(per * phi + delta));
            dpot = -k * per * sin(per * phi + delta);
        } else {
            double diff = phi - delta;
            if (diff < -kPi) diff += 2.0 * kPi;
            else if (diff > kPi) diff -= 2.0 * kPi;
            E[2] += k * diff * diff;
            dpot = 2.0 * k * diff;
        }
        const double fg = dot(Fv, G), hg = dot(H, G);
        const V3 d1 = (-Gn / A2) * A, d4 = (Gn / B2) * B;
        const V3 d2 = ((Gn / A2) * A + (fg / (A2 * Gn)) * A) - (hg / (B2 * Gn)) * B;
        const V3 d3 = ((-Gn / B2) * B - (fg / (A2 * Gn)) * A) + (hg / (B2 * Gn)) * B;
        c.add(a1, -dpot * d1);
        c.add(a2, -dpot * d2);
        c.add(a3, -dpot * d3);
        c.add(a4, -dpot * d4);
    }
    return 0;
}
