/*
 * mdrl_bonded.cu — bonded terms (bonds, angles with Urey-Bradley, dihedrals) on sm_103a.
 *
 * The reference evaluates them in a separate engine whose forces are summed with the
 * range-limited ones before the motion update (Bonded/Bonded_Top.v; the units state ProtoMol's
 * algorithm in comments: Bonded/calc_bond_v2.v:40-95, Bonded/calc_angle_v2.v:55-290,
 * Bonded/calcTorsion_v2.v:70-285).  Here one thread evaluates one term in FP32 and adds each
 * atom's force to the same accumulators as the pair kernel (int64 fixed point 2^-24: exact and
 * order-free, so the sum does not depend on the order of the pair and bonded kernels), after the
 * pair kernel and before the kick / unsort.  Terms name atoms by user index; the cell-order
 * position of each user index is rebuilt after every binning (k_invert).
 *
 * Forms, per term (kcal/mol, Angstrom, radian):
 *   bond      E = k (r - r0)^2,                       F_i = -2 k (r - r0) r_ij / r,  F_j = -F_i
 *   angle     E = k_t (theta - theta0)^2 + k_ub (d13 - s0)^2, theta = atan2(|r12 x r32|, r12.r32),
 *             dtheta/dr1 = (cos r12^ - r32^) / (sin d12) (the ProtoMol gradient of the RTL's
 *             comments), the vertex takes minus the sum of the end forces
 *   dihedral  E = k (1 + cos(n phi + delta)) (n > 0), k (phi - delta)^2 with the difference in
 *             [-pi, pi] (n = 0); phi is the IUPAC angle (ProtoMol's -atan2(c.b, a.b)); gradient of
 *             Blondel & Karplus, J. Comput. Chem. 17 (1996) 1132, which has no 1/sin(phi) factor.
 * Vectors between bonded atoms take the one-wrap periodic rule per axis, with the box edge taken
 * off the far coordinate before the difference (bsub1), and a bond's stretch r - r0 comes from a
 * compensated r^2 - r0^2 (norm2_hilo): FP32 terms, but a stiff bond at its rest length (water
 * O-H, 553 kcal/mol/A^2 at 0.9572 A) keeps its force to FP32 precision.  Degenerate geometry (a
 * zero bond length, an angle within 1e-6 of 0 or pi in sine, collinear dihedral atoms) adds no
 * force.  Energies are summed per CTA in FP64 and over CTAs in a fixed order (k_bonded_energy).
 */
#include <math.h>

#include <vector>

#include "mdrl_ctx.cuh"
#include "mdrl_force.cuh"

namespace mdrl {

constexpr int kBondedThreads = 256;

struct BondedState {
    int nb = 0, na = 0, nd = 0;
    int max_atom = -1;
    int2 *d_bi = nullptr;
    float4 *d_bp = nullptr;   /* k, r0, hi and lo parts of r0^2 */
    int4 *d_ai = nullptr;     /* i, j (vertex), l */
    float4 *d_ap = nullptr;   /* k_theta, theta0, k_ub, s0 */
    int4 *d_di = nullptr;
    float4 *d_dp = nullptr;   /* k, n, delta, 0 */
    double *d_epart = nullptr;
    int nblocks = 0;
};

struct BondedDev {
    int nb, na, nd;
    const int2 *bi;
    const float4 *bp;
    const int4 *ai;
    const float4 *ap;
    const int4 *di;
    const float4 *dp;
};

static __global__ void k_invert(int n, const int *__restrict__ pid, int *__restrict__ inv) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) inv[pid[k]] = k;
}

/* a - b with the one-wrap rule decided on fl(a - b), but the box edge taken off the coordinate
 * that lies beyond the half box before the two are subtracted: a - L is exact for a > L/2
 * (Sterbenz), and the final difference is of two small numbers.  Subtracting L from fl(a - b)
 * instead would keep the rounding of the difference of two far-apart coordinates (up to
 * ulp(L)/2), which a stiff bond turns into a force error of 2 k ulp(L)/2. */
__device__ __forceinline__ float bsub1(float a, float b, float L, float h) {
    const float d = __fsub_rn(a, b);
    if (d > h) return __fsub_rn(__fsub_rn(a, L), b);
    if (d < -h) return __fsub_rn(a, __fsub_rn(b, L));
    return d;
}
__device__ __forceinline__ float3 bsub(float4 a, float4 b, const Geom &g) {
    return make_float3(bsub1(a.x, b.x, g.L[0], g.h[0]), bsub1(a.y, b.y, g.L[1], g.h[1]),
                       bsub1(a.z, b.z, g.L[2], g.h[2]));
}
/* s + e = a + b exactly (Knuth's two-sum) */
__device__ __forceinline__ float two_sum(float a, float b, float &e) {
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    return s;
}
/* r^2 of v as an unevaluated sum hi + lo (products split exactly with fma, the sum with two-sum):
 * about twice FP32's precision, so that r^2 - r0^2 of a bond near its rest length keeps its digits */
__device__ __forceinline__ float norm2_hilo(float3 v, float &lo) {
    const float px = __fmul_rn(v.x, v.x), py = __fmul_rn(v.y, v.y), pz = __fmul_rn(v.z, v.z);
    const float ex = __fmaf_rn(v.x, v.x, -px), ey = __fmaf_rn(v.y, v.y, -py), ez = __fmaf_rn(v.z, v.z, -pz);
    float t1, t2;
    const float s1 = two_sum(px, py, t1);
    const float s = two_sum(s1, pz, t2);
    lo = __fadd_rn(__fadd_rn(__fadd_rn(__fadd_rn(t1, t2), ex), ey), ez);
    return s;
}
__device__ __forceinline__ float bdot(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ float3 bcross(float3 a, float3 b) {
    return make_float3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ float3 bscale(float s, float3 a) { return make_float3(s * a.x, s * a.y, s * a.z); }
__device__ __forceinline__ float3 badd(float3 a, float3 b) { return make_float3(a.x + b.x, a.y + b.y, a.z + b.z); }

template <int ACC>
__device__ __forceinline__ void badd_force(unsigned long long *F64, float *F32, int n, int k, float3 f,
                                           unsigned *err) {
    flush_force<ACC>(F64, F32, n, k, f.x, f.y, f.z, err);
}

template <int ACC>
static __global__ void __launch_bounds__(kBondedThreads)
k_bonded(BondedDev b, int n, const int *__restrict__ inv, const float4 *__restrict__ pos, Geom g,
         unsigned long long *__restrict__ F64, float *__restrict__ F32, double *__restrict__ epart,
         unsigned *__restrict__ err) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    float eb = 0.0f, ea = 0.0f, ed = 0.0f;
    if (t < b.nb) {
        const int2 at = b.bi[t];
        const float4 p = b.bp[t];
        const int i = inv[at.x], j = inv[at.y];
        const float3 r = bsub(pos[i], pos[j], g);
        /* d - r0 = (d^2 - r0^2) / (d + r0) with d^2 and r0^2 (host, FP64) as hi + lo pairs: the
         * difference of the hi parts is exact near the rest length, so the stretch of a stiff bond
         * at equilibrium keeps FP32's relative precision instead of ulp(r0) */
        float lo;
        const float hi = norm2_hilo(r, lo);
        const float d = sqrtf(hi);
        const float den = __fadd_rn(d, p.y);   /* 0 only for d = r0 = 0 */
        const float dd = den > 0.0f ? __fadd_rn(__fsub_rn(hi, p.z), __fsub_rn(lo, p.w)) / den : 0.0f;
        eb = p.x * dd * dd;
        if (d > 0.0f) {
            const float3 fi = bscale(-2.0f * p.x * dd / d, r);
            badd_force<ACC>(F64, F32, n, i, fi, err);
            badd_force<ACC>(F64, F32, n, j, bscale(-1.0f, fi), err);
        }
    } else if (t < b.nb + b.na) {
        const int4 at = b.ai[t - b.nb];
        const float4 p = b.ap[t - b.nb];
        const int i = inv[at.x], j = inv[at.y], l = inv[at.z];
        const float4 pj = pos[j];
        const float3 r12 = bsub(pos[i], pj, g), r32 = bsub(pos[l], pj, g);
        const float3 r13 = make_float3(r12.x - r32.x, r12.y - r32.y, r12.z - r32.z);
        const float d12 = sqrtf(bdot(r12, r12)), d32 = sqrtf(bdot(r32, r32)), d13 = sqrtf(bdot(r13, r13));
        const float3 cr = bcross(r12, r32);
        const float crn = sqrtf(bdot(cr, cr)), dt = bdot(r12, r32);
        const float theta = atan2f(crn, dt);
        const float dth = theta - p.y, dub = d13 - p.w;
        ea = p.x * dth * dth + p.z * dub * dub;
        float3 f1 = make_float3(0.f, 0.f, 0.f), f3 = f1;
        if (d12 > 0.0f && d32 > 0.0f) {
            const float sn = crn / (d12 * d32), cs = dt / (d12 * d32);
            if (sn > 1e-6f) {
                const float dpot = 2.0f * p.x * dth;
                const float3 u12 = bscale(1.0f / d12, r12), u32 = bscale(1.0f / d32, r32);
                f1 = bscale(-dpot / (sn * d12), make_float3(cs * u12.x - u32.x, cs * u12.y - u32.y, cs * u12.z - u32.z));
                f3 = bscale(-dpot / (sn * d32), make_float3(cs * u32.x - u12.x, cs * u32.y - u12.y, cs * u32.z - u12.z));
            }
        }
        if (p.z != 0.0f && d13 > 0.0f) {
            const float3 ub = bscale(2.0f * p.z * dub / d13, r13);
            f1 = make_float3(f1.x - ub.x, f1.y - ub.y, f1.z - ub.z);
            f3 = badd(f3, ub);
        }
        badd_force<ACC>(F64, F32, n, i, f1, err);
        badd_force<ACC>(F64, F32, n, l, f3, err);
        badd_force<ACC>(F64, F32, n, j, bscale(-1.0f, badd(f1, f3)), err);
    } else if (t < b.nb + b.na + b.nd) {
        const int4 at = b.di[t - b.nb - b.na];
        const float4 p = b.dp[t - b.nb - b.na];
        const int a1 = inv[at.x], a2 = inv[at.y], a3 = inv[at.z], a4 = inv[at.w];
        const float4 p2 = pos[a2], p3 = pos[a3];
        const float3 Fv = bsub(pos[a1], p2, g), G = bsub(p2, p3, g), H = bsub(pos[a4], p3, g);
        const float3 A = bcross(Fv, G), B = bcross(H, G);
        const float A2 = bdot(A, A), B2 = bdot(B, B), Gn = sqrtf(bdot(G, G));
        if (A2 > 1e-12f && B2 > 1e-12f && Gn > 1e-6f) {
            const float ab = sqrtf(A2 * B2);
            const float cosp = bdot(A, B) / ab, sinp = bdot(bcross(B, A), G) / (ab * Gn);
            const float phi = atan2f(sinp, cosp);
            float dpot;
            if (p.y > 0.0f) {
                const float arg = p.y * phi + p.z;
                ed = p.x * (1.0f + cosf(arg));
                dpot = -p.x * p.y * sinf(arg);
            } else {
                const float pi = 3.14159265358979f;
                float diff = phi - p.z;
                if (diff < -pi) diff += 2.0f * pi;
                else if (diff > pi) diff -= 2.0f * pi;
                ed = p.x * diff * diff;
                dpot = 2.0f * p.x * diff;
            }
            const float fg = bdot(Fv, G), hg = bdot(H, G);
            const float ca = Gn / A2, cb = Gn / B2, sa = fg / (A2 * Gn), sb = hg / (B2 * Gn);
            const float3 d1 = bscale(-ca, A), d4 = bscale(cb, B);
            const float3 d2 = make_float3((ca + sa) * A.x - sb * B.x, (ca + sa) * A.y - sb * B.y, (ca + sa) * A.z - sb * B.z);
            const float3 d3 = make_float3((sb - cb) * B.x - sa * A.x, (sb - cb) * B.y - sa * A.y, (sb - cb) * B.z - sa * A.z);
            badd_force<ACC>(F64, F32, n, a1, bscale(-dpot, d1), err);
            badd_force<ACC>(F64, F32, n, a2, bscale(-dpot, d2), err);
            badd_force<ACC>(F64, F32, n, a3, bscale(-dpot, d3), err);
            badd_force<ACC>(F64, F32, n, a4, bscale(-dpot, d4), err);
        }
    }
    if (!epart) return;
    /* per-CTA energies in FP64, reduced in a fixed order */
    __shared__ double s_e[kBondedThreads / 32][3];
    double e0 = eb, e1 = ea, e2 = ed;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        e0 += __shfl_xor_sync(0xffffffffu, e0, o);
        e1 += __shfl_xor_sync(0xffffffffu, e1, o);
        e2 += __shfl_xor_sync(0xffffffffu, e2, o);
    }
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 0) { s_e[w][0] = e0; s_e[w][1] = e1; s_e[w][2] = e2; }
    __syncthreads();
    if (threadIdx.x < 3) {
        double s = 0.0;
        for (int k = 0; k < kBondedThreads / 32; ++k) s += s_e[k][threadIdx.x];
        epart[3 * blockIdx.x + threadIdx.x] = s;
    }
}

static __global__ void k_bonded_energy(int nblocks, const double *__restrict__ epart, DevTotals *tot) {
    const int lane = threadIdx.x;
    double e[3] = {0.0, 0.0, 0.0};
    for (int b = lane; b < nblocks; b += 32)
        for (int k = 0; k < 3; ++k) e[k] += epart[3 * b + k];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
        for (int k = 0; k < 3; ++k) e[k] += __shfl_xor_sync(0xffffffffu, e[k], o);
    if (lane == 0) { tot->e_bond = e[0]; tot->e_angle = e[1]; tot->e_dihedral = e[2]; }
}

void bonded_free(mdrl_ctx *c) {
    BondedState *s = c->bonded;
    if (!s) return;
    cudaFree(s->d_bi); cudaFree(s->d_bp); cudaFree(s->d_ai); cudaFree(s->d_ap);
    cudaFree(s->d_di); cudaFree(s->d_dp); cudaFree(s->d_epart);
    delete s;
    c->bonded = nullptr;
}

mdrl_status bonded_check_atoms(const mdrl_ctx *c, int n) {
    if (c->bonded && c->bonded->max_atom >= n) {
        set_error("bonded terms name atom " + std::to_string(c->bonded->max_atom) + " but the call has " +
                  std::to_string(n) + " particles");
        return MDRL_ERR_INVALID_ARG;
    }
    return MDRL_OK;
}

mdrl_status bonded_enqueue(mdrl_ctx *c, int n, const float4 *pos, const int *pid, unsigned long long *F64,
                           float *F32, bool energy) {
    BondedState *s = c->bonded;
    if (!s || n <= 0) return MDRL_OK;
    const int nt = s->nb + s->na + s->nd;
    k_invert<<<nblk(n, 256), 256, 0, c->stream>>>(n, pid, c->d_inv);
    const BondedDev b{s->nb, s->na, s->nd, s->d_bi, s->d_bp, s->d_ai, s->d_ap, s->d_di, s->d_dp};
    const int blocks = s->nblocks;
    (void)nt;
    double *ep = energy ? s->d_epart : nullptr;
    switch (c->p.accum) {
    case MDRL_ACC_FP32_ATOMIC:
        k_bonded<1><<<blocks, kBondedThreads, 0, c->stream>>>(b, n, c->d_inv, pos, c->g, F64, F32, ep, c->d_err);
        break;
    case MDRL_ACC_KAHAN:
        k_bonded<2><<<blocks, kBondedThreads, 0, c->stream>>>(b, n, c->d_inv, pos, c->g, F64, F32, ep, c->d_err);
        break;
    default:
        k_bonded<0><<<blocks, kBondedThreads, 0, c->stream>>>(b, n, c->d_inv, pos, c->g, F64, F32, ep, c->d_err);
    }
    MDRL_CUDA(cudaGetLastError());
    return MDRL_OK;
}

mdrl_status bonded_add_energy(mdrl_ctx *c, int n) {
    const BondedState *s = c->bonded;
    if (!s || n <= 0) return MDRL_OK;
    k_bonded_energy<<<1, 32, 0, c->stream>>>(s->nblocks, s->d_epart, c->d_tot);
    MDRL_CUDA(cudaGetLastError());
    return MDRL_OK;
}

}  // namespace mdrl

using namespace mdrl;

template <typename T>
static mdrl_status upload(T **dst, const std::vector<T> &v) {
    if (v.empty()) return MDRL_OK;
    MDRL_CUDA(cudaMalloc(dst, sizeof(T) * v.size()));
    MDRL_CUDA(cudaMemcpy(*dst, v.data(), sizeof(T) * v.size(), cudaMemcpyHostToDevice));
    return MDRL_OK;
}

extern "C" mdrl_status mdrl_set_bonded(mdrl_ctx *c, int nbonds, const int *bond_atoms, const double *bond_params,
                                       int nangles, const int *angle_atoms, const double *angle_params,
                                       int ndihedrals, const int *dihedral_atoms, const double *dihedral_params) {
    if (!c || nbonds < 0 || nangles < 0 || ndihedrals < 0 || (nbonds && (!bond_atoms || !bond_params)) ||
        (nangles && (!angle_atoms || !angle_params)) || (ndihedrals && (!dihedral_atoms || !dihedral_params))) {
        set_error("mdrl_set_bonded: null or invalid argument");
        return MDRL_ERR_INVALID_ARG;
    }
    if ((long long)nbonds + nangles + ndihedrals > (1ll << 30)) {
        set_error("mdrl_set_bonded: too many terms");
        return MDRL_ERR_INVALID_ARG;
    }
    int max_atom = -1;
    auto atoms_ok = [&](const int *a, long long cnt) {
        for (long long k = 0; k < cnt; ++k) {
            if (a[k] < 0) return false;
            max_atom = a[k] > max_atom ? a[k] : max_atom;
        }
        return true;
    };
    auto finite = [](const double *p, long long cnt) {
        for (long long k = 0; k < cnt; ++k)
            if (!std::isfinite(p[k])) return false;
        return true;
    };
    if (!atoms_ok(bond_atoms, 2ll * nbonds) || !atoms_ok(angle_atoms, 3ll * nangles) ||
        !atoms_ok(dihedral_atoms, 4ll * ndihedrals)) {
        set_error("mdrl_set_bonded: negative atom index");
        return MDRL_ERR_INVALID_ARG;
    }
    if (!finite(bond_params, 2ll * nbonds) || !finite(angle_params, 4ll * nangles) ||
        !finite(dihedral_params, 3ll * ndihedrals)) {
        set_error("mdrl_set_bonded: parameters must be finite");
        return MDRL_ERR_INVALID_ARG;
    }
    for (int t = 0; t < ndihedrals; ++t) {
        const double per = dihedral_params[3 * t + 1];
        if (per < 0.0 || per > 12.0 || per != (double)(int)per) {
            set_error("mdrl_set_bonded: dihedral periodicity must be an integer in [0, 12]");
            return MDRL_ERR_INVALID_ARG;
        }
    }
    if (c->have_state && max_atom >= c->n) {
        set_error("mdrl_set_bonded: atom index beyond the state's particles");
        return MDRL_ERR_INVALID_ARG;
    }
    MDRL_CUDA(cudaSetDevice(c->p.device));
    MDRL_CUDA(cudaStreamSynchronize(c->stream));
    bonded_free(c);
    c->graph_n = -1;   /* re-capture the step graphs */
    const long long nt = (long long)nbonds + nangles + ndihedrals;
    if (nt == 0) return MDRL_OK;
    std::vector<int2> bi(nbonds);
    std::vector<float4> bp(nbonds);
    for (int t = 0; t < nbonds; ++t) {
        bi[t] = make_int2(bond_atoms[2 * t], bond_atoms[2 * t + 1]);
        const double r0 = bond_params[2 * t + 1], r0sq = r0 * r0;
        const float hi = (float)r0sq;
        bp[t] = make_float4((float)bond_params[2 * t], (float)r0, hi, (float)(r0sq - (double)hi));
    }
    std::vector<int4> ai(nangles), di(ndihedrals);
    std::vector<float4> ap(nangles), dp(ndihedrals);
    for (int t = 0; t < nangles; ++t) {
        ai[t] = make_int4(angle_atoms[3 * t], angle_atoms[3 * t + 1], angle_atoms[3 * t + 2], 0);
        ap[t] = make_float4((float)angle_params[4 * t], (float)angle_params[4 * t + 1],
                            (float)angle_params[4 * t + 2], (float)angle_params[4 * t + 3]);
    }
    for (int t = 0; t < ndihedrals; ++t) {
        di[t] = make_int4(dihedral_atoms[4 * t], dihedral_atoms[4 * t + 1], dihedral_atoms[4 * t + 2],
                          dihedral_atoms[4 * t + 3]);
        dp[t] = make_float4((float)dihedral_params[3 * t], (float)dihedral_params[3 * t + 1],
                            (float)dihedral_params[3 * t + 2], 0.0f);
    }
    BondedState *s = new BondedState;
    c->bonded = s;
    s->nb = nbonds; s->na = nangles; s->nd = ndihedrals;
    s->max_atom = max_atom;
    s->nblocks = nblk((int)nt, kBondedThreads);
    MDRL_TRY(upload(&s->d_bi, bi)); MDRL_TRY(upload(&s->d_bp, bp));
    MDRL_TRY(upload(&s->d_ai, ai)); MDRL_TRY(upload(&s->d_ap, ap));
    MDRL_TRY(upload(&s->d_di, di)); MDRL_TRY(upload(&s->d_dp, dp));
    MDRL_CUDA(cudaMalloc(&s->d_epart, sizeof(double) * 3 * (size_t)s->nblocks));
    return MDRL_OK;
}

extern "C" mdrl_status mdrl_time_bonded(mdrl_ctx *c, float *ms) {
    if (!c || !ms) { set_error("mdrl_time_bonded: null argument"); return MDRL_ERR_INVALID_ARG; }
    if (!c->have_state) { set_error("mdrl_time_bonded: call mdrl_set_state first"); return MDRL_ERR_STATE; }
    MDRL_CUDA(cudaSetDevice(c->p.device));
    const int n = c->n, a = c->cur;
    /* scratch accumulators: the state's forces stay as they are */
    const bool fp32 = c->p.accum != MDRL_ACC_FIXED64;
    if (fp32 && !c->d_Fscr32) MDRL_TRY(dalloc(&c->d_Fscr32, 6 * (size_t)c->cap));
    if (!fp32 && !c->d_Fscr64) MDRL_TRY(dalloc(&c->d_Fscr64, 3 * (size_t)c->cap));
    if (fp32) MDRL_CUDA(cudaMemsetAsync(c->d_Fscr32, 0, sizeof(float) * 6 * (size_t)n, c->stream));
    else MDRL_CUDA(cudaMemsetAsync(c->d_Fscr64, 0, sizeof(unsigned long long) * 3 * (size_t)n, c->stream));
    MDRL_CUDA(cudaEventRecord(c->ev0, c->stream));
    MDRL_TRY(bonded_enqueue(c, n, c->d_pos[a], c->d_id[a], c->d_Fscr64, c->d_Fscr32, false));
    MDRL_CUDA(cudaEventRecord(c->ev1, c->stream));
    MDRL_CUDA(cudaStreamSynchronize(c->stream));
    MDRL_CUDA(cudaEventElapsedTime(ms, c->ev0, c->ev1));
    return MDRL_OK;
}

extern "C" mdrl_status mdrl_get_bonded_counts(mdrl_ctx *c, int *nbonds, int *nangles, int *ndihedrals) {
    if (!c) { set_error("mdrl_get_bonded_counts: null context"); return MDRL_ERR_INVALID_ARG; }
    const BondedState *s = c->bonded;
    if (nbonds) *nbonds = s ? s->nb : 0;
    if (nangles) *nangles = s ? s->na : 0;
    if (ndihedrals) *ndihedrals = s ? s->nd : 0;
    return MDRL_OK;
}
