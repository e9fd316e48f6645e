/*
 * mdrl_pme.cu — long-range electrostatics by smooth particle-mesh Ewald (PME).
 *
 * No counterpart on the reference's RL path, which truncates Coulomb at rc; its Long_Range/ RTL
 * (coeff64.sv: B-spline basis coefficients of a particle on a 4x4x4 grid patch; Top_Electro.sv:
 * a 16^3 grid and FFT cores) is a partial PME pipeline.  With PME on, the pair kernel's Coulomb
 * table slots hold the Ewald real-space pair (erfc-screened, fitted like the other tables), and
 * every force evaluation adds the reciprocal-space forces of the smooth PME method (Essmann et
 * al., J. Chem. Phys. 103, 8577 (1995)):
 *
 *   spread    Q(k) = sum_i q_i prod_a M_p(u_ia - k_a)  (cardinal B-splines of order p, u = K x / L)
 *             into an int64 fixed-point grid (2^-40 e): exact sums, so the grid does not depend
 *             on the order of the atomic adds;
 *   solve     X = FFT(Q) (cuFFT R2C), X *= G, phi = IFFT(X) (C2R), with
 *             G(m) = ke exp(-pi^2 m^2 / beta^2) / (pi V m^2) * |b1(m1) b2(m2) b3(m3)|^2, G(0) = 0,
 *             E_rec = 1/2 sum_m G(m) |X(m)|^2;
 *   gather    F_i = -q_i sum_k grad_i(prod_a M_p) phi(k), added to the particle's accumulator
 *             (one thread per particle, after the pair kernel's atomics in stream order);
 *   constants E_self = -ke beta / sqrt(pi) sum q^2, E_background = -ke pi Q^2 / (2 V beta^2).
 *
 * The 3-D transforms are cuFFT (a plain library transform, as cuBLAS would be for a plain GEMM);
 * spreading, the influence function, the energy reduction and the gather are kernels here.
 */
#include <cuda_runtime.h>
#include <cufft.h>

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdio>
#include <string>
#include <vector>

#include "mdrl_ctx.cuh"

using namespace mdrl;

namespace mdrl {

constexpr float kPmeFix = 1099511627776.0f;          /* 2^40 grid units per e */
constexpr float kPmeFixInv = 9.094947017729282e-13f; /* 2^-40 */
constexpr int kPmeEnergyBlocks = 256;

struct PmeState {
    mdrl_pme_params p;          /* resolved: beta and grid filled in */
    int K[3] = {0, 0, 0};
    int nreal = 0, ncplx = 0;
    cufftHandle fwd = 0, bwd = 0;
    unsigned long long *d_qfix = nullptr;   /* K0*K1*K2 int64 charge grid */
    float *d_real = nullptr;                /* charge grid, then phi */
    cufftComplex *d_cplx = nullptr;         /* K0*K1*(K2/2+1) */
    float *d_green = nullptr;               /* influence function over the half spectrum */
    double *d_epart = nullptr;              /* [kPmeEnergyBlocks] reciprocal-energy partials */
    double *d_qpart = nullptr;              /* [2 * blocks] sum q, sum q^2 partials */
    int qblocks = 0;
    double volume = 0.0;
};

/* theta[j] = M_p(w + j), dtheta[j] = M_p'(w + j) for j < p (grid point floor(u) - j), w in [0, 1):
 * the cardinal B-spline recursion M_m(x) = (x M_{m-1}(x) + (m - x) M_{m-1}(x - 1)) / (m - 1),
 * M_2(x) = 1 - |x - 1|, and M_m'(x) = M_{m-1}(x) - M_{m-1}(x - 1). */
template <int P>
__device__ __forceinline__ void bspline(float w, float (&th)[P], float (&dth)[P]) {
    float a[P];
#pragma unroll
    for (int j = 0; j < P; ++j) a[j] = 0.0f;
    a[0] = w;
    a[1] = 1.0f - w;
#pragma unroll
    for (int m = 3; m <= P; ++m) {
        if (m == P) {
#pragma unroll
            for (int j = 0; j < P; ++j) dth[j] = a[j] - (j > 0 ? a[j - 1] : 0.0f);
        }
        float b[P];
        const float inv = 1.0f / (float)(m - 1);
#pragma unroll
        for (int j = 0; j < P; ++j) {
            const float x = w + (float)j;
            const float lo = j > 0 ? a[j - 1] : 0.0f;
            b[j] = (j < m ? (x * a[j] + ((float)m - x) * lo) * inv : 0.0f);
        }
#pragma unroll
        for (int j = 0; j < P; ++j) a[j] = b[j];
    }
#pragma unroll
    for (int j = 0; j < P; ++j) th[j] = a[j];
}

struct PmeGeom {
    int K[3];
    float scale[3];   /* K / L */
};

__device__ __forceinline__ int wrapk(int k, int K) { return k < 0 ? k + K : (k >= K ? k - K : k); }

template <int P>
__global__ void k_pme_spread(int n, const float4 *__restrict__ pos, PmeGeom pg,
                             unsigned long long *__restrict__ qfix, double *__restrict__ qpart) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    float q = 0.0f;
    if (i < n) {
        const float4 r = pos[i];
        q = r.w;
        if (q != 0.0f) {
            float th[3][P], dth[P];
            int k0[3];
            const float rr[3] = {r.x, r.y, r.z};
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                const float u = rr[a] * pg.scale[a];
                const float fl = floorf(u);
                /* positions outside [0, L) are reported by the binning; keep the grid index in
                 * range whatever the input (k0 - j stays in [-P, K]) */
                k0[a] = min(max((int)fl, 0), pg.K[a]);
                bspline<P>(fminf(fmaxf(u - fl, 0.0f), 1.0f), th[a], dth);
            }
#pragma unroll
            for (int j0 = 0; j0 < P; ++j0) {
                const int g0 = wrapk(k0[0] - j0, pg.K[0]) * pg.K[1];
                const float q0 = q * th[0][j0];
#pragma unroll
                for (int j1 = 0; j1 < P; ++j1) {
                    const int g1 = (g0 + wrapk(k0[1] - j1, pg.K[1])) * pg.K[2];
                    const float q1 = q0 * th[1][j1];
#pragma unroll
                    for (int j2 = 0; j2 < P; ++j2) {
                        const float v = q1 * th[2][j2];
                        /* v 2^40 is exact in FP32 (a power-of-two scale), so rounding it to an
                         * integer gives the same value as the same product in FP64 would, without
                         * FP64 arithmetic (slow on this part) */
                        atomicAdd(qfix + g1 + wrapk(k0[2] - j2, pg.K[2]),
                                  (unsigned long long)__float2ll_rn(v * kPmeFix));
                    }
                }
            }
        }
    }
    if (qpart) {   /* sum q and sum q^2 of the block, fixed order */
        __shared__ double s[2][256];
        s[0][threadIdx.x] = q;
        s[1][threadIdx.x] = (double)q * (double)q;
        __syncthreads();
        for (int o = 128; o > 0; o >>= 1) {
            if ((int)threadIdx.x < o) { s[0][threadIdx.x] += s[0][threadIdx.x + o]; s[1][threadIdx.x] += s[1][threadIdx.x + o]; }
            __syncthreads();
        }
        if (threadIdx.x == 0) { qpart[2 * blockIdx.x] = s[0][0]; qpart[2 * blockIdx.x + 1] = s[1][0]; }
    }
}

__global__ void k_pme_unfix(int nreal, const unsigned long long *__restrict__ qfix, float *__restrict__ real) {
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nreal; k += gridDim.x * blockDim.x)
        real[k] = (float)(long long)qfix[k] * kPmeFixInv;
}

/* X *= G over the half spectrum; with energy, E partials: entries with 0 < m2 < K2/2 stand for
 * two conjugate entries of the full spectrum. */
__global__ void k_pme_convolve(int ncplx, int K2h, int K2, cufftComplex *__restrict__ X,
                               const float *__restrict__ G, double *__restrict__ epart) {
    double e = 0.0;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < ncplx; k += gridDim.x * blockDim.x) {
        const cufftComplex x = X[k];
        const float g = G[k];
        if (epart) {
            const int m2 = k % K2h;
            const double w = (m2 == 0 || (2 * m2 == K2)) ? 1.0 : 2.0;
            e += w * (double)g * ((double)x.x * x.x + (double)x.y * x.y);
        }
        X[k] = make_cuComplex(x.x * g, x.y * g);
    }
    if (!epart) return;
    __shared__ double s[256];
    s[threadIdx.x] = e;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) s[threadIdx.x] += s[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) epart[blockIdx.x] = 0.5 * s[0];
}

template <int P, int ACC>
__global__ void k_pme_gather(int n, const float4 *__restrict__ pos, PmeGeom pg, const float *__restrict__ phi,
                             unsigned long long *__restrict__ F64, float *__restrict__ F32, unsigned *__restrict__ err) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 r = pos[i];
    if (r.w == 0.0f) return;
    float th[3][P], dth[3][P];
    int k0[3];
    const float rr[3] = {r.x, r.y, r.z};
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const float u = rr[a] * pg.scale[a];
        const float fl = floorf(u);
        k0[a] = min(max((int)fl, 0), pg.K[a]);
        bspline<P>(fminf(fmaxf(u - fl, 0.0f), 1.0f), th[a], dth[a]);
    }
    float fx = 0.0f, fy = 0.0f, fz = 0.0f;
#pragma unroll
    for (int j0 = 0; j0 < P; ++j0) {
        const int g0 = wrapk(k0[0] - j0, pg.K[0]) * pg.K[1];
#pragma unroll
        for (int j1 = 0; j1 < P; ++j1) {
            const int g1 = (g0 + wrapk(k0[1] - j1, pg.K[1])) * pg.K[2];
#pragma unroll
            for (int j2 = 0; j2 < P; ++j2) {
                const float v = __ldg(phi + g1 + wrapk(k0[2] - j2, pg.K[2]));
                fx += dth[0][j0] * th[1][j1] * th[2][j2] * v;
                fy += th[0][j0] * dth[1][j1] * th[2][j2] * v;
                fz += th[0][j0] * th[1][j1] * dth[2][j2] * v;
            }
        }
    }
    fx *= -r.w * pg.scale[0];
    fy *= -r.w * pg.scale[1];
    fz *= -r.w * pg.scale[2];
    if (ACC == MDRL_ACC_FIXED64) {
        check_force(err, fx, fy, fz);
        F64[i] += to_fixed(fx);
        F64[(size_t)n + i] += to_fixed(fy);
        F64[2 * (size_t)n + i] += to_fixed(fz);
    } else {
        /* the high planes; with compensation the low planes take the rounding of the add */
        if (!(isfinite(fx) && isfinite(fy) && isfinite(fz))) atomicOr(err, kErrForce);
        const float add[3] = {fx, fy, fz};
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            float *hi = F32 + (size_t)a * n + i;
            const float s = *hi + add[a];
            if (ACC == MDRL_ACC_KAHAN) {
                const float bb = s - *hi;
                F32[(size_t)(a + 3) * n + i] += (*hi - (s - bb)) + (add[a] - bb);
            }
            *hi = s;
        }
    }
}

/* E_rec + E_self + E_background added to the totals' Coulomb energy (fixed order). */
__global__ void k_pme_energy(int neb, const double *__restrict__ epart, int nqb, const double *__restrict__ qpart,
                             double ke, double beta, double volume, DevTotals *tot) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    double e = 0.0, q = 0.0, q2 = 0.0;
    for (int b = 0; b < neb; ++b) e += epart[b];
    for (int b = 0; b < nqb; ++b) { q += qpart[2 * b]; q2 += qpart[2 * b + 1]; }
    const double pi = 3.14159265358979323846;
    tot->e_coul += e - ke * beta / sqrt(pi) * q2 - ke * pi * q * q / (2.0 * volume * beta * beta);
}

/* ---- host ---------------------------------------------------------------------------------- */

static bool fft_friendly(int k) {
    for (int f : {2, 3, 5, 7})
        while (k % f == 0) k /= f;
    return k == 1;
}

static int grid_points(double L, double spacing, int order) {
    int k = std::max(2 * order, (int)std::ceil(L / spacing));
    while (!fft_friendly(k)) ++k;
    return k;
}

/* |b(m)|^2 of Essmann et al. eq. 4.4 for one axis: 1 / |sum_{k=0}^{p-2} M_p(k+1) e^{2 pi i m k / K}|^2;
 * where the sum vanishes (odd p at m = K/2) the neighbours' mean is used. */
static std::vector<double> bspline_moduli(int K, int p) {
    std::vector<double> M(p + 1, 0.0);   /* M_p at integers 1..p-1 */
    {
        std::vector<double> a(p + 1, 0.0);
        a[1] = 1.0;                       /* M_2(1) = 1, M_2 elsewhere on the integers 0 */
        for (int m = 3; m <= p; ++m) {
            std::vector<double> b(p + 1, 0.0);
            for (int x = 1; x < m; ++x) b[x] = (x * a[x] + (m - x) * a[x - 1]) / (m - 1);
            a = b;
        }
        M = a;
    }
    std::vector<double> out(K);
    const double pi = 3.14159265358979323846;
    for (int m = 0; m < K; ++m) {
        std::complex<double> s(0.0, 0.0);
        for (int k = 0; k <= p - 2; ++k) s += M[k + 1] * std::exp(std::complex<double>(0.0, 2.0 * pi * m * k / K));
        const double d = std::norm(s);
        out[m] = d > 1e-10 ? 1.0 / d : -1.0;
    }
    for (int m = 0; m < K; ++m)
        if (out[m] < 0.0) out[m] = 0.5 * (out[(m + K - 1) % K] + out[(m + 1) % K]);
    return out;
}

static double beta_for(double rc, double tol) {
    double lo = 0.0, hi = 10.0 / rc;
    for (int it = 0; it < 200; ++it) {
        const double mid = 0.5 * (lo + hi);
        if (std::erfc(mid * rc) > tol) lo = mid; else hi = mid;
    }
    return 0.5 * (lo + hi);
}

void pme_free(mdrl_ctx *c) {
    PmeState *s = c->pme;
    if (!s) return;
    if (s->fwd) cufftDestroy(s->fwd);
    if (s->bwd) cufftDestroy(s->bwd);
    dfree(&s->d_qfix); dfree(&s->d_real); dfree(&s->d_cplx); dfree(&s->d_green);
    dfree(&s->d_epart); dfree(&s->d_qpart);
    delete s;
    c->pme = nullptr;
}

#define PME_FFT(call)                                                                     \
    do {                                                                                  \
        cufftResult r_ = (call);                                                          \
        if (r_ != CUFFT_SUCCESS) {                                                        \
            set_error(std::string(#call) + ": cuFFT error " + std::to_string((int)r_));   \
            return MDRL_ERR_CUDA;                                                         \
        }                                                                                 \
    } while (0)

mdrl_status pme_setup(mdrl_ctx *c, const mdrl_pme_params *in) {
    char buf[256];
    mdrl_pme_params p = *in;
    if (p.order != 4 && p.order != 6) { set_error("PME: order must be 4 or 6"); return MDRL_ERR_INVALID_ARG; }
    if (!(c->p.coulomb_k != 0.0)) { set_error("PME: coulomb_k is 0 (no charges to solve for)"); return MDRL_ERR_INVALID_ARG; }
    const double rc = (double)(float)c->p.cutoff;
    if (p.beta <= 0.0) {
        if (!(p.tolerance > 0.0 && p.tolerance < 1.0)) { set_error("PME: tolerance must be in (0, 1)"); return MDRL_ERR_INVALID_ARG; }
        p.beta = beta_for(rc, p.tolerance);
    }
    if (!std::isfinite(p.beta) || p.beta > 100.0) { set_error("PME: beta out of range"); return MDRL_ERR_INVALID_ARG; }
    for (int d = 0; d < 3; ++d) {
        if (p.grid[d] <= 0) {
            if (!(p.spacing > 0.0)) { set_error("PME: spacing must be positive"); return MDRL_ERR_INVALID_ARG; }
            p.grid[d] = grid_points(c->p.box[d], p.spacing, p.order);
        }
        if (p.grid[d] < 2 * p.order || p.grid[d] > 1024) {
            snprintf(buf, sizeof buf, "PME: grid[%d] = %d must be in [2*order, 1024]", d, p.grid[d]);
            set_error(buf);
            return MDRL_ERR_INVALID_ARG;
        }
    }
    pme_free(c);
    PmeState *s = new PmeState();
    c->pme = s;
    s->p = p;
    for (int d = 0; d < 3; ++d) s->K[d] = p.grid[d];
    const int K2h = s->K[2] / 2 + 1;
    s->nreal = s->K[0] * s->K[1] * s->K[2];
    s->ncplx = s->K[0] * s->K[1] * K2h;
    s->volume = c->p.box[0] * c->p.box[1] * c->p.box[2];
    mdrl_status st;
    auto fail = [&](mdrl_status e) { pme_free(c); return e; };
    if ((st = dalloc(&s->d_qfix, (size_t)s->nreal)) != MDRL_OK) return fail(st);
    if ((st = dalloc(&s->d_real, (size_t)s->nreal)) != MDRL_OK) return fail(st);
    if ((st = dalloc(&s->d_cplx, (size_t)s->ncplx)) != MDRL_OK) return fail(st);
    if ((st = dalloc(&s->d_green, (size_t)s->ncplx)) != MDRL_OK) return fail(st);
    if ((st = dalloc(&s->d_epart, (size_t)kPmeEnergyBlocks)) != MDRL_OK) return fail(st);
    /* influence function, FP64 on the host */
    std::vector<double> b[3];
    for (int d = 0; d < 3; ++d) b[d] = bspline_moduli(s->K[d], p.order);
    std::vector<float> G((size_t)s->ncplx);
    const double pi = 3.14159265358979323846, ke = c->p.coulomb_k;
    for (int k0 = 0; k0 < s->K[0]; ++k0)
        for (int k1 = 0; k1 < s->K[1]; ++k1)
            for (int k2 = 0; k2 < K2h; ++k2) {
                const int m0 = k0 <= s->K[0] / 2 ? k0 : k0 - s->K[0];
                const int m1 = k1 <= s->K[1] / 2 ? k1 : k1 - s->K[1];
                const int m2 = k2;
                const double mx = m0 / c->p.box[0], my = m1 / c->p.box[1], mz = m2 / c->p.box[2];
                const double m2s = mx * mx + my * my + mz * mz;
                double g = 0.0;
                if (m2s > 0.0)
                    g = ke * std::exp(-pi * pi * m2s / (p.beta * p.beta)) / (pi * s->volume * m2s) * b[0][k0] * b[1][k1] *
                        b[2][k2];
                G[((size_t)k0 * s->K[1] + k1) * K2h + k2] = (float)g;
            }
    cudaError_t e = cudaMemcpy(s->d_green, G.data(), sizeof(float) * G.size(), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) { set_error(std::string("PME: ") + cudaGetErrorString(e)); return fail(MDRL_ERR_CUDA); }
    if (cufftPlan3d(&s->fwd, s->K[0], s->K[1], s->K[2], CUFFT_R2C) != CUFFT_SUCCESS ||
        cufftPlan3d(&s->bwd, s->K[0], s->K[1], s->K[2], CUFFT_C2R) != CUFFT_SUCCESS ||
        cufftSetStream(s->fwd, c->stream) != CUFFT_SUCCESS || cufftSetStream(s->bwd, c->stream) != CUFFT_SUCCESS) {
        set_error("PME: cuFFT plan creation failed");
        return fail(MDRL_ERR_CUDA);
    }
    return MDRL_OK;
}

/* The reciprocal-space part of one force evaluation, enqueued on the context stream after the
 * pair kernel (pos: the cell-sorted particles the pair kernel used; forces added in place). */
mdrl_status pme_enqueue(mdrl_ctx *c, int n, const float4 *pos, unsigned long long *F64, float *F32, bool energy) {
    PmeState *s = c->pme;
    if (!s || n <= 0) return MDRL_OK;
    PmeGeom pg;
    for (int d = 0; d < 3; ++d) {
        pg.K[d] = s->K[d];
        pg.scale[d] = (float)((double)s->K[d] / c->p.box[d]);
    }
    const int qb = nblk(n, 256);
    if (energy && qb > s->qblocks) {
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        MDRL_CUDA(cudaStreamIsCapturing(c->stream, &cs));
        if (cs != cudaStreamCaptureStatusNone) {
            set_error("PME: energy partials not allocated before graph capture");
            return MDRL_ERR_STATE;
        }
        MDRL_TRY(dalloc(&s->d_qpart, 2 * (size_t)qb));
        s->qblocks = qb;
    }
    MDRL_CUDA(cudaMemsetAsync(s->d_qfix, 0, sizeof(unsigned long long) * s->nreal, c->stream));
    double *qpart = energy ? s->d_qpart : nullptr;
    if (s->p.order == 6) k_pme_spread<6><<<qb, 256, 0, c->stream>>>(n, pos, pg, s->d_qfix, qpart);
    else k_pme_spread<4><<<qb, 256, 0, c->stream>>>(n, pos, pg, s->d_qfix, qpart);
    const int gb = std::min(nblk(s->nreal, 256), 4 * std::max(1, c->num_sms));
    k_pme_unfix<<<gb, 256, 0, c->stream>>>(s->nreal, s->d_qfix, s->d_real);
    MDRL_CUDA(cudaGetLastError());
    PME_FFT(cufftExecR2C(s->fwd, s->d_real, s->d_cplx));
    k_pme_convolve<<<kPmeEnergyBlocks, 256, 0, c->stream>>>(s->ncplx, s->K[2] / 2 + 1, s->K[2], s->d_cplx,
                                                            s->d_green, energy ? s->d_epart : nullptr);
    MDRL_CUDA(cudaGetLastError());
    PME_FFT(cufftExecC2R(s->bwd, s->d_cplx, s->d_real));
    const int acc = c->p.accum;
    if (s->p.order == 6) {
        if (acc == MDRL_ACC_FIXED64) k_pme_gather<6, MDRL_ACC_FIXED64><<<qb, 256, 0, c->stream>>>(n, pos, pg, s->d_real, F64, F32, c->d_err);
        else if (acc == MDRL_ACC_KAHAN) k_pme_gather<6, MDRL_ACC_KAHAN><<<qb, 256, 0, c->stream>>>(n, pos, pg, s->d_real, F64, F32, c->d_err);
        else k_pme_gather<6, MDRL_ACC_FP32_ATOMIC><<<qb, 256, 0, c->stream>>>(n, pos, pg, s->d_real, F64, F32, c->d_err);
    } else {
        if (acc == MDRL_ACC_FIXED64) k_pme_gather<4, MDRL_ACC_FIXED64><<<qb, 256, 0, c->stream>>>(n, pos, pg, s->d_real, F64, F32, c->d_err);
        else if (acc == MDRL_ACC_KAHAN) k_pme_gather<4, MDRL_ACC_KAHAN><<<qb, 256, 0, c->stream>>>(n, pos, pg, s->d_real, F64, F32, c->d_err);
        else k_pme_gather<4, MDRL_ACC_FP32_ATOMIC><<<qb, 256, 0, c->stream>>>(n, pos, pg, s->d_real, F64, F32, c->d_err);
    }
    MDRL_CUDA(cudaGetLastError());
    return MDRL_OK;
}

/* After the totals kernel: add the reciprocal, self and background energies (with energies on). */
mdrl_status pme_add_energy(mdrl_ctx *c, int n) {
    PmeState *s = c->pme;
    if (!s || n <= 0) return MDRL_OK;
    k_pme_energy<<<1, 32, 0, c->stream>>>(kPmeEnergyBlocks, s->d_epart, nblk(n, 256), s->d_qpart, c->p.coulomb_k,
                                          s->p.beta, s->volume, c->d_tot);
    MDRL_CUDA(cudaGetLastError());
    return MDRL_OK;
}

}  // namespace mdrl

extern "C" void mdrl_default_pme_params(mdrl_pme_params *p) {
    if (!p) return;
    p->beta = 0.0;
    p->tolerance = 1e-5;
    p->spacing = 1.0;
    p->grid[0] = p->grid[1] = p->grid[2] = 0;
    p->order = 4;
}

extern "C" mdrl_status mdrl_get_pme(mdrl_ctx *c, mdrl_pme_params *p, int *enabled) {
    if (!c) { set_error("mdrl_get_pme: null context"); return MDRL_ERR_INVALID_ARG; }
    if (enabled) *enabled = c->pme ? 1 : 0;
    if (p && c->pme) *p = c->pme->p;
    return MDRL_OK;
}
