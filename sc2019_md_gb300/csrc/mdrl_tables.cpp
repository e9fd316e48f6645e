/*
 * mdrl_tables.cpp — FP64 generation of the interpolation tables and the per-type-pair
 * multipliers.
 *
 * Tables follow MatlabScripts/LJ_no_smooth_poly_interpolation_function.m:182-378 and
 * LJ_Coulomb_no_smooth_poly_interpolation_function.m:337-405: the r2 axis is cut into
 * power-of-two segments [2^m, 2^(m+1)), each segment into `bins` equal bins, and in every bin a
 * least-squares polynomial of the requested order is fitted through `samples` points
 * x_i = bin_start + i * bin_width / samples (i = 0..samples-1).  The reference fits in MATLAB
 * single precision; here the fit is FP64 (Householder QR on the bin-local variable
 * t = (x - bin_start) / bin_width, then an exact change of variable back to powers of r2), and
 * only the final coefficients are rounded to FP32.
 *
 * The functions are unit-prefactor powers of r2 (x = r2):
 *   r^-14 = x^-7, r^-8 = x^-4, r^-3 = x^-1.5, r^-12 = x^-6, r^-6 = x^-3, r^-1 = x^-0.5,
 * or, with Ewald splitting for the long-range solver, the real-space Coulomb pair in the r^-3 and
 * r^-1 slots, and the per-pair prefactors (A14 = 48*eps*sig^12, B8 = -24*eps*sig^6, A12 = 4*eps*sig^12,
 * B6 = -4*eps*sig^6, QQ = ke*qi*qj) multiply the table values in the kernel, as the reference's
 * LJ+Coulomb pipeline does with its p_a, p_b, p_qq ports
 * (SC/RL_Evaluate_Pairs_1st_Order.v:53-55,361-395).
 */
#include "mdrl_internal.h"

#include <cmath>
#include <vector>

namespace mdrl {

static const double kExponent[kNumFunc] = {-7.0, -4.0, -1.5, -6.0, -3.0, -0.5};

/* log2 of a power of two (the bin widths 2^(min_log2 + s) / bins). */
static int ilog2_exact(double w) {
    int e;
    std::frexp(w, &e);
    return e - 1;
}

/* Least-squares fit of degree `order` to (t_i, y_i), i < m, by Householder QR.  Returns
 * coefficients a[0..order] of a0 + a1 t + ... */
static void lsq_fit(int m, int order, const double *t, const double *y, double *a) {
    const int nc = order + 1;
    std::vector<double> V((size_t)m * nc), b(y, y + m);
    for (int i = 0; i < m; ++i) {
        double p = 1.0;
        for (int k = 0; k < nc; ++k) { V[(size_t)i * nc + k] = p; p *= t[i]; }
    }
    for (int k = 0; k < nc; ++k) {
        double norm = 0.0;
        for (int i = k; i < m; ++i) norm += V[(size_t)i * nc + k] * V[(size_t)i * nc + k];
        norm = std::sqrt(norm);
        const double akk = V[(size_t)k * nc + k];
        const double alpha = akk > 0 ? -norm : norm;
        std::vector<double> v(m, 0.0);
        for (int i = k; i < m; ++i) v[i] = V[(size_t)i * nc + k];
        v[k] -= alpha;
        double vnorm2 = 0.0;
        for (int i = k; i < m; ++i) vnorm2 += v[i] * v[i];
        if (vnorm2 == 0.0) continue;
        for (int c = k; c < nc; ++c) {
            double dot = 0.0;
            for (int i = k; i < m; ++i) dot += v[i] * V[(size_t)i * nc + c];
            const double s = 2.0 * dot / vnorm2;
            for (int i = k; i < m; ++i) V[(size_t)i * nc + c] -= s * v[i];
        }
        double dot = 0.0;
        for (int i = k; i < m; ++i) dot += v[i] * b[i];
        const double s = 2.0 * dot / vnorm2;
        for (int i = k; i < m; ++i) b[i] -= s * v[i];
    }
    for (int k = nc - 1; k >= 0; --k) {
        double s = b[k];
        for (int c = k + 1; c < nc; ++c) s -= V[(size_t)k * nc + c] * a[c];
        a[k] = s / V[(size_t)k * nc + k];
    }
}

/* Unit function f of the table set at x = r2: powers of x, or with Ewald splitting (beta > 0) the
 * real-space Coulomb pair (r^-3 -> (erfc(beta r)/r + 2 beta/sqrt(pi) exp(-beta^2 r^2)) / r^2, the
 * force over r; r^-1 -> erfc(beta r)/r, the energy). */
static double unit_function(int f, double x, double beta) {
    if (beta > 0.0 && (f == kF3 || f == kF1)) {
        const double r = std::sqrt(x);
        const double e = std::erfc(beta * r) / r;
        if (f == kF1) return e;
        return (e + 2.0 * beta / std::sqrt(3.14159265358979323846) * std::exp(-beta * beta * x)) / x;
    }
    return std::pow(x, kExponent[f]);
}

void fit_tables(int order, int nseg, int bins, int min_log2, int samples, std::vector<float> *out, double beta,
                bool local) {
    const int nidx = nseg * bins;
    const int nc = order + 1;
    out->assign((size_t)kNumFunc * nc * nidx, 0.0f);
    std::vector<double> t(samples), y(samples), a(nc), c(nc);
    for (int f = 0; f < kNumFunc; ++f) {
        for (int s = 0; s < nseg; ++s) {
            const double seg_lo = std::ldexp(1.0, min_log2 + s);
            const double width = seg_lo / bins;
            for (int j = 0; j < bins; ++j) {
                const double x0 = seg_lo + j * width;
                for (int i = 0; i < samples; ++i) {
                    t[i] = (double)i / samples;
                    y[i] = unit_function(f, x0 + t[i] * width, beta);
                }
                lsq_fit(samples, order, t.data(), y.data(), a.data());
                const int idx = s * bins + j;
                if (local) {
                    /* p = sum_m a_m (u / w)^m with u = x - x0: coefficients a_m / w^m (w is a
                     * power of two, so the scaling is exact) */
                    for (int m = 0; m < nc; ++m)
                        (*out)[((size_t)f * nc + m) * nidx + idx] = (float)std::ldexp(a[m], -m * ilog2_exact(width));
                    continue;
                }
                /* p(x) = sum_m a_m ((x - x0)/w)^m  ->  sum_k c_k x^k */
                for (int k = 0; k < nc; ++k) c[k] = 0.0;
                for (int m = 0; m < nc; ++m) {
                    const double am = a[m] / std::pow(width, m);
                    double binom = 1.0; /* C(m, k) */
                    for (int k = 0; k <= m; ++k) {
                        c[k] += am * binom * std::pow(-x0, m - k);
                        binom = binom * (m - k) / (k + 1);
                    }
                }
                for (int k = 0; k < nc; ++k)
                    (*out)[((size_t)f * nc + k) * nidx + idx] = (float)c[k];
            }
        }
    }
}

void mix_pair_coefficients(const mdrl_params &p, std::vector<float> *pc, std::vector<double> *pc64) {
    const int T = p.ntypes;
    pc->assign((size_t)T * T * 4, 0.0f);
    if (pc64) pc64->assign((size_t)T * T * 4, 0.0);
    for (int a = 0; a < T; ++a) {
        for (int b = 0; b < T; ++b) {
            const double sig = 0.5 * (p.sigma[a] + p.sigma[b]);
            const double eps = std::sqrt(p.epsilon[a] * p.epsilon[b]);
            const double s6 = std::pow(sig, 6.0), s12 = s6 * s6;
            const double v[4] = {48.0 * eps * s12, -24.0 * eps * s6, 4.0 * eps * s12, -4.0 * eps * s6};
            for (int k = 0; k < 4; ++k) {
                (*pc)[((size_t)a * T + b) * 4 + k] = (float)v[k];
                if (pc64) (*pc64)[((size_t)a * T + b) * 4 + k] = v[k];
            }
        }
    }
}

}  // namespace mdrl
