/*
 * mdrl_cmodel.cu — the drop-in for the reference C model, int MD_Evaluation_Model()
 * (Range_Limited/C_Model_ForceEval/MD_Evaluation_Model.h:1, .cpp:9-205), on the GPU.
 *
 * The reference runs an all-pairs O(N^2) FP32 LJ force with minimum-image PBC, a symplectic
 * Euler update and prints the energies of every iteration.  This file keeps its constants and
 * its rounding: every float expression is evaluated in the reference's types and order with
 * separately rounded intrinsics, and pow(float, int) -- which C++ evaluates in double and the
 * reference stores to float -- is the correctly rounded double power (exact products and a
 * double-double product for the 6th and 7th powers) converted to float.  Each reference
 * particle's force is summed over j in index order by one thread, and the energies are summed
 * over i in index order, so the printed values match the reference line for line.
 */
#include <cuda_runtime.h>

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "mdrl_internal.h"

using namespace mdrl;

namespace {

struct CConst {
    float eps, sig12, sig6, mass, dt, rc2, box;
};

struct DD { double h, l; };

__device__ __forceinline__ DD two_prod(double a, double b) {
    const double p = __dmul_rn(a, b);
    return {p, __fma_rn(a, b, -p)};
}

__device__ __forceinline__ DD dd_mul(DD a, DD b) {
    const double p = __dmul_rn(a.h, b.h);
    double e = __fma_rn(a.h, b.h, -p);
    e = __fma_rn(a.h, b.l, e);
    e = __fma_rn(a.l, b.h, e);
    const double s = __dadd_rn(p, e);
    return {s, __dsub_rn(e, __dsub_rn(s, p))};
}

/* (float)pow((double)x, k) for k = 3, 4, 6, 7 with x a float. */
__device__ __forceinline__ void cpow(float xf, float &p3, float &p4, float &p6, float &p7) {
    const double x = (double)xf;
    const double x2 = __dmul_rn(x, x);         /* exact: 48 significant bits */
    const DD x3 = two_prod(x2, x);              /* exact */
    const DD x4 = two_prod(x2, x2);             /* exact */
    const DD x6 = dd_mul(x3, x3);
    const DD x7 = dd_mul(x4, x3);
    p3 = __double2float_rn(x3.h);
    p4 = __double2float_rn(x4.h);
    p6 = __double2float_rn(__dadd_rn(x6.h, x6.l));
    p7 = __double2float_rn(__dadd_rn(x7.h, x7.l));
}

/* dx -= L * (int)(dx/L +- 0.5)  (MD_Evaluation_Model.cpp:81-98) */
__device__ __forceinline__ float cmin_image(float d, float L) {
    const double q = (double)__fdiv_rn(d, L);
    const int k = (d >= 0.0f) ? (int)__dadd_rn(q, 0.5) : (int)__dsub_rn(q, 0.5);
    return __fsub_rn(d, __fmul_rn(L, (float)k));
}

/* Force, energy and the velocity update of particle i (.cpp:63-150). */
__global__ void k_cm_force(int n, const float *__restrict__ pos, float *__restrict__ vel,
                           float *__restrict__ F, float *__restrict__ ev, float *__restrict__ ek,
                           int *__restrict__ counts, CConst k) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float rx = pos[3 * i], ry = pos[3 * i + 1], rz = pos[3 * i + 2];
    float E = 0.0f, fx = 0.0f, fy = 0.0f, fz = 0.0f;
    int nb = 0;
    const float e4 = __fmul_rn(4.0f, k.eps), e48 = __fmul_rn(48.0f, k.eps), e24 = __fmul_rn(24.0f, k.eps);
    const float c12 = __fmul_rn(e4, k.sig12), c6 = __fmul_rn(e4, k.sig6);
    const float c14 = __fmul_rn(e48, k.sig12), c8 = __fmul_rn(e24, k.sig6);
    for (int j = 0; j < n; ++j) {
        const float dx = cmin_image(__fsub_rn(rx, pos[3 * j]), k.box);
        const float dy = cmin_image(__fsub_rn(ry, pos[3 * j + 1]), k.box);
        const float dz = cmin_image(__fsub_rn(rz, pos[3 * j + 2]), k.box);
        const float r2 = __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
        if (r2 > 0.0f && r2 <= k.rc2) {
            ++nb;
            const float inv_r2 = __fdiv_rn(1.0f, r2);
            float p3, p4, p6, p7;
            cpow(inv_r2, p3, p4, p6, p7);
            const float vdw12 = __fmul_rn(c12, p6), vdw6 = __fmul_rn(c6, p3);
            const float vdw14 = __fmul_rn(c14, p7), vdw8 = __fmul_rn(c8, p4);
            const float Fv = __fsub_rn(vdw14, vdw8), Ev = __fsub_rn(vdw12, vdw6);
            fx = __fadd_rn(fx, __fmul_rn(Fv, dx));
            fy = __fadd_rn(fy, __fmul_rn(Fv, dy));
            fz = __fadd_rn(fz, __fmul_rn(Fv, dz));
            E = __fadd_rn(E, Ev);
        }
    }
    F[3 * i] = fx; F[3 * i + 1] = fy; F[3 * i + 2] = fz;
    ev[i] = E;
    if (counts) counts[i] = nb;
    const float ax = __fdiv_rn(fx, k.mass), ay = __fdiv_rn(fy, k.mass), az = __fdiv_rn(fz, k.mass);
    float vx = vel[3 * i], vy = vel[3 * i + 1], vz = vel[3 * i + 2];
    vx = __fadd_rn(vx, __fmul_rn(ax, k.dt));
    vy = __fadd_rn(vy, __fmul_rn(ay, k.dt));
    vz = __fadd_rn(vz, __fmul_rn(az, k.dt));
    const float v2 = __fadd_rn(__fadd_rn(__fmul_rn(vx, vx), __fmul_rn(vy, vy)), __fmul_rn(vz, vz));
    ek[i] = __double2float_rn(__dmul_rn(__dmul_rn(0.5, (double)k.mass), (double)v2));
    vel[3 * i] = vx; vel[3 * i + 1] = vy; vel[3 * i + 2] = vz;
}

/* System energies summed over i in order (.cpp:152-158). */
__global__ void k_cm_energy(int n, const float *__restrict__ ev, const float *__restrict__ ek,
                            float *__restrict__ out) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    float se = 0.0f, sk = 0.0f;
    for (int i = 0; i < n; ++i) { se = __fadd_rn(se, ev[i]); sk = __fadd_rn(sk, ek[i]); }
    out[0] = __double2float_rn(__dmul_rn((double)se, 0.5));
    out[1] = sk;
}

/* x += v dt with one wrap into [0, L) (.cpp:164-202). */
__global__ void k_cm_move(int n, float *__restrict__ pos, const float *__restrict__ vel, CConst k) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= 3 * n) return;
    float p = __fadd_rn(pos[i], __fmul_rn(vel[i], k.dt));
    if (p < 0.0f) p = __fadd_rn(p, k.box);
    else if (p >= k.box) p = __fsub_rn(p, k.box);
    pos[i] = p;
}

struct DevBuf {
    void *p = nullptr;
    ~DevBuf() { if (p) cudaFree(p); }
};

}  // namespace

#define CM_CUDA(call)                                                                    \
    do {                                                                                 \
        cudaError_t e_ = (call);                                                         \
        if (e_ != cudaSuccess) {                                                         \
            set_error(std::string(#call) + ": " + cudaGetErrorString(e_));               \
            return MDRL_ERR_CUDA;                                                        \
        }                                                                                \
    } while (0)

extern "C" mdrl_status mdrl_cmodel_run(int n, int iters, float box, float cutoff, float *pos, float *vel,
                                       float *energy, int *counts) {
    if (n <= 0 || iters < 0 || !(box > 0.0f) || !(cutoff > 0.0f) || !pos || !vel || (iters > 0 && !energy)) {
        set_error("mdrl_cmodel_run: invalid argument");
        return MDRL_ERR_INVALID_ARG;
    }
    /* The reference's constants (.cpp:14-24), in its types. */
    CConst k;
    k.eps = (float)(1.995996 * 1.995996);
    const float sigma = (float)(0.1675 * 2);
    k.sig12 = (float)std::pow((double)sigma, 12.0);
    k.sig6 = (float)std::pow((double)sigma, 6.0);
    const float weight = 39.95f, nav = 6.022e23f;
    k.mass = weight / nav / 1000;
    k.dt = (float)2E-15;
    k.rc2 = cutoff * cutoff;
    k.box = box;
    DevBuf dpos, dvel, dF, dev, dek, dout, dcnt;
    const size_t b3 = sizeof(float) * 3 * (size_t)n;
    CM_CUDA(cudaMalloc(&dpos.p, b3));
    CM_CUDA(cudaMalloc(&dvel.p, b3));
    CM_CUDA(cudaMalloc(&dF.p, b3));
    CM_CUDA(cudaMalloc(&dev.p, sizeof(float) * n));
    CM_CUDA(cudaMalloc(&dek.p, sizeof(float) * n));
    CM_CUDA(cudaMalloc(&dout.p, sizeof(float) * 2 * (size_t)(iters > 0 ? iters : 1)));
    if (counts) CM_CUDA(cudaMalloc(&dcnt.p, sizeof(int) * n));
    CM_CUDA(cudaMemcpy(dpos.p, pos, b3, cudaMemcpyHostToDevice));
    CM_CUDA(cudaMemcpy(dvel.p, vel, b3, cudaMemcpyHostToDevice));
    const int blocks = (n + 127) / 128;
    for (int it = 0; it < iters; ++it) {
        k_cm_force<<<blocks, 128>>>(n, (float *)dpos.p, (float *)dvel.p, (float *)dF.p, (float *)dev.p,
                                    (float *)dek.p, (int *)dcnt.p, k);
        k_cm_energy<<<1, 32>>>(n, (float *)dev.p, (float *)dek.p, (float *)dout.p + 2 * it);
        k_cm_move<<<(3 * n + 255) / 256, 256>>>(n, (float *)dpos.p, (float *)dvel.p, k);
    }
    CM_CUDA(cudaGetLastError());
    CM_CUDA(cudaDeviceSynchronize());
    CM_CUDA(cudaMemcpy(pos, dpos.p, b3, cudaMemcpyDeviceToHost));
    CM_CUDA(cudaMemcpy(vel, dvel.p, b3, cudaMemcpyDeviceToHost));
    if (iters > 0) CM_CUDA(cudaMemcpy(energy, dout.p, sizeof(float) * 2 * iters, cudaMemcpyDeviceToHost));
    if (counts) CM_CUDA(cudaMemcpy(counts, dcnt.p, sizeof(int) * n, cudaMemcpyDeviceToHost));
    return MDRL_OK;
}

/* The reference reads an argon PDB: five header lines, then one atom per line whose 7th-9th
 * whitespace-separated fields are x, y, z (.cpp:38-55). */
extern "C" int MD_Evaluation_Model(void) {
    const char *path = std::getenv("MDRL_INPUT");
    if (!path || !*path) {
        set_error("MD_Evaluation_Model: set MDRL_INPUT to the argon PDB file");
        return 0;
    }
    const char *ns = std::getenv("MDRL_N");
    const char *is = std::getenv("MDRL_ITERS");
    const int n = ns ? std::atoi(ns) : 500;
    const int iters = is ? std::atoi(is) : 100;
    if (n <= 0 || iters < 0) { set_error("MD_Evaluation_Model: bad MDRL_N or MDRL_ITERS"); return 0; }
    FILE *fp = std::fopen(path, "r");
    if (!fp) { set_error(std::string("MD_Evaluation_Model: cannot open ") + path); return 0; }
    std::vector<float> pos(3 * (size_t)n, 0.0f), vel(3 * (size_t)n, 0.0f);
    char line[1024];
    for (int i = 0; i < 5; ++i)
        if (!std::fgets(line, sizeof line, fp)) break;
    int got = 0;
    for (int i = 0; i < n; ++i) {
        if (!std::fgets(line, sizeof line, fp)) break;
        float x, y, z;
        if (std::sscanf(line, "%*s %*s %*s %*s %*s %*s %f %f %f", &x, &y, &z) == 3) {
            pos[3 * i] = x; pos[3 * i + 1] = y; pos[3 * i + 2] = z;
            ++got;
        }
    }
    std::fclose(fp);
    if (got != n) {
        set_error("MD_Evaluation_Model: the PDB holds fewer atoms than MDRL_N");
        return 0;
    }
    std::vector<float> energy(2 * (size_t)(iters > 0 ? iters : 1));
    if (mdrl_cmodel_run(n, iters, 24.0f, 8.0f, pos.data(), vel.data(), energy.data(), nullptr) != MDRL_OK)
        return 0;
    for (int it = 0; it < iters; ++it)
        std::printf("Iteration %d, System energy is %f, Kinetic Energy is %f\n", it, energy[2 * it],
                    energy[2 * it + 1]);
    std::fflush(stdout);
    return 1;
}
