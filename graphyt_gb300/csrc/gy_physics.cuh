// gy_physics.cuh -- per-particle constitutive and damage updates in FP32 registers.
//
// Each function restates one reference routine (ConstitutiveModels.cpp, DamageModels.cpp)
// including its literal constants (1/3 written as 0.3333 / 0.33333 / 0.33, pi = 3.14159).
#pragma once

#include "gy_common.cuh"

namespace gy {

struct Constit {
    float s[6];      // stress, updated in place
    float e[6];      // strain after e += edot*dt
    float r[6];      // strain rate from G2P
    float ep[6];     // plastic strain
    float eqps;      // accumulated plastic strain
    float dmg;       // damage (turbulence flag for model 5)
    float smax;
    float mass, rho; // for Grady-Kipp's volume and model 5's kinetic energy
    float v[3];
};

// elastic, ConstitutiveModels.cpp:3-30
__device__ __forceinline__ void cm_elastic(Constit &c, const DevMaterial &M, float dt)
{
    const float vol = 0.3333f * (c.r[0] + c.r[1] + c.r[2]);
    const float twoG = 2.0f * M.G, threeKv = 3.0f * M.K * vol;
    c.s[0] += (twoG * (c.r[0] - vol) + threeKv) * dt;
    c.s[1] += (twoG * (c.r[1] - vol) + threeKv) * dt;
    c.s[2] += (twoG * (c.r[2] - vol) + threeKv) * dt;
    c.s[3] += (twoG * c.r[3]) * dt;
    c.s[4] += (twoG * c.r[4]) * dt;
    c.s[5] += (twoG * c.r[5]) * dt;
}

// Newtonian liquid, ConstitutiveModels.cpp:33-64: pressure from the accumulated strain,
// viscous stress = mu * rate * dt (the reference multiplies by dt).  With raw_dev set the
// normal rates are used unsplit, as model 5 does (ConstitutiveModels.cpp:77-82).
__device__ __forceinline__ void cm_newtonian(Constit &c, float K, float mu, float dt, int is3d, bool raw_dev)
{
    const float vol = raw_dev ? 0.0f : 0.33333f * (c.r[0] + c.r[1] + c.r[2]);
    const float P = K * (c.e[0] + c.e[1] + c.e[2]);
    const float k43 = (float)(2.0 - (2.0 / 3.0));
    c.s[0] = P + mu * k43 * (c.r[0] - vol) * dt;
    c.s[1] = P + mu * k43 * (c.r[1] - vol) * dt;
    c.s[3] = 2.0f * mu * c.r[3] * dt;
    if (is3d) {
        c.s[2] = P + mu * k43 * (c.r[2] - vol) * dt;
        c.s[4] = 2.0f * mu * c.r[4] * dt;
        c.s[5] = 2.0f * mu * c.r[5] * dt;
    }
}

// turbulent liquid, ConstitutiveModels.cpp:66-126 (turbulence flag kept in damage)
__device__ __forceinline__ void cm_turbulent(Constit &c, const DevMaterial &M, float dt, int is3d)
{
    float mu = M.viscosity;
    if (c.dmg == 1.0f) mu = M.viscosity / 2.0f;
    const float KE = 0.5f * c.mass * (c.v[0] * c.v[0] + c.v[1] * c.v[1] + c.v[2] * c.v[2]);
    const float VE = 0.5f * M.viscosity * (c.r[3] * c.r[3] + c.r[4] * c.r[4] + c.r[5] * c.r[5]);
    const float crit = KE - VE - M.turb_stress;
    if (crit > 0.0f) c.dmg = 1.0f;
    if (crit <= 0.0f) { c.dmg = 0.0f; mu = M.viscosity; }
    cm_newtonian(c, M.K, mu, dt, is3d, true);
}

// von Mises perfect plasticity, ConstitutiveModels.cpp:131-234
__device__ __forceinline__ void cm_perfect_plastic(Constit &c, const DevMaterial &M, float dt, int is3d)
{
    const float G = M.G, K = M.K;
    const float vol = 0.33f * (c.r[0] + c.r[1] + c.r[2]);
    float t[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    t[0] = c.s[0] + (2.0f * G * (c.r[0] - vol) + 3.0f * K * vol) * dt;
    t[1] = c.s[1] + (2.0f * G * (c.r[1] - vol) + 3.0f * K * vol) * dt;
    if (is3d) {
        t[2] = c.s[2] + (2.0f * G * (c.r[2] - vol) + 3.0f * K * vol) * dt;
        t[4] = c.s[4] + (2.0f * G * c.r[4]) * dt;
        t[5] = c.s[5] + (2.0f * G * c.r[5]) * dt;
    }
    t[3] = c.s[3] + (2.0f * G * c.r[3]) * dt;
    const float q = sqrtf(0.5f * (t[0] - t[1]) * (t[0] - t[1]) + 0.5f * (t[1] - t[2]) * (t[1] - t[2]) +
                          0.5f * (t[2] - t[0]) * (t[2] - t[0]) + t[3] * t[3] + t[4] * t[4] + t[5] * t[5]);
    if (q > M.yield) {
        const float dL = (q - M.yield) / (3.0f * G);
        const float cf = dL * (0.5f / q);
        float p[6];
        p[0] = cf * (2.0f * t[0] - t[1] - t[2]);
        p[1] = cf * (2.0f * t[1] - t[2] - t[0]);
        p[2] = cf * (2.0f * t[2] - t[0] - t[1]);
        p[3] = cf * (6.0f * t[3]);
        p[4] = cf * (6.0f * t[4]);
        p[5] = cf * (6.0f * t[5]);
        c.eqps += dt * sqrtf(0.5f * (p[0] - p[1]) * (p[0] - p[1]) + 0.5f * (p[1] - p[2]) * (p[1] - p[2]) +
                             0.5f * (p[2] - p[0]) * (p[2] - p[0]) + p[3] * p[3] + p[4] * p[4] + p[5] * p[5]);
        float el[6];
#pragma unroll
        for (int k = 0; k < 6; k++) {
            c.ep[k] += p[k];
            el[k] = c.r[k] - p[k] / dt;
        }
        c.s[0] += (2.0f * G * (el[0] - vol) + 3.0f * K * vol) * dt;
        c.s[1] += (2.0f * G * (el[1] - vol) + 3.0f * K * vol) * dt;
        c.s[3] += (2.0f * G * el[3]) * dt;
        if (is3d) {
            c.s[2] += (2.0f * G * (el[2] - vol) + 3.0f * K * vol) * dt;
            c.s[4] += (2.0f * G * el[4]) * dt;
            c.s[5] += (2.0f * G * el[5]) * dt;
        }
    } else {
#pragma unroll
        for (int k = 0; k < 6; k++) c.s[k] = t[k];
    }
}

// Drucker-Prager with linear cohesion softening, ConstitutiveModels.cpp:238-428.
// The yield function along the return, Fp(dL) = sqrt(J2) - G dL + eta (p - eta_bar K dL)
// - xi c(dL), is linear in dL between the kinks of the softened cohesion
// c(dL) = max(c - (eqps + xi dL) c/eps_cr, c/10), so the reference's Newton loop (tolerance
// 1e-8, <= 200 iterations, :321-344) lands on the root in two or three iterations in FP64.
// In FP32 that tolerance is out of reach; the same Newton iteration is run here to a
// relative residual of 1e-6 or four iterations, which reaches the same root of the
// piecewise-linear function.  The apex branch (:347-395) is treated the same way.
__device__ __forceinline__ void cm_drucker_prager(Constit &c, const DevMaterial &M, float dt)
{
    const float G = M.G, K = M.K, coh = M.cohesion, ecr = M.crit_strain;
    const float eta = M.eta, xi = M.xi, etab = M.eta_bar;
    const float vol = 0.3333f * (c.r[0] + c.r[1] + c.r[2]);
    float t[6];
    t[0] = c.s[0] + (2.0f * G * (c.r[0] - vol) + 3.0f * K * vol) * dt;
    t[1] = c.s[1] + (2.0f * G * (c.r[1] - vol) + 3.0f * K * vol) * dt;
    t[2] = c.s[2] + (2.0f * G * (c.r[2] - vol) + 3.0f * K * vol) * dt;
    t[3] = c.s[3] + (2.0f * G * c.r[3]) * dt;
    t[4] = c.s[4] + (2.0f * G * c.r[4]) * dt;
    t[5] = c.s[5] + (2.0f * G * c.r[5]) * dt;
    const float I1 = (1.0f / 3.0f) * (t[0] + t[1] + t[2]);  // mean stress
    const float sxx = t[0] - I1, syy = t[1] - I1, szz = t[2] - I1, sxy = t[3], syz = t[4], sxz = t[5];
    const float J2 = 0.5f * (sxx * sxx + syy * syy + szz * szz + 2.0f * sxy * sxy + 2.0f * syz * syz + 2.0f * sxz * sxz);
    const float sqJ = sqrtf(J2);
    const float F = sqJ + eta * I1 - xi * coh;
    const bool yield = M.damage ? (F > 0.0f && I1 < 0.0f) : (F > 0.0f);
    if (!yield) {
#pragma unroll
        for (int k = 0; k < 6; k++) c.s[k] = t[k];
        return;
    }
    const float H = coh / ecr, cfloor = coh / 10.0f;
    float dL = 0.0f;
    for (int it = 0; it < 4; it++) {
        float cv = coh - (c.eqps + xi * dL) * H;
        float dc = -H;
        if (cv < cfloor) { cv = cfloor; dc = 0.0f; }
        const float Fp = sqJ - G * dL + eta * (I1 - etab * K * dL) - xi * cv;
        const float dFp = -G - K * eta * etab - xi * xi * dc;
        const float step = Fp / dFp;
        dL = dL - step;
        if (fabsf(Fp) <= 1e-6f * fabsf(cv)) break;
    }
    const float Gapex = sqJ - G * dL;
    if (Gapex < 0.0f && !M.damage) {
        float de = 0.0f;
        for (int it = 0; it < 4; it++) {
            float cv = coh - (c.eqps + (xi / eta) * de) * H;
            float dc = -H;
            if (cv < cfloor) { cv = cfloor; dc = 0.0f; }
            const float Gp = cv * (xi / etab) - I1 + K * de;
            const float dGp = (xi / eta) * dc * (xi / etab) + K;
            de = de - Gp / dGp;
            if (fabsf(Gp) <= 1e-6f * fabsf(cv)) break;
        }
        if (de >= 0.0f) {
            const float pm = I1 - K * de;
            c.s[0] = pm; c.s[1] = pm; c.s[2] = pm;
            c.s[3] = 0.0f; c.s[4] = 0.0f; c.s[5] = 0.0f;
            c.eqps += de * (xi / eta);
            c.ep[0] += de * (etab / 3.0f);
            c.ep[1] += de * (etab / 3.0f);
            c.ep[2] += de * (etab / 3.0f);
        }
        // de < 0: the reference leaves the stress at its previous value (:376-378)
    } else {
        const float f = 1.0f - G * dL / sqJ;
        const float pm = I1 - K * etab * dL;
        c.s[0] = f * sxx + pm; c.s[1] = f * syy + pm; c.s[2] = f * szz + pm;
        c.s[3] = f * sxy; c.s[4] = f * syz; c.s[5] = f * sxz;
        c.eqps += dL * xi;
        const float hj = 0.5f / J2;
        c.ep[0] += dL * (hj * sxx + etab / 3.0f);
        c.ep[1] += dL * (hj * syy + etab / 3.0f);
        c.ep[2] += dL * (hj * szz + etab / 3.0f);
        c.ep[3] += dL * hj * sxy;
        c.ep[4] += dL * hj * syz;
        c.ep[5] += dL * hj * sxz;
    }
}

// The elastic trial stress of the Drucker-Prager update (ConstitutiveModels.cpp:254-300) and
// its yield test (:300-307: with damage on, only compressive states yield); t receives the
// trial stress.
__device__ __forceinline__ bool dp_trial_yields(const Constit &c, const DevMaterial &M, float dt, float t[6])
{
    const float G = M.G, K = M.K;
    const float vol = 0.3333f * (c.r[0] + c.r[1] + c.r[2]);
    t[0] = c.s[0] + (2.0f * G * (c.r[0] - vol) + 3.0f * K * vol) * dt;
    t[1] = c.s[1] + (2.0f * G * (c.r[1] - vol) + 3.0f * K * vol) * dt;
    t[2] = c.s[2] + (2.0f * G * (c.r[2] - vol) + 3.0f * K * vol) * dt;
    t[3] = c.s[3] + (2.0f * G * c.r[3]) * dt;
    t[4] = c.s[4] + (2.0f * G * c.r[4]) * dt;
    t[5] = c.s[5] + (2.0f * G * c.r[5]) * dt;
    const float I1 = (1.0f / 3.0f) * (t[0] + t[1] + t[2]);
    const float sxx = t[0] - I1, syy = t[1] - I1, szz = t[2] - I1;
    const float J2 = 0.5f * (sxx * sxx + syy * syy + szz * szz + 2.0f * t[3] * t[3] + 2.0f * t[4] * t[4] +
                             2.0f * t[5] * t[5]);
    const float F = sqrtf(J2) + M.eta * I1 - M.xi * M.cohesion;
    return M.damage ? (F > 0.0f && I1 < 0.0f) : (F > 0.0f);
}

// Residual of the Drucker-Prager yield function at a stress and accumulated plastic strain,
// with the softened cohesion max(c - eqps c / eps_cr, c / 10) (ConstitutiveModels.cpp:321-344):
// the exact return mapping lands on F = 0.
__device__ __forceinline__ float dp_residual(const float s[6], float eqps, const DevMaterial &M)
{
    const float I1 = (1.0f / 3.0f) * (s[0] + s[1] + s[2]);
    const float sxx = s[0] - I1, syy = s[1] - I1, szz = s[2] - I1;
    const float J2 = 0.5f * (sxx * sxx + syy * syy + szz * szz + 2.0f * s[3] * s[3] + 2.0f * s[4] * s[4] +
                             2.0f * s[5] * s[5]);
    const float cv = fmaxf(M.cohesion - eqps * (M.cohesion / M.crit_strain), M.cohesion / 10.0f);
    return sqrtf(J2) + M.eta * I1 - M.xi * cv;
}

// Symmetric 3x3 eigen-decomposition by cyclic Jacobi rotations (FP32).  A is overwritten;
// on return A[i][i] hold the eigenvalues and V's columns the eigenvectors.  The reference
// uses JAMA's tred2+tql2 (eig3.cpp:258-267); the damaged stress V diag(s') V^T depends
// only on the eigenpairs, not on the method.
__device__ __forceinline__ void sym_eigen3(float A[3][3], float V[3][3])
{
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
        for (int j = 0; j < 3; j++) V[i][j] = (i == j) ? 1.0f : 0.0f;
    for (int sweep = 0; sweep < 8; sweep++) {
        const float off = fabsf(A[0][1]) + fabsf(A[0][2]) + fabsf(A[1][2]);
        const float dg = fabsf(A[0][0]) + fabsf(A[1][1]) + fabsf(A[2][2]);
        if (off <= 1e-9f * dg || off == 0.0f) break;
#pragma unroll
        for (int pq = 0; pq < 3; pq++) {
            const int p = pq == 2 ? 1 : 0;
            const int q = pq == 0 ? 1 : 2;
            const float apq = A[p][q];
            if (apq == 0.0f) continue;
            const float theta = (A[q][q] - A[p][p]) / (2.0f * apq);
            const float tt = copysignf(1.0f, theta) / (fabsf(theta) + sqrtf(theta * theta + 1.0f));
            const float cs = rsqrtf(tt * tt + 1.0f), sn = tt * cs;
#pragma unroll
            for (int k = 0; k < 3; k++) {
                const float akp = A[k][p], akq = A[k][q];
                A[k][p] = cs * akp - sn * akq;
                A[k][q] = sn * akp + cs * akq;
            }
#pragma unroll
            for (int k = 0; k < 3; k++) {
                const float apk = A[p][k], aqk = A[q][k];
                A[p][k] = cs * apk - sn * aqk;
                A[q][k] = sn * apk + cs * aqk;
            }
#pragma unroll
            for (int k = 0; k < 3; k++) {
                const float vkp = V[k][p], vkq = V[k][q];
                V[k][p] = cs * vkp - sn * vkq;
                V[k][q] = sn * vkp + cs * vkq;
            }
        }
    }
}

// Activation strain of the particle's weakest flaw, e_min = w (V k)^(-1/m) (DamageModels.cpp:
// 102-103 with w = 1), evaluated as exp(-(ln V + ln k)/m) so V*k never overflows.  w is the
// particle's flaw scale (a per-particle Weibull draw) where the handle has a flaw table.
__device__ __forceinline__ float gk_emin(const Constit &c, const DevMaterial &M, const float *flaw, int pid)
{
    const float vol = c.mass / c.rho;
    const float emin = expf(-(logf(vol) + M.gk_logk) / M.gk_m);
    return flaw ? emin * __ldg(flaw + pid) : emin;
}

// Largest eigenvalue of a symmetric 3x3 matrix (xx yy zz xy yz xz), by the trigonometric
// solution of the characteristic cubic (O. K. Smith, "Eigenvalues of a symmetric 3 x 3
// matrix", Comm. ACM 4(4), 1961): with q = tr/3 and B = (A - q I) / p, p^2 = |A - q I|^2 / 6,
// the eigenvalues are q + 2 p cos(acos(det(B) / 2) / 3 + 2 pi k / 3); k = 0 is the largest.
__device__ __forceinline__ float sym3_max_eigenvalue(const float s[6])
{
    const float q = (s[0] + s[1] + s[2]) * (1.0f / 3.0f);
    const float a = s[0] - q, b = s[1] - q, c = s[2] - q;
    const float off = s[3] * s[3] + s[4] * s[4] + s[5] * s[5];
    const float p2 = (a * a + b * b + c * c + 2.0f * off) * (1.0f / 6.0f);
    if (!(p2 > 0.0f)) return q;  // a multiple of the identity
    const float p = sqrtf(p2), ip = 1.0f / p;
    const float ba = a * ip, bb = b * ip, bc = c * ip, bxy = s[3] * ip, byz = s[4] * ip, bxz = s[5] * ip;
    const float det = ba * (bb * bc - byz * byz) - bxy * (bxy * bc - byz * bxz) + bxz * (bxy * byz - bb * bxz);
    const float r = fminf(fmaxf(0.5f * det, -1.0f), 1.0f);
    return q + 2.0f * p * cosf(acosf(r) * (1.0f / 3.0f));
}

// Grady-Kipp damage, 3D branch of DamageModels.cpp:71-150.  The largest principal stress
// decides whether damage grows; most stressed particles stop there, so it comes from the
// closed form above, and the eigen-decomposition runs only when damage grows and the stress
// is rebuilt from the principal values (without growth V diag(s) V^T is the stress itself,
// which the reference recomputes with rounding only).
__device__ __forceinline__ void dm_grady_kipp3(Constit &c, const DevMaterial &M, float dt, const float *flaw, int pid)
{
    const float chk = fabsf(c.s[0] + c.s[1] + c.s[2] + c.s[3] + c.s[4] + c.s[5]);
    if (!(chk > 1e-3f)) return;
    const float smx = fmaxf(sym3_max_eigenvalue(c.s), 0.0f);
    c.smax = smx;
    if (!(smx > 1e-3f)) return;
    const float eff = smx / (M.K + 4.0f * M.G / 3.0f);
    if (!(eff > gk_emin(c, M, flaw, pid))) return;
    float A[3][3] = {{c.s[0], c.s[3], c.s[5]}, {c.s[3], c.s[1], c.s[4]}, {c.s[5], c.s[4], c.s[2]}};
    float V[3][3];
    sym_eigen3(A, V);
    float p[3] = {A[0][0], A[1][1], A[2][2]};
    const float rate = M.gk_rate_coef * powf(eff, M.gk_m / 3.0f);
    const float root = cbrtf(c.dmg) + dt * rate;
    float D = root * root * root;
    if (D > 1.0f) D = 1.0f;
    c.dmg = D;
#pragma unroll
    for (int i = 0; i < 3; i++)
        if (p[i] > 0.0f) p[i] = (1.0f - D) * p[i];
    float R[3][3];
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
        for (int j = 0; j < 3; j++) R[i][j] = V[i][0] * p[0] * V[j][0] + V[i][1] * p[1] * V[j][1] + V[i][2] * p[2] * V[j][2];
    c.s[0] = R[0][0]; c.s[1] = R[1][1]; c.s[2] = R[2][2];
    c.s[3] = R[0][1]; c.s[4] = R[1][2]; c.s[5] = R[0][2];
}

// Grady-Kipp, 2D branch of DamageModels.cpp:11-70 (principal axes in closed form).
__device__ __forceinline__ void dm_grady_kipp2(Constit &c, const DevMaterial &M, float dt, const float *flaw, int pid)
{
    float sxx = c.s[0], syy = c.s[1], sxy = c.s[3], szz = c.s[2];
    float th;
    if (fabsf(sxx - syy) < 1e-5f) th = 3.14159f / 4.0f;
    else th = 0.5f * atanf(2.0f * sxy / (sxx - syy));
    const float cs = cosf(th), sn = sinf(th);
    float s1 = sxx * cs * cs + syy * sn * sn + 2.0f * cs * sn * sxy;
    float s2 = sxx * sn * sn + syy * cs * cs - 2.0f * cs * sn * sxy;
    const float smx = fmaxf(s1, fmaxf(s2, 0.0f));
    c.smax = smx;
    bool rebuilt = false;
    if (smx > 1e-3f) {
        const float eff = smx / (M.K + 4.0f * M.G / 3.0f);
        if (eff > gk_emin(c, M, flaw, pid)) {
            const float rate = M.gk_rate_coef * powf(eff, M.gk_m / 3.0f);
            const float root = cbrtf(c.dmg) + dt * rate;
            float D = root * root * root;
            if (D > 1.0f) D = 1.0f;
            c.dmg = D;
            if (s1 > 0.0f) s1 = (1.0f - D) * s1;
            if (s2 > 0.0f) s2 = (1.0f - D) * s2;
            rebuilt = true;
        }
    }
    if (c.dmg == 1.0f) {
        if (s1 > 0.0f) s1 = 0.0f;
        if (s2 > 0.0f) s2 = 0.0f;
        rebuilt = true;
    }
    if (rebuilt) {
        sxx = s1 * cs * cs + s2 * sn * sn;
        syy = s1 * sn * sn + s2 * cs * cs;
        sxy = (s1 - s2) * cs * sn;
        szz = 0.0f;
    }
    c.s[0] = sxx; c.s[1] = syy; c.s[2] = szz; c.s[3] = sxy;
}

// constitutiveModel dispatch (TimeIntegration.cpp:120-143) and applyDamage (:165-173); flaw
// (may be null) is the per-particle flaw scale table, pid the particle's insertion index
__device__ __forceinline__ void constitutive_update(Constit &c, const DevMaterial &M, float dt, int is3d,
                                                    const float *flaw, int pid)
{
    switch (M.model) {
    case 1: cm_elastic(c, M, dt); break;
    case 2: cm_newtonian(c, M.K, M.viscosity, dt, is3d, false); break;
    case 3: cm_perfect_plastic(c, M, dt, is3d); break;
    case 4: cm_drucker_prager(c, M, dt); break;
    case 5: cm_turbulent(c, M, dt, is3d); break;
    default: break;
    }
    if (M.damage && M.damage_model == 1) {
        if (is3d) dm_grady_kipp3(c, M, dt, flaw, pid);
        else dm_grady_kipp2(c, M, dt, flaw, pid);
    }
}

}  // namespace gy
