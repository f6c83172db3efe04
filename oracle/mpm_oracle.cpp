// mpm_oracle.cpp - CPU restatement of warpmpm's explicit MLS/APIC substep.
//
// TEST INFRASTRUCTURE ONLY. This library is the parity checker for the CUDA
// engine in mpm_engine_gb300/ and the CPU baseline timed by bench.py. Nothing in
// the product imports, links or calls it.
//
// It restates, in fp32 with the reference's operation order, the Warp kernels of
// kks32/mpm-engine (src/warpmpm/kernels/mpm_utils.py, mpm_solver_warp.py) and the
// tick schedule of MPM_Simulator_WARP.p2g2p_fused_tick / p2g2p. Citations are
// file:line within that project. Compile with -ffp-contract=off so every
// multiply and add rounds separately, as written.
//
// Parity status: the glass SDF, cup fill, material parameter mapping and
// block-sort keys are pinned against fixtures generated from the reference's own
// Python modules (tests/golden/). The per-substep arithmetic (svd3, pow/log/exp,
// atomic order) lives in the third-party package warp-lang 1.14.0
// (uv.lock:1159-1160), which is not installed here, so step-level parity is
// unpinned: it is anchored on the reference's physics-gate assertions
// (tests/test_engine.py, test_analytic_benchmarks.py, test_pour.py,
// test_sdf_collider.py, test_material_review_fixes.py, test_periodic_chute.py,
// test_tabulated_material.py, test_sparse_blocks.py, test_particle_sort.py,
// test_cdf_mask.py), restated in tests/ on this oracle and on the CUDA engine.
//
// Precision: the restated arithmetic is written over the scalar type Real, float
// by default (the reference's fp32 and operation order: the parity checker). The
// same source built with -DORACLE_REAL=double is a second library with the
// rounding taken out: its particle arrays, grid and accumulators are float64, and
// the tests use it as a noise-free forward for finite-difference checks of the
// engine's adjoint (literal constants keep their fp32 values, so both builds
// describe the same model).
//
// svd3: warp's svd3 is not vendored. This file uses its own method: a cyclic
// Jacobi eigen-solve of F^T F in float64, descending sort, then a Givens QR of
// F V, giving U and V proper rotations and sigma_3 carrying the sign of det F
// (the convention the reference's abs()/max() guards at mpm_utils.py:134-136,
// 266 and the det-flip at :1273-1281 are written against).

#include "../include/gbmpm.h"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstddef>
#include <cstring>
#include <numeric>
#include <vector>
#include <functional>
#ifdef _OPENMP
#include <omp.h>
#endif

#ifndef ORACLE_REAL
#define ORACLE_REAL float
#endif

namespace {

using Real = ORACLE_REAL;

// The particle arrays in the oracle's precision: gbmpm_particles with Real fields
// (the caller's arrays are float32 or float64 to match the build).
struct RP {
    int32_t n;
    Real *x, *v;
    Real *C, *F, *F_trial, *L, *stress;
    Real *mass, *vol, *density, *Jp;
    Real *mu, *lam, *yield_stress;
    int32_t *material, *selection;
    Real *cov, *init_cov;
    int32_t *cdf_tag;
    int32_t *rigid_id;
    Real *x_ref;
    int32_t *mod_mask;
};
inline RP to_rp(const gbmpm_particles& P) {
    auto r = [](float* f) { return reinterpret_cast<Real*>(f); };
    RP o;
    o.n = P.n;
    o.x = r(P.x); o.v = r(P.v); o.C = r(P.C); o.F = r(P.F); o.F_trial = r(P.F_trial); o.L = r(P.L);
    o.stress = r(P.stress); o.mass = r(P.mass); o.vol = r(P.vol); o.density = r(P.density); o.Jp = r(P.Jp);
    o.mu = r(P.mu); o.lam = r(P.lam); o.yield_stress = r(P.yield_stress);
    o.material = P.material; o.selection = P.selection; o.cov = r(P.cov); o.init_cov = r(P.init_cov);
    o.cdf_tag = P.cdf_tag; o.rigid_id = P.rigid_id; o.x_ref = r(P.x_ref); o.mod_mask = P.mod_mask;
    return o;
}

struct V3 { Real v[3]; Real& operator[](int i) { return v[i]; } Real operator[](int i) const { return v[i]; } };
struct M3 { Real m[3][3]; };

inline V3 mkv(Real a, Real b, Real c) { V3 r; r.v[0] = a; r.v[1] = b; r.v[2] = c; return r; }
inline M3 zero33() { M3 r; std::memset(&r, 0, sizeof r); return r; }
inline M3 ident33() { M3 r = zero33(); r.m[0][0] = r.m[1][1] = r.m[2][2] = 1.0f; return r; }
inline M3 diag33(Real a, Real b, Real c) { M3 r = zero33(); r.m[0][0] = a; r.m[1][1] = b; r.m[2][2] = c; return r; }
// loads and stores from either precision: the particle arrays are Real, collider
// and rigid-body records float
template <class T> inline M3 load33(const T* p) {
    M3 r;
    for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j) r.m[i][j] = (Real)p[3 * i + j];
    return r;
}
template <class T> inline void store33(T* p, const M3& a) {
    for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j) p[3 * i + j] = (T)a.m[i][j];
}
template <class T> inline V3 load3(const T* p) { return mkv((Real)p[0], (Real)p[1], (Real)p[2]); }
template <class T> inline void store3(T* p, const V3& a) { p[0] = (T)a[0]; p[1] = (T)a[1]; p[2] = (T)a[2]; }

inline V3 vadd(V3 a, V3 b) { return mkv(a[0] + b[0], a[1] + b[1], a[2] + b[2]); }
inline V3 vsub(V3 a, V3 b) { return mkv(a[0] - b[0], a[1] - b[1], a[2] - b[2]); }
inline V3 vscale(V3 a, Real s) { return mkv(a[0] * s, a[1] * s, a[2] * s); }
inline V3 vdivs(V3 a, Real s) { return mkv(a[0] / s, a[1] / s, a[2] / s); }
inline Real vdot(V3 a, V3 b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
inline Real vlen(V3 a) { return std::sqrt(vdot(a, a)); }
inline V3 vcross(V3 a, V3 b) {
    return mkv(a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]);
}
inline V3 vnormalize(V3 a) {
    Real l = vlen(a);
    if (l > 0.0f) return vdivs(a, l);
    return mkv(0, 0, 0);
}

// wp.log, wp.exp and wp.pow in fp32 as their correctly rounded values: each is
// evaluated in double by this file's own method and rounded once to Real. That is
// the correctly rounded float except when the exact value lies within about 1e-16
// of a float rounding boundary. The method is written here operation by operation
// (no libm), so the deterministic GPU passes, which state the same operations in the
// same order, return the same bits.
//   log x = k ln2 + 2 atanh(s), x = m 2^k with m in [1/sqrt 2, sqrt 2), s = (m - 1)/(m + 1),
//           the atanh series to s^23 (|s| <= 0.1716: the next term is below 1e-18);
//   exp x = 2^k exp(r), k = round(x / ln2), r = x - k ln2 (|r| <= 0.35), the Taylor
//           series to r^17 in Horner form (the next term is below 1e-22).
inline double dlog(double x) {
    if (!(x > 0.0) || x == HUGE_VAL) return (x == 0.0) ? -HUGE_VAL : (x == HUGE_VAL ? x : NAN);
    int k = 0;
    double m = std::frexp(x, &k);
    if (m < 0.70710678118654752440) { m = m * 2.0; k = k - 1; }
    const double s = (m - 1.0) / (m + 1.0);
    const double s2 = s * s;
    double t = 1.0 / 23.0;
    for (int j = 21; j >= 1; j -= 2) t = 1.0 / (double)j + s2 * t;
    return (double)k * 0.69314718055994530942 + 2.0 * s * t;
}
inline double dexp(double x) {
    if (x != x) return x;
    if (x > 709.0) return HUGE_VAL;
    if (x < -745.0) return 0.0;
    const double kd = std::floor(x * 1.44269504088896340736 + 0.5);
    const double r = x - kd * 0.69314718055994530942;
    double t = 1.0;
    for (int j = 17; j >= 1; --j) t = 1.0 + r * t / (double)j;
    return std::ldexp(t, (int)kd);
}
inline Real logr(Real x) { return (Real)dlog((double)x); }
inline Real expr(Real x) { return (Real)dexp((double)x); }
inline Real powr(Real x, Real y) { return (Real)dexp((double)y * dlog((double)x)); }

// wp.sin, wp.cos and wp.acos of the particle rotation modifier, the same way:
//   sin, cos: x = q pi/2 + r, q = round(x 2/pi) (|r| <= pi/4 for the angles the
//             modifier forms), then the Taylor series of sin r to r^21 and of cos r to
//             r^20 in nested form (the next terms are below 1e-23), and the quadrant;
//   acos c = pi/2 - asin c for |c| <= 1/2, 2 asin sqrt((1 - c)/2) above 1/2 and
//            pi - 2 asin sqrt((1 + c)/2) below -1/2, with the Taylor series of asin z
//            (|z| <= 1/2) to z^51 in Horner form (the next term is below 1e-18).
inline double dsincos(double x, bool want_cos) {
    if (!(x == x) || x == HUGE_VAL || x == -HUGE_VAL) return NAN;
    const double q = std::floor(x * 0.63661977236758134308 + 0.5);
    const double r = x - q * 1.57079632679489661923;
    const double r2 = r * r;
    double ts = 1.0, tc = 1.0;
    for (int k = 10; k >= 1; --k) {
        ts = 1.0 - r2 * ts / (double)((2 * k) * (2 * k + 1));
        tc = 1.0 - r2 * tc / (double)((2 * k - 1) * (2 * k));
    }
    const double sn = r * ts;
    int n = (int)((long long)q & 3);
    if (want_cos) n = (n + 1) & 3;   // cos x = sin(x + pi/2)
    return n == 0 ? sn : (n == 1 ? tc : (n == 2 ? -sn : -tc));
}
inline double dasin_half(double z) {   // |z| <= 1/2
    double coef[26];
    double a = 1.0;   // (2n)! / (4^n (n!)^2)
    for (int n = 0; n < 26; ++n) {
        coef[n] = a / (double)(2 * n + 1);
        a = a * (double)(2 * n + 1) / (double)(2 * n + 2);
    }
    const double z2 = z * z;
    double t = coef[25];
    for (int n = 24; n >= 0; --n) t = coef[n] + z2 * t;
    return z * t;
}
inline double dacos(double c) {
    if (!(c >= -1.0 && c <= 1.0)) return NAN;
    if (c > 0.5) return 2.0 * dasin_half(std::sqrt((1.0 - c) * 0.5));
    if (c < -0.5) return 3.14159265358979323846 - 2.0 * dasin_half(std::sqrt((1.0 + c) * 0.5));
    return 1.57079632679489661923 - dasin_half(c);
}
inline Real sinr(Real x) { return (Real)dsincos((double)x, false); }
inline Real cosr(Real x) { return (Real)dsincos((double)x, true); }
inline Real acosr(Real c) { return (Real)dacos((double)c); }

// warp mat*mat: t[i][j] += a[i][k]*b[k][j], k ascending from zero
inline M3 mmul(const M3& a, const M3& b) {
    M3 t = zero33();
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
            for (int k = 0; k < 3; ++k) t.m[i][j] = t.m[i][j] + a.m[i][k] * b.m[k][j];
    return t;
}
inline V3 mvmul(const M3& a, V3 b) {
    V3 r;
    for (int i = 0; i < 3; ++i) r[i] = a.m[i][0] * b[0] + a.m[i][1] * b[1] + a.m[i][2] * b[2];
    return r;
}
inline M3 mT(const M3& a) {
    M3 r;
    for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j) r.m[i][j] = a.m[j][i];
    return r;
}
inline M3 madd(const M3& a, const M3& b) {
    M3 r; for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j) r.m[i][j] = a.m[i][j] + b.m[i][j]; return r;
}
inline M3 msub(const M3& a, const M3& b) {
    M3 r; for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j) r.m[i][j] = a.m[i][j] - b.m[i][j]; return r;
}
inline M3 mscale(const M3& a, Real s) {
    M3 r; for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j) r.m[i][j] = a.m[i][j] * s; return r;
}
inline M3 outer(V3 a, V3 b) {
    M3 r; for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j) r.m[i][j] = a[i] * b[j]; return r;
}
// warp determinant(mat33) = dot(row0, cross(row1, row2))
inline Real mdet(const M3& a) {
    V3 r0 = mkv(a.m[0][0], a.m[0][1], a.m[0][2]);
    V3 r1 = mkv(a.m[1][0], a.m[1][1], a.m[1][2]);
    V3 r2 = mkv(a.m[2][0], a.m[2][1], a.m[2][2]);
    return vdot(r0, vcross(r1, r2));
}

// ---------------------------------------------------------------- svd3 -----
void svd3_impl(const M3& Fin, M3& U, V3& s, M3& V) {
    double A[3][3], B[3][3], W[3][3], Vd[3][3], Q[3][3];
    for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j) A[i][j] = Fin.m[i][j];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            double acc = 0.0;
            for (int k = 0; k < 3; ++k) acc += A[k][i] * A[k][j];
            B[i][j] = acc;
            Vd[i][j] = (i == j) ? 1.0 : 0.0;
        }
    // cyclic Jacobi on the symmetric B = A^T A
    for (int sweep = 0; sweep < 40; ++sweep) {
        double off = B[0][1] * B[0][1] + B[0][2] * B[0][2] + B[1][2] * B[1][2];
        double dia = B[0][0] * B[0][0] + B[1][1] * B[1][1] + B[2][2] * B[2][2];
        if (off <= 1e-32 * dia || off == 0.0) break;
        for (int p = 0; p < 2; ++p)
            for (int q = p + 1; q < 3; ++q) {
                if (B[p][q] == 0.0) continue;
                double theta = (B[q][q] - B[p][p]) / (2.0 * B[p][q]);
                double t = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
                double c = 1.0 / std::sqrt(t * t + 1.0), sn = t * c;
                for (int k = 0; k < 3; ++k) {  // B = J^T B J
                    double bkp = B[k][p], bkq = B[k][q];
                    B[k][p] = c * bkp - sn * bkq;
                    B[k][q] = sn * bkp + c * bkq;
                }
                for (int k = 0; k < 3; ++k) {
                    double bpk = B[p][k], bqk = B[q][k];
                    B[p][k] = c * bpk - sn * bqk;
                    B[q][k] = sn * bpk + c * bqk;
                }
                for (int k = 0; k < 3; ++k) {
                    double vkp = Vd[k][p], vkq = Vd[k][q];
                    Vd[k][p] = c * vkp - sn * vkq;
                    Vd[k][q] = sn * vkp + c * vkq;
                }
            }
    }
    // descending eigenvalues
    int ord[3] = {0, 1, 2};
    std::sort(ord, ord + 3, [&](int a, int b) { return B[a][a] > B[b][b]; });
    double Vs[3][3];
    for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j) Vs[i][j] = Vd[i][ord[j]];
    double dv = Vs[0][0] * (Vs[1][1] * Vs[2][2] - Vs[1][2] * Vs[2][1]) -
                Vs[0][1] * (Vs[1][0] * Vs[2][2] - Vs[1][2] * Vs[2][0]) +
                Vs[0][2] * (Vs[1][0] * Vs[2][1] - Vs[1][1] * Vs[2][0]);
    if (dv < 0) for (int i = 0; i < 3; ++i) Vs[i][2] = -Vs[i][2];
    // W = A V, then Givens QR: W = Q R with Q a proper rotation
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            double acc = 0.0;
            for (int k = 0; k < 3; ++k) acc += A[i][k] * Vs[k][j];
            W[i][j] = acc;
            Q[i][j] = (i == j) ? 1.0 : 0.0;
        }
    const int pr[3][2] = {{0, 1}, {0, 2}, {1, 2}};  // zero W[1][0], W[2][0], W[2][1]
    for (int g = 0; g < 3; ++g) {
        int a = pr[g][0], b = pr[g][1], col = (g < 2) ? 0 : 1;
        double x = W[a][col], y = W[b][col];
        double r = std::sqrt(x * x + y * y);   // O(1) entries: no overflow guard needed
        double c = 1.0, sn = 0.0;
        if (r > 0.0) { c = x / r; sn = y / r; }
        for (int k = 0; k < 3; ++k) {  // rows a, b of W: G W
            double wa = W[a][k], wb = W[b][k];
            W[a][k] = c * wa + sn * wb;
            W[b][k] = -sn * wa + c * wb;
        }
        for (int k = 0; k < 3; ++k) {  // Q = Q G^T
            double qa = Q[k][a], qb = Q[k][b];
            Q[k][a] = c * qa + sn * qb;
            Q[k][b] = -sn * qa + c * qb;
        }
    }
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) { U.m[i][j] = (Real)Q[i][j]; V.m[i][j] = (Real)Vs[i][j]; }
    s[0] = (Real)W[0][0]; s[1] = (Real)W[1][1]; s[2] = (Real)W[2][2];
}

// ------------------------------------------------------------ model view ---
struct Model {
    const gbmpm_model* m;
    Real dx, inv_dx;
};

struct Parts {
    const RP* p;
};

// --------------------------------------------------------- stress laws -----
// kirchoff_stress_FCR (mpm_utils.py:8-15)
M3 stress_fcr(const M3& F, const M3& U, const M3& V, Real J, Real mu, Real lam) {
    M3 R = mmul(U, mT(V));
    M3 t = mmul(mscale(msub(F, R), 2.0f * mu), mT(F));
    Real d = lam * J * (J - 1.0f);
    M3 id = ident33();
    return madd(t, mscale(id, d));
}
// kirchoff_stress_water (mpm_utils.py:17-25)
M3 stress_water(Real J, Real bulk) {
    const Real gamma = 1.1f;
    Real pressure = -bulk * (powr(J, -gamma) - 1.0f);
    M3 c = mscale(ident33(), pressure);
    return mscale(c, J);
}
// deviatoric strain rate shared by the newtonian and tabulated laws (mpm_utils.py:40-49)
void dev_rate(const M3& L, M3& Ddev, Real& gd) {
    const Real eps = 0.02f;
    M3 D = mscale(madd(L, mT(L)), 0.5f);
    Real trd = (D.m[0][0] + D.m[1][1] + D.m[2][2]) / 3.0f;
    Ddev = msub(D, mscale(ident33(), trd));
    Real dd = 0.0f;
    for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j) dd = dd + Ddev.m[i][j] * Ddev.m[i][j];
    gd = std::sqrt(2.0f * dd + eps * eps);
}
// kirchoff_stress_newtonian (mpm_utils.py:27-54)
M3 stress_newtonian(Real J, Real bulk, const M3& L, Real eta, Real tau_y, Real pk, Real pn) {
    const Real gamma = 1.1f;
    Real pressure = -bulk * (powr(J, -gamma) - 1.0f);
    M3 Ddev; Real gd;
    dev_rate(L, Ddev, gd);
    Real eta_app = eta + tau_y / gd + pk * powr(gd, pn - 1.0f);
    M3 c = madd(mscale(ident33(), pressure), mscale(Ddev, 2.0f * eta_app));
    return mscale(c, J);
}
// kirchoff_stress_tabulated (mpm_utils.py:56-85)
M3 stress_tabulated(Real J, Real bulk, const M3& L, const float* table, Real smin, Real smax, int n) {
    const Real gamma = 1.1f;
    Real pressure = -bulk * (powr(J, -gamma) - 1.0f);
    M3 Ddev; Real gd;
    dev_rate(L, Ddev, gd);
    Real s = logr(gd) * 0.43429448190325176f;
    Real idx = (s - smin) / (smax - smin) * (Real)(n - 1);
    idx = std::min<Real>(std::max<Real>(idx, 0.0f), (Real)(n - 1) - 1.0e-6f);
    int i0 = (int)std::floor(idx);
    Real frac = idx - (Real)i0;
    Real eta_app = table[i0] * (1.0f - frac) + table[i0 + 1] * frac;
    M3 c = madd(mscale(ident33(), pressure), mscale(Ddev, 2.0f * eta_app));
    return mscale(c, J);
}
// kirchoff_stress_drucker_prager (mpm_utils.py:109-124)
M3 stress_dp(const M3& F, const M3& U, const M3& V, V3 sig, Real mu, Real lam) {
    Real l0 = logr(sig[0]), l1 = logr(sig[1]), l2 = logr(sig[2]);
    Real lsum = l0 + l1 + l2;
    Real c0 = 2.0f * mu * logr(sig[0]) * (1.0f / sig[0]) + lam * lsum * (1.0f / sig[0]);
    Real c1 = 2.0f * mu * logr(sig[1]) * (1.0f / sig[1]) + lam * lsum * (1.0f / sig[1]);
    Real c2 = 2.0f * mu * logr(sig[2]) * (1.0f / sig[2]) + lam * lsum * (1.0f / sig[2]);
    return mmul(mmul(mmul(U, diag33(c0, c1, c2)), mT(V)), mT(F));
}
// kirchoff_stress_hencky (mpm_utils.py:228-243)
M3 stress_hencky(const M3& U, V3 sig, Real mu, Real lam) {
    Real e0 = logr(std::max<Real>(sig[0], 1e-6f)), e1 = logr(std::max<Real>(sig[1], 1e-6f)),
          e2 = logr(std::max<Real>(sig[2], 1e-6f));
    Real tr = e0 + e1 + e2;
    M3 t = diag33(2.0f * mu * e0 + lam * tr, 2.0f * mu * e1 + lam * tr, 2.0f * mu * e2 + lam * tr);
    return mmul(mmul(U, t), mT(U));
}
// mu_i_phi_pressure (mpm_utils.py:421-430)
Real mu_i_phi_pressure(const gbmpm_model* m, int mat, Real J, Real Jp_ref) {
    Real K = m->E[mat] / (3.0f * (1.0f - 2.0f * m->nu[mat]));
    Real p = K * (Jp_ref / std::max<Real>(J, 1e-6f) - 1.0f);
    return std::max<Real>(p, 0.0f);
}
// kirchoff_stress_mu_i_phi (mpm_utils.py:525-540)
M3 stress_mu_i_phi(const M3& U, V3 sig, Real G, Real p_comp) {
    Real s0 = std::max<Real>(sig[0], 1e-6f), s1 = std::max<Real>(sig[1], 1e-6f), s2 = std::max<Real>(sig[2], 1e-6f);
    Real e0 = logr(s0), e1 = logr(s1), e2 = logr(s2);
    Real J = s0 * s1 * s2;
    Real mean = (e0 + e1 + e2) / 3.0f;
    Real iso = -p_comp * J;
    M3 t = diag33(2.0f * G * (e0 - mean) + iso, 2.0f * G * (e1 - mean) + iso, 2.0f * G * (e2 - mean) + iso);
    return mmul(mmul(U, t), mT(U));
}

// ------------------------------------------------------- return maps -------
// von_mises_return_mapping (mpm_utils.py:127-170); with_damage (:172-225)
M3 rm_von_mises(const M3& Ft, const RP* P, const gbmpm_model* m, int p, int mat, bool damage) {
    M3 U, V; V3 so;
    svd3_impl(Ft, U, so, V);
    V3 sig = mkv(std::max<Real>(so[0], 0.01f), std::max<Real>(so[1], 0.01f), std::max<Real>(so[2], 0.01f));
    V3 eps = mkv(logr(sig[0]), logr(sig[1]), logr(sig[2]));
    Real temp = (eps[0] + eps[1] + eps[2]) / 3.0f;
    Real mu = P->mu[p], lam = P->lam[p];
    Real tr = eps[0] + eps[1] + eps[2];
    V3 tau = vadd(vscale(eps, 2.0f * mu), vscale(mkv(1, 1, 1), lam * tr));
    Real sum_tau = tau[0] + tau[1] + tau[2];
    V3 cond = mkv(tau[0] - sum_tau / 3.0f, tau[1] - sum_tau / 3.0f, tau[2] - sum_tau / 3.0f);
    if (vlen(cond) > P->yield_stress[p]) {
        if (damage && P->yield_stress[p] <= 0) return Ft;
        V3 eh = vsub(eps, mkv(temp, temp, temp));
        Real ehn = vlen(eh) + 1e-6f;
        Real dg = ehn - P->yield_stress[p] / (2.0f * mu);
        eps = vsub(eps, vscale(eh, dg / ehn));
        if (damage) {
            P->yield_stress[p] = P->yield_stress[p] - m->softening[mat] * vlen(vscale(eh, dg / ehn));
            if (P->yield_stress[p] <= 0) { P->mu[p] = 0.0f; P->lam[p] = 0.0f; }
        }
        M3 se = diag33(expr(eps[0]), expr(eps[1]), expr(eps[2]));
        M3 Fe = mmul(mmul(U, se), mT(V));
        if (m->hardening[mat] > 0.5f)
            P->yield_stress[p] = P->yield_stress[p] + 2.0f * P->mu[p] * m->xi[mat] * dg;
        return Fe;
    }
    return Ft;
}

// mu_i_return_mapping (mpm_utils.py:246-324) and the tabulated variant (:327-407)
M3 rm_mu_i(const M3& Ft, const RP* P, const gbmpm_model* m, int p, int mat, Real dt, bool tab) {
    M3 U, V; V3 sig;
    svd3_impl(Ft, U, sig, V);
    V3 sc = mkv(std::max<Real>(std::fabs(sig[0]), 1e-6f), std::max<Real>(std::fabs(sig[1]), 1e-6f),
                std::max<Real>(std::fabs(sig[2]), 1e-6f));
    V3 eps = mkv(logr(sc[0]), logr(sc[1]), logr(sc[2]));
    Real tr = eps[0] + eps[1] + eps[2];
    M3 Fe = Ft;
    if (tr >= 0.0f) {
        Fe = mmul(U, mT(V));
    } else {
        Real G = P->mu[p], lam = P->lam[p];
        Real J = sc[0] * sc[1] * sc[2];
        Real mean = tr / 3.0f;
        Real d0 = eps[0] - mean, d1 = eps[1] - mean, d2 = eps[2] - mean;
        Real dn = std::sqrt(d0 * d0 + d1 * d1 + d2 * d2);
        Real pK = -(2.0f * G / 3.0f + lam) * tr;
        Real tbK = 2.0f * G * dn / std::sqrt(2.0f);
        Real pC = pK / J;
        Real mu_s = m->muI_mu_s[mat], dmu = m->muI_delta_mu[mat], I0 = m->muI_I0[mat];
        Real thresh = tab ? m->eta_table[0] : mu_s;
        if (tbK > thresh * pK) {
            Real Ic = m->muI_d[mat] * std::sqrt(m->muI_rho_s[mat] / pC);
            Real lo = 0.0f, hi = tbK / (G * dt);
            for (int it = 0; it < 48; ++it) {
                Real mid = 0.5f * (lo + hi);
                Real Im = mid * Ic;
                Real mu_mid;
                if (!tab) {
                    mu_mid = mu_s + dmu * Im / (Im + I0);
                } else {
                    Real s = logr(std::max<Real>(Im, 1e-12f)) * 0.43429448190325176f;
                    Real idx = (s - m->eta_table_smin) / (m->eta_table_smax - m->eta_table_smin) *
                                (Real)(m->eta_table_n - 1);
                    idx = std::min<Real>(std::max<Real>(idx, 0.0f), (Real)(m->eta_table_n - 1) - 1.0e-6f);
                    int i0 = (int)std::floor(idx);
                    Real fr = idx - (Real)i0;
                    mu_mid = m->eta_table[i0] * (1.0f - fr) + m->eta_table[i0 + 1] * fr;
                }
                Real g = tbK - G * dt * mid - mu_mid * pK;
                if (g > 0.0f) lo = mid; else hi = mid;
            }
            Real gdp = 0.5f * (lo + hi);
            Real tbn = tbK - G * dt * gdp;
            Real scale = tbn / std::max<Real>(tbK, 1e-20f);
            Real e0 = d0 * scale + mean, e1 = d1 * scale + mean, e2 = d2 * scale + mean;
            Fe = mmul(mmul(U, diag33(expr(e0), expr(e1), expr(e2))), mT(V));
        }
    }
    return Fe;
}

// j_cs_of_I (mpm_utils.py:410-418)
Real j_cs_of_I(const gbmpm_model* m, int mat, Real I) {
    Real I0 = m->muI_I0[mat], chi = m->muI_phi_chi[mat];
    Real denom = std::max<Real>(1.0f - chi * I / (I + I0), 1e-3f);
    return 1.0f / denom;
}

// mu_i_phi_return_mapping (mpm_utils.py:433-522)
M3 rm_mu_i_phi(const M3& Ft, const RP* P, const gbmpm_model* m, int p, int mat, Real dt) {
    M3 U, V; V3 sig;
    svd3_impl(Ft, U, sig, V);
    V3 sc = mkv(std::max<Real>(std::fabs(sig[0]), 1e-6f), std::max<Real>(std::fabs(sig[1]), 1e-6f),
                std::max<Real>(std::fabs(sig[2]), 1e-6f));
    V3 eps = mkv(logr(sc[0]), logr(sc[1]), logr(sc[2]));
    Real J = sc[0] * sc[1] * sc[2];
    Real tr = eps[0] + eps[1] + eps[2];
    Real mean = tr / 3.0f;
    Real d0 = eps[0] - mean, d1 = eps[1] - mean, d2 = eps[2] - mean;
    Real dn = std::sqrt(d0 * d0 + d1 * d1 + d2 * d2);
    Real G = P->mu[p];
    Real Jp_ref = P->Jp[p];
    if (Jp_ref < 0.5f) Jp_ref = 1.0f;
    Real pc = mu_i_phi_pressure(m, mat, J, Jp_ref);
    const Real beta = 8.0f;
    M3 Fe = Ft;
    P->Jp[p] = Jp_ref;
    if (pc <= 0.0f) {
        Real si = expr(mean);
        Fe = mmul(mmul(U, diag33(si, si, si)), mT(V));
    } else {
        Real pK = pc * J;
        Real tbK = 2.0f * G * dn / std::sqrt(2.0f);
        Real mu_s = m->muI_mu_s[mat], dmu = m->muI_delta_mu[mat], I0 = m->muI_I0[mat];
        if (tbK > mu_s * pK) {
            Real Ic = m->muI_d[mat] * std::sqrt(m->muI_rho_s[mat] / pc);
            Real lo = 0.0f, hi = tbK / (G * dt);
            for (int it = 0; it < 48; ++it) {
                Real mid = 0.5f * (lo + hi);
                Real Im = mid * Ic;
                Real mu_mid = mu_s + dmu * Im / (Im + I0);
                Real g = tbK - G * dt * mid - mu_mid * pK;
                if (g > 0.0f) lo = mid; else hi = mid;
            }
            Real gdp = 0.5f * (lo + hi);
            Real Ir = gdp * Ic;
            Real dgam = std::min<Real>(beta * gdp * dt, 1.0f);
            Real jcs = j_cs_of_I(m, mat, Ir);
            P->Jp[p] = Jp_ref + dgam * (jcs - Jp_ref);
            Real tbn = tbK - G * dt * gdp;
            Real scale = tbn / std::max<Real>(tbK, 1e-20f);
            Real e0 = d0 * scale + mean, e1 = d1 * scale + mean, e2 = d2 * scale + mean;
            Fe = mmul(mmul(U, diag33(expr(e0), expr(e1), expr(e2))), mT(V));
        }
    }
    return Fe;
}

// sand_return_mapping (mpm_utils.py:543-580)
M3 rm_sand(const M3& Ft, const RP* P, const gbmpm_model* m, int p, int mat) {
    M3 U, V; V3 sig;
    svd3_impl(Ft, U, sig, V);
    V3 eps = mkv(logr(std::max<Real>(std::fabs(sig[0]), 1e-14f)), logr(std::max<Real>(std::fabs(sig[1]), 1e-14f)),
                 logr(std::max<Real>(std::fabs(sig[2]), 1e-14f)));
    Real tr = eps[0] + eps[1] + eps[2];
    V3 eh = vsub(eps, mkv(tr / 3.0f, tr / 3.0f, tr / 3.0f));
    Real ehn = vlen(eh);
    Real mu = P->mu[p], lam = P->lam[p];
    Real dg = ehn + (3.0f * lam + 2.0f * mu) / (2.0f * mu) * tr * m->alpha[mat];
    M3 Fe = Ft;
    if (dg <= 0) Fe = Ft;
    if (dg > 0 && tr > 0) Fe = mmul(U, mT(V));
    if (dg > 0 && tr <= 0) {
        V3 H = vsub(eps, vscale(eh, dg / ehn));
        Fe = mmul(mmul(U, diag33(expr(H[0]), expr(H[1]), expr(H[2]))), mT(V));
    }
    return Fe;
}

// CPIC (CDF) state; its kernels follow the collider section
constexpr int kOwnerShift = 8;
constexpr int kOwnerMask = 3 << kOwnerShift;

struct CdfState {
    int n_grid = 0, nb = 0, n = 0;
    std::vector<int32_t> tag, tag_prev, block;
    std::vector<Real> d, d_prev;
    gbmpm_cdf rec[GBMPM_MAX_CDF];
    Real c_cur[4][3] = {}, v_cur[4][3] = {}, w_cur[4][3] = {};
    Real c_prev[4][3] = {}, v_prev[4][3] = {}, w_prev[4][3] = {};
    Real fric[4] = {};
    int type[4] = {};
    bool dirty[4] = {}, active[4] = {}, has_prev_box[4] = {};
    int prev_box[4][6] = {};
    bool stale_set = false;
    int stale_box[6] = {};
    bool lane_prev_stale = false;
    int stamp_count = 0;
    void alloc(int ng) {
        n_grid = ng;
        nb = (ng + 3) / 4;
        size_t N = (size_t)ng * ng * ng;
        tag.assign(N, 0); tag_prev.assign(N, 0);
        d.assign(N, 1.0e9f); d_prev.assign(N, 1.0e9f);
        block.assign((size_t)nb * nb * nb, 0);
    }
    size_t idx(int x, int y, int z) const { return ((size_t)x * n_grid + y) * n_grid + z; }
    void sync_lane(int l) {  // _sync_cdf_lane (mpm_solver_warp.py:2883-2905)
        const gbmpm_cdf& r = rec[l];
        for (int a = 0; a < 3; ++a) { c_cur[l][a] = r.center[a]; v_cur[l][a] = r.velocity[a]; w_cur[l][a] = r.omega[a]; }
        fric[l] = r.friction;
        type[l] = r.surface_type;
    }
    void copy_lane_prev() {
        std::memcpy(c_prev, c_cur, sizeof c_cur);
        std::memcpy(v_prev, v_cur, sizeof v_cur);
        std::memcpy(w_prev, w_cur, sizeof w_cur);
        lane_prev_stale = false;
    }
};

inline bool cdf_incompatible(int pc, int nt);
bool cdf_stencil_near(const CdfState& S, const int* b);
struct Weights;
int cdf_particle_tag(const CdfState& S, const Weights& W, bool use_prev);
int cdf_persist(int old, int fresh);
V3 cdf_ghost(const CdfState& S, const gbmpm_model* M, Real dt, V3 xp, V3 vp, int pc, const Weights& W);

// ----------------------------------------------------- particle stages -----
struct Weights {
    int base[3];
    Real fx[3];
    Real w[3][3];   // w[axis][i]
    Real dw[3][3];
};

inline void bspline(const Real* x, Real inv_dx, Weights& W) {
    for (int a = 0; a < 3; ++a) {
        Real gp = x[a] * inv_dx;
        W.base[a] = (int)std::floor(gp - 0.5f);
        W.fx[a] = gp - (Real)W.base[a];
        Real fx = W.fx[a];
        Real wa = 1.5f - fx, wb = fx - 1.0f, wc = fx - 0.5f;
        W.w[a][0] = wa * wa * 0.5f;
        W.w[a][1] = (0.0f - wb * wb) + 0.75f;
        W.w[a][2] = wc * wc * 0.5f;
        W.dw[a][0] = fx - 1.5f;
        W.dw[a][1] = -2.0f * (fx - 1.0f);
        W.dw[a][2] = fx - 0.5f;
    }
}

// compute_dweight (mpm_utils.py:601-610)
inline V3 dweight(const Weights& W, int i, int j, int k, Real inv_dx) {
    V3 d = mkv(W.dw[0][i] * W.w[1][j] * W.w[2][k], W.w[0][i] * W.dw[1][j] * W.w[2][k],
               W.w[0][i] * W.w[1][j] * W.dw[2][k]);
    return vscale(d, inv_dx);
}

struct Grid {
    int n = 0;
    std::vector<Real> m, vin, vout;   // m[n^3], vin/vout[n^3][3]
    // box of nodes written since the last zero: [lo, hi) per axis
    int lo[3], hi[3];
    int plo[3], phi[3];
    void resize(int nn) {
        if (n == nn) return;
        n = nn;
        size_t N = (size_t)nn * nn * nn;
        m.assign(N, 0.0f); vin.assign(3 * N, 0.0f); vout.assign(3 * N, 0.0f);
        reset_box();
        for (int a = 0; a < 3; ++a) { plo[a] = nn; phi[a] = 0; }
    }
    void reset_box() { for (int a = 0; a < 3; ++a) { lo[a] = n; hi[a] = 0; } }
    size_t idx(int x, int y, int z) const { return ((size_t)x * n + y) * n + z; }
};

thread_local const char* g_err = "";

struct Ctx {
    const RP* P;
    const gbmpm_model* M;
    Grid* G;
    Real dt;
    bool atomic;   // parallel mode
    int oob;
    CdfState* cdf = nullptr;     // CPIC lanes (null or n == 0: feature off)
    Real* cdf_wrench = nullptr; // [4][6] blocked-deposit reaction
};

inline int wrapx(int ix, int n) { return ((ix % n) + n) % n; }

// p2g_particle (mpm_utils.py:819-916), CDF branch omitted (no CDF colliders)
void p2g_particle(Ctx& c, int p) {
    const RP* P = c.P;
    const gbmpm_model* M = c.M;
    Grid& G = *c.G;
    M3 stress = load33(P->stress + 9 * (size_t)p);
    Weights W;
    bspline(P->x + 3 * (size_t)p, M->inv_dx, W);
    int n = G.n;
    for (int a = 0; a < 3; ++a) {
        int b0 = W.base[a], b1 = W.base[a] + 2;
        if (a == 0 && M->periodic_x) continue;
        if (b0 < 0 || b1 >= n) { c.oob = 1; return; }
    }
    M3 C = load33(P->C + 9 * (size_t)p);
    Real r = M->rpic_damping;
    C = madd(mscale(C, 1.0f - r), mscale(msub(C, mT(C)), r / 2.0f));
    if (r < -0.001f) C = zero33();
    Real mass = P->mass[p], vol = P->vol[p];
    V3 v = load3(P->v + 3 * (size_t)p);
    M3 fs = mscale(stress, -vol);
    int pc = 0;
    if (c.cdf && c.cdf->n > 0 && cdf_stencil_near(*c.cdf, W.base))
        pc = cdf_persist(P->cdf_tag ? P->cdf_tag[p] : 0, cdf_particle_tag(*c.cdf, W, false));
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
            for (int k = 0; k < 3; ++k) {
                V3 dpos = vscale(vsub(mkv((Real)i, (Real)j, (Real)k), mkv(W.fx[0], W.fx[1], W.fx[2])), M->dx);
                int ix = W.base[0] + i, iy = W.base[1] + j, iz = W.base[2] + k;
                if (M->periodic_x) ix = wrapx(ix, n);
                Real weight = W.w[0][i] * W.w[1][j] * W.w[2][k];
                V3 dwt = dweight(W, i, j, k, M->inv_dx);
                V3 ef = mvmul(fs, dwt);
                V3 add = vadd(vscale(vadd(v, mvmul(C, dpos)), weight * mass), vscale(ef, c.dt));
                size_t id = G.idx(ix, iy, iz);
                Real dm = weight * mass;
                if (pc != 0) {
                    int nt = c.cdf->tag[id];
                    if (cdf_incompatible(pc, nt)) {   // blocked deposit = reaction on the sheet
                        int own = (nt >> kOwnerShift) & 3;
                        V3 xw = mkv((Real)ix * M->dx, (Real)iy * M->dx, (Real)iz * M->dx);
                        V3 tq = vcross(vsub(xw, load3(c.cdf->c_cur[own])), add);
                        Real* acc = c.cdf_wrench + 6 * own;
                        for (int a = 0; a < 3; ++a) {
                            if (c.atomic) {
#pragma omp atomic
                                acc[a] += add[a];
#pragma omp atomic
                                acc[3 + a] += tq[a];
                            } else {
                                acc[a] += add[a];
                                acc[3 + a] += tq[a];
                            }
                        }
                        continue;
                    }
                }
                if (c.atomic) {
#pragma omp atomic
                    G.vin[3 * id + 0] += add[0];
#pragma omp atomic
                    G.vin[3 * id + 1] += add[1];
#pragma omp atomic
                    G.vin[3 * id + 2] += add[2];
#pragma omp atomic
                    G.m[id] += dm;
                } else {
                    G.vin[3 * id + 0] += add[0];
                    G.vin[3 * id + 1] += add[1];
                    G.vin[3 * id + 2] += add[2];
                    G.m[id] += dm;
                }
            }
}

// update_cov (mpm_utils.py:613-633)
void update_cov(const RP* P, int p, const M3& gv, Real dt) {
    Real* c6 = P->cov + 6 * (size_t)p;
    M3 cn;
    cn.m[0][0] = c6[0]; cn.m[0][1] = c6[1]; cn.m[0][2] = c6[2];
    cn.m[1][0] = c6[1]; cn.m[1][1] = c6[3]; cn.m[1][2] = c6[4];
    cn.m[2][0] = c6[2]; cn.m[2][1] = c6[4]; cn.m[2][2] = c6[5];
    M3 nn = madd(cn, mscale(madd(mmul(gv, cn), mmul(cn, mT(gv))), dt));
    c6[0] = nn.m[0][0]; c6[1] = nn.m[0][1]; c6[2] = nn.m[0][2];
    c6[3] = nn.m[1][1]; c6[4] = nn.m[1][2]; c6[5] = nn.m[2][2];
}

// g2p_particle (mpm_utils.py:944-1043), CDF branch omitted
void g2p_particle(Ctx& c, int p) {
    const RP* P = c.P;
    const gbmpm_model* M = c.M;
    Grid& G = *c.G;
    Weights W;
    bspline(P->x + 3 * (size_t)p, M->inv_dx, W);
    int n = G.n;
    for (int a = 0; a < 3; ++a) {
        if (a == 0 && M->periodic_x) continue;
        if (W.base[a] < 0 || W.base[a] + 2 >= n) { c.oob = 1; return; }
    }
    int pc = 0;
    V3 ghost = mkv(0, 0, 0);
    if (c.cdf && c.cdf->n > 0) {
        if (cdf_stencil_near(*c.cdf, W.base))
            pc = cdf_persist(P->cdf_tag ? P->cdf_tag[p] : 0, cdf_particle_tag(*c.cdf, W, true));
        if (P->cdf_tag) P->cdf_tag[p] = pc;
        if (pc != 0)
            ghost = cdf_ghost(*c.cdf, M, c.dt, load3(P->x + 3 * (size_t)p), load3(P->v + 3 * (size_t)p), pc, W);
    }
    V3 nv = mkv(0, 0, 0);
    M3 nC = zero33(), nF = zero33();
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
            for (int k = 0; k < 3; ++k) {
                int ix = W.base[0] + i, iy = W.base[1] + j, iz = W.base[2] + k;
                if (M->periodic_x) ix = wrapx(ix, n);
                V3 dpos = vsub(mkv((Real)i, (Real)j, (Real)k), mkv(W.fx[0], W.fx[1], W.fx[2]));
                Real weight = W.w[0][i] * W.w[1][j] * W.w[2][k];
                size_t id = G.idx(ix, iy, iz);
                V3 gv = load3(&G.vout[3 * id]);
                if (pc != 0 && cdf_incompatible(pc, c.cdf->tag_prev[id])) gv = ghost;
                nv = vadd(nv, vscale(gv, weight));
                nC = madd(nC, mscale(outer(gv, dpos), weight * M->inv_dx * 4.0f));
                V3 dwt = dweight(W, i, j, k, M->inv_dx);
                nF = madd(nF, outer(gv, dwt));
            }
    store3(P->v + 3 * (size_t)p, nv);
    V3 x = load3(P->x + 3 * (size_t)p);
    V3 xn = vadd(x, vscale(nv, c.dt));
    if (M->periodic_x) {
        Real lx = (Real)n * M->dx;
        if (xn[0] < 0.0f) xn[0] = xn[0] + lx;
        if (xn[0] >= lx) xn[0] = xn[0] - lx;
    }
    store3(P->x + 3 * (size_t)p, xn);
    store33(P->C + 9 * (size_t)p, nC);
    store33(P->L + 9 * (size_t)p, nF);
    M3 Ft = mmul(madd(ident33(), mscale(nF, c.dt)), load33(P->F + 9 * (size_t)p));
    store33(P->F_trial + 9 * (size_t)p, Ft);
    if (M->update_cov_with_F && P->cov) update_cov(P, p, nF, c.dt);
}

// stress_update_particle (mpm_utils.py:1056-1149)
void stress_particle(Ctx& c, int p) {
    const RP* P = c.P;
    const gbmpm_model* M = c.M;
    int mat = P->material[p];
    M3 Ft = load33(P->F_trial + 9 * (size_t)p);
    M3 F;
    if (mat == 1) F = rm_von_mises(Ft, P, M, p, mat, false);
    else if (mat == 2) F = rm_sand(Ft, P, M, p, mat);
    else if (mat == 5) F = rm_von_mises(Ft, P, M, p, mat, true);
    else if (mat == 9) F = rm_mu_i(Ft, P, M, p, mat, c.dt, false);
    else if (mat == 13) F = rm_mu_i(Ft, P, M, p, mat, c.dt, true);
    else if (mat == 11) F = rm_mu_i_phi(Ft, P, M, p, mat, c.dt);
    else if (mat == 6 || mat == 10 || mat == 12) {
        Real J = mdet(Ft);
        Real Jc = powr(J, 1.0f / 3.0f);
        F = diag33(Jc, Jc, Jc);
    } else if (mat == 7 || mat == 8) F = ident33();
    else F = Ft;
    store33(P->F + 9 * (size_t)p, F);

    Real J = mdet(F);
    M3 U = zero33(), V = zero33(); V3 sig = mkv(0, 0, 0);
    M3 st = zero33();
    if (mat != 6 && mat != 7 && mat != 8 && mat != 10 && mat != 12) svd3_impl(F, U, sig, V);
    if (mat == 0 || mat == 5) st = stress_fcr(F, U, V, J, P->mu[p], P->lam[p]);
    if (mat == 1) st = stress_hencky(U, sig, P->mu[p], P->lam[p]);
    if (mat == 2) st = stress_dp(F, U, V, sig, P->mu[p], P->lam[p]);
    if (mat == 6) st = stress_water(J, M->bulk[mat]);
    if (mat == 10)
        st = stress_newtonian(J, M->bulk[mat], load33(P->L + 9 * (size_t)p), M->plastic_viscosity[mat],
                              P->yield_stress[p], M->hardening[mat], M->softening[mat]);
    if (mat == 12)
        st = stress_tabulated(J, M->bulk[mat], load33(P->L + 9 * (size_t)p), M->eta_table, M->eta_table_smin,
                              M->eta_table_smax, M->eta_table_n);
    if (mat == 9 || mat == 13) st = stress_hencky(U, sig, P->mu[p], P->lam[p]);
    if (mat == 11) {
        Real Jr = P->Jp[p];
        if (Jr < 0.5f) Jr = 1.0f;
        Real pc = mu_i_phi_pressure(M, mat, J, Jr);
        st = stress_mu_i_phi(U, sig, P->mu[p], pc);
    }
    st = mscale(madd(st, mT(st)), 0.5f);
    // warp divides by 2.0 (:1148); x*0.5 and x/2 round identically
    store33(P->stress + 9 * (size_t)p, st);
}

// ------------------------------------------------------------ colliders -----
// capped_cylinder_sdf / revolved_glass_sdf (mpm_solver_warp.py:29-57)
Real capped_cyl(Real r, Real z, Real rad, Real z0, Real z1) {
    Real zc = 0.5f * (z0 + z1), hh = 0.5f * (z1 - z0);
    Real dr = r - rad, dz = std::fabs(z - zc) - hh;
    Real dro = std::max<Real>(dr, 0.0f), dzo = std::max<Real>(dz, 0.0f);
    Real outside = std::sqrt(dro * dro + dzo * dzo);
    Real inside = std::min<Real>(std::max<Real>(dr, dz), 0.0f);
    return outside + inside;
}
Real glass_sdf(V3 l, const gbmpm_collider& c) {
    Real r = std::sqrt(l[0] * l[0] + l[1] * l[1]);
    Real d_outer = capped_cyl(r, l[2], c.outer_radius, -c.half_height, c.half_height);
    Real d_cav = capped_cyl(r, l[2], c.inner_radius - c.fillet_radius, c.inner_floor_z + c.fillet_radius,
                             c.half_height + c.outer_radius) - c.fillet_radius;
    return std::max(d_outer, -d_cav);
}

// sdf_trilerp (mpm_solver_warp.py:60-74)
template <class T> Real trilerp(const T* vals, int res, V3 f, int stride, int comp) {
    Real fi = std::min<Real>(std::max<Real>(f[0], 0.0f), (Real)res - 1.0001f);
    Real fj = std::min<Real>(std::max<Real>(f[1], 0.0f), (Real)res - 1.0001f);
    Real fk = std::min<Real>(std::max<Real>(f[2], 0.0f), (Real)res - 1.0001f);
    int i = (int)std::floor(fi), j = (int)std::floor(fj), k = (int)std::floor(fk);
    Real tx = fi - (Real)i, ty = fj - (Real)j, tz = fk - (Real)k;
    auto at = [&](int a, int b, int cc) { return vals[(((size_t)a * res + b) * res + cc) * stride + comp]; };
    Real c00 = at(i, j, k) * (1.0f - tx) + at(i + 1, j, k) * tx;
    Real c01 = at(i, j, k + 1) * (1.0f - tx) + at(i + 1, j, k + 1) * tx;
    Real c10 = at(i, j + 1, k) * (1.0f - tx) + at(i + 1, j + 1, k) * tx;
    Real c11 = at(i, j + 1, k + 1) * (1.0f - tx) + at(i + 1, j + 1, k + 1) * tx;
    Real c0 = c00 * (1.0f - ty) + c10 * ty;
    Real c1 = c01 * (1.0f - ty) + c11 * ty;
    return c0 * (1.0f - tz) + c1 * tz;
}

// warp quat_rotate / quat_rotate_inv: x(2w^2-1) +/- 2w(q x x) + 2q(q.x)
template <class T> V3 qrot(const T q[4], V3 x, bool inv) {
    V3 qv = mkv(q[0], q[1], q[2]);
    Real w = q[3];
    Real c = 2.0f * w * w - 1.0f;
    V3 a = vscale(x, c);
    V3 b = vscale(vscale(vcross(qv, x), w), 2.0f);
    V3 d = vscale(vscale(qv, vdot(qv, x)), 2.0f);
    return inv ? vadd(vsub(a, b), d) : vadd(vadd(a, b), d);
}

struct NodeCtx {
    Real time;
    Real dt;
    const gbmpm_model* M;
};

// one collider applied to one node; returns true when the node was handled
void collide_node(const gbmpm_collider& c, int gx, int gy, int gz, Real m, Real* vout, const NodeCtx& nc,
                  Real* acc /* force[3], torque[3] fp32 */, bool atomic) {
    const gbmpm_model* M = nc.M;
    Real dx = M->dx;
    if (m <= 0.0f) return;   // mass gate (mpm_solver_warp.py:1942 and the other collide kernels)
    bool live = nc.time >= c.start_time && nc.time < c.end_time;
    auto addacc = [&](int i, Real v) {
        if (atomic) {
#pragma omp atomic
            acc[i] += v;
        } else {
            acc[i] += v;
        }
    };
    switch (c.kind) {
    case GBMPM_COLLIDER_PLANE: {  // mpm_solver_warp.py:1929-1992
        if (!live) return;
        V3 off = mkv((Real)gx * dx - c.point[0], (Real)gy * dx - c.point[1], (Real)gz * dx - c.point[2]);
        V3 n = mkv(c.normal[0], c.normal[1], c.normal[2]);
        Real dp = vdot(off, n);
        if (dp < 0.0f) {
            if (c.surface_type == 0) {
                vout[0] = vout[1] = vout[2] = 0.0f;
            } else if (c.surface_type == 11) {
                if ((Real)gz * dx < 0.4f || (Real)gz * dx > 0.53f) {
                    vout[0] = vout[1] = vout[2] = 0.0f;
                } else {
                    V3 vi = load3(vout);
                    V3 r = vscale(mkv(vi[0], 0.0f, vi[2]), 0.3f);
                    store3(vout, r);
                }
            } else {
                V3 v = load3(vout);
                Real nc_ = vdot(v, n);
                if (c.surface_type == 1) v = vsub(v, vscale(n, nc_));
                else v = vsub(v, vscale(n, std::min<Real>(nc_, 0.0f)));
                if (nc_ < 0.0f && vlen(v) > 1e-20f) {
                    Real s = std::max<Real>(0.0f, vlen(v) + nc_ * c.friction);
                    v = vscale(vnormalize(v), s);
                }
                store3(vout, v);
            }
        }
        return;
    }
    case GBMPM_COLLIDER_BOX: {  // mpm_solver_warp.py:2053-2088
        if (live) {
            V3 off = mkv((Real)gx * dx - c.point[0], (Real)gy * dx - c.point[1], (Real)gz * dx - c.point[2]);
            if (std::fabs(off[0]) < c.size[0] && std::fabs(off[1]) < c.size[1] && std::fabs(off[2]) < c.size[2]) {
                V3 vf = load3(vout);
                V3 vb = mkv(c.velocity[0], c.velocity[1], c.velocity[2]);
                V3 imp = vscale(vsub(vf, vb), m);
                addacc(0, imp[0]); addacc(1, imp[1]); addacc(2, imp[2]);
                store3(vout, vb);
            }
        } else if (c.reset == 1) {
            if (nc.time < c.end_time + 15.0f * nc.dt) vout[0] = vout[1] = vout[2] = 0.0f;
        }
        return;
    }
    case GBMPM_COLLIDER_CUP: {  // mpm_solver_warp.py:2161-2225
        if (!live) return;
        V3 xn = mkv((Real)gx * dx, (Real)gy * dx, (Real)gz * dx);
        V3 rel = vsub(xn, mkv(c.point[0], c.point[1], c.point[2]));
        M3 R = load33(c.rot);
        V3 local = mvmul(mT(R), rel);
        Real sdf = glass_sdf(local, c);
        if (sdf < c.contact_band) {
            V3 vs = vadd(mkv(c.velocity[0], c.velocity[1], c.velocity[2]),
                         vcross(mkv(c.omega[0], c.omega[1], c.omega[2]), rel));
            V3 vin = load3(vout);
            V3 vnew = vs;
            if (sdf > -c.sticky_depth) {
                vnew = vin;
                Real h = 0.25f * dx;
                V3 nl = mkv(glass_sdf(vadd(local, mkv(h, 0, 0)), c) - glass_sdf(vsub(local, mkv(h, 0, 0)), c),
                            glass_sdf(vadd(local, mkv(0, h, 0)), c) - glass_sdf(vsub(local, mkv(0, h, 0)), c),
                            glass_sdf(vadd(local, mkv(0, 0, h)), c) - glass_sdf(vsub(local, mkv(0, 0, h)), c));
                Real nl_len = vlen(nl);
                if (nl_len > 1.0e-12f) {
                    V3 n = mvmul(R, vdivs(nl, nl_len));
                    V3 vr = vsub(vin, vs);
                    Real vn = vdot(vr, n);
                    if (vn < 0.0f) {
                        V3 vt = vsub(vr, vscale(n, vn));
                        Real vtl = vlen(vt);
                        if (vtl > 1.0e-20f) vt = vscale(vdivs(vt, vtl), std::max<Real>(vtl + c.friction * vn, 0.0f));
                        vnew = vadd(vs, vt);
                    }
                }
            }
            V3 imp = vscale(vsub(vin, vnew), m);
            V3 tq = vcross(rel, imp);
            for (int i = 0; i < 3; ++i) { addacc(i, imp[i]); addacc(3 + i, tq[i]); }
            store3(vout, vnew);
        }
        return;
    }
    case GBMPM_COLLIDER_WALLS: {  // mpm_solver_warp.py:2294-2359
        if (!live) return;
        const int pad = 3;
        int n = M->n_grid;
        if (gx < pad && vout[0] < 0) vout[0] = 0.0f;
        if (gx >= n - pad && vout[0] > 0) vout[0] = 0.0f;
        if (gy < pad && vout[1] < 0) vout[1] = 0.0f;
        if (gy >= n - pad && vout[1] > 0) vout[1] = 0.0f;
        if (gz < pad && vout[2] < 0) vout[2] = 0.0f;
        if (gz >= n - pad && vout[2] > 0) vout[2] = 0.0f;
        return;
    }
    case GBMPM_COLLIDER_SDF: {  // mpm_solver_warp.py:2680-2736
        if (!live) return;
        V3 xw = mkv((Real)gx * dx, (Real)gy * dx, (Real)gz * dx);
        V3 rel = vsub(xw, mkv(c.point[0], c.point[1], c.point[2]));
        V3 body = qrot(c.quat, rel, true);
        V3 f = mkv((body[0] - c.sdf_origin[0]) / c.sdf_cell, (body[1] - c.sdf_origin[1]) / c.sdf_cell,
                   (body[2] - c.sdf_origin[2]) / c.sdf_cell);
        Real rf = (Real)c.sdf_res - 1.0f;
        bool inside = f[0] >= 0.0f && f[1] >= 0.0f && f[2] >= 0.0f && f[0] <= rf && f[1] <= rf && f[2] <= rf;
        if (!inside) return;
        Real sd = trilerp(c.sdf_val, c.sdf_res, f, 1, 0);
        if (sd <= c.band) {
            V3 g = mkv(trilerp(c.sdf_grad, c.sdf_res, f, 3, 0), trilerp(c.sdf_grad, c.sdf_res, f, 3, 1),
                       trilerp(c.sdf_grad, c.sdf_res, f, 3, 2));
            if (vlen(g) > 1.0e-12f) {
                V3 nw = qrot(c.quat, vnormalize(g), false);
                V3 vs = vadd(mkv(c.velocity[0], c.velocity[1], c.velocity[2]),
                             vcross(mkv(c.omega[0], c.omega[1], c.omega[2]), rel));
                V3 vf = load3(vout);
                V3 vr = vsub(vf, vs);
                Real vn = vdot(vr, nw);
                V3 vnew = vf;
                if (c.surface_type == 0) vnew = vs;
                else if (c.surface_type == 1) vnew = vadd(vs, vsub(vr, vscale(nw, vn)));
                else if (vn < 0.0f) {
                    V3 vt = vsub(vr, vscale(nw, vn));
                    Real tl = vlen(vt);
                    if (tl > 1.0e-12f) vt = vscale(vt, std::max<Real>(0.0f, tl + c.friction * vn) / tl);
                    vnew = vadd(vs, vt);
                }
                V3 imp = vscale(vsub(vf, vnew), m);
                V3 tq = vcross(rel, imp);
                for (int i = 0; i < 3; ++i) { addacc(i, imp[i]); addacc(3 + i, tq[i]); }
                store3(vout, vnew);
            }
        }
        return;
    }
    default: return;
    }
}

// host pose integration, the modify_bc callables (float64 arithmetic on the fp32
// struct values, rounded back to fp32)
void integrate_pose(gbmpm_collider& c, double time, double dt) {
    bool live = time >= (double)c.start_time && time < (double)c.end_time;
    if (!live) return;
    if (c.kind == GBMPM_COLLIDER_BOX || c.kind == GBMPM_COLLIDER_CUP || c.kind == GBMPM_COLLIDER_SDF) {
        // box: mpm_solver_warp.py:2090-2096; cup: :2227-2233; sdf: :2756
        for (int i = 0; i < 3; ++i) c.point[i] = (Real)((double)c.point[i] + dt * (double)c.velocity[i]);
    }
    if (c.kind == GBMPM_COLLIDER_CUP) {  // Rodrigues on the float64 shadow (:2234-2254)
        double w[3] = {c.omega[0], c.omega[1], c.omega[2]};
        double wn = std::sqrt(w[0] * w[0] + w[1] * w[1] + w[2] * w[2]);
        double ang = wn * dt;
        if (ang > 1.0e-12) {
            double ax[3] = {w[0] / wn, w[1] / wn, w[2] / wn};
            double K[3][3] = {{0.0, -ax[2], ax[1]}, {ax[2], 0.0, -ax[0]}, {-ax[1], ax[0], 0.0}};
            double K2[3][3], Ri[3][3], Rn[3][3];
            for (int i = 0; i < 3; ++i)
                for (int j = 0; j < 3; ++j) {
                    double acc = 0.0;
                    for (int k = 0; k < 3; ++k) acc += K[i][k] * K[k][j];
                    K2[i][j] = acc;
                }
            double s = std::sin(ang), cc = 1.0 - std::cos(ang);
            for (int i = 0; i < 3; ++i)
                for (int j = 0; j < 3; ++j) Ri[i][j] = ((i == j) ? 1.0 : 0.0) + s * K[i][j] + cc * K2[i][j];
            for (int i = 0; i < 3; ++i)
                for (int j = 0; j < 3; ++j) {
                    double acc = 0.0;
                    for (int k = 0; k < 3; ++k) acc += Ri[i][k] * c.rot64[3 * k + j];
                    Rn[i][j] = acc;
                }
            for (int i = 0; i < 3; ++i)
                for (int j = 0; j < 3; ++j) { c.rot64[3 * i + j] = Rn[i][j]; c.rot[3 * i + j] = (Real)Rn[i][j]; }
        }
    }
    if (c.kind == GBMPM_COLLIDER_SDF) {  // _omega_step_quat (mpm_solver_warp.py:198-210)
        double w[3] = {c.omega[0], c.omega[1], c.omega[2]};
        double sp = std::sqrt(w[0] * w[0] + w[1] * w[1] + w[2] * w[2]);
        double q[4] = {c.quat[0], c.quat[1], c.quat[2], c.quat[3]};
        if (!(sp * dt < 1e-12)) {
            double half = 0.5 * sp * dt;
            double sh = std::sin(half);
            double d[4] = {w[0] / sp * sh, w[1] / sp * sh, w[2] / sp * sh, std::cos(half)};
            double r[4] = {d[3] * q[0] + d[0] * q[3] + d[1] * q[2] - d[2] * q[1],
                           d[3] * q[1] - d[0] * q[2] + d[1] * q[3] + d[2] * q[0],
                           d[3] * q[2] + d[0] * q[1] - d[1] * q[0] + d[2] * q[3],
                           d[3] * q[3] - d[0] * q[0] - d[1] * q[1] - d[2] * q[2]};
            double nr = std::sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2] + r[3] * r[3]);
            for (int i = 0; i < 4; ++i) c.quat[i] = (Real)(r[i] / nr);
        }
    }
}

// ------------------------------------------------------------ CPIC (CDF) -----
// Thin-boundary colliders: node tag bits (bit 2l valid, 2l+1 side, owner lane in
// bits 8..9), owner distance, the previous stamp's copies and a 4^3 occupancy
// mask (mpm_solver_warp.py:94-183, mpm_utils.py:648-816).
// cdf_pair_incompatible (mpm_utils.py:648-654)
inline bool cdf_incompatible(int pc, int nt) { return ((pc & nt & 0x55) & ((pc ^ nt) >> 1)) != 0; }

// cdf_stencil_near (mpm_utils.py:657-675)
bool cdf_stencil_near(const CdfState& S, const int* b) {
    for (int bi = b[0] >> 2; bi <= (b[0] + 2) >> 2; ++bi)
        for (int bj = b[1] >> 2; bj <= (b[1] + 2) >> 2; ++bj)
            for (int bk = b[2] >> 2; bk <= (b[2] + 2) >> 2; ++bk)
                if (S.block[((size_t)bi * S.nb + bj) * S.nb + bk] != 0) return true;
    return false;
}

// cdf_particle_tag (mpm_utils.py:678-713)
int cdf_particle_tag(const CdfState& S, const Weights& W, bool use_prev) {
    Real votes[4] = {0.f, 0.f, 0.f, 0.f};
    int seen = 0;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
            for (int k = 0; k < 3; ++k) {
                size_t id = S.idx(W.base[0] + i, W.base[1] + j, W.base[2] + k);
                int t = use_prev ? S.tag_prev[id] : S.tag[id];
                Real dd = use_prev ? S.d_prev[id] : S.d[id];
                if (t == 0) continue;
                Real weight = W.w[0][i] * W.w[1][j] * W.w[2][k];
                for (int lane = 0; lane < 4; ++lane)
                    if ((t >> (2 * lane)) & 1) {
                        seen |= 1 << (2 * lane);
                        Real sgn = ((t >> (2 * lane + 1)) & 1) ? 1.0f : -1.0f;
                        votes[lane] = votes[lane] + weight * dd * sgn;
                    }
            }
    int pc = 0;
    for (int lane = 0; lane < 4; ++lane)
        if ((seen >> (2 * lane)) & 1) {
            pc |= 1 << (2 * lane);
            if (votes[lane] >= 0.0f) pc |= 1 << (2 * lane + 1);
        }
    return pc;
}

// cdf_persist_tag (mpm_utils.py:716-730)
int cdf_persist(int old, int fresh) {
    int pc = 0;
    for (int lane = 0; lane < 4; ++lane)
        if ((fresh >> (2 * lane)) & 1) {
            pc |= 1 << (2 * lane);
            pc |= ((old >> (2 * lane)) & 1) ? (old & (1 << (2 * lane + 1))) : (fresh & (1 << (2 * lane + 1)));
        }
    return pc;
}

// cdf_particle_ghost (mpm_utils.py:733-816)
V3 cdf_ghost(const CdfState& S, const gbmpm_model* M, Real dt, V3 xp, V3 vp, int pc, const Weights& W) {
    Real d_hat = 0.0f;
    V3 n_acc = mkv(0, 0, 0);
    Real best_w = 0.0f;
    int lane_p = 0;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
            for (int k = 0; k < 3; ++k) {
                size_t id = S.idx(W.base[0] + i, W.base[1] + j, W.base[2] + k);
                int t = S.tag_prev[id];
                if (t == 0) continue;
                int own = (t >> kOwnerShift) & 3;
                if (((t >> (2 * own)) & 1) == 0) continue;
                Real weight = W.w[0][i] * W.w[1][j] * W.w[2][k];
                Real sgn = ((t >> (2 * own + 1)) & 1) ? 1.0f : -1.0f;
                Real dd = S.d_prev[id];
                d_hat = d_hat + weight * sgn * dd;
                V3 dwt = dweight(W, i, j, k, M->inv_dx);
                n_acc = vadd(n_acc, vscale(vscale(dwt, sgn), dd));
                if (weight > best_w) { best_w = weight; lane_p = own; }
            }
    V3 g = mkv(M->gravity[0], M->gravity[1], M->gravity[2]);
    V3 v_free = vadd(vp, vscale(g, dt));
    V3 ghost = v_free;
    if (vlen(n_acc) > 1.0e-12f) {
        V3 n_hat = vnormalize(n_acc);
        Real side = ((pc >> (2 * lane_p + 1)) & 1) ? 1.0f : -1.0f;
        V3 n_par = vscale(n_hat, side);
        V3 rel = vsub(xp, load3(S.c_prev[lane_p]));
        V3 v_surf = vadd(load3(S.v_prev[lane_p]), vcross(load3(S.w_prev[lane_p]), rel));
        V3 v_rel = vsub(v_free, v_surf);
        Real vn = vdot(v_rel, n_par);
        V3 v_tan = vsub(v_rel, vscale(n_par, vn));
        Real c = 0.0f;
        Real d_side = d_hat * side;
        Real eps = 0.05f * M->dx;
        if (d_side < eps) c = std::min((eps - d_side) / dt, 0.5f * M->dx / dt);
        int stype = S.type[lane_p];
        if (stype == 0) {
            ghost = vadd(v_surf, vscale(n_par, c));
        } else if (stype == 1) {
            ghost = vadd(vadd(v_surf, v_tan), vscale(n_par, c));
        } else {
            Real dvn = std::max<Real>(-vn, 0.0f) + c;
            Real tlen = vlen(v_tan);
            if (tlen > 1.0e-12f && dvn > 0.0f) {
                Real sc = std::max<Real>(0.0f, tlen - S.fric[lane_p] * dvn) / tlen;
                v_tan = vscale(v_tan, sc);
            }
            ghost = vadd(vadd(vadd(v_surf, v_tan), vscale(n_par, std::max<Real>(vn, 0.0f))), vscale(n_par, c));
        }
    }
    return ghost;
}

// the CDF collider's grid box (cdf_aabb, mpm_solver_warp.py:2860-2870 with halo 2)
bool cdf_lane_box(const gbmpm_cdf& r, const gbmpm_model* M, int* box) {
    double qx = r.quat[0], qy = r.quat[1], qz = r.quat[2], qw = r.quat[3];
    double R[3][3] = {{1 - 2 * (qy * qy + qz * qz), 2 * (qx * qy - qz * qw), 2 * (qx * qz + qy * qw)},
                      {2 * (qx * qy + qz * qw), 1 - 2 * (qx * qx + qz * qz), 2 * (qy * qz - qx * qw)},
                      {2 * (qx * qz - qy * qw), 2 * (qy * qz + qx * qw), 1 - 2 * (qx * qx + qy * qy)}};
    double ext = (r.res - 1) * (double)r.cell;
    double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
    for (int a = 0; a < 2; ++a)
        for (int b = 0; b < 2; ++b)
            for (int c = 0; c < 2; ++c) {
                double cr[3] = {(double)r.origin[0] + a * ext, (double)r.origin[1] + b * ext, (double)r.origin[2] + c * ext};
                for (int i = 0; i < 3; ++i) {
                    double p = (double)r.center[i] + R[i][0] * cr[0] + R[i][1] * cr[1] + R[i][2] * cr[2];
                    lo[i] = std::min(lo[i], p);
                    hi[i] = std::max(hi[i], p);
                }
            }
    double dx = (double)M->grid_lim / M->n_grid;   // python Real grid_lim / n_grid
    for (int i = 0; i < 3; ++i) {
        int l = std::max(0, (int)std::floor(lo[i] / dx) - 2);
        int h = std::min(M->n_grid, (int)std::ceil(hi[i] / dx) + 2 + 1);
        if (h - l <= 0) return false;
        box[i] = l;
        box[3 + i] = h;   // exclusive
    }
    return true;
}

// cdf_stamp kernel body (mpm_solver_warp.py:146-183) for one lane over a box
void cdf_stamp_lane(CdfState& S, const gbmpm_model* M, const gbmpm_cdf& r, int lane, Real time_f, const int* box) {
    if (time_f < r.start_time || time_f >= r.end_time) return;
    Real rf = (Real)r.res - 1.0f;
    for (int x = box[0]; x < box[3]; ++x)
        for (int y = box[1]; y < box[4]; ++y)
            for (int z = box[2]; z < box[5]; ++z) {
                V3 xw = mkv((Real)x * M->dx, (Real)y * M->dx, (Real)z * M->dx);
                V3 rel = vsub(xw, mkv(r.center[0], r.center[1], r.center[2]));
                V3 body = qrot(r.quat, rel, true);
                V3 f = mkv((body[0] - r.origin[0]) / r.cell, (body[1] - r.origin[1]) / r.cell,
                           (body[2] - r.origin[2]) / r.cell);
                if (f[0] < 0.0f || f[1] < 0.0f || f[2] < 0.0f || f[0] > rf || f[1] > rf || f[2] > rf) continue;
                Real ok = trilerp(r.valid, r.res, f, 1, 0);
                if (ok < 0.999f) continue;
                Real dd = trilerp(r.values, r.res, f, 1, 0);
                Real ud = std::fabs(dd);
                if (ud > r.band) continue;
                int side = dd >= 0.0f ? 1 : 0;
                size_t id = S.idx(x, y, z);
                int t = S.tag[id];
                t = t | (1 << (2 * lane)) | (side << (2 * lane + 1));
                if (ud < S.d[id]) {
                    S.d[id] = ud;
                    t = (t ^ (t & kOwnerMask)) | (lane << kOwnerShift);
                }
                S.tag[id] = t;
            }
}

void cdf_copy_prev_box(CdfState& S, const int* box) {
    for (int x = box[0]; x < box[3]; ++x)
        for (int y = box[1]; y < box[4]; ++y)
            for (int z = box[2]; z < box[5]; ++z) {
                size_t id = S.idx(x, y, z);
                S.tag_prev[id] = S.tag[id];
                S.d_prev[id] = S.d[id];
            }
}

// _stamp_cdf (mpm_solver_warp.py:3040-3098)
void cdf_stamp(CdfState& S, const gbmpm_model* M, double time, bool lag_prev) {
    if (S.n == 0) return;
    if (S.stale_set) { cdf_copy_prev_box(S, S.stale_box); S.stale_set = false; }
    for (int l = 0; l < S.n; ++l) {
        bool act = time >= (double)S.rec[l].start_time && time < (double)S.rec[l].end_time;
        if (act != S.active[l]) { S.active[l] = act; S.dirty[l] = true; }
    }
    bool any = false;
    for (int l = 0; l < S.n; ++l) any = any || S.dirty[l];
    if (!any) return;
    // _cdf_dirty_box: union of the dirty lanes' boxes and the boxes of their last stamps
    int box[6] = {INT32_MAX, INT32_MAX, INT32_MAX, INT32_MIN, INT32_MIN, INT32_MIN};
    bool have = false;
    auto grow = [&](const int* b) {
        for (int i = 0; i < 3; ++i) { box[i] = std::min(box[i], b[i]); box[3 + i] = std::max(box[3 + i], b[3 + i]); }
        have = true;
    };
    for (int l = 0; l < S.n; ++l) {
        if (!S.dirty[l]) continue;
        int b[6];
        bool ok = cdf_lane_box(S.rec[l], M, b);
        if (ok) grow(b);
        if (S.has_prev_box[l]) grow(S.prev_box[l]);
        S.has_prev_box[l] = ok;
        if (ok) std::memcpy(S.prev_box[l], b, sizeof b);
    }
    for (int l = 0; l < S.n; ++l) S.dirty[l] = false;
    if (!have) return;
    S.stamp_count++;
    for (int x = box[0]; x < box[3]; ++x)
        for (int y = box[1]; y < box[4]; ++y)
            for (int z = box[2]; z < box[5]; ++z) {
                size_t id = S.idx(x, y, z);
                S.tag[id] = 0;
                S.d[id] = 1.0e9f;
            }
    Real tf = (Real)time;
    for (int l = 0; l < S.n; ++l) {
        int lb[6];
        if (!cdf_lane_box(S.rec[l], M, lb)) continue;
        int clip[6];
        bool empty = false;
        for (int i = 0; i < 3; ++i) {
            clip[i] = std::max(box[i], lb[i]);
            clip[3 + i] = std::min(box[3 + i], lb[3 + i]);
            if (clip[3 + i] <= clip[i]) empty = true;
        }
        if (!empty) cdf_stamp_lane(S, M, S.rec[l], l, tf, clip);
    }
    if (lag_prev) { S.stale_set = true; std::memcpy(S.stale_box, box, sizeof box); }
    else cdf_copy_prev_box(S, box);
    // cdf_block_mask over the blocks of the box (cur OR prev)
    for (int bi = box[0] >> 2; bi <= (box[3] - 1) >> 2; ++bi)
        for (int bj = box[1] >> 2; bj <= (box[4] - 1) >> 2; ++bj)
            for (int bk = box[2] >> 2; bk <= (box[5] - 1) >> 2; ++bk) {
                int occ = 0;
                for (int i = 0; i < 4; ++i)
                    for (int j = 0; j < 4; ++j)
                        for (int k = 0; k < 4; ++k) {
                            int ci = (bi << 2) + i, cj = (bj << 2) + j, ck = (bk << 2) + k;
                            if (ci < S.n_grid && cj < S.n_grid && ck < S.n_grid) {
                                size_t id = S.idx(ci, cj, ck);
                                occ = occ | S.tag[id] | S.tag_prev[id];
                            }
                        }
                S.block[((size_t)bi * S.nb + bj) * S.nb + bk] = occ;
            }
}

// _integrate_cdf_poses (mpm_solver_warp.py:3107-3148)
void cdf_integrate(CdfState& S, double time, double dt, bool lag_prev) {
    if (S.n == 0) return;
    if (lag_prev && S.lane_prev_stale) S.copy_lane_prev();
    for (int l = 0; l < S.n; ++l) {
        gbmpm_cdf& r = S.rec[l];
        if (!(time >= (double)r.start_time && time < (double)r.end_time)) continue;
        if (r.velocity[0] == 0.0f && r.velocity[1] == 0.0f && r.velocity[2] == 0.0f && r.omega[0] == 0.0f &&
            r.omega[1] == 0.0f && r.omega[2] == 0.0f)
            continue;
        for (int a = 0; a < 3; ++a) r.center[a] = (Real)((double)r.center[a] + dt * (double)r.velocity[a]);
        double w[3] = {r.omega[0], r.omega[1], r.omega[2]};
        double sp = std::sqrt(w[0] * w[0] + w[1] * w[1] + w[2] * w[2]);
        if (!(sp * dt < 1e-12)) {
            double q[4] = {r.quat[0], r.quat[1], r.quat[2], r.quat[3]};
            double half = 0.5 * sp * dt, sh = std::sin(half);
            double dq[4] = {w[0] / sp * sh, w[1] / sp * sh, w[2] / sp * sh, std::cos(half)};
            double o[4] = {dq[3] * q[0] + dq[0] * q[3] + dq[1] * q[2] - dq[2] * q[1],
                           dq[3] * q[1] - dq[0] * q[2] + dq[1] * q[3] + dq[2] * q[0],
                           dq[3] * q[2] + dq[0] * q[1] - dq[1] * q[0] + dq[2] * q[3],
                           dq[3] * q[3] - dq[0] * q[0] - dq[1] * q[1] - dq[2] * q[2]};
            double nr = std::sqrt(o[0] * o[0] + o[1] * o[1] + o[2] * o[2] + o[3] * o[3]);
            for (int i = 0; i < 4; ++i) r.quat[i] = (Real)(o[i] / nr);
        }
        S.sync_lane(l);
        S.dirty[l] = true;
        S.lane_prev_stale = true;
    }
    if (!lag_prev && S.lane_prev_stale) S.copy_lane_prev();
}

// ---------------------------------------------------------- tick driver -----
struct Oracle {
    Grid G;
};
Oracle g_oracle;

template <class Fn> void par_for(int n, bool par, Fn fn) {
    if (par) {
#pragma omp parallel for schedule(static)
        for (int i = 0; i < n; ++i) fn(i);
    } else {
        for (int i = 0; i < n; ++i) fn(i);
    }
}

void track_box(Grid& G, const RP* P, const gbmpm_model* M) {
    // nodes the coming scatter can touch: every selected particle's stencil
    G.reset_box();
    int lo[3] = {G.n, G.n, G.n}, hi[3] = {0, 0, 0};
    for (int p = 0; p < P->n; ++p) {
        if (P->selection && P->selection[p] != 0) continue;
        for (int a = 0; a < 3; ++a) {
            Real gp = P->x[3 * (size_t)p + a] * M->inv_dx;
            int b = (int)std::floor(gp - 0.5f);
            if (a == 0 && M->periodic_x) { lo[0] = 0; hi[0] = G.n; continue; }
            lo[a] = std::min(lo[a], std::max(b, 0));
            hi[a] = std::max(hi[a], std::min(b + 3, G.n));
        }
    }
    for (int a = 0; a < 3; ++a) { G.lo[a] = lo[a]; G.hi[a] = hi[a]; }
}

void zero_box(Grid& G, const int* lo, const int* hi, bool m_vin, bool vout) {
    for (int x = lo[0]; x < hi[0]; ++x)
        for (int y = lo[1]; y < hi[1]; ++y)
            for (int z = lo[2]; z < hi[2]; ++z) {
                size_t id = G.idx(x, y, z);
                if (m_vin) { G.m[id] = 0.0f; G.vin[3 * id] = G.vin[3 * id + 1] = G.vin[3 * id + 2] = 0.0f; }
                if (vout) { G.vout[3 * id] = G.vout[3 * id + 1] = G.vout[3 * id + 2] = 0.0f; }
            }
}

// grid_normalization_and_gravity (mpm_utils.py:927-941), add_damping_via_grid
// (:1287-1295) and the collider kernels, over the box of touched nodes
void grid_update(Grid& G, const gbmpm_model* M, gbmpm_collider* cols, int ncol, Real* wrench, Real time_f,
                 Real dt, bool par) {
    int nx = G.hi[0] - G.lo[0];
    if (nx <= 0) return;
    NodeCtx nc{time_f, dt, M};
    auto row = [&](int xi) {
        int x = G.lo[0] + xi;
        for (int y = G.lo[1]; y < G.hi[1]; ++y)
            for (int z = G.lo[2]; z < G.hi[2]; ++z) {
                size_t id = G.idx(x, y, z);
                Real m = G.m[id];
                if (m > 1e-15f) {
                    Real inv = 1.0f / m;
                    for (int a = 0; a < 3; ++a) G.vout[3 * id + a] = G.vin[3 * id + a] * inv + dt * M->gravity[a];
                }
            }
    };
    par_for(nx, par, row);
    if (M->grid_v_damping_scale < 1.0f) {
        par_for(nx, par, [&](int xi) {
            int x = G.lo[0] + xi;
            for (int y = G.lo[1]; y < G.hi[1]; ++y)
                for (int z = G.lo[2]; z < G.hi[2]; ++z) {
                    size_t id = G.idx(x, y, z);
                    for (int a = 0; a < 3; ++a) G.vout[3 * id + a] = G.vout[3 * id + a] * M->grid_v_damping_scale;
                }
        });
    }
    for (int k = 0; k < ncol; ++k) {
        par_for(nx, par, [&](int xi) {
            int x = G.lo[0] + xi;
            for (int y = G.lo[1]; y < G.hi[1]; ++y)
                for (int z = G.lo[2]; z < G.hi[2]; ++z) {
                    size_t id = G.idx(x, y, z);
                    collide_node(cols[k], x, y, z, G.m[id], &G.vout[3 * id], nc, wrench + 6 * k, par);
                }
        });
    }
}

// ---- rigid bodies and particle modifiers (split pipeline order) ----------------
struct RigidState {
    std::vector<gbmpm_rigid_body> bodies;
    std::vector<gbmpm_rigid_surface> surf;
    std::vector<gbmpm_modifier> mods;
};
RigidState g_rigid;

// pre-P2G operations and velocity modifiers (mpm_solver_warp.py:1182-1196,
// 2385-2540) on every selected particle whose mod_mask bit is set: impulses first,
// then velocity overrides, each in list order, on the float32 window [start, end)
void apply_modifiers(const RP* P, int p, Real time_f, Real dt) {
    const int mask = P->mod_mask ? P->mod_mask[p] : 0;
    if (!mask) return;
    Real* v = P->v + 3 * (size_t)p;
    const Real* x = P->x + 3 * (size_t)p;
    for (int pass = 0; pass < 2; ++pass)
        for (size_t m = 0; m < g_rigid.mods.size(); ++m) {
            const gbmpm_modifier& d = g_rigid.mods[m];
            if (!((mask >> m) & 1) || (d.kind == 0) != (pass == 0)) continue;
            if (!(time_f >= d.start_time && time_f < d.end_time)) continue;
            if (d.kind == 0) {
                const Real mass = P->mass[p];
                for (int a = 0; a < 3; ++a) v[a] = v[a] + (d.vec[a] / mass) * dt;
            } else if (d.kind == 1) {
                for (int a = 0; a < 3; ++a) v[a] = d.vec[a];
            } else {
                Real off[3], hz[3];
                for (int a = 0; a < 3; ++a) off[a] = x[a] - d.point[a];
                const Real on = off[0] * d.normal[0] + off[1] * d.normal[1] + off[2] * d.normal[2];
                for (int a = 0; a < 3; ++a) hz[a] = off[a] - on * d.normal[a];
                const Real hd = std::sqrt(hz[0] * hz[0] + hz[1] * hz[1] + hz[2] * hz[2]);
                const Real cosine = (off[0] * d.axis1[0] + off[1] * d.axis1[1] + off[2] * d.axis1[2]) / hd;
                Real theta = acosr(std::min<Real>(std::max<Real>(cosine, -1.0f), 1.0f));
                if (!(off[0] * d.axis2[0] + off[1] * d.axis2[1] + off[2] * d.axis2[2] > 0.0f)) theta = -theta;
                const Real a1 = -hd * sinr(theta) * d.rotation_scale;
                const Real a2 = hd * cosr(theta) * d.rotation_scale;
                for (int a = 0; a < 3; ++a) v[a] = a1 * d.axis1[a] + a2 * d.axis2[a] + d.translation_scale * d.normal[a];
            }
        }
}

template <class A, class B>
inline void rmul(const A* a, const B* b, Real* c) {   // row-major 3x3 product
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
            c[3 * i + j] = (Real)a[3 * i] * (Real)b[j] + (Real)a[3 * i + 1] * (Real)b[3 + j] +
                           (Real)a[3 * i + 2] * (Real)b[6 + j];
}
template <class A, class B>
inline void rmulT(const A* a, const B* b, Real* c) {  // a b^T
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
            c[3 * i + j] = (Real)a[3 * i] * (Real)b[3 * j] + (Real)a[3 * i + 1] * (Real)b[3 * j + 1] +
                           (Real)a[3 * i + 2] * (Real)b[3 * j + 2];
}

// the rigid tail of one substep (_p2g2p_tail, mpm_solver_warp.py:1338-1367):
// rigid_g2p_accumulate, rigid_body_integrate, _apply_rigid_restitution (deepest
// particle by float64 distance, lowest index on a tie) and rigid_particle_update
void rigid_tail(const RP* P, const gbmpm_model* M, Grid& G, double time, Real dt,
                const std::function<bool(int)>& sel) {
    const int nb = (int)g_rigid.bodies.size();
    if (nb == 0) return;
    std::vector<double> acc(6 * (size_t)nb, 0.0);
    for (int p = 0; p < P->n; ++p) {
        if (!sel(p) || P->material[p] != 8) continue;
        Weights W;
        bspline(P->x + 3 * (size_t)p, M->inv_dx, W);
        Real vi[3] = {0.0f, 0.0f, 0.0f};
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j)
                for (int k = 0; k < 3; ++k) {
                    const Real w = W.w[0][i] * W.w[1][j] * W.w[2][k];
                    const size_t id = G.idx(W.base[0] + i, W.base[1] + j, W.base[2] + k);
                    for (int a = 0; a < 3; ++a) vi[a] = vi[a] + G.vout[3 * id + a] * w;
                }
        const int b = P->rigid_id[p];
        const Real m = P->mass[p];
        const Real* x = P->x + 3 * (size_t)p;
        const Real r[3] = {x[0] - g_rigid.bodies[b].x_cm[0], x[1] - g_rigid.bodies[b].x_cm[1],
                            x[2] - g_rigid.bodies[b].x_cm[2]};
        const Real pm[3] = {vi[0] * m, vi[1] * m, vi[2] * m};
        const Real am[3] = {r[1] * pm[2] - r[2] * pm[1], r[2] * pm[0] - r[0] * pm[2], r[0] * pm[1] - r[1] * pm[0]};
        for (int a = 0; a < 3; ++a) { acc[6 * b + a] += pm[a]; acc[6 * b + 3 + a] += am[a]; }
    }
    for (int b = 0; b < nb; ++b) {
        gbmpm_rigid_body& r = g_rigid.bodies[b];
        Real v[3], w[3], T1[9], Iw[9];
        for (int a = 0; a < 3; ++a) v[a] = (Real)acc[6 * b + a] / r.mass;
        rmul(r.R, r.inv_inertia, T1);
        rmulT(T1, r.R, Iw);
        const Real L[3] = {(Real)acc[6 * b + 3], (Real)acc[6 * b + 4], (Real)acc[6 * b + 5]};
        for (int i = 0; i < 3; ++i) w[i] = Iw[3 * i] * L[0] + Iw[3 * i + 1] * L[1] + Iw[3 * i + 2] * L[2];
        for (int a = 0; a < 3; ++a) r.x_cm[a] = r.x_cm[a] + v[a] * dt;
        const Real Wk[9] = {0.0f, -w[2], w[1], w[2], 0.0f, -w[0], -w[1], w[0], 0.0f};
        Real WR[9], Rn[9];
        rmul(Wk, r.R, WR);
        for (int i = 0; i < 9; ++i) Rn[i] = r.R[i] + WR[i] * dt;
        M3 Rm = load33(Rn), U, V;
        V3 sg;
        svd3_impl(Rm, U, sg, V);
        store33(r.R, mmul(U, mT(V)));
        for (int a = 0; a < 3; ++a) { r.v_cm[a] = v[a]; r.omega[a] = w[a]; }
        // world positions once, from the integrated pose; each surface's deepest
        // particle is taken there and shifted by the pushes of the surfaces before
        // it (the reference adds each push to its world positions)
        const Real xc0[3] = {r.x_cm[0], r.x_cm[1], r.x_cm[2]};
        double pacc[3] = {0.0, 0.0, 0.0};
        for (const gbmpm_rigid_surface& sf : g_rigid.surf) {
            if (!(time >= sf.start_time && time < sf.end_time)) continue;
            double dmin = 0.0;
            int pmin = -1;
            for (int p = 0; p < P->n; ++p) {
                if (!sel(p) || P->material[p] != 8 || P->rigid_id[p] != b) continue;
                const Real* xr = P->x_ref + 3 * (size_t)p;
                double d = 0.0;
                for (int i = 0; i < 3; ++i) {
                    const Real xw = xc0[i] + (r.R[3 * i] * xr[0] + r.R[3 * i + 1] * xr[1] + r.R[3 * i + 2] * xr[2]);
                    d += ((double)xw - sf.point[i]) * sf.normal[i];
                }
                if (pmin < 0 || d < dmin) { dmin = d; pmin = p; }
            }
            if (pmin < 0) continue;
            dmin += pacc[0] * sf.normal[0] + pacc[1] * sf.normal[1] + pacc[2] * sf.normal[2];
            if (!(dmin < 0.0)) continue;
            const double* n = sf.normal;
            const Real* xr = P->x_ref + 3 * (size_t)pmin;
            double xc[3];
            for (int i = 0; i < 3; ++i) {
                const Real xw = xc0[i] + (r.R[3 * i] * xr[0] + r.R[3 * i + 1] * xr[1] + r.R[3 * i + 2] * xr[2]);
                const double push = -dmin * n[i];
                pacc[i] += push;
                xc[i] = (double)xw + pacc[i];
                r.x_cm[i] = (Real)((double)r.x_cm[i] + push);
            }
            Real Iwf[9];
            rmul(r.R, r.inv_inertia, T1);
            rmulT(T1, r.R, Iwf);
            auto mv = [&](const double* a, double* o) {
                for (int i = 0; i < 3; ++i) o[i] = (double)Iwf[3 * i] * a[0] + (double)Iwf[3 * i + 1] * a[1] + (double)Iwf[3 * i + 2] * a[2];
            };
            auto cross = [](const double* a, const double* c, double* o) {
                o[0] = a[1] * c[2] - a[2] * c[1];
                o[1] = a[2] * c[0] - a[0] * c[2];
                o[2] = a[0] * c[1] - a[1] * c[0];
            };
            double rr[3], om[3], vc[3], tmp[3];
            for (int i = 0; i < 3; ++i) { rr[i] = xc[i] - (double)r.x_cm[i]; om[i] = r.omega[i]; }
            cross(om, rr, tmp);
            for (int i = 0; i < 3; ++i) vc[i] = (double)r.v_cm[i] + tmp[i];
            const double vn = vc[0] * n[0] + vc[1] * n[1] + vc[2] * n[2];
            if (!(vn < 0.0)) continue;
            const double Mb = r.mass;
            double rxn[3], q[3], qq[3], dw[3];
            cross(rr, n, rxn);
            mv(rxn, q);
            cross(q, rr, qq);
            const double Jn = -(1.0 + sf.restitution) * vn / (1.0 / Mb + (qq[0] * n[0] + qq[1] * n[1] + qq[2] * n[2]));
            const double jr[3] = {Jn * rxn[0], Jn * rxn[1], Jn * rxn[2]};
            mv(jr, dw);
            for (int i = 0; i < 3; ++i) {
                r.v_cm[i] = (Real)((double)r.v_cm[i] + (Jn / Mb) * n[i]);
                r.omega[i] = (Real)((double)r.omega[i] + dw[i]);
            }
            if (sf.friction > 0.0) {
                double vt[3];
                for (int i = 0; i < 3; ++i) vt[i] = vc[i] - vn * n[i];
                const double vtm = std::sqrt(vt[0] * vt[0] + vt[1] * vt[1] + vt[2] * vt[2]);
                if (vtm > 1e-10) {
                    const double th[3] = {vt[0] / vtm, vt[1] / vtm, vt[2] / vtm};
                    double rxt[3], q2[3], qq2[3];
                    cross(rr, th, rxt);
                    mv(rxt, q2);
                    cross(q2, rr, qq2);
                    const double dent = 1.0 / Mb + (qq2[0] * th[0] + qq2[1] * th[1] + qq2[2] * th[2]);
                    const double Jt = std::min(vtm / dent, sf.friction * Jn);
                    const double jt[3] = {Jt * rxt[0], Jt * rxt[1], Jt * rxt[2]};
                    mv(jt, dw);
                    for (int i = 0; i < 3; ++i) {
                        r.v_cm[i] = (Real)((double)r.v_cm[i] - (Jt / Mb) * th[i]);
                        r.omega[i] = (Real)((double)r.omega[i] - dw[i]);
                    }
                }
            }
        }
    }
    for (int p = 0; p < P->n; ++p) {
        if (!sel(p) || P->material[p] != 8) continue;
        const gbmpm_rigid_body& r = g_rigid.bodies[P->rigid_id[p]];
        const Real* xr = P->x_ref + 3 * (size_t)p;
        Real* x = P->x + 3 * (size_t)p;
        Real* v = P->v + 3 * (size_t)p;
        for (int i = 0; i < 3; ++i)
            x[i] = r.x_cm[i] + (r.R[3 * i] * xr[0] + r.R[3 * i + 1] * xr[1] + r.R[3 * i + 2] * xr[2]);
        const Real rr[3] = {x[0] - r.x_cm[0], x[1] - r.x_cm[1], x[2] - r.x_cm[2]};
        v[0] = r.v_cm[0] + (r.omega[1] * rr[2] - r.omega[2] * rr[1]);
        v[1] = r.v_cm[1] + (r.omega[2] * rr[0] - r.omega[0] * rr[2]);
        v[2] = r.v_cm[2] + (r.omega[0] * rr[1] - r.omega[1] * rr[0]);
        const Real Cm[9] = {0.0f, -r.omega[2], r.omega[1], r.omega[2], 0.0f, -r.omega[0], -r.omega[1], r.omega[0], 0.0f};
        const Real I[9] = {1.0f, 0.0f, 0.0f, 0.0f, 1.0f, 0.0f, 0.0f, 0.0f, 1.0f};
        std::memcpy(P->C + 9 * (size_t)p, Cm, sizeof Cm);
        std::memcpy(P->F + 9 * (size_t)p, I, sizeof I);
    }
}

}  // namespace

extern "C" {

const char* gbmpm_oracle_last_error(void) { return g_err; }

int gbmpm_oracle_set_rigid(const gbmpm_rigid_body* bodies, int32_t nb, const gbmpm_rigid_surface* surf, int32_t ns) {
    g_rigid.bodies.assign(bodies, bodies + nb);
    g_rigid.surf.assign(surf, surf + ns);
    return GBMPM_OK;
}
int gbmpm_oracle_get_rigid(gbmpm_rigid_body* bodies, int32_t nb) {
    for (int b = 0; b < nb && b < (int)g_rigid.bodies.size(); ++b) bodies[b] = g_rigid.bodies[b];
    return GBMPM_OK;
}
int gbmpm_oracle_set_modifiers(const gbmpm_modifier* mods, int32_t n) {
    g_rigid.mods.assign(mods, mods + n);
    return GBMPM_OK;
}

// the oracle's own double sin (kind 0), cos (1) and acos (2) of n arguments, for the
// tests that check them against the host's libm
void gbmpm_oracle_trig(const double* x, int64_t n, int32_t kind, double* out) {
    for (int64_t i = 0; i < n; ++i)
        out[i] = kind == 2 ? dacos(x[i]) : dsincos(x[i], kind == 1);
}

// sizes and field offsets of the include/gbmpm.h records, so tests can check
// the ctypes mirror against the C compiler's layout
void gbmpm_oracle_abi_layout(int64_t* out) {
    out[0] = sizeof(gbmpm_particles);
    out[1] = sizeof(gbmpm_grid);
    out[2] = sizeof(gbmpm_model);
    out[3] = sizeof(gbmpm_collider);
    out[4] = offsetof(gbmpm_model, eta_table);
    out[5] = offsetof(gbmpm_model, eta_table_smax);
    out[6] = offsetof(gbmpm_collider, sdf_val);
    out[7] = offsetof(gbmpm_collider, rot64);
    out[8] = offsetof(gbmpm_particles, init_cov);
    out[9] = offsetof(gbmpm_model, material_mask);
}

void gbmpm_oracle_svd3(const Real* F, Real* U, Real* s, Real* V) {
    M3 f = load33(F), u, v; V3 sg;
    svd3_impl(f, u, sg, v);
    store33(U, u); store33(V, v); s[0] = sg[0]; s[1] = sg[1]; s[2] = sg[2];
}

Real gbmpm_oracle_glass_sdf(const gbmpm_collider* c, const Real* local) {
    return glass_sdf(load3(local), *c);
}

void gbmpm_oracle_integrate_pose(gbmpm_collider* c, double time, double dt) { integrate_pose(*c, time, dt); }

// One control tick (MPM_Simulator_WARP.p2g2p_fused_tick, mpm_solver_warp.py:1379-1546,
// or S calls of p2g2p, :1092-1281, when fused == 0). wrench: [ncol][6] fp32
// accumulators. threads <= 1 runs serially and deterministically.
// CPIC lane state of one scene (tag grids, lane poses, stamp bookkeeping)
void* gbmpm_oracle_cdf_new(int32_t n_grid) {
    CdfState* S = new CdfState();
    S->alloc(n_grid);
    return S;
}
void gbmpm_oracle_cdf_free(void* st) { delete static_cast<CdfState*>(st); }
int32_t gbmpm_oracle_cdf_stamp_count(void* st) { return static_cast<CdfState*>(st)->stamp_count; }
// current node tags and owner distances (grid_cdf_tag / grid_cdf_d), n_grid^3 each
void gbmpm_oracle_cdf_grids(void* st, int32_t* tag, Real* d) {
    CdfState& S = *static_cast<CdfState*>(st);
    if (tag) std::memcpy(tag, S.tag.data(), S.tag.size() * sizeof(int32_t));
    if (d) std::memcpy(d, S.d.data(), S.d.size() * sizeof(Real));
}

// add_cdf_collider / set_cdf_pose (mpm_solver_warp.py:2819-2953): lanes beyond the
// current count are new; an existing lane whose centre or quaternion changed is
// marked for restamping, and any pose or rate change refreshes the lane arrays.
int gbmpm_oracle_cdf_set(void* st, const gbmpm_cdf* lanes, int32_t n, double time) {
    CdfState& S = *static_cast<CdfState*>(st);
    if (n < S.n || n > GBMPM_MAX_CDF) { g_err = "lanes can only be added (max 4)"; return GBMPM_ERR_ARG; }
    for (int l = 0; l < n; ++l) {
        const gbmpm_cdf& r = lanes[l];
        if (l >= S.n) {
            S.rec[l] = r;
            S.dirty[l] = true;
            S.active[l] = time >= (double)r.start_time && time < (double)r.end_time;
            S.has_prev_box[l] = false;
            S.sync_lane(l);
            continue;
        }
        gbmpm_cdf& o = S.rec[l];
        bool moved = std::memcmp(o.center, r.center, sizeof o.center) != 0 || std::memcmp(o.quat, r.quat, sizeof o.quat) != 0;
        bool synced = std::memcmp(o.velocity, r.velocity, sizeof o.velocity) != 0 ||
                      std::memcmp(o.omega, r.omega, sizeof o.omega) != 0;
        S.rec[l] = r;
        if (moved) S.dirty[l] = true;
        if (moved || synced) { S.sync_lane(l); S.lane_prev_stale = true; }
    }
    S.n = n;
    return GBMPM_OK;
}

int gbmpm_oracle_cdf_get(void* st, gbmpm_cdf* lanes, int32_t n) {
    CdfState& S = *static_cast<CdfState*>(st);
    for (int l = 0; l < n && l < S.n; ++l) lanes[l] = S.rec[l];
    return GBMPM_OK;
}

// The particle record's float pointers address Real arrays (float32, or float64 in
// the double build); wrench and cdf_wrench are Real accumulators.
int gbmpm_oracle_tick(const gbmpm_particles* Pin, const gbmpm_model* M, gbmpm_collider* cols, int32_t ncol,
                      Real* wrench, double* time, double dt, int32_t substeps, int32_t fused, int32_t threads,
                      void* cdf_state, Real* cdf_wrench) {
    if (!Pin || !M || !time || substeps < 1) { g_err = "bad argument"; return GBMPM_ERR_ARG; }
    const RP rp = to_rp(*Pin);
    const RP* P = &rp;
    bool par = threads > 1;
#ifdef _OPENMP
    if (par) omp_set_num_threads(threads);
#else
    par = false;
#endif
    Grid& G = g_oracle.G;
    G.resize(M->n_grid);
    Real dtf = (Real)dt;
    Ctx c{P, M, &G, dtf, par, 0};
    CdfState* S = static_cast<CdfState*>(cdf_state);
    if (S && S->n > 0) {
        if (S->n_grid != M->n_grid) { g_err = "cdf state grid differs from the model"; return GBMPM_ERR_ARG; }
        c.cdf = S;
        c.cdf_wrench = cdf_wrench;
    } else {
        S = nullptr;
    }
    const int n = P->n;
    auto sel = [&](int p) { return !P->selection || P->selection[p] == 0; };
    const std::function<bool(int)> self_fn = sel;
    // rigid bodies and particle modifiers run the split pipeline, as Solver.step does
    // (core/solver.py:440-453)
    const bool rigid = !g_rigid.bodies.empty() && P->rigid_id && P->x_ref;
    const bool mods = !g_rigid.mods.empty() && P->mod_mask;
    if (rigid || mods) fused = 0;
    int prev_lo[3], prev_hi[3];
    for (int s = 0; s < substeps; ++s) {
        Real tf = (Real)*time;
        const double t_sub = *time;
        for (int a = 0; a < 3; ++a) { prev_lo[a] = G.lo[a]; prev_hi[a] = G.hi[a]; }
        if (S) cdf_stamp(*S, M, *time, fused != 0);
        if (!fused || s == 0) {
            // zero_grid over the previous touched box, stress, p2g
            if (prev_hi[0] > prev_lo[0]) zero_box(G, prev_lo, prev_hi, true, true);
            if (!fused && s > 0) { /* split pipeline: g2p already ran at the end of s-1 */ }
            if (mods) for (int p = 0; p < n; ++p) if (sel(p)) apply_modifiers(P, p, tf, dtf);
            par_for(n, par, [&](int p) { if (sel(p)) stress_particle(c, p); });
            track_box(G, P, M);
            par_for(n, par, [&](int p) { if (sel(p)) p2g_particle(c, p); });
        } else {
            // zero_grid_m_vin, g2p_stress_p2g, zero_grid_vout
            if (prev_hi[0] > prev_lo[0]) zero_box(G, prev_lo, prev_hi, true, false);
            par_for(n, par, [&](int p) {
                if (!sel(p)) return;
                int mat = P->material[p];
                if (mat != 7 && mat != 8) g2p_particle(c, p);
            });
            if (prev_hi[0] > prev_lo[0]) zero_box(G, prev_lo, prev_hi, false, true);
            par_for(n, par, [&](int p) { if (sel(p)) stress_particle(c, p); });
            track_box(G, P, M);
            par_for(n, par, [&](int p) { if (sel(p)) p2g_particle(c, p); });
        }
        grid_update(G, M, cols, ncol, wrench, tf, dtf, par);
        for (int k = 0; k < ncol; ++k) integrate_pose(cols[k], *time, dt);
        if (S) cdf_integrate(*S, *time, dt, fused != 0);
        *time = *time + dt;
        if (!fused) {
            par_for(n, par, [&](int p) {
                if (!sel(p)) return;
                int mat = P->material[p];
                if (mat != 7 && mat != 8) g2p_particle(c, p);
            });
            if (rigid) rigid_tail(P, M, G, t_sub, dtf, self_fn);
        }
    }
    if (fused) {
        if (S && S->stale_set) { cdf_copy_prev_box(*S, S->stale_box); S->stale_set = false; }
        par_for(n, par, [&](int p) {
            if (!sel(p)) return;
            int mat = P->material[p];
            if (mat != 7 && mat != 8) g2p_particle(c, p);
        });
    }
    if (c.oob) { g_err = "particle stencil left the grid"; return GBMPM_ERR_BOUNDS; }
    return GBMPM_OK;
}

// Block-key sort permutation (core/solver.py:458-465): float64 floor, >> 2,
// lexicographic key, stable argsort; returns 0 (perm untouched) when sorted.
int32_t gbmpm_oracle_sort_perm(const Real* x, int32_t n, double dx, int32_t n_grid, int64_t* keys_out,
                               int32_t* perm_out) {
    std::vector<int64_t> keys(n);
    int64_t nb = (n_grid >> 2) + 2;
    for (int p = 0; p < n; ++p) {
        int64_t b[3];
        for (int a = 0; a < 3; ++a) {
            double q = (double)x[3 * (size_t)p + a] / dx - 0.5;
            b[a] = ((int64_t)std::floor(q)) >> 2;
        }
        keys[p] = (b[0] * nb + b[1]) * nb + b[2];
    }
    if (keys_out) std::copy(keys.begin(), keys.end(), keys_out);
    bool sorted = true;
    for (int p = 1; p < n; ++p) if (keys[p] < keys[p - 1]) { sorted = false; break; }
    if (sorted) return 0;
    std::vector<int32_t> perm(n);
    std::iota(perm.begin(), perm.end(), 0);
    std::stable_sort(perm.begin(), perm.end(), [&](int32_t a, int32_t b) { return keys[a] < keys[b]; });
    std::copy(perm.begin(), perm.end(), perm_out);
    return 1;
}

// Active blocks (mpm_utils.py:1506-1544): mark with fp32 int() truncation,
// dilate by one block, count current and union-with-previous. prev/cur are
// int32[bd^3] (cur is written); counts = {current, union}.
void gbmpm_oracle_blocks(const Real* x, int32_t n, Real inv_dx, int32_t n_grid, const int32_t* prev, int32_t* cur,
                         int32_t* counts) {
    int bd = (n_grid + 3) / 4;
    std::vector<int32_t> raw((size_t)bd * bd * bd, 0);
    for (int p = 0; p < n; ++p) {
        int b[3];
        for (int a = 0; a < 3; ++a) {
            int v = (int)(x[3 * (size_t)p + a] * inv_dx - 0.5f);
            v = v >> 2;
            b[a] = std::min(std::max(v, 0), bd - 1);
        }
        raw[((size_t)b[0] * bd + b[1]) * bd + b[2]] = 1;
    }
    int cc = 0, uc = 0;
    for (int x0 = 0; x0 < bd; ++x0)
        for (int y0 = 0; y0 < bd; ++y0)
            for (int z0 = 0; z0 < bd; ++z0) {
                int on = 0;
                for (int i = -1; i <= 1; ++i)
                    for (int j = -1; j <= 1; ++j)
                        for (int k = -1; k <= 1; ++k) {
                            int xi = std::min(std::max(x0 + i, 0), bd - 1);
                            int yj = std::min(std::max(y0 + j, 0), bd - 1);
                            int zk = std::min(std::max(z0 + k, 0), bd - 1);
                            if (raw[((size_t)xi * bd + yj) * bd + zk] == 1) on = 1;
                        }
                size_t id = ((size_t)x0 * bd + y0) * bd + z0;
                cur[id] = on;
                if (on) ++cc;
                if (on || (prev && prev[id] == 1)) ++uc;
            }
    counts[0] = cc;
    counts[1] = uc;
}

// compute_R_from_F (mpm_utils.py:1256-1285): stores R^T
void gbmpm_oracle_R(const Real* F_trial, int32_t n, Real* R_out) {
    for (int p = 0; p < n; ++p) {
        M3 F = load33(F_trial + 9 * (size_t)p), U, V; V3 s;
        svd3_impl(F, U, s, V);
        if (mdet(U) < 0.0f) for (int i = 0; i < 3; ++i) U.m[i][2] = -U.m[i][2];
        if (mdet(V) < 0.0f) for (int i = 0; i < 3; ++i) V.m[i][2] = -V.m[i][2];
        store33(R_out + 9 * (size_t)p, mT(mmul(U, mT(V))));
    }
}

// compute_cov_from_F (mpm_utils.py:1234-1253)
void gbmpm_oracle_cov(const Real* F_trial, const Real* init_cov, int32_t n, Real* cov_out) {
    for (int p = 0; p < n; ++p) {
        M3 F = load33(F_trial + 9 * (size_t)p);
        const Real* c = init_cov + 6 * (size_t)p;
        M3 I0;
        I0.m[0][0] = c[0]; I0.m[0][1] = c[1]; I0.m[0][2] = c[2];
        I0.m[1][0] = c[1]; I0.m[1][1] = c[3]; I0.m[1][2] = c[4];
        I0.m[2][0] = c[2]; I0.m[2][1] = c[4]; I0.m[2][2] = c[5];
        M3 r = mmul(mmul(F, I0), mT(F));
        Real* o = cov_out + 6 * (size_t)p;
        o[0] = r.m[0][0]; o[1] = r.m[0][1]; o[2] = r.m[0][2];
        o[3] = r.m[1][1]; o[4] = r.m[1][2]; o[5] = r.m[2][2];
    }
}

}  // extern "C"
