// The deterministic particle passes (GBMPM_TICK_DETERMINISTIC).
//
// Every operation here rounds once: this translation unit is compiled with
// --fmad=false, so no product is contracted into an FMA, and each expression is
// written in the operation order of the fp32 statement of the reference's kernels
// (mpm_utils.py). Logarithms, exponentials and powers are evaluated in double by this
// file's own method and rounded once, and the SVD runs in double. The P2G deposits are not added with atomics: each particle writes its
// 27 contributions as records keyed by node, a stable radix sort groups them by
// node in particle order, and one thread per node adds its group in that order.
//
// So a tick on this path is bit-for-bit reproducible run to run, and it equals, bit
// for bit, a single-threaded CPU statement of the same arithmetic in the same order.
// It is a verification mode: simple one-thread-per-item kernels over the caller's
// particle order, several times slower than the tiled path.
//
// Scope: every material law (ids 0-2, 5, 6, 9-13), with the grid pass's colliders;
// the host rejects rigid bodies (7, 8), CDF lanes and particle modifiers.
#include "common.cuh"

namespace gbmpm {
namespace {

constexpr int kDetThreads = 256;

// ---- 3x3 algebra, row-major float[9], in the reference's operation order ----

// warp mat*mat: t[i][j] = ((0 + a[i][0] b[0][j]) + a[i][1] b[1][j]) + a[i][2] b[2][j]
__device__ __forceinline__ void d_mmul(const float *a, const float *b, float *t) {
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            float acc = 0.0f;
#pragma unroll
            for (int k = 0; k < 3; ++k) acc = acc + a[3 * i + k] * b[3 * k + j];
            t[3 * i + j] = acc;
        }
}
__device__ __forceinline__ void d_trans(const float *a, float *t) {
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) t[3 * i + j] = a[3 * j + i];
}
// warp mat*vec: r[i] = (a[i][0] b0 + a[i][1] b1) + a[i][2] b2
__device__ __forceinline__ void d_mvmul(const float *a, const float *b, float *r) {
#pragma unroll
    for (int i = 0; i < 3; ++i) r[i] = a[3 * i] * b[0] + a[3 * i + 1] * b[1] + a[3 * i + 2] * b[2];
}
// warp determinant: dot(row0, cross(row1, row2))
__device__ __forceinline__ float d_det(const float *a) {
    const float c0 = a[4] * a[8] - a[5] * a[7];
    const float c1 = a[5] * a[6] - a[3] * a[8];
    const float c2 = a[3] * a[7] - a[4] * a[6];
    return a[0] * c0 + a[1] * c1 + a[2] * c2;
}
// wp.log, wp.exp and wp.pow in fp32 as their correctly rounded values: evaluated in
// double by this file's own method, operation by operation, and rounded once. The
// CPU statement of the same method returns the same double, bit for bit.
//   log x = k ln2 + 2 atanh(s), x = m 2^k with m in [1/sqrt 2, sqrt 2), s = (m - 1)/(m + 1),
//           the atanh series to s^23 (|s| <= 0.1716: the next term is below 1e-18);
//   exp x = 2^k exp(r), k = round(x / ln2), r = x - k ln2 (|r| <= 0.35), the Taylor
//           series to r^17 in Horner form (the next term is below 1e-22).
// Measured against the host libm over 2e6 arguments: 3.7e-16 and 9.4e-16 relative.
__device__ __forceinline__ double d_dlog(double x) {
    if (!(x > 0.0) || isinf(x)) return (x == 0.0) ? -HUGE_VAL : (isinf(x) ? x : (double)NAN);
    int k = 0;
    double m = frexp(x, &k);
    if (m < 0.70710678118654752440) { m = m * 2.0; k = k - 1; }
    const double s = (m - 1.0) / (m + 1.0);
    const double s2 = s * s;
    double t = 1.0 / 23.0;
    for (int j = 21; j >= 1; j -= 2) t = 1.0 / (double)j + s2 * t;
    return (double)k * 0.69314718055994530942 + 2.0 * s * t;
}
__device__ __forceinline__ double d_dexp(double x) {
    if (x != x) return x;
    if (x > 709.0) return HUGE_VAL;
    if (x < -745.0) return 0.0;
    const double kd = floor(x * 1.44269504088896340736 + 0.5);
    const double r = x - kd * 0.69314718055994530942;
    double t = 1.0;
    for (int j = 17; j >= 1; --j) t = 1.0 + r * t / (double)j;
    return ldexp(t, (int)kd);
}
__device__ __forceinline__ float d_log(float x) { return (float)d_dlog((double)x); }
__device__ __forceinline__ float d_exp(float x) { return (float)d_dexp((double)x); }
__device__ __forceinline__ float d_pow(float x, float y) { return (float)d_dexp((double)y * d_dlog((double)x)); }

// wp.sin, wp.cos and wp.acos of the particle rotation modifier, the same way (the CPU
// statement of the same method returns the same double, bit for bit):
//   sin, cos: x = q pi/2 + r, q = round(x 2/pi) (|r| <= pi/4 for the angles the
//             modifier forms), then the Taylor series of sin r to r^21 and of cos r to
//             r^20 in nested form (the next terms are below 1e-23), and the quadrant;
//   acos c = pi/2 - asin c for |c| <= 1/2, 2 asin sqrt((1 - c)/2) above 1/2 and
//            pi - 2 asin sqrt((1 + c)/2) below -1/2, with the Taylor series of asin z
//            (|z| <= 1/2) to z^51 in Horner form (the next term is below 1e-18).
// Measured against the host libm over 2e6 arguments: within 2.2e-16 (sin, cos) and
// 8.9e-16 (acos), and the same float after rounding.
__device__ __forceinline__ double d_dsincos(double x, bool want_cos) {
    if (!(x == x) || isinf(x)) return (double)NAN;
    const double q = floor(x * 0.63661977236758134308 + 0.5);
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
__device__ __forceinline__ double d_dasin_half(double z) {   // |z| <= 1/2
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
__device__ __forceinline__ double d_dacos(double c) {
    if (!(c >= -1.0 && c <= 1.0)) return (double)NAN;
    if (c > 0.5) return 2.0 * d_dasin_half(sqrt((1.0 - c) * 0.5));
    if (c < -0.5) return 3.14159265358979323846 - 2.0 * d_dasin_half(sqrt((1.0 + c) * 0.5));
    return 1.57079632679489661923 - d_dasin_half(c);
}
__device__ __forceinline__ float d_sin(float x) { return (float)d_dsincos((double)x, false); }
__device__ __forceinline__ float d_cos(float x) { return (float)d_dsincos((double)x, true); }
__device__ __forceinline__ float d_acos(float c) { return (float)d_dacos((double)c); }

// ---- SVD: this project's cyclic Jacobi eigen-solve of F^T F, then a Givens QR of
// F V, in double throughout (the tiled path's method, without its FP32 first try)
__device__ void d_svd3(const float *F, float *U, float *s, float *Vo) {
    double A[3][3], B[3][3], V[3][3], W[3][3], Q[3][3];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) A[i][j] = (double)F[3 * i + j];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            double acc = 0.0;
            for (int k = 0; k < 3; ++k) acc = acc + A[k][i] * A[k][j];
            B[i][j] = acc;
            V[i][j] = (i == j) ? 1.0 : 0.0;
        }
    for (int sweep = 0; sweep < 40; ++sweep) {
        const double off = B[0][1] * B[0][1] + B[0][2] * B[0][2] + B[1][2] * B[1][2];
        const double dia = B[0][0] * B[0][0] + B[1][1] * B[1][1] + B[2][2] * B[2][2];
        if (off <= 1e-32 * dia || off == 0.0) break;
        for (int p = 0; p < 2; ++p)
            for (int q = p + 1; q < 3; ++q) {
                if (B[p][q] == 0.0) continue;
                const double theta = (B[q][q] - B[p][p]) / (2.0 * B[p][q]);
                const double t = (theta >= 0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
                const double c = 1.0 / sqrt(t * t + 1.0), sn = t * c;
                for (int k = 0; k < 3; ++k) {   // B = J^T B J
                    const double bkp = B[k][p], bkq = B[k][q];
                    B[k][p] = c * bkp - sn * bkq;
                    B[k][q] = sn * bkp + c * bkq;
                }
                for (int k = 0; k < 3; ++k) {
                    const double bpk = B[p][k], bqk = B[q][k];
                    B[p][k] = c * bpk - sn * bqk;
                    B[q][k] = sn * bpk + c * bqk;
                }
                for (int k = 0; k < 3; ++k) {
                    const double vkp = V[k][p], vkq = V[k][q];
                    V[k][p] = c * vkp - sn * vkq;
                    V[k][q] = sn * vkp + c * vkq;
                }
            }
    }
    // eigenvalues descending, a stable insertion sort (equal values keep their order)
    int ord[3] = {0, 1, 2};
    for (int i = 1; i < 3; ++i) {
        const int val = ord[i];
        int j = i;
        while (j > 0 && B[val][val] > B[ord[j - 1]][ord[j - 1]]) { ord[j] = ord[j - 1]; --j; }
        ord[j] = val;
    }
    double Vs[3][3];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) Vs[i][j] = V[i][ord[j]];
    const double dv = Vs[0][0] * (Vs[1][1] * Vs[2][2] - Vs[1][2] * Vs[2][1]) -
                      Vs[0][1] * (Vs[1][0] * Vs[2][2] - Vs[1][2] * Vs[2][0]) +
                      Vs[0][2] * (Vs[1][0] * Vs[2][1] - Vs[1][1] * Vs[2][0]);
    if (dv < 0)
        for (int i = 0; i < 3; ++i) Vs[i][2] = -Vs[i][2];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            double acc = 0.0;
            for (int k = 0; k < 3; ++k) acc = acc + A[i][k] * Vs[k][j];
            W[i][j] = acc;
            Q[i][j] = (i == j) ? 1.0 : 0.0;
        }
    const int pr[3][2] = {{0, 1}, {0, 2}, {1, 2}};   // zero W[1][0], W[2][0], W[2][1]
    for (int g = 0; g < 3; ++g) {
        const int a = pr[g][0], b = pr[g][1], col = (g < 2) ? 0 : 1;
        const double x = W[a][col], y = W[b][col];
        const double r = sqrt(x * x + y * y);
        double c = 1.0, sn = 0.0;
        if (r > 0.0) { c = x / r; sn = y / r; }
        for (int k = 0; k < 3; ++k) {
            const double wa = W[a][k], wb = W[b][k];
            W[a][k] = c * wa + sn * wb;
            W[b][k] = -sn * wa + c * wb;
        }
        for (int k = 0; k < 3; ++k) {
            const double qa = Q[k][a], qb = Q[k][b];
            Q[k][a] = c * qa + sn * qb;
            Q[k][b] = -sn * qa + c * qb;
        }
    }
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) { U[3 * i + j] = (float)Q[i][j]; Vo[3 * i + j] = (float)Vs[i][j]; }
    s[0] = (float)W[0][0]; s[1] = (float)W[1][1]; s[2] = (float)W[2][2];
}

// U diag(d0, d1, d2) W^T as the reference writes it: full 3x3 products with the zeros
__device__ __forceinline__ void d_udwt(const float *U, float d0, float d1, float d2, const float *W, float *out) {
    const float D[9] = {d0, 0.0f, 0.0f, 0.0f, d1, 0.0f, 0.0f, 0.0f, d2};
    float UD[9], WT[9];
    d_mmul(U, D, UD);
    d_trans(W, WT);
    d_mmul(UD, WT, out);
}
__device__ __forceinline__ float d_len3(float a, float b, float c) { return sqrtf(a * a + b * b + c * c); }
__device__ __forceinline__ float d_max(float a, float b) { return (a < b) ? b : a; }   // std::max
__device__ __forceinline__ float d_min(float a, float b) { return (b < a) ? b : a; }   // std::min

// a table over [smin, smax] sampled at n points, linear in between (mpm_utils.py:62-70)
__device__ __forceinline__ float d_table(const float *tab, int n, float smin, float smax, float s) {
    float idx = (s - smin) / (smax - smin) * (float)(n - 1);
    idx = d_min(d_max(idx, 0.0f), (float)(n - 1) - 1.0e-6f);
    const int i0 = (int)floorf(idx);
    const float fr = idx - (float)i0;
    return tab[i0] * (1.0f - fr) + tab[i0 + 1] * fr;
}

// ---- return maps (mpm_utils.py:127-580); each may update the particle's yield, mu,
// lam or Jp as the reference's do
// von_mises_return_mapping (:127-170), with_damage (:172-225)
__device__ void d_rm_von_mises(const PK &k, int p, int mat, bool damage, const float *Ft, float *Fe) {
    const MatTables &T = *k.tab;
    float U[9], so[3], V[9];
    d_svd3(Ft, U, so, V);
    const float sig[3] = {d_max(so[0], 0.01f), d_max(so[1], 0.01f), d_max(so[2], 0.01f)};
    float eps[3] = {d_log(sig[0]), d_log(sig[1]), d_log(sig[2])};
    const float temp = (eps[0] + eps[1] + eps[2]) / 3.0f;
    const float mu = k.mu[p], lam = k.lam[p];
    const float tr = eps[0] + eps[1] + eps[2];
    float tau[3];
    for (int a = 0; a < 3; ++a) tau[a] = eps[a] * (2.0f * mu) + 1.0f * (lam * tr);
    const float sum_tau = tau[0] + tau[1] + tau[2];
    const float cond[3] = {tau[0] - sum_tau / 3.0f, tau[1] - sum_tau / 3.0f, tau[2] - sum_tau / 3.0f};
    for (int i = 0; i < 9; ++i) Fe[i] = Ft[i];
    float ys = k.ys[p];
    if (!(d_len3(cond[0], cond[1], cond[2]) > ys)) return;
    if (damage && ys <= 0) return;
    const float eh[3] = {eps[0] - temp, eps[1] - temp, eps[2] - temp};
    const float ehn = d_len3(eh[0], eh[1], eh[2]) + 1e-6f;
    const float dg = ehn - ys / (2.0f * mu);
    const float f = dg / ehn;
    for (int a = 0; a < 3; ++a) eps[a] = eps[a] - eh[a] * f;
    if (damage) {
        ys = ys - T.softening[mat] * d_len3(eh[0] * f, eh[1] * f, eh[2] * f);
        if (ys <= 0) { k.mu[p] = 0.0f; k.lam[p] = 0.0f; }
    }
    d_udwt(U, d_exp(eps[0]), d_exp(eps[1]), d_exp(eps[2]), V, Fe);
    if (T.hardening[mat] > 0.5f) ys = ys + 2.0f * k.mu[p] * T.xi[mat] * dg;
    k.ys[p] = ys;
}

// the 48-step bisection of mu_i_return_mapping (:300-312), as the reference runs it
__device__ float d_mu_i_bisect(const PK &k, bool tab, float tbK, float G, float pK, float Ic, float mu_s, float dmu,
                               float I0) {
    float lo = 0.0f, hi = tbK / (G * k.dt);
    for (int it = 0; it < 48; ++it) {
        const float mid = 0.5f * (lo + hi);
        const float Im = mid * Ic;
        float mu_mid;
        if (!tab) mu_mid = mu_s + dmu * Im / (Im + I0);
        else mu_mid = d_table(k.eta, k.eta_n, k.eta_smin, k.eta_smax, d_log(d_max(Im, 1e-12f)) * 0.43429448190325176f);
        const float g = tbK - G * k.dt * mid - mu_mid * pK;
        if (g > 0.0f) lo = mid; else hi = mid;
    }
    return 0.5f * (lo + hi);
}

// mu_i_return_mapping (:246-324) and its tabulated variant (:327-407)
__device__ void d_rm_mu_i(const PK &k, int p, int mat, bool tab, const float *Ft, float *Fe) {
    const MatTables &T = *k.tab;
    float U[9], sig[3], V[9];
    d_svd3(Ft, U, sig, V);
    const float sc[3] = {d_max(fabsf(sig[0]), 1e-6f), d_max(fabsf(sig[1]), 1e-6f), d_max(fabsf(sig[2]), 1e-6f)};
    const float eps[3] = {d_log(sc[0]), d_log(sc[1]), d_log(sc[2])};
    const float tr = eps[0] + eps[1] + eps[2];
    for (int i = 0; i < 9; ++i) Fe[i] = Ft[i];
    if (tr >= 0.0f) {
        float VT[9];
        d_trans(V, VT);
        d_mmul(U, VT, Fe);
        return;
    }
    const float G = k.mu[p], lam = k.lam[p];
    const float J = sc[0] * sc[1] * sc[2];
    const float mean = tr / 3.0f;
    const float d0 = eps[0] - mean, d1 = eps[1] - mean, d2 = eps[2] - mean;
    const float dn = sqrtf(d0 * d0 + d1 * d1 + d2 * d2);
    const float pK = -(2.0f * G / 3.0f + lam) * tr;
    const float tbK = 2.0f * G * dn / sqrtf(2.0f);
    const float pC = pK / J;
    const float mu_s = T.mu_s[mat], dmu = T.dmu[mat], I0 = T.I0[mat];
    const float thresh = tab ? k.eta[0] : mu_s;
    if (!(tbK > thresh * pK)) return;
    const float Ic = T.d[mat] * sqrtf(T.rho_s[mat] / pC);
    const float gdp = d_mu_i_bisect(k, tab, tbK, G, pK, Ic, mu_s, dmu, I0);
    const float tbn = tbK - G * k.dt * gdp;
    const float scale = tbn / d_max(tbK, 1e-20f);
    d_udwt(U, d_exp(d0 * scale + mean), d_exp(d1 * scale + mean), d_exp(d2 * scale + mean), V, Fe);
}

// mu_i_phi_pressure (:421-430), j_cs_of_I (:410-418)
__device__ __forceinline__ float d_mu_i_phi_pressure(const MatTables &T, int mat, float J, float Jr) {
    const float K = T.E[mat] / (3.0f * (1.0f - 2.0f * T.nu[mat]));
    const float pr = K * (Jr / d_max(J, 1e-6f) - 1.0f);
    return d_max(pr, 0.0f);
}

// mu_i_phi_return_mapping (:433-522)
__device__ void d_rm_mu_i_phi(const PK &k, int p, int mat, const float *Ft, float *Fe) {
    const MatTables &T = *k.tab;
    float U[9], sig[3], V[9];
    d_svd3(Ft, U, sig, V);
    const float sc[3] = {d_max(fabsf(sig[0]), 1e-6f), d_max(fabsf(sig[1]), 1e-6f), d_max(fabsf(sig[2]), 1e-6f)};
    const float eps[3] = {d_log(sc[0]), d_log(sc[1]), d_log(sc[2])};
    const float J = sc[0] * sc[1] * sc[2];
    const float tr = eps[0] + eps[1] + eps[2];
    const float mean = tr / 3.0f;
    const float d0 = eps[0] - mean, d1 = eps[1] - mean, d2 = eps[2] - mean;
    const float dn = sqrtf(d0 * d0 + d1 * d1 + d2 * d2);
    const float G = k.mu[p];
    float Jr = k.Jp[p];
    if (Jr < 0.5f) Jr = 1.0f;
    const float pc = d_mu_i_phi_pressure(T, mat, J, Jr);
    const float beta = 8.0f;
    for (int i = 0; i < 9; ++i) Fe[i] = Ft[i];
    k.Jp[p] = Jr;
    if (pc <= 0.0f) {
        const float si = d_exp(mean);
        d_udwt(U, si, si, si, V, Fe);
        return;
    }
    const float pK = pc * J;
    const float tbK = 2.0f * G * dn / sqrtf(2.0f);
    const float mu_s = T.mu_s[mat], dmu = T.dmu[mat], I0 = T.I0[mat];
    if (!(tbK > mu_s * pK)) return;
    const float Ic = T.d[mat] * sqrtf(T.rho_s[mat] / pc);
    const float gdp = d_mu_i_bisect(k, false, tbK, G, pK, Ic, mu_s, dmu, I0);
    const float Ir = gdp * Ic;
    const float dgam = d_min(beta * gdp * k.dt, 1.0f);
    const float denom = d_max(1.0f - T.phi_chi[mat] * Ir / (Ir + I0), 1e-3f);
    const float jcs = 1.0f / denom;
    k.Jp[p] = Jr + dgam * (jcs - Jr);
    const float tbn = tbK - G * k.dt * gdp;
    const float scale = tbn / d_max(tbK, 1e-20f);
    d_udwt(U, d_exp(d0 * scale + mean), d_exp(d1 * scale + mean), d_exp(d2 * scale + mean), V, Fe);
}

// sand_return_mapping (:543-580)
__device__ void d_rm_sand(const PK &k, int p, int mat, const float *Ft, float *Fe) {
    const MatTables &T = *k.tab;
    float U[9], sig[3], V[9];
    d_svd3(Ft, U, sig, V);
    const float eps[3] = {d_log(d_max(fabsf(sig[0]), 1e-14f)), d_log(d_max(fabsf(sig[1]), 1e-14f)),
                          d_log(d_max(fabsf(sig[2]), 1e-14f))};
    const float tr = eps[0] + eps[1] + eps[2];
    const float eh[3] = {eps[0] - tr / 3.0f, eps[1] - tr / 3.0f, eps[2] - tr / 3.0f};
    const float ehn = d_len3(eh[0], eh[1], eh[2]);
    const float mu = k.mu[p], lam = k.lam[p];
    const float dg = ehn + (3.0f * lam + 2.0f * mu) / (2.0f * mu) * tr * T.alpha[mat];
    for (int i = 0; i < 9; ++i) Fe[i] = Ft[i];
    if (dg > 0 && tr > 0) {
        float VT[9];
        d_trans(V, VT);
        d_mmul(U, VT, Fe);
    }
    if (dg > 0 && tr <= 0) {
        const float f = dg / ehn;
        d_udwt(U, d_exp(eps[0] - eh[0] * f), d_exp(eps[1] - eh[1] * f), d_exp(eps[2] - eh[2] * f), V, Fe);
    }
}

// ---- quadratic B-spline weights (p2g_particle / g2p_particle, mpm_utils.py:830-850)
struct DetStencil {
    int base[3];
    float fx[3], w[3][3], dw[3][3];   // w[axis][node]
};
__device__ __forceinline__ void d_stencil(const float *x, float inv_dx, DetStencil &S) {
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const float gp = x[a] * inv_dx;
        S.base[a] = (int)floorf(gp - 0.5f);
        const float fx = gp - (float)S.base[a];
        S.fx[a] = fx;
        const float wa = 1.5f - fx, wb = fx - 1.0f, wc = fx - 0.5f;
        S.w[a][0] = wa * wa * 0.5f;
        S.w[a][1] = (0.0f - wb * wb) + 0.75f;
        S.w[a][2] = wc * wc * 0.5f;
        S.dw[a][0] = fx - 1.5f;
        S.dw[a][1] = -2.0f * (fx - 1.0f);
        S.dw[a][2] = fx - 0.5f;
    }
}
__device__ __forceinline__ bool d_inside(const DetStencil &S, int ng, int periodic_x) {
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        if (a == 0 && periodic_x) continue;
        if (S.base[a] < 0 || S.base[a] + 2 >= ng) return false;
    }
    return true;
}
__device__ __forceinline__ int d_wrap(int i, int n) { return ((i % n) + n) % n; }
// compute_dweight (mpm_utils.py:601-610)
__device__ __forceinline__ void d_dweight(const DetStencil &S, int i, int j, int k, float inv_dx, float *d) {
    d[0] = S.dw[0][i] * S.w[1][j] * S.w[2][k] * inv_dx;
    d[1] = S.w[0][i] * S.dw[1][j] * S.w[2][k] * inv_dx;
    d[2] = S.w[0][i] * S.w[1][j] * S.dw[2][k] * inv_dx;
}

// ---- G2P (g2p_particle, mpm_utils.py:944-1043): v, C, x, L and F_trial --------
__global__ void __launch_bounds__(kDetThreads) k_det_g2p(PK k, int reset_lists) {
    if (reset_lists && blockIdx.x == 0 && threadIdx.x == 0) {
        k.blk_count[0] = 0;
        k.blk_count[1] = 0;
    }
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= k.n) return;
    if (k.sel && k.sel[p] != 0) return;
    const float x[3] = {k.x[3 * p], k.x[3 * p + 1], k.x[3 * p + 2]};
    DetStencil S;
    d_stencil(x, k.inv_dx, S);
    if (!d_inside(S, k.ng, k.periodic_x)) { set_status(k.status, GBMPM_FLAG_STENCIL_OOB); return; }
    float nv[3] = {0.0f, 0.0f, 0.0f}, nC[9], nF[9];
#pragma unroll
    for (int i = 0; i < 9; ++i) { nC[i] = 0.0f; nF[i] = 0.0f; }
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
            for (int kk = 0; kk < 3; ++kk) {
                int ix = S.base[0] + i;
                if (k.periodic_x) ix = d_wrap(ix, k.ng);
                const int iy = S.base[1] + j, iz = S.base[2] + kk;
                const float dpos[3] = {(float)i - S.fx[0], (float)j - S.fx[1], (float)kk - S.fx[2]};
                const float weight = S.w[0][i] * S.w[1][j] * S.w[2][kk];
                const float4 g4 = k.gv[((size_t)ix * k.ng + iy) * k.ng + iz];
                const float gv[3] = {g4.x, g4.y, g4.z};
#pragma unroll
                for (int a = 0; a < 3; ++a) nv[a] = nv[a] + gv[a] * weight;
                const float sc = weight * k.inv_dx * 4.0f;
#pragma unroll
                for (int a = 0; a < 3; ++a)
#pragma unroll
                    for (int b = 0; b < 3; ++b) nC[3 * a + b] = nC[3 * a + b] + gv[a] * dpos[b] * sc;
                float dwt[3];
                d_dweight(S, i, j, kk, k.inv_dx, dwt);
#pragma unroll
                for (int a = 0; a < 3; ++a)
#pragma unroll
                    for (int b = 0; b < 3; ++b) nF[3 * a + b] = nF[3 * a + b] + gv[a] * dwt[b];
            }
    float xn[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) xn[a] = x[a] + nv[a] * k.dt;
    if (k.periodic_x) {
        const float lx = (float)k.ng * k.dx;
        if (xn[0] < 0.0f) xn[0] = xn[0] + lx;
        if (xn[0] >= lx) xn[0] = xn[0] - lx;
    }
#pragma unroll
    for (int a = 0; a < 3; ++a) { k.v[3 * p + a] = nv[a]; k.x[3 * p + a] = xn[a]; }
    float A[9], Fo[9], Ft[9];
#pragma unroll
    for (int i = 0; i < 9; ++i) {
        k.C[9 * (size_t)p + i] = nC[i];
        k.L[9 * (size_t)p + i] = nF[i];
        A[i] = ((i % 4 == 0) ? 1.0f : 0.0f) + nF[i] * k.dt;
        Fo[i] = k.F[9 * (size_t)p + i];
    }
    d_mmul(A, Fo, Ft);
#pragma unroll
    for (int i = 0; i < 9; ++i) k.Ft[9 * (size_t)p + i] = Ft[i];
    if (k.update_cov && k.cov) {   // update_cov (mpm_utils.py:613-633)
        float *c6 = k.cov + 6 * (size_t)p;
        const float cn[9] = {c6[0], c6[1], c6[2], c6[1], c6[3], c6[4], c6[2], c6[4], c6[5]};
        float gT[9], a1[9], a2[9];
        d_trans(nF, gT);
        d_mmul(nF, cn, a1);
        d_mmul(cn, gT, a2);
        float nn[9];
#pragma unroll
        for (int i = 0; i < 9; ++i) nn[i] = cn[i] + (a1[i] + a2[i]) * k.dt;
        c6[0] = nn[0]; c6[1] = nn[1]; c6[2] = nn[2]; c6[3] = nn[4]; c6[4] = nn[5]; c6[5] = nn[8];
    }
}

// ---- stress (stress_update_particle, mpm_utils.py:1056-1149) --------------------
// the fluids' pressure and deviatoric rate (mpm_utils.py:17-85)
__device__ __forceinline__ float d_eos(float J, float bulk) { return -bulk * (d_pow(J, -1.1f) - 1.0f); }
__device__ __forceinline__ void d_dev_rate(const float *L, float *Dd, float &gd) {
    float D[9];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) D[3 * i + j] = (L[3 * i + j] + L[3 * j + i]) * 0.5f;
    const float trd = (D[0] + D[4] + D[8]) / 3.0f;
    for (int i = 0; i < 9; ++i) Dd[i] = D[i] - ((i % 4 == 0) ? 1.0f : 0.0f) * trd;
    float dd = 0.0f;
    for (int i = 0; i < 9; ++i) dd = dd + Dd[i] * Dd[i];
    const float eps = 0.02f;
    gd = sqrtf(2.0f * dd + eps * eps);
}
// Hencky (mpm_utils.py:228-243): U diag(2 mu e + lam tr e) U^T
__device__ void d_stress_hencky(const float *U, const float *sig, float mu, float lam, float *st) {
    const float e0 = d_log(d_max(sig[0], 1e-6f)), e1 = d_log(d_max(sig[1], 1e-6f)), e2 = d_log(d_max(sig[2], 1e-6f));
    const float tr = e0 + e1 + e2;
    d_udwt(U, 2.0f * mu * e0 + lam * tr, 2.0f * mu * e1 + lam * tr, 2.0f * mu * e2 + lam * tr, U, st);
}
// Drucker-Prager (mpm_utils.py:109-124): U diag(c) V^T F^T
__device__ void d_stress_dp(const float *F, const float *U, const float *V, const float *sig, float mu, float lam,
                            float *st) {
    const float l0 = d_log(sig[0]), l1 = d_log(sig[1]), l2 = d_log(sig[2]);
    const float lsum = l0 + l1 + l2;
    float c[3];
    for (int a = 0; a < 3; ++a)
        c[a] = 2.0f * mu * d_log(sig[a]) * (1.0f / sig[a]) + lam * lsum * (1.0f / sig[a]);
    float UDV[9], FT[9];
    d_udwt(U, c[0], c[1], c[2], V, UDV);
    d_trans(F, FT);
    d_mmul(UDV, FT, st);
}
// mu(I)-Phi(I) (mpm_utils.py:525-540)
__device__ void d_stress_mu_i_phi(const float *U, const float *sig, float G, float pc, float *st) {
    const float s0 = d_max(sig[0], 1e-6f), s1 = d_max(sig[1], 1e-6f), s2 = d_max(sig[2], 1e-6f);
    const float e0 = d_log(s0), e1 = d_log(s1), e2 = d_log(s2);
    const float J = s0 * s1 * s2;
    const float mean = (e0 + e1 + e2) / 3.0f;
    const float iso = -pc * J;
    d_udwt(U, 2.0f * G * (e0 - mean) + iso, 2.0f * G * (e1 - mean) + iso, 2.0f * G * (e2 - mean) + iso, U, st);
}

__global__ void __launch_bounds__(kDetThreads) k_det_stress(PK k) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= k.n) return;
    if (k.sel && k.sel[p] != 0) return;
    const int mat = k.mat[p];
    const MatTables &T = *k.tab;
    float Ft[9], F[9], st[9];
    for (int i = 0; i < 9; ++i) Ft[i] = k.Ft[9 * (size_t)p + i];
    // the return map (or the fluids' volumetric F)
    if (mat == 1 || mat == 5) {
        d_rm_von_mises(k, p, mat, mat == 5, Ft, F);
    } else if (mat == 2) {
        d_rm_sand(k, p, mat, Ft, F);
    } else if (mat == 9 || mat == 13) {
        d_rm_mu_i(k, p, mat, mat == 13, Ft, F);
    } else if (mat == 11) {
        d_rm_mu_i_phi(k, p, mat, Ft, F);
    } else if (mat == 6 || mat == 10 || mat == 12) {   // the fluids keep only the volume: F = J^(1/3) I
        const float Jc = d_pow(d_det(Ft), 1.0f / 3.0f);
        for (int i = 0; i < 9; ++i) F[i] = (i % 4 == 0) ? Jc : 0.0f;
    } else {
        for (int i = 0; i < 9; ++i) F[i] = Ft[i];
    }
    for (int i = 0; i < 9; ++i) k.F[9 * (size_t)p + i] = F[i];
    const float J = d_det(F);
    float U[9], sg[3], V[9];
    if (mat != 6 && mat != 10 && mat != 12) d_svd3(F, U, sg, V);
    const float mu = k.mu[p], lam = k.lam[p];
    if (mat == 0 || mat == 5) {   // kirchoff_stress_FCR (mpm_utils.py:8-15)
        float Vt[9], R[9], D[9], FT[9];
        d_trans(V, Vt);
        d_mmul(U, Vt, R);
        for (int i = 0; i < 9; ++i) D[i] = (F[i] - R[i]) * (2.0f * mu);
        d_trans(F, FT);
        d_mmul(D, FT, st);
        const float d = lam * J * (J - 1.0f);
        for (int i = 0; i < 9; ++i) st[i] = st[i] + ((i % 4 == 0) ? 1.0f : 0.0f) * d;
    } else if (mat == 1 || mat == 9 || mat == 13) {
        d_stress_hencky(U, sg, mu, lam, st);
    } else if (mat == 2) {
        d_stress_dp(F, U, V, sg, mu, lam, st);
    } else if (mat == 11) {
        float Jr = k.Jp[p];
        if (Jr < 0.5f) Jr = 1.0f;
        d_stress_mu_i_phi(U, sg, mu, d_mu_i_phi_pressure(T, mat, J, Jr), st);
    } else {   // the fluids (mpm_utils.py:17-85)
        const float pressure = d_eos(J, T.bulk[mat]);
        float c[9];
        if (mat == 6) {   // water
            for (int i = 0; i < 9; ++i) c[i] = ((i % 4 == 0) ? 1.0f : 0.0f) * pressure;
        } else {          // Newtonian / Bingham / Herschel-Bulkley, tabulated viscosity
            float Dd[9], gd;
            d_dev_rate(k.L + 9 * (size_t)p, Dd, gd);
            float eta_app;
            if (mat == 10)
                eta_app = T.pv[mat] + k.ys[p] / gd + T.hardening[mat] * d_pow(gd, T.softening[mat] - 1.0f);
            else
                eta_app = d_table(k.eta, k.eta_n, k.eta_smin, k.eta_smax, d_log(gd) * 0.43429448190325176f);
            for (int i = 0; i < 9; ++i) c[i] = ((i % 4 == 0) ? 1.0f : 0.0f) * pressure + Dd[i] * (2.0f * eta_app);
        }
        for (int i = 0; i < 9; ++i) st[i] = c[i] * J;
    }
    float stT[9];
    d_trans(st, stT);
    for (int i = 0; i < 9; ++i) k.S[9 * (size_t)p + i] = (st[i] + stT[i]) * 0.5f;
}

// ---- particle modifiers before P2G (the pre-P2G operations and velocity modifiers
// of p2g2p, mpm_solver_warp.py:1182-1196; kernels :2385-2540): impulses first, then
// velocity overrides, each in list order, on the float32 window [start, end), in the
// oracle's order of operations. The stress update reads no velocity, so applying
// them in the P2G pass equals applying them before the stress update.
__device__ void d_modifiers(const PK &k, int mask, const float *x, float mass, float *v) {
    const float t = (float)k.sub_time[k.sub];
    for (int pass = 0; pass < 2; ++pass)
        for (int m = 0; m < k.n_mods; ++m) {
            const gbmpm_modifier &d = k.mods[m];
            if (!((mask >> m) & 1) || (d.kind == 0) != (pass == 0)) continue;
            if (!(t >= d.start_time && t < d.end_time)) continue;
            if (d.kind == 0) {
                for (int a = 0; a < 3; ++a) v[a] = v[a] + (d.vec[a] / mass) * k.dt;
            } else if (d.kind == 1) {
                for (int a = 0; a < 3; ++a) v[a] = d.vec[a];
            } else {
                float off[3], hz[3];
                for (int a = 0; a < 3; ++a) off[a] = x[a] - d.point[a];
                const float on = off[0] * d.normal[0] + off[1] * d.normal[1] + off[2] * d.normal[2];
                for (int a = 0; a < 3; ++a) hz[a] = off[a] - on * d.normal[a];
                const float hd = sqrtf(hz[0] * hz[0] + hz[1] * hz[1] + hz[2] * hz[2]);
                const float cosine = (off[0] * d.axis1[0] + off[1] * d.axis1[1] + off[2] * d.axis1[2]) / hd;
                float theta = d_acos(d_min(d_max(cosine, -1.0f), 1.0f));
                if (!(off[0] * d.axis2[0] + off[1] * d.axis2[1] + off[2] * d.axis2[2] > 0.0f)) theta = -theta;
                const float a1 = -hd * d_sin(theta) * d.rotation_scale;
                const float a2 = hd * d_cos(theta) * d.rotation_scale;
                for (int a = 0; a < 3; ++a) v[a] = a1 * d.axis1[a] + a2 * d.axis2[a] + d.translation_scale * d.normal[a];
            }
        }
}

// ---- P2G records (p2g_particle, mpm_utils.py:819-916) ---------------------------
// Record p * 27 + (i * 9 + j * 3 + k) holds the deposit of particle p into node
// (base + (i, j, k)): key = node index, val = (momentum and force impulse, mass).
// A particle that deposits nothing keys its records past the last node.
__global__ void __launch_bounds__(kDetThreads) k_det_p2g(PK k, unsigned long long *key, int *idx, float4 *val) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= k.n) return;
    const unsigned long long none = (unsigned long long)k.ng * k.ng * k.ng;
    const size_t r0 = (size_t)p * 27;
    auto skip = [&]() {
        for (int s = 0; s < 27; ++s) { key[r0 + s] = none; idx[r0 + s] = (int)(r0 + s); }
    };
    if (k.sel && k.sel[p] != 0) { skip(); return; }
    const float x[3] = {k.x[3 * p], k.x[3 * p + 1], k.x[3 * p + 2]};
    float v[3] = {k.v[3 * p], k.v[3 * p + 1], k.v[3 * p + 2]};
    if (k.n_mods && k.mod_mask && k.mod_mask[p]) {
        d_modifiers(k, k.mod_mask[p], x, k.mass[p], v);
        for (int a = 0; a < 3; ++a) k.v[3 * (size_t)p + a] = v[a];
    }
    DetStencil S;
    d_stencil(x, k.inv_dx, S);
    if (!d_inside(S, k.ng, k.periodic_x)) {
        set_status(k.status, GBMPM_FLAG_STENCIL_OOB);
        skip();
        return;
    }
    float C0[9], CT[9], C[9], fs[9];
#pragma unroll
    for (int i = 0; i < 9; ++i) C0[i] = k.C[9 * (size_t)p + i];
    d_trans(C0, CT);
    const float r = k.rpic;
#pragma unroll
    for (int i = 0; i < 9; ++i) C[i] = C0[i] * (1.0f - r) + (C0[i] - CT[i]) * (r / 2.0f);
    if (r < -0.001f) {
#pragma unroll
        for (int i = 0; i < 9; ++i) C[i] = 0.0f;
    }
    const float mass = k.mass[p], vol = k.vol[p];
#pragma unroll
    for (int i = 0; i < 9; ++i) fs[i] = k.S[9 * (size_t)p + i] * -vol;
    int s = 0;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
            for (int kk = 0; kk < 3; ++kk, ++s) {
                const float dpos[3] = {((float)i - S.fx[0]) * k.dx, ((float)j - S.fx[1]) * k.dx,
                                       ((float)kk - S.fx[2]) * k.dx};
                int ix = S.base[0] + i;
                if (k.periodic_x) ix = d_wrap(ix, k.ng);
                const int iy = S.base[1] + j, iz = S.base[2] + kk;
                const float weight = S.w[0][i] * S.w[1][j] * S.w[2][kk];
                float dwt[3], ef[3], cd[3];
                d_dweight(S, i, j, kk, k.inv_dx, dwt);
                d_mvmul(fs, dwt, ef);
                d_mvmul(C, dpos, cd);
                const float wm = weight * mass;
                float add[3];
#pragma unroll
                for (int a = 0; a < 3; ++a) add[a] = (v[a] + cd[a]) * wm + ef[a] * k.dt;
                key[r0 + s] = ((unsigned long long)ix * k.ng + iy) * k.ng + iz;
                idx[r0 + s] = (int)(r0 + s);
                val[r0 + s] = make_float4(add[0], add[1], add[2], weight * mass);
            }
}

// ---- per-node sums in particle order ---------------------------------------------
// After the stable sort by node, the records of one node are contiguous and in
// particle order; the thread at the first record of a node adds them from zero,
// as the serial deposit loop does, writes the node and marks its 4^3 block.
__global__ void __launch_bounds__(kDetThreads) k_det_segsum(PK k, const unsigned long long *key, const int *idx,
                                                            const float4 *val, int n_rec) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_rec) return;
    const unsigned long long node = key[i];
    const unsigned long long none = (unsigned long long)k.ng * k.ng * k.ng;
    if (node >= none || (i > 0 && key[i - 1] == node)) return;
    float4 acc = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    for (int j = i; j < n_rec && key[j] == node; ++j) {
        const float4 d = val[idx[j]];
        acc.x = acc.x + d.x;
        acc.y = acc.y + d.y;
        acc.z = acc.z + d.z;
        acc.w = acc.w + d.w;
    }
    k.gmv[node] = acc;
    const int gz = (int)(node % k.ng), gy = (int)((node / k.ng) % k.ng), gx = (int)(node / ((size_t)k.ng * k.ng));
    const int b = ((gx >> 2) * k.bd + (gy >> 2)) * k.bd + (gz >> 2);
    if (k.blk_flag[b] == 0 && atomicExch(&k.blk_flag[b], 1) == 0) k.blk_list[atomicAdd(k.blk_count, 1)] = b;
}

inline int det_grid(long long n) { return (int)std::max<long long>(1, (n + kDetThreads - 1) / kDetThreads); }

}  // namespace

void det_launch_g2p(const PK &k, bool reset_lists, cudaStream_t s) {
    k_det_g2p<<<det_grid(k.n), kDetThreads, 0, s>>>(k, reset_lists ? 1 : 0);
}
void det_launch_stress(const PK &k, cudaStream_t s) { k_det_stress<<<det_grid(k.n), kDetThreads, 0, s>>>(k); }
void det_launch_p2g(const PK &k, unsigned long long *key, int *idx, float4 *val, cudaStream_t s) {
    k_det_p2g<<<det_grid(k.n), kDetThreads, 0, s>>>(k, key, idx, val);
}
void det_launch_segsum(const PK &k, const unsigned long long *key, const int *idx, const float4 *val, int n_rec,
                       cudaStream_t s) {
    k_det_segsum<<<det_grid(n_rec), kDetThreads, 0, s>>>(k, key, idx, val, n_rec);
}

}  // namespace gbmpm
