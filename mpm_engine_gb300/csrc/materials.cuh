// Material laws: the Kirchhoff stress of the viscous laws and the return maps of
// the solid laws (mpm_utils.py:8-633, 1056-1149), evaluated per particle by the
// stress update of the particle pass.
//
// Included by gbmpm.cu inside namespace gbmpm, after the constants and helpers
// and before the host code; it is not a standalone header.

// ------------------------------------------------------- material laws -----
// Kirchhoff stress of the viscous laws (mpm_utils.py:17-85)
__device__ __forceinline__ void dev_rate(const float *L, float *Dd, float &gd) {
    float D[9];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) D[3 * i + j] = 0.5f * (L[3 * i + j] + L[3 * j + i]);
    float trd = (D[0] + D[4] + D[8]) / 3.0f;
    float dd = 0.0f;
#pragma unroll
    for (int i = 0; i < 9; ++i) {
        Dd[i] = D[i] - ((i % 4 == 0) ? trd : 0.0f);
        dd += Dd[i] * Dd[i];
    }
    gd = sqrtf(2.0f * dd + 0.02f * 0.02f);
}

// x^y for x near 1 (the volume ratios of the fluid laws), as 1 + expm1(y log1p(x - 1)).
// x - 1 is exact for x in [0.5, 2], and the small term carries about one ulp of its
// own size, far below the final rounding next to 1: the result is the correctly
// rounded power except in rare near-ties, as an accurate C library's powf gives it.
// Near 1 a powf with a few ulps of error would differ from that rounding often, and
// the stiff equation of state (K (J^-1.1 - 1), K ~ 1e6 Pa) turns each ulp into a
// visible pressure difference. Away from [0.5, 2] this is powf.
__device__ __forceinline__ float pow_near1(float x, float y) {
    if (!(x > 0.5f && x < 2.0f)) return powf(x, y);
    return 1.0f + expm1f(y * log1pf(x - 1.0f));
}

__device__ __forceinline__ float eos_pressure(float J, float bulk) { return -bulk * (pow_near1(J, -1.1f) - 1.0f); }

__device__ __forceinline__ float table_lerp(const float *tab, int n, float smin, float smax, float s) {
    float idx = (s - smin) / (smax - smin) * (float)(n - 1);
    idx = fminf(fmaxf(idx, 0.0f), (float)(n - 1) - 1.0e-6f);
    int i0 = (int)floorf(idx);
    float fr = idx - (float)i0;
    return tab[i0] * (1.0f - fr) + tab[i0 + 1] * fr;
}

// Hencky stress U diag(2 mu eps + lam tr eps) U^T (mpm_utils.py:228-243)
__device__ __forceinline__ void stress_hencky(const float *U, const float *sig, float mu, float lam, float *out) {
    float e0 = logf(fmaxf(sig[0], 1e-6f)), e1 = logf(fmaxf(sig[1], 1e-6f)), e2 = logf(fmaxf(sig[2], 1e-6f));
    float tr = e0 + e1 + e2;
    udvt(U, 2.0f * mu * e0 + lam * tr, 2.0f * mu * e1 + lam * tr, 2.0f * mu * e2 + lam * tr, U, out);
}

// the friction law mu(I): mu_s + dmu I / (I + I0), or the table over log10 I
template <bool TAB>
__device__ __forceinline__ float mu_of_i(float Im, float mu_s, float dmu, float I0, const float *tab, int tn, float smin,
                                         float smax) {
    if (!TAB) return mu_s + dmu * Im / (Im + I0);
    return table_lerp(tab, tn, smin, smax, logf(fmaxf(Im, 1e-12f)) * 0.43429448190325176f);
}

// The root of g(gdp) = tau_bar - G dt gdp - mu(gdp Ic) p (mpm_utils.py:300-312) for the
// parametric law mu(I) = mu_s + dmu I / (I + I0), in closed form. With a = G dt,
// T = tau_bar - mu_s p (> 0 on the plastic branch) and q = dmu p, g = 0 is the
// quadratic a Ic gdp^2 - B gdp - T I0 = 0 with B = Ic (T - q) - a I0, whose positive
// root is (B + sqrt(B^2 + 4 a Ic T I0)) / (2 a Ic); for B < 0 it is taken as
// 2 T I0 / (sqrt(...) - B), which does not cancel. The reference bisects instead
// (48 steps, about 33 before fp32 exhausts the bracket). Over 20,000 random inputs
// spanning the press's range the returned stress tau_bar - a gdp agrees with the
// bisection's within 2.4e-7 relative (two ulps), and the pass drops the bisection's
// dependent chain of divisions.
__device__ __forceinline__ float mu_i_root(float tbK, float G, float dt, float pK, float Ic, float mu_s, float dmu,
                                           float I0) {
    const float a = G * dt, T = tbK - mu_s * pK, q = dmu * pK;
    const float B = Ic * (T - q) - a * I0;
    const float disc = sqrtf(B * B + 4.0f * a * Ic * (T * I0));
    const float r = (B >= 0.0f) ? (B + disc) / (2.0f * a * Ic) : (2.0f * T * I0) / (disc - B);
    return fminf(fmaxf(r, 0.0f), tbK / a);
}

// the 48-step bisection on g(gdp) = tau_bar - G dt gdp - mu(I) p (mpm_utils.py:300-312).
// Once the midpoint rounds to one end of the bracket, the step it takes leaves the
// bracket where every later step leaves it too (the midpoint repeats, so does the
// comparison), and the loop stops there: the result is bit for bit that of all 48
// steps, which fp32 exhausts after about 24 + log2(hi / root) of them.
template <bool TAB>
__device__ __forceinline__ float mu_i_bisect(float tbK, float G, float dt, float pK, float Ic, float mu_s, float dmu,
                                             float I0, const float *tab, int tn, float smin, float smax) {
    float lo = 0.0f, hi = tbK / (G * dt);
    for (int it = 0; it < 48; ++it) {
        const float mid = 0.5f * (lo + hi);
        const bool at_end = mid == lo || mid == hi;
        float mu_mid = mu_of_i<TAB>(mid * Ic, mu_s, dmu, I0, tab, tn, smin, smax);
        float g = tbK - G * dt * mid - mu_mid * pK;
        if (g > 0.0f) lo = mid; else hi = mid;
        if (at_end) break;
    }
    return 0.5f * (lo + hi);
}
template <bool TAB>
__device__ __forceinline__ float mu_i_bisect(float tbK, float G, float dt, float pK, float Ic, float mu_s, float dmu,
                                             float I0, const PK &k) {
    return mu_i_bisect<TAB>(tbK, G, dt, pK, Ic, mu_s, dmu, I0, k.eta, k.eta_n, k.eta_smin, k.eta_smax);
}

// Return map F_trial -> F and Kirchhoff stress for one particle
// (stress_update_particle, mpm_utils.py:1056-1149).
template <bool SOLIDS>
__device__ __forceinline__ void stress_update(const PK &k, int p, int mat, const float *Ft, const float *L, float *F,
                                              float *S) {
    const MatTables &T = *k.tab;
    if (!SOLIDS || mat == 6 || mat == 10 || mat == 12 || mat == 7 || mat == 8) {
        float J;
        if (mat == 7 || mat == 8) {
#pragma unroll
            for (int i = 0; i < 9; ++i) F[i] = (i % 4 == 0) ? 1.0f : 0.0f;
            J = 1.0f;
        } else {
            float Jt = det3(Ft);
            float Jc = pow_near1(Jt, 1.0f / 3.0f);
#pragma unroll
            for (int i = 0; i < 9; ++i) F[i] = (i % 4 == 0) ? Jc : 0.0f;
            J = Jc * Jc * Jc;
        }
        if (mat == 7 || mat == 8) {
#pragma unroll
            for (int i = 0; i < 9; ++i) S[i] = 0.0f;
            return;
        }
        float pr = eos_pressure(J, T.bulk[mat]);
        if (mat == 6) {
#pragma unroll
            for (int i = 0; i < 9; ++i) S[i] = (i % 4 == 0) ? J * pr : 0.0f;
            return;
        }
        float Dd[9], gd;
        dev_rate(L, Dd, gd);
        float eta_app;
        if (mat == 10) {
            // tau_y / gd and K gd^(n-1) are exactly zero when tau_y or K is zero
            const float ys = k.ys[p], Kp = T.hardening[mat];
            eta_app = T.pv[mat] + (ys != 0.0f ? ys / gd : 0.0f) + (Kp != 0.0f ? Kp * powf(gd, T.softening[mat] - 1.0f) : 0.0f);
        }
        else eta_app = table_lerp(k.eta, k.eta_n, k.eta_smin, k.eta_smax, logf(gd) * 0.43429448190325176f);
        float two_eta = 2.0f * eta_app;
#pragma unroll
        for (int i = 0; i < 9; ++i) S[i] = J * (((i % 4 == 0) ? pr : 0.0f) + two_eta * Dd[i]);
        return;
    }
    if constexpr (SOLIDS) {
        float U[9], V[9], sig[3];
        float mu = k.mu[p], lam = k.lam[p];
        // ---- return mapping
        if (mat == 1 || mat == 5) {  // von Mises (mpm_utils.py:127-225)
            svd3(Ft, U, sig, V);
            float e0 = logf(fmaxf(sig[0], 0.01f)), e1 = logf(fmaxf(sig[1], 0.01f)), e2 = logf(fmaxf(sig[2], 0.01f));
            float tr = e0 + e1 + e2;
            float temp = tr / 3.0f;
            float t0 = 2.0f * mu * e0 + lam * tr, t1 = 2.0f * mu * e1 + lam * tr, t2 = 2.0f * mu * e2 + lam * tr;
            float st = (t0 + t1 + t2) / 3.0f;
            float c0 = t0 - st, c1 = t1 - st, c2 = t2 - st;
            float y = k.ys[p];
            bool done = false;
            if (sqrtf(c0 * c0 + c1 * c1 + c2 * c2) > y) {
                if (mat == 5 && y <= 0.0f) {
#pragma unroll
                    for (int i = 0; i < 9; ++i) F[i] = Ft[i];
                    done = true;
                } else {
                    float h0 = e0 - temp, h1 = e1 - temp, h2 = e2 - temp;
                    float hn = sqrtf(h0 * h0 + h1 * h1 + h2 * h2) + 1e-6f;
                    float dg = hn - y / (2.0f * mu);
                    float r = dg / hn;
                    e0 -= r * h0; e1 -= r * h1; e2 -= r * h2;
                    if (mat == 5) {
                        float rh0 = r * h0, rh1 = r * h1, rh2 = r * h2;
                        y = y - T.softening[mat] * sqrtf(rh0 * rh0 + rh1 * rh1 + rh2 * rh2);
                        if (y <= 0.0f) { mu = 0.0f; lam = 0.0f; k.mu[p] = 0.0f; k.lam[p] = 0.0f; }
                    }
                    sig[0] = expf(e0); sig[1] = expf(e1); sig[2] = expf(e2);
                    udvt(U, sig[0], sig[1], sig[2], V, F);
                    if (T.hardening[mat] > 0.5f) y = y + 2.0f * mu * T.xi[mat] * dg;
                    k.ys[p] = y;
                    done = true;
                }
            }
            if (!done) {
#pragma unroll
                for (int i = 0; i < 9; ++i) F[i] = Ft[i];
            }
        } else if (mat == 2) {  // Drucker-Prager sand (mpm_utils.py:543-580)
            svd3(Ft, U, sig, V);
            float e0 = logf(fmaxf(fabsf(sig[0]), 1e-14f)), e1 = logf(fmaxf(fabsf(sig[1]), 1e-14f)),
                  e2 = logf(fmaxf(fabsf(sig[2]), 1e-14f));
            float tr = e0 + e1 + e2;
            float h0 = e0 - tr / 3.0f, h1 = e1 - tr / 3.0f, h2 = e2 - tr / 3.0f;
            float hn = sqrtf(h0 * h0 + h1 * h1 + h2 * h2);
            float dg = hn + (3.0f * lam + 2.0f * mu) / (2.0f * mu) * tr * T.alpha[mat];
            if (dg <= 0.0f) {
#pragma unroll
                for (int i = 0; i < 9; ++i) F[i] = Ft[i];
            } else if (tr > 0.0f) {
                sig[0] = sig[1] = sig[2] = 1.0f;
                udvt(U, 1.0f, 1.0f, 1.0f, V, F);
            } else {
                float r = dg / hn;
                sig[0] = expf(e0 - h0 * r); sig[1] = expf(e1 - h1 * r); sig[2] = expf(e2 - h2 * r);
                udvt(U, sig[0], sig[1], sig[2], V, F);
            }
        } else if (mat == 9 || mat == 13 || mat == 11) {  // mu(I) family (mpm_utils.py:246-522)
            svd3(Ft, U, sig, V);
            float s0 = fmaxf(fabsf(sig[0]), 1e-6f), s1 = fmaxf(fabsf(sig[1]), 1e-6f), s2 = fmaxf(fabsf(sig[2]), 1e-6f);
            float e0 = logf(s0), e1 = logf(s1), e2 = logf(s2);
            float tr = e0 + e1 + e2;
            float mean = tr / 3.0f;
            float d0 = e0 - mean, d1 = e1 - mean, d2 = e2 - mean;
            float dn = sqrtf(d0 * d0 + d1 * d1 + d2 * d2);
            float J = s0 * s1 * s2;
#pragma unroll
            for (int i = 0; i < 9; ++i) F[i] = Ft[i];
            if (mat != 11) {
                if (tr >= 0.0f) {
                    sig[0] = sig[1] = sig[2] = 1.0f;
                    udvt(U, 1.0f, 1.0f, 1.0f, V, F);
                } else {
                    float pK = -(2.0f * mu / 3.0f + lam) * tr;
                    float tbK = 2.0f * mu * dn / sqrtf(2.0f);
                    float pC = pK / J;
                    float thr = (mat == 13) ? k.eta[0] : T.mu_s[mat];
                    if (tbK > thr * pK) {
                        float Ic = T.d[mat] * sqrtf(T.rho_s[mat] / pC);
                        float gdp = (mat == 13) ? mu_i_bisect<true>(tbK, mu, k.dt, pK, Ic, 0, 0, 0, k)
                                                : mu_i_root(tbK, mu, k.dt, pK, Ic, T.mu_s[mat], T.dmu[mat], T.I0[mat]);
                        float sc = (tbK - mu * k.dt * gdp) / fmaxf(tbK, 1e-20f);
                        sig[0] = expf(d0 * sc + mean); sig[1] = expf(d1 * sc + mean); sig[2] = expf(d2 * sc + mean);
                        udvt(U, sig[0], sig[1], sig[2], V, F);
                    }
                }
            } else {
                float Jr = k.Jp[p];
                if (Jr < 0.5f) Jr = 1.0f;
                float K = T.E[mat] / (3.0f * (1.0f - 2.0f * T.nu[mat]));
                float pc = fmaxf(K * (Jr / fmaxf(J, 1e-6f) - 1.0f), 0.0f);
                float jp_new = Jr;
                if (pc <= 0.0f) {
                    float si = expf(mean);
                    sig[0] = sig[1] = sig[2] = si;
                    udvt(U, si, si, si, V, F);
                } else {
                    float pK = pc * J;
                    float tbK = 2.0f * mu * dn / sqrtf(2.0f);
                    if (tbK > T.mu_s[mat] * pK) {
                        float Ic = T.d[mat] * sqrtf(T.rho_s[mat] / pc);
                        float gdp = mu_i_root(tbK, mu, k.dt, pK, Ic, T.mu_s[mat], T.dmu[mat], T.I0[mat]);
                        float Ir = gdp * Ic;
                        float dgam = fminf(8.0f * gdp * k.dt, 1.0f);
                        float jcs = 1.0f / fmaxf(1.0f - T.phi_chi[mat] * Ir / (Ir + T.I0[mat]), 1e-3f);
                        jp_new = Jr + dgam * (jcs - Jr);
                        float sc = (tbK - mu * k.dt * gdp) / fmaxf(tbK, 1e-20f);
                        sig[0] = expf(d0 * sc + mean); sig[1] = expf(d1 * sc + mean); sig[2] = expf(d2 * sc + mean);
                        udvt(U, sig[0], sig[1], sig[2], V, F);
                    }
                }
                k.Jp[p] = jp_new;
            }
        } else {  // jelly (0) and any unknown id: F = F_trial
#pragma unroll
            for (int i = 0; i < 9; ++i) F[i] = Ft[i];
        }
        // ---- stress of the returned F. Every return map above leaves (U, sig, V) a
        // singular value decomposition of the F it returns: F_trial's own when it
        // returns F_trial (bit for bit what a second svd3 gives), else U diag(sig) V^T
        // with the projected values, whose descending order the projections keep. So
        // only the maps without an SVD of their own (FCR jelly) factor F here.
        float J = det3(F);
        if (!(mat == 1 || mat == 5 || mat == 2 || mat == 9 || mat == 13 || mat == 11)) svd3(F, U, sig, V);
        if (mat == 0 || mat == 5) {  // FCR (mpm_utils.py:8-15)
            float R[9], FR[9];
            mmT(U, V, R);
#pragma unroll
            for (int i = 0; i < 9; ++i) FR[i] = 2.0f * mu * (F[i] - R[i]);
            mmT(FR, F, S);
            float dl = lam * J * (J - 1.0f);
            S[0] += dl; S[4] += dl; S[8] += dl;
        } else if (mat == 1 || mat == 9 || mat == 13) {
            stress_hencky(U, sig, mu, lam, S);
        } else if (mat == 2) {  // Drucker-Prager stress (mpm_utils.py:109-124)
            float l0 = logf(sig[0]), l1 = logf(sig[1]), l2 = logf(sig[2]);
            float ls = l0 + l1 + l2;
            float c0 = (2.0f * mu * l0 + lam * ls) / sig[0];
            float c1 = (2.0f * mu * l1 + lam * ls) / sig[1];
            float c2 = (2.0f * mu * l2 + lam * ls) / sig[2];
            float T1[9];
            udvt(U, c0, c1, c2, V, T1);
            mmT(T1, F, S);
        } else if (mat == 11) {  // mu(I)-Phi(I) stress (mpm_utils.py:525-540)
            float Jr = k.Jp[p];
            if (Jr < 0.5f) Jr = 1.0f;
            float K = T.E[mat] / (3.0f * (1.0f - 2.0f * T.nu[mat]));
            float pc = fmaxf(K * (Jr / fmaxf(J, 1e-6f) - 1.0f), 0.0f);
            float s0 = fmaxf(sig[0], 1e-6f), s1 = fmaxf(sig[1], 1e-6f), s2 = fmaxf(sig[2], 1e-6f);
            float e0 = logf(s0), e1 = logf(s1), e2 = logf(s2);
            float Jc = s0 * s1 * s2;
            float mean = (e0 + e1 + e2) / 3.0f;
            float iso = -pc * Jc;
            udvt(U, 2.0f * mu * (e0 - mean) + iso, 2.0f * mu * (e1 - mean) + iso, 2.0f * mu * (e2 - mean) + iso, U, S);
        } else {
#pragma unroll
            for (int i = 0; i < 9; ++i) S[i] = 0.0f;
        }
        // symmetrize (mpm_utils.py:1148)
        float s01 = 0.5f * (S[1] + S[3]), s02 = 0.5f * (S[2] + S[6]), s12 = 0.5f * (S[5] + S[7]);
        S[1] = S[3] = s01; S[2] = S[6] = s02; S[5] = S[7] = s12;
    }
}
