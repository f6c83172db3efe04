// Reverse-mode adjoint of the explicit MLS/APIC substep (split schedule:
// stress -> P2G -> grid update + colliders -> G2P) for the elastic (FCR, id 0), von
// Mises (id 1, optional hardening), water (id 6) and Newtonian / Bingham /
// Herschel-Bulkley (id 10) materials, with plane, cuboid, domain-wall, revolved-SDF
// cup and mesh-SDF colliders. The reference has no adjoint; the forward it differentiates is the one
// restated by the rest of this file (mpm_utils.py:819-1158, mpm_solver_warp.py:
// 1092-1281).
//
// One substep maps the particle state s = (x, v, C, F_trial, L, yield) to s' with
// per-particle parameters (mu, lam) and the per-type viscosity (L feeds the viscous
// stress of the next substep). Given the adjoint of s' the kernels below
// produce the adjoint of s and accumulate the adjoints of mu and lam:
//
//   forward recompute   k_adj_stress_fwd (F_trial -> F, Kirchhoff stress),
//                       k_adj_p2g_fwd (scatter {m v, m}), k_adj_grid_fwd (normalize,
//                       gravity, damping, colliders in list order)
//   G2P adjoint         k_adj_g2p_bwd: x' = x + dt v', v' = sum w v_i,
//                       C' = 4/dx^2 sum w v_i r_i^T, F_trial' = (I + dt L) F,
//                       L = sum v_i grad(w_i)^T  -> grid v adjoint (scatter), F adjoint,
//                       x adjoint through w, grad(w) (Hessian) and r_i = x_i - x_p
//   grid adjoint        k_adj_grid_bwd: colliders in reverse order, then
//                       v = mom/m + dt g  -> adjoints of mom and m per node
//   P2G adjoint         k_adj_p2g_bwd: mom_i = sum w m (v + C r_i) + dt A grad(w_i),
//                       A = -vol stress, m_i = sum w m  -> adjoints of v, C, x and the
//                       stress; then the stress law and the return map back to
//                       F_trial, yield, mu and lam.
//
// Every SVD-based map (the FCR rotation R = U V^T, the von Mises return
// F = U diag(exp(eps')) V^T and the Hencky stress written as G(F) F^T) is an
// isotropic matrix function G(F) = U diag(g(sigma)) V^T with g symmetric in sigma;
// iso_adjoint propagates through all of them with the closed-form rotation terms
// (g_i - g_j)/(s_i - s_j) and (g_i + g_j)/(s_i + s_j), using the coincident-value
// limit of the first when two singular values (nearly) coincide.

namespace gbmpm {

struct AdjK {
    // state at the start of the substep (caller layout: x[n][3], C[n][9] ...)
    const float *x, *v, *C, *Ft, *Lst, *ys, *Jp;
    const MatTables *tab;
    const float *mass, *vol, *mu, *lam;   // mu, lam: the state at the start of the substep
    const int *mat, *sel;
    const float *eta_tab;                 // viscosity / mu(I) table of the tabulated laws (ids 12, 13)
    int eta_n;
    float eta_smin, eta_smax;
    int n;
    // per-particle scratch: projected F, stress, adjoint of the projected F
    float *Fp, *S, *Fpb;
    // grid scratch (dense n^3): {mom, m}, {v}, {v adjoint}, {mom adjoint, m adjoint}
    float4 *gmv, *gv, *gvb, *gmb;
    int ng;
    float dx, inv_dx, dt;
    float grav[3];
    float damp;
    float hard1, xi1;   // von Mises hardening switch and xi (material table, id 1)
    // adjoints: in = end of the substep, out = start of the substep
    float *xb, *vb, *Cb, *Ftb, *Lb, *ysb, *Jpb;
    float *mub, *lamb, *pvb;   // accumulated over substeps (pvb: Newtonian viscosity)
    // colliders of this substep
    int ncol;
    const ColDev *cols;
    const PoseRec *poses;
    // kinematic cuboids: adjoint of each collider's force accumulator at this
    // substep ([ncol][3], or null) and the accumulated adjoint of each collider's
    // velocity ([ncol][3], or null)
    const float *col_force_b;
    float *col_vel_b;
    // node box of the segment ({lo x, y, z, hi x, y, z}, inclusive): every stencil of
    // the segment's particles lies inside it, so the grid kernels visit only it
    const int *box;
};

// the index-th node of the segment's box
__device__ __forceinline__ bool box_node(const int *box, size_t index, int ng, int &gx, int &gy, int &gz, size_t &id) {
    const int ex = box[3] - box[0] + 1, ey = box[4] - box[1] + 1, ez = box[5] - box[2] + 1;
    if (ex <= 0 || ey <= 0 || ez <= 0 || index >= (size_t)ex * ey * ez) return false;
    gz = box[2] + (int)(index % ez);
    gy = box[1] + (int)((index / ez) % ey);
    gx = box[0] + (int)(index / ((size_t)ez * ey));
    id = ((size_t)gx * ng + gy) * ng + gz;
    return true;
}
__device__ __forceinline__ size_t box_count(const int *box) {
    const int ex = box[3] - box[0] + 1, ey = box[4] - box[1] + 1, ez = box[5] - box[2] + 1;
    return (ex <= 0 || ey <= 0 || ez <= 0) ? 0 : (size_t)ex * ey * ez;
}

// c = a^T b
__device__ __forceinline__ void mTm(const float *a, const float *b, float *c) {
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) c[3 * i + j] = a[i] * b[j] + a[3 + i] * b[3 + j] + a[6 + i] * b[6 + j];
}

// Adjoint of G(F) = U diag(g) V^T at F = U diag(s) V^T, g symmetric in s with
// Jacobian Jg[i][j] = dg_i/ds_j: adds to Fb the pull-back of Gb and returns the
// diagonal of U^T Gb V (the adjoint of g) in yd.
__device__ void iso_adjoint(const float *U, const float *s, const float *V, const float *g, const float (&Jg)[3][3],
                            const float *Gb, float *Fb, float *yd) {
    float T[9], Y[9], M[9];
    mTm(U, Gb, T);
    mm(T, V, Y);
#pragma unroll
    for (int i = 0; i < 3; ++i) yd[i] = Y[4 * i];
#pragma unroll
    for (int j = 0; j < 3; ++j) M[4 * j] = Jg[0][j] * Y[0] + Jg[1][j] * Y[4] + Jg[2][j] * Y[8];
    const int P[3][2] = {{0, 1}, {0, 2}, {1, 2}};
#pragma unroll
    for (int q = 0; q < 3; ++q) {
        const int i = P[q][0], j = P[q][1];
        const float d = s[i] - s[j], su = s[i] + s[j];
        const float sc = fmaxf(fabsf(s[i]), fabsf(s[j]));
        const float a = (fabsf(d) > 1e-3f * sc) ? (g[i] - g[j]) / d
                                                : 0.5f * (Jg[i][i] - Jg[i][j] + Jg[j][j] - Jg[j][i]);
        const float b = (fabsf(su) > 1e-6f) ? (g[i] + g[j]) / su : 0.0f;
        const float ap = 0.5f * (a + b), am = 0.5f * (a - b);
        const float yij = Y[3 * i + j], yji = Y[3 * j + i];
        M[3 * i + j] = ap * yij + am * yji;
        M[3 * j + i] = ap * yji + am * yij;
    }
    float W[9], R[9];
    mm(U, M, W);
    mmT(W, V, R);
#pragma unroll
    for (int i = 0; i < 9; ++i) Fb[i] += R[i];
}

// cofactor matrix: d det(F) / dF
__device__ __forceinline__ void cofactor(const float *F, float *c) {
    c[0] = F[4] * F[8] - F[5] * F[7];
    c[1] = F[5] * F[6] - F[3] * F[8];
    c[2] = F[3] * F[7] - F[4] * F[6];
    c[3] = F[2] * F[7] - F[1] * F[8];
    c[4] = F[0] * F[8] - F[2] * F[6];
    c[5] = F[1] * F[6] - F[0] * F[7];
    c[6] = F[1] * F[5] - F[2] * F[4];
    c[7] = F[2] * F[3] - F[0] * F[5];
    c[8] = F[0] * F[4] - F[1] * F[3];
}

// von Mises return map of one particle (mpm_utils.py:127-170) as the engine's
// stress pass computes it; returns true on the plastic branch.
__device__ bool vm_return(const float *Ft, float mu, float lam, float ys, float *U, float *sg, float *V, float *eps,
                          float *Fp) {
    svd3(Ft, U, sg, V);
    eps[0] = logf(fmaxf(sg[0], 0.01f));
    eps[1] = logf(fmaxf(sg[1], 0.01f));
    eps[2] = logf(fmaxf(sg[2], 0.01f));
    const float tr = eps[0] + eps[1] + eps[2];
    const float temp = tr / 3.0f;
    const float t0 = 2.0f * mu * eps[0] + lam * tr, t1 = 2.0f * mu * eps[1] + lam * tr, t2 = 2.0f * mu * eps[2] + lam * tr;
    const float st = (t0 + t1 + t2) / 3.0f;
    const float c0 = t0 - st, c1 = t1 - st, c2 = t2 - st;
    if (!(sqrtf(c0 * c0 + c1 * c1 + c2 * c2) > ys)) {
#pragma unroll
        for (int i = 0; i < 9; ++i) Fp[i] = Ft[i];
        return false;
    }
    const float h0 = eps[0] - temp, h1 = eps[1] - temp, h2 = eps[2] - temp;
    const float hn = sqrtf(h0 * h0 + h1 * h1 + h2 * h2) + 1e-6f;
    const float r = (hn - ys / (2.0f * mu)) / hn;
    udvt(U, expf(eps[0] - r * h0), expf(eps[1] - r * h1), expf(eps[2] - r * h2), V, Fp);
    return true;
}

// slope of table_lerp in its argument (0 where the lookup is clamped)
__device__ __forceinline__ float table_slope(const float *tab, int n, float smin, float smax, float s) {
    const float idx = (s - smin) / (smax - smin) * (float)(n - 1);
    if (!(idx > 0.0f && idx < (float)(n - 1) - 1.0e-6f)) return 0.0f;
    const int i0 = (int)floorf(idx);
    return (tab[i0 + 1] - tab[i0]) * (float)(n - 1) / (smax - smin);
}

// Drucker-Prager return map (mpm_utils.py:543-580) as the engine's stress pass
// computes it: 0 elastic (F = F_trial), 1 apex (F = U V^T), 2 onto the cone.
__device__ int dp_return(const float *Ft, float mu, float lam, float alpha, float *U, float *sg, float *V, float *e,
                         float *h, float &hn, float *Fp) {
    svd3(Ft, U, sg, V);
#pragma unroll
    for (int i = 0; i < 3; ++i) e[i] = logf(fmaxf(fabsf(sg[i]), 1e-14f));
    const float tr = e[0] + e[1] + e[2];
#pragma unroll
    for (int i = 0; i < 3; ++i) h[i] = e[i] - tr / 3.0f;
    hn = sqrtf(h[0] * h[0] + h[1] * h[1] + h[2] * h[2]);
    const float dg = hn + (3.0f * lam + 2.0f * mu) / (2.0f * mu) * tr * alpha;
    if (dg <= 0.0f) {
#pragma unroll
        for (int i = 0; i < 9; ++i) Fp[i] = Ft[i];
        return 0;
    }
    if (tr > 0.0f) {
        udvt(U, 1.0f, 1.0f, 1.0f, V, Fp);
        return 1;
    }
    const float r = dg / hn;
    udvt(U, expf(e[0] - h[0] * r), expf(e[1] - h[1] * r), expf(e[2] - h[2] * r), V, Fp);
    return 2;
}

// mu(I) return map (ids 9 and 13; mpm_utils.py:246-522) as the engine's stress pass
// computes it: 0 below the yield surface (F = F_trial), 1 tension (F = U V^T), 2
// flow with the rate gdp from the bisection. MuI keeps what the adjoint needs.
struct MuI {
    float s[3], e[3], d[3], dn, tr, mean, J, pK, tbK, pC, Ic, gdp, sc;
};
__device__ int mui_return(const AdjK &a, int mat, const float *Ft, float mu, float lam, float *U, float *sg, float *V,
                          MuI &m, float *Fp) {
    const MatTables &T = *a.tab;
    svd3(Ft, U, sg, V);
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        m.s[i] = fmaxf(fabsf(sg[i]), 1e-6f);
        m.e[i] = logf(m.s[i]);
    }
    m.tr = m.e[0] + m.e[1] + m.e[2];
    m.mean = m.tr / 3.0f;
#pragma unroll
    for (int i = 0; i < 3; ++i) m.d[i] = m.e[i] - m.mean;
    m.dn = sqrtf(m.d[0] * m.d[0] + m.d[1] * m.d[1] + m.d[2] * m.d[2]);
    m.J = m.s[0] * m.s[1] * m.s[2];
#pragma unroll
    for (int i = 0; i < 9; ++i) Fp[i] = Ft[i];
    if (m.tr >= 0.0f) {
        udvt(U, 1.0f, 1.0f, 1.0f, V, Fp);
        return 1;
    }
    m.pK = -(2.0f * mu / 3.0f + lam) * m.tr;
    m.tbK = 2.0f * mu * m.dn / sqrtf(2.0f);
    m.pC = m.pK / m.J;
    const float thr = (mat == 13) ? a.eta_tab[0] : T.mu_s[mat];
    if (!(m.tbK > thr * m.pK)) return 0;
    m.Ic = T.d[mat] * sqrtf(T.rho_s[mat] / m.pC);
    m.gdp = (mat == 13) ? mu_i_bisect<true>(m.tbK, mu, a.dt, m.pK, m.Ic, 0.0f, 0.0f, 0.0f, a.eta_tab, a.eta_n,
                                            a.eta_smin, a.eta_smax)
                        : mu_i_root(m.tbK, mu, a.dt, m.pK, m.Ic, T.mu_s[mat], T.dmu[mat], T.I0[mat]);
    m.sc = (m.tbK - mu * a.dt * m.gdp) / fmaxf(m.tbK, 1e-20f);
    udvt(U, expf(m.d[0] * m.sc + m.mean), expf(m.d[1] * m.sc + m.mean), expf(m.d[2] * m.sc + m.mean), V, Fp);
    return 2;
}

// Reverse of the mu(I) flow branch: from gb (adjoint of the returned singular
// values g) to sb (adjoint of the trial singular values) and the mu, lam adjoints.
// The rate gdp is the root of f = tbK - mu dt gdp - mu_I(gdp Ic) pK, so its
// sensitivities follow from the implicit function theorem: d gdp = -df / f_gdp.
__device__ void mui_reverse(const AdjK &a, int mat, const MuI &m, const float *sg, float mu, float lam, const float *gb,
                            float *sb, float &mub, float &lamb) {
    const MatTables &T = *a.tab;
    float epb[3], db[3];
    float scb = 0.0f, meanb = 0.0f;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        epb[i] = gb[i] * expf(m.d[i] * m.sc + m.mean);
        db[i] = epb[i] * m.sc;
        scb += epb[i] * m.d[i];
        meanb += epb[i];
    }
    // sc = (tbK - mu dt gdp) / tbK (tbK > 0 on this branch)
    float tbKb = scb * mu * a.dt * m.gdp / (m.tbK * m.tbK);
    const float gdpb = -scb * mu * a.dt / m.tbK;
    mub += -scb * a.dt * m.gdp / m.tbK;
    const float I = m.gdp * m.Ic;
    float muI, dmuI;
    if (mat == 13) {
        muI = mu_of_i<true>(I, 0.0f, 0.0f, 0.0f, a.eta_tab, a.eta_n, a.eta_smin, a.eta_smax);
        dmuI = (I > 1e-12f) ? table_slope(a.eta_tab, a.eta_n, a.eta_smin, a.eta_smax,
                                           logf(I) * 0.43429448190325176f) * 0.43429448190325176f / I
                            : 0.0f;
    } else {
        muI = mu_of_i<false>(I, T.mu_s[mat], T.dmu[mat], T.I0[mat], nullptr, 0, 0.0f, 0.0f);
        dmuI = T.dmu[mat] * T.I0[mat] / ((I + T.I0[mat]) * (I + T.I0[mat]));
    }
    const float fg = -mu * a.dt - dmuI * m.Ic * m.pK;
    const float kf = (fg != 0.0f) ? -gdpb / fg : 0.0f;
    tbKb += kf;
    mub += kf * (-a.dt * m.gdp);
    float pKb = kf * (-muI);
    const float Icb = kf * (-dmuI * m.gdp * m.pK);
    // Ic = d sqrt(rho_s / pC), pC = pK / J
    const float pCb = Icb * (-0.5f * m.Ic / m.pC);
    pKb += pCb / m.J;
    const float Jb = -pCb * m.pK / (m.J * m.J);
    // pK = -(2 mu / 3 + lam) tr, tbK = 2 mu dn / sqrt 2
    mub += pKb * (-2.0f * m.tr / 3.0f) + tbKb * 2.0f * m.dn / sqrtf(2.0f);
    lamb += pKb * (-m.tr);
    const float trb = pKb * (-(2.0f * mu / 3.0f + lam)) + meanb / 3.0f;
    const float dnb = tbKb * 2.0f * mu / sqrtf(2.0f);
    if (m.dn > 0.0f) {
#pragma unroll
        for (int i = 0; i < 3; ++i) db[i] += dnb * m.d[i] / m.dn;
    }
    const float dsum = (db[0] + db[1] + db[2]) / 3.0f;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        const float eb = db[i] - dsum + trb;
        const float s_b = eb / m.s[i] + Jb * m.J / m.s[i];
        sb[i] = (fabsf(sg[i]) > 1e-6f) ? (sg[i] > 0.0f ? s_b : -s_b) : 0.0f;
    }
}

// mu(I)-Phi(I) return map (id 11; mpm_utils.py:375-522) as the engine's stress pass
// computes it, with the packing state Jp: 0 no compaction pressure (F = U e^mean V^T),
// 1 below the yield surface (F = F_trial), 2 flow (rate gdp from the bisection, Jp
// relaxing toward the critical-state value). MuIPhi keeps what the adjoint needs.
struct MuIPhi {
    float s[3], e[3], d[3], dn, mean, J, Jr, K, pc, pK, tbK, Ic, gdp, Ir, dgam, jcs, q, sc;
    bool jr_clamped;
};
__device__ int muiphi_return(const AdjK &a, const float *Ft, float mu, float jp, float *U, float *sg, float *V,
                             MuIPhi &m, float *Fp, float &jp_new) {
    const MatTables &T = *a.tab;
    const int mat = 11;
    svd3(Ft, U, sg, V);
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        m.s[i] = fmaxf(fabsf(sg[i]), 1e-6f);
        m.e[i] = logf(m.s[i]);
    }
    m.mean = (m.e[0] + m.e[1] + m.e[2]) / 3.0f;
#pragma unroll
    for (int i = 0; i < 3; ++i) m.d[i] = m.e[i] - m.mean;
    m.dn = sqrtf(m.d[0] * m.d[0] + m.d[1] * m.d[1] + m.d[2] * m.d[2]);
    m.J = m.s[0] * m.s[1] * m.s[2];
    m.jr_clamped = jp < 0.5f;
    m.Jr = m.jr_clamped ? 1.0f : jp;
    m.K = T.E[mat] / (3.0f * (1.0f - 2.0f * T.nu[mat]));
    m.pc = fmaxf(m.K * (m.Jr / fmaxf(m.J, 1e-6f) - 1.0f), 0.0f);
    jp_new = m.Jr;
#pragma unroll
    for (int i = 0; i < 9; ++i) Fp[i] = Ft[i];
    if (m.pc <= 0.0f) {
        const float si = expf(m.mean);
        udvt(U, si, si, si, V, Fp);
        return 0;
    }
    m.pK = m.pc * m.J;
    m.tbK = 2.0f * mu * m.dn / sqrtf(2.0f);
    if (!(m.tbK > T.mu_s[mat] * m.pK)) return 1;
    m.Ic = T.d[mat] * sqrtf(T.rho_s[mat] / m.pc);
    m.gdp = mu_i_root(m.tbK, mu, a.dt, m.pK, m.Ic, T.mu_s[mat], T.dmu[mat], T.I0[mat]);
    m.Ir = m.gdp * m.Ic;
    m.dgam = fminf(8.0f * m.gdp * a.dt, 1.0f);
    m.q = 1.0f - T.phi_chi[mat] * m.Ir / (m.Ir + T.I0[mat]);
    m.jcs = 1.0f / fmaxf(m.q, 1e-3f);
    jp_new = m.Jr + m.dgam * (m.jcs - m.Jr);
    m.sc = (m.tbK - mu * a.dt * m.gdp) / fmaxf(m.tbK, 1e-20f);
    udvt(U, expf(m.d[0] * m.sc + m.mean), expf(m.d[1] * m.sc + m.mean), expf(m.d[2] * m.sc + m.mean), V, Fp);
    return 2;
}

// Reverse of the mu(I)-Phi(I) flow branch: from gb (adjoint of the returned singular
// values) and jpb (adjoint of the new Jp) to sb (adjoint of the trial singular
// values), mu and the clamped old Jp (jrb). gdp is the root of
// f = tbK - mu dt gdp - mu_I(gdp Ic) pK, differentiated implicitly.
__device__ void muiphi_reverse(const AdjK &a, const MuIPhi &m, const float *sg, float mu, const float *gb, float jpb,
                               float *sb, float &mub, float &jrb) {
    const MatTables &T = *a.tab;
    const int mat = 11;
    float db[3], scb = 0.0f, meanb = 0.0f;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        const float epb = gb[i] * expf(m.d[i] * m.sc + m.mean);
        db[i] = epb * m.sc;
        scb += epb * m.d[i];
        meanb += epb;
    }
    float tbKb = scb * mu * a.dt * m.gdp / (m.tbK * m.tbK);
    float gdpb = -scb * mu * a.dt / m.tbK;
    mub += -scb * a.dt * m.gdp / m.tbK;
    // Jp' = Jr + dgam (jcs - Jr), dgam = min(8 gdp dt, 1), jcs = 1 / max(q, 1e-3)
    jrb += jpb * (1.0f - m.dgam);
    const float dgamb = jpb * (m.jcs - m.Jr), jcsb = jpb * m.dgam;
    if (8.0f * m.gdp * a.dt < 1.0f) gdpb += dgamb * 8.0f * a.dt;
    float Irb = 0.0f;
    if (m.q > 1e-3f) {
        const float qb = -jcsb / (m.q * m.q);
        Irb = qb * (-T.phi_chi[mat] * T.I0[mat] / ((m.Ir + T.I0[mat]) * (m.Ir + T.I0[mat])));
    }
    gdpb += Irb * m.Ic;
    float Icb = Irb * m.gdp;
    const float muI = mu_of_i<false>(m.Ir, T.mu_s[mat], T.dmu[mat], T.I0[mat], nullptr, 0, 0.0f, 0.0f);
    const float dmuI = T.dmu[mat] * T.I0[mat] / ((m.Ir + T.I0[mat]) * (m.Ir + T.I0[mat]));
    const float fg = -mu * a.dt - dmuI * m.Ic * m.pK;
    const float kf = (fg != 0.0f) ? -gdpb / fg : 0.0f;
    tbKb += kf;
    mub += kf * (-a.dt * m.gdp);
    const float pKb = kf * (-muI);
    Icb += kf * (-dmuI * m.gdp * m.pK);
    // Ic = d sqrt(rho_s / pc), pK = pc J, pc = K (Jr / J - 1)
    float pcb = Icb * (-0.5f * m.Ic / m.pc) + pKb * m.J;
    float Jb = pKb * m.pc;
    jrb += pcb * m.K / m.J;
    Jb += pcb * (-m.K * m.Jr / (m.J * m.J));
    // tbK = 2 mu dn / sqrt 2
    mub += tbKb * 2.0f * m.dn / sqrtf(2.0f);
    const float dnb = tbKb * 2.0f * mu / sqrtf(2.0f);
    if (m.dn > 0.0f) {
#pragma unroll
        for (int i = 0; i < 3; ++i) db[i] += dnb * m.d[i] / m.dn;
    }
    const float dsum = (db[0] + db[1] + db[2]) / 3.0f;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        const float eb = db[i] - dsum + meanb / 3.0f;
        const float s_b = eb / m.s[i] + Jb * m.J / m.s[i];
        sb[i] = (fabsf(sg[i]) > 1e-6f) ? (sg[i] > 0.0f ? s_b : -s_b) : 0.0f;
    }
}

// The return map of a solid particle and the (mu, lam) its stress then uses: von
// Mises with softening (id 5) zeroes both once the yield stress is used up. Returns
// the yield stress after the substep in *ys_out.
__device__ void solid_return(const AdjK &a, int mat, const float *Ft, float mu, float lam, float ys, float jp,
                             float *Fp, float &mus, float &lams, float &ys_out, float &jp_out) {
    const MatTables &T = *a.tab;
    float U[9], V[9], sg[3], e[3];
    mus = mu;
    lams = lam;
    ys_out = ys;
    jp_out = jp;
    if (mat == 11) {
        MuIPhi m;
        muiphi_return(a, Ft, mu, jp, U, sg, V, m, Fp, jp_out);
        return;
    }
    if (mat == 1 || mat == 5) {
        if (mat == 5 && ys <= 0.0f) {
#pragma unroll
            for (int i = 0; i < 9; ++i) Fp[i] = Ft[i];
            return;
        }
        if (!vm_return(Ft, mu, lam, ys, U, sg, V, e, Fp)) return;
        const float mean = (e[0] + e[1] + e[2]) / 3.0f;
        const float h0 = e[0] - mean, h1 = e[1] - mean, h2 = e[2] - mean;
        const float hn = sqrtf(h0 * h0 + h1 * h1 + h2 * h2) + 1e-6f;
        const float dg = hn - ys / (2.0f * mu);
        float y = ys;
        if (mat == 5) {
            const float r = dg / hn;
            const float rh0 = r * h0, rh1 = r * h1, rh2 = r * h2;
            y = y - T.softening[mat] * sqrtf(rh0 * rh0 + rh1 * rh1 + rh2 * rh2);
            if (y <= 0.0f) { mus = 0.0f; lams = 0.0f; }
        }
        if (T.hardening[mat] > 0.5f) y = y + 2.0f * mus * T.xi[mat] * dg;
        ys_out = y;
    } else if (mat == 2) {
        float h[3], hn;
        dp_return(Ft, mu, lam, T.alpha[mat], U, sg, V, e, h, hn, Fp);
    } else if (mat == 9 || mat == 13) {
        MuI m;
        mui_return(a, mat, Ft, mu, lam, U, sg, V, m, Fp);
    } else {
#pragma unroll
        for (int i = 0; i < 9; ++i) Fp[i] = Ft[i];
    }
}

// mu(I)-Phi(I) stress (mpm_utils.py:525-540): U diag(2 mu (e - mean) - pc Jc) U^T,
// e = log max(sigma, 1e-6), pc = max(K (Jr / J - 1), 0) with the new Jp, symmetrized
__device__ void muiphi_stress(const AdjK &a, const float *F, float mu, float jp, float *S) {
    const MatTables &T = *a.tab;
    float U[9], V[9], sg[3], Tm[9];
    const float J = det3(F);
    svd3(F, U, sg, V);
    const float Jr = (jp < 0.5f) ? 1.0f : jp;
    const float K = T.E[11] / (3.0f * (1.0f - 2.0f * T.nu[11]));
    const float pc = fmaxf(K * (Jr / fmaxf(J, 1e-6f) - 1.0f), 0.0f);
    const float s0 = fmaxf(sg[0], 1e-6f), s1 = fmaxf(sg[1], 1e-6f), s2 = fmaxf(sg[2], 1e-6f);
    const float e0 = logf(s0), e1 = logf(s1), e2 = logf(s2);
    const float Jc = s0 * s1 * s2;
    const float mean = (e0 + e1 + e2) / 3.0f;
    const float iso = -pc * Jc;
    udvt(U, 2.0f * mu * (e0 - mean) + iso, 2.0f * mu * (e1 - mean) + iso, 2.0f * mu * (e2 - mean) + iso, U, Tm);
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) S[3 * i + j] = 0.5f * (Tm[3 * i + j] + Tm[3 * j + i]);
}

// Kirchhoff stress of the projected F (FCR for ids 0 and 5, Hencky otherwise), symmetrized
__device__ void adj_stress(int mat, const float *F, float mu, float lam, float *S) {
    float U[9], V[9], sg[3], T[9];
    svd3(F, U, sg, V);
    if (mat == 0 || mat == 5) {
        float R[9], FR[9];
        mmT(U, V, R);
#pragma unroll
        for (int i = 0; i < 9; ++i) FR[i] = 2.0f * mu * (F[i] - R[i]);
        mmT(FR, F, T);
        const float J = det3(F);
        const float dl = lam * J * (J - 1.0f);
        T[0] += dl; T[4] += dl; T[8] += dl;
    } else {
        stress_hencky(U, sg, mu, lam, T);
    }
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) S[3 * i + j] = 0.5f * (T[3 * i + j] + T[3 * j + i]);
}

// Fluid stress (water id 6; Newtonian / Bingham / Herschel-Bulkley id 10) as the
// engine's stress pass computes it: F reset to J^(1/3) I, tau = J (p I + 2 eta dev D).
struct FluidTerms {
    float Jt, Jc, J, pr, gd, eta, Dd[9];
};
__device__ void fluid_stress(const AdjK &k, int p, int mat, const float *Ft, const float *L, FluidTerms &f, float *Fp,
                             float *S) {
    const MatTables &T = *k.tab;
    f.Jt = det3(Ft);
    f.Jc = pow_near1(f.Jt, 1.0f / 3.0f);
    f.J = f.Jc * f.Jc * f.Jc;
#pragma unroll
    for (int i = 0; i < 9; ++i) Fp[i] = (i % 4 == 0) ? f.Jc : 0.0f;
    f.pr = eos_pressure(f.J, T.bulk[mat]);
    if (mat == 6) {
        f.gd = 1.0f; f.eta = 0.0f;
#pragma unroll
        for (int i = 0; i < 9; ++i) { f.Dd[i] = 0.0f; S[i] = (i % 4 == 0) ? f.J * f.pr : 0.0f; }
        return;
    }
    dev_rate(L, f.Dd, f.gd);
    if (mat == 12) {
        f.eta = table_lerp(k.eta_tab, k.eta_n, k.eta_smin, k.eta_smax, logf(f.gd) * 0.43429448190325176f);
    } else {
        const float ys = k.ys[p], Kp = T.hardening[mat];
        f.eta = T.pv[mat] + (ys != 0.0f ? ys / f.gd : 0.0f) +
                (Kp != 0.0f ? Kp * powf(f.gd, T.softening[mat] - 1.0f) : 0.0f);
    }
    const float two_eta = 2.0f * f.eta;
#pragma unroll
    for (int i = 0; i < 9; ++i) S[i] = f.J * (((i % 4 == 0) ? f.pr : 0.0f) + two_eta * f.Dd[i]);
}

// The per-particle adjoint kernels run 128-thread CTAs with register caps that let
// 4 to 6 CTAs share an SM: scenes of a batch reverse side by side, and the batched
// identification workload's reverse pass measured 1.015 -> 0.946 s (uncapped, the
// reverse scatter took 150 registers and three CTAs an SM).
__global__ void __launch_bounds__(128, 6) k_adj_stress_fwd(AdjK k) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= k.n || (k.sel && k.sel[p] != 0)) return;
    float Ft[9], Fp[9], S[9];
#pragma unroll
    for (int i = 0; i < 9; ++i) Ft[i] = k.Ft[9 * (size_t)p + i];
    const int mat = k.mat[p];
    const float mu = k.mu[p], lam = k.lam[p];
    if (mat == 6 || mat == 10 || mat == 12) {
        float L[9];
#pragma unroll
        for (int i = 0; i < 9; ++i) L[i] = k.Lst[9 * (size_t)p + i];
        FluidTerms f;
        fluid_stress(k, p, mat, Ft, L, f, Fp, S);
#pragma unroll
        for (int i = 0; i < 9; ++i) { k.Fp[9 * (size_t)p + i] = Fp[i]; k.S[9 * (size_t)p + i] = S[i]; }
        return;
    }
    float mus, lams, ys_out, jp_out;
    solid_return(k, mat, Ft, mu, lam, k.ys[p], k.Jp[p], Fp, mus, lams, ys_out, jp_out);
    if (mat == 11) muiphi_stress(k, Fp, mus, jp_out, S);
    else adj_stress(mat, Fp, mus, lams, S);
#pragma unroll
    for (int i = 0; i < 9; ++i) { k.Fp[9 * (size_t)p + i] = Fp[i]; k.S[9 * (size_t)p + i] = S[i]; }
}

// grad(w) and the Hessian of w with respect to x_p for node (i, j, kk)
__device__ __forceinline__ void weight_derivs(const Stencil &s, float inv_dx, int i, int j, int kk, float &w, float *g,
                                              float *H) {
    const float dd[3] = {1.0f, -2.0f, 1.0f};
    const float w0 = s.w[0][i], w1 = s.w[1][j], w2 = s.w[2][kk];
    const float d0 = s.dw[0][i], d1 = s.dw[1][j], d2 = s.dw[2][kk];
    w = w0 * w1 * w2;
    g[0] = d0 * w1 * w2 * inv_dx;
    g[1] = w0 * d1 * w2 * inv_dx;
    g[2] = w0 * w1 * d2 * inv_dx;
    const float i2 = inv_dx * inv_dx;
    H[0] = dd[i] * w1 * w2 * i2;
    H[4] = w0 * dd[j] * w2 * i2;
    H[8] = w0 * w1 * dd[kk] * i2;
    H[1] = H[3] = d0 * d1 * w2 * i2;
    H[2] = H[6] = d0 * w1 * d2 * i2;
    H[5] = H[7] = w0 * d1 * d2 * i2;
}

__global__ void __launch_bounds__(128, 6) k_adj_p2g_fwd(AdjK a, PK k) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= a.n || (a.sel && a.sel[p] != 0)) return;
    float x[3] = {a.x[3 * p], a.x[3 * p + 1], a.x[3 * p + 2]};
    float v[3] = {a.v[3 * p], a.v[3 * p + 1], a.v[3 * p + 2]};
    float C[9], S[9];
#pragma unroll
    for (int i = 0; i < 9; ++i) { C[i] = a.C[9 * (size_t)p + i]; S[i] = a.S[9 * (size_t)p + i]; }
    Stencil s;
    stencil(x, a.inv_dx, s);
    if (!stencil_ok(s, a.ng, 0)) { set_status(k.status, GBMPM_FLAG_STENCIL_OOB); return; }
    p2g_core(k, s, p, v, C, S, [&](int i, int j, int kk, float4 val) {
        atomicAdd(a.gmv + ((size_t)(s.b[0] + i) * a.ng + (s.b[1] + j)) * a.ng + (s.b[2] + kk), val);
    });
}

__device__ __forceinline__ GK adj_gk(const AdjK &a) {
    GK g{};
    g.ng = a.ng;
    g.dx = a.dx;
    g.dt = a.dt;
    for (int i = 0; i < 3; ++i) g.g[i] = a.grav[i];
    g.damp = a.damp;
    return g;
}

// normalized, damped velocity before the colliders; m <= 1e-15 leaves zero
__device__ __forceinline__ void grid_pre(const AdjK &a, float4 mv, float *v) {
    v[0] = v[1] = v[2] = 0.0f;
    if (mv.w > 1e-15f) {
        const float inv = 1.0f / mv.w;
        v[0] = mv.x * inv + a.dt * a.grav[0];
        v[1] = mv.y * inv + a.dt * a.grav[1];
        v[2] = mv.z * inv + a.dt * a.grav[2];
    }
    if (a.damp < 1.0f) { v[0] *= a.damp; v[1] *= a.damp; v[2] *= a.damp; }
}

// The segment's node box: every particle stencil of every saved substep state
// (base cell to base + 2 per axis), as an inclusive node range clamped to the grid.
__global__ void k_adj_box_init(int *box, int ng) {
    if (threadIdx.x == 0) { box[0] = box[1] = box[2] = ng; box[3] = box[4] = box[5] = -1; }
}
__global__ void k_adj_box(const float *states, size_t per, int n, int substeps, float inv_dx, int ng, int *box) {
    int lo[3] = {ng, ng, ng}, hi[3] = {-1, -1, -1};
    const size_t total = (size_t)n * substeps;
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < total; t += (size_t)gridDim.x * blockDim.x) {
        const size_t i = t / n, p = t % n;
        const float *x = states + per * i + 3 * p;
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            const int b = (int)floorf(x[d] * inv_dx - 0.5f);
            lo[d] = min(lo[d], max(b, 0));
            hi[d] = max(hi[d], min(b + 2, ng - 1));
        }
    }
#pragma unroll
    for (int d = 0; d < 3; ++d) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            lo[d] = min(lo[d], __shfl_xor_sync(0xffffffffu, lo[d], o));
            hi[d] = max(hi[d], __shfl_xor_sync(0xffffffffu, hi[d], o));
        }
    }
    if ((threadIdx.x & 31) == 0) {
#pragma unroll
        for (int d = 0; d < 3; ++d) { atomicMin(box + d, lo[d]); atomicMax(box + 3 + d, hi[d]); }
    }
}
// zero the accumulated grids (momentum and mass, the velocity adjoint) inside the box
__global__ void k_adj_zero_box(AdjK a) {
    const size_t N = box_count(a.box);
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < N; t += (size_t)gridDim.x * blockDim.x) {
        int gx, gy, gz;
        size_t id;
        if (!box_node(a.box, t, a.ng, gx, gy, gz, id)) break;
        a.gmv[id] = make_float4(0.f, 0.f, 0.f, 0.f);
        a.gvb[id] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
}

__global__ void k_adj_grid_fwd(AdjK a) {
    const size_t N = box_count(a.box);
    const GK gk = adj_gk(a);
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < N; t += (size_t)gridDim.x * blockDim.x) {
        int gx, gy, gz;
        size_t id;
        if (!box_node(a.box, t, a.ng, gx, gy, gz, id)) break;
        const float4 mv = a.gmv[id];
        if (mv.w == 0.0f) { a.gv[id] = make_float4(0.f, 0.f, 0.f, 0.f); continue; }
        float v[3], acc[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
        grid_pre(a, mv, v);
        for (int c = 0; c < a.ncol; ++c)
            if (mv.w > 0.0f && a.poses[c].mode != 0) collide(a.cols[c], a.poses[c], gx, gy, gz, mv.w, v, gk, acc);
        a.gv[id] = make_float4(v[0], v[1], v[2], 0.0f);
    }
}

__global__ void __launch_bounds__(128, 5) k_adj_g2p_bwd(AdjK a) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= a.n || (a.sel && a.sel[p] != 0)) return;
    const float x[3] = {a.x[3 * p], a.x[3 * p + 1], a.x[3 * p + 2]};
    float Fp[9], Ftb[9], Cb[9];
#pragma unroll
    for (int i = 0; i < 9; ++i) {
        Fp[i] = a.Fp[9 * (size_t)p + i];
        Ftb[i] = a.Ftb[9 * (size_t)p + i];
        Cb[i] = a.Cb[9 * (size_t)p + i];
    }
    float xb[3], vt[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        xb[d] = a.xb[3 * p + d];
        vt[d] = a.vb[3 * p + d] + a.dt * xb[d];   // adjoint of v' (x' = x + dt v')
    }
    float Lb[9];   // adjoint of L: the state's L' (viscous stress next substep) and F_trial' = (I + dt L) F
    mmT(Ftb, Fp, Lb);
#pragma unroll
    for (int i = 0; i < 9; ++i) Lb[i] = Lb[i] * a.dt + a.Lb[9 * (size_t)p + i];
    Stencil s;
    stencil(x, a.inv_dx, s);
    if (!stencil_ok(s, a.ng, 0)) return;
    const float c4 = 4.0f * a.inv_dx * a.inv_dx;
    float L[9] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
            for (int kk = 0; kk < 3; ++kk) {
                const size_t id = ((size_t)(s.b[0] + i) * a.ng + (s.b[1] + j)) * a.ng + (s.b[2] + kk);
                const float4 g4 = a.gv[id];
                const float vi[3] = {g4.x, g4.y, g4.z};
                float w, g[3], H[9];
                weight_derivs(s, a.inv_dx, i, j, kk, w, g, H);
                const float r[3] = {((float)i - s.fx[0]) * a.dx, ((float)j - s.fx[1]) * a.dx, ((float)kk - s.fx[2]) * a.dx};
#pragma unroll
                for (int u = 0; u < 3; ++u)
#pragma unroll
                    for (int q = 0; q < 3; ++q) L[3 * u + q] += vi[u] * g[q];
                float vib[3], Cbr[3], CbTv[3], LbTv[3];
#pragma unroll
                for (int u = 0; u < 3; ++u) {
                    Cbr[u] = Cb[3 * u] * r[0] + Cb[3 * u + 1] * r[1] + Cb[3 * u + 2] * r[2];
                    CbTv[u] = Cb[u] * vi[0] + Cb[3 + u] * vi[1] + Cb[6 + u] * vi[2];
                    LbTv[u] = Lb[u] * vi[0] + Lb[3 + u] * vi[1] + Lb[6 + u] * vi[2];
                    vib[u] = w * vt[u] + c4 * w * Cbr[u] + (Lb[3 * u] * g[0] + Lb[3 * u + 1] * g[1] + Lb[3 * u + 2] * g[2]);
                }
                atomicAdd(a.gvb + id, make_float4(vib[0], vib[1], vib[2], 0.0f));
                const float vv = vt[0] * vi[0] + vt[1] * vi[1] + vt[2] * vi[2];
                const float vCr = vi[0] * Cbr[0] + vi[1] * Cbr[1] + vi[2] * Cbr[2];
#pragma unroll
                for (int d = 0; d < 3; ++d)
                    xb[d] += (vv + c4 * vCr) * g[d] - c4 * w * CbTv[d] +
                             (H[3 * d] * LbTv[0] + H[3 * d + 1] * LbTv[1] + H[3 * d + 2] * LbTv[2]);
            }
    // adjoint of the projected F: (I + dt L)^T F_trial'-adjoint
    float A[9], Fb[9];
#pragma unroll
    for (int i = 0; i < 9; ++i) A[i] = ((i % 4 == 0) ? 1.0f : 0.0f) + a.dt * L[i];
    mTm(A, Ftb, Fb);
#pragma unroll
    for (int i = 0; i < 9; ++i) a.Fpb[9 * (size_t)p + i] = Fb[i];
#pragma unroll
    for (int d = 0; d < 3; ++d) a.xb[3 * p + d] = xb[d];
}

// Adjoint of the separable contact response v = v_s + v_t max(0, |v_t| + mu v_n)/|v_t|
// applied when v_n = v_r . n < 0 (identity otherwise), with v_r = v - v_s and
// v_t = v_r - v_n n; vb: adjoint of the output in, of the input velocity out.
__device__ __forceinline__ void coulomb_adj(const float *vr, const float *n, float mu, float tl_eps, float *vb) {
    const float vn = vr[0] * n[0] + vr[1] * n[1] + vr[2] * n[2];
    if (!(vn < 0.0f)) return;
    const float vt[3] = {vr[0] - vn * n[0], vr[1] - vn * n[1], vr[2] - vn * n[2]};
    const float tl = sqrtf(vt[0] * vt[0] + vt[1] * vt[1] + vt[2] * vt[2]);
    float tb[3] = {vb[0], vb[1], vb[2]}, nb = 0.0f;
    if (tl > tl_eps) {
        if (tl + mu * vn <= 0.0f) { vb[0] = vb[1] = vb[2] = 0.0f; return; }
        const float th[3] = {vt[0] / tl, vt[1] / tl, vt[2] / tl};
        const float thv = th[0] * vb[0] + th[1] * vb[1] + th[2] * vb[2];
        const float f = mu * vn / tl;
#pragma unroll
        for (int d = 0; d < 3; ++d) tb[d] = vb[d] + f * (vb[d] - th[d] * thv);
        nb = mu * thv;
    }
    const float ntb = n[0] * tb[0] + n[1] * tb[1] + n[2] * tb[2];
#pragma unroll
    for (int d = 0; d < 3; ++d) vb[d] = tb[d] - n[d] * ntb + n[d] * nb;
}

// Adjoint of one collider at one node: vb holds the adjoint of the collider's
// output velocity on entry and of its input velocity vin on return. A kinematic
// cuboid also takes fb, the adjoint of its force accumulator (acc += m (vin - vel)),
// and adds to velb (its velocity's adjoint) and mb (the node mass's adjoint).
__device__ void collide_adj(const ColDev &c, const PoseRec &P, int gx, int gy, int gz, const float *vin, float *vb,
                            const AdjK &a, float m, const float *fb, float *velb, float &mb) {
    const float dx = a.dx;
    switch (c.kind) {
    case GBMPM_COLLIDER_PLANE: {   // the forward's contact test, rounded as it rounds it
        const float o0 = __fsub_rn(__fmul_rn((float)gx, dx), P.p[0]), o1 = __fsub_rn(__fmul_rn((float)gy, dx), P.p[1]),
                    o2 = __fsub_rn(__fmul_rn((float)gz, dx), P.p[2]);
        const float dp = dot3_rn(o0, c.normal[0], o1, c.normal[1], o2, c.normal[2]);
        if (!(dp < 0.0f)) return;
        if (c.surface == 0) { vb[0] = vb[1] = vb[2] = 0.0f; return; }
        if (c.surface == 11) {
            if ((float)gz * dx < 0.4f || (float)gz * dx > 0.53f) { vb[0] = vb[1] = vb[2] = 0.0f; }
            else { vb[0] *= 0.3f; vb[1] = 0.0f; vb[2] *= 0.3f; }
            return;
        }
        const float *n = c.normal;
        const float nc = dot3_rn(vin[0], n[0], vin[1], n[1], vin[2], n[2]);
        const bool slip = c.surface == 1;
        const float sub = slip ? nc : fminf(nc, 0.0f);
        const float w[3] = {__fsub_rn(vin[0], __fmul_rn(n[0], sub)), __fsub_rn(vin[1], __fmul_rn(n[1], sub)),
                            __fsub_rn(vin[2], __fmul_rn(n[2], sub))};
        const float len = __fsqrt_rn(dot3_rn(w[0], w[0], w[1], w[1], w[2], w[2]));
        float wb[3] = {vb[0], vb[1], vb[2]}, ncb = 0.0f;
        if (nc < 0.0f && len > 1e-20f) {
            const float t = __fadd_rn(len, __fmul_rn(nc, c.friction));
            if (t <= 0.0f) {
                wb[0] = wb[1] = wb[2] = 0.0f;
            } else {   // v = w + mu nc w/|w|
                const float wh[3] = {w[0] / len, w[1] / len, w[2] / len};
                const float whv = wh[0] * vb[0] + wh[1] * vb[1] + wh[2] * vb[2];
                const float f = c.friction * nc / len;
#pragma unroll
                for (int d = 0; d < 3; ++d) wb[d] = vb[d] + f * (vb[d] - wh[d] * whv);
                ncb = c.friction * whv;
            }
        }
        const float ds = (slip || nc < 0.0f) ? 1.0f : 0.0f;   // d sub / d nc
        const float nw = n[0] * wb[0] + n[1] * wb[1] + n[2] * wb[2];
#pragma unroll
        for (int d = 0; d < 3; ++d) vb[d] = wb[d] + n[d] * (ncb - ds * nw);
        return;
    }
    case GBMPM_COLLIDER_BOX: {   // v = vel, acc += m (vin - vel) inside (mpm_solver_warp.py:2053-2088)
        if (P.mode == 2) { vb[0] = vb[1] = vb[2] = 0.0f; return; }
        const float o0 = __fsub_rn(__fmul_rn((float)gx, dx), P.p[0]), o1 = __fsub_rn(__fmul_rn((float)gy, dx), P.p[1]),
                    o2 = __fsub_rn(__fmul_rn((float)gz, dx), P.p[2]);
        if (fabsf(o0) < c.size[0] && fabsf(o1) < c.size[1] && fabsf(o2) < c.size[2]) {
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                const float f = fb ? fb[d] : 0.0f;
                velb[d] += vb[d] - f * m;
                mb += f * (vin[d] - c.vel[d]);
                vb[d] = f * m;
            }
        }
        return;
    }
    case GBMPM_COLLIDER_CUP: {   // mpm_solver_warp.py:2161-2225
        const float rel[3] = {(float)gx * dx - P.p[0], (float)gy * dx - P.p[1], (float)gz * dx - P.p[2]};
        const float *R = P.r;
        const float l0 = R[0] * rel[0] + R[3] * rel[1] + R[6] * rel[2];
        const float l1 = R[1] * rel[0] + R[4] * rel[1] + R[7] * rel[2];
        const float l2 = R[2] * rel[0] + R[5] * rel[1] + R[8] * rel[2];
        const float sdf = glass_sdf(l0, l1, l2, c);
        if (!(sdf < c.band_c)) return;
        if (!(sdf > -c.sticky)) { vb[0] = vb[1] = vb[2] = 0.0f; return; }   // grabbed: v = v_solid
        const float h = 0.25f * dx;
        float n0 = glass_sdf(l0 + h, l1, l2, c) - glass_sdf(l0 - h, l1, l2, c);
        float n1 = glass_sdf(l0, l1 + h, l2, c) - glass_sdf(l0, l1 - h, l2, c);
        float n2 = glass_sdf(l0, l1, l2 + h, c) - glass_sdf(l0, l1, l2 - h, c);
        const float nl = sqrtf(n0 * n0 + n1 * n1 + n2 * n2);
        if (!(nl > 1.0e-12f)) return;
        n0 /= nl; n1 /= nl; n2 /= nl;
        const float n[3] = {R[0] * n0 + R[1] * n1 + R[2] * n2, R[3] * n0 + R[4] * n1 + R[5] * n2,
                            R[6] * n0 + R[7] * n1 + R[8] * n2};
        const float vs[3] = {c.vel[0] + (c.omega[1] * rel[2] - c.omega[2] * rel[1]),
                             c.vel[1] + (c.omega[2] * rel[0] - c.omega[0] * rel[2]),
                             c.vel[2] + (c.omega[0] * rel[1] - c.omega[1] * rel[0])};
        const float vr[3] = {vin[0] - vs[0], vin[1] - vs[1], vin[2] - vs[2]};
        coulomb_adj(vr, n, c.friction, 1.0e-20f, vb);
        return;
    }
    case GBMPM_COLLIDER_SDF: {   // mpm_solver_warp.py:2680-2736
        const float rel[3] = {(float)gx * dx - P.p[0], (float)gy * dx - P.p[1], (float)gz * dx - P.p[2]};
        float body[3];
        qrot(P.q, rel, body, true);
        const float f0 = (body[0] - c.origin[0]) / c.cell, f1 = (body[1] - c.origin[1]) / c.cell,
                    f2 = (body[2] - c.origin[2]) / c.cell;
        const float rf = (float)c.sdf_res - 1.0f;
        if (!(f0 >= 0.0f && f1 >= 0.0f && f2 >= 0.0f && f0 <= rf && f1 <= rf && f2 <= rf)) return;
        if (!(trilerp(c.sdf_val, c.sdf_res, f0, f1, f2, 1, 0) <= c.band)) return;
        float g[3] = {trilerp(c.sdf_grad, c.sdf_res, f0, f1, f2, 3, 0), trilerp(c.sdf_grad, c.sdf_res, f0, f1, f2, 3, 1),
                      trilerp(c.sdf_grad, c.sdf_res, f0, f1, f2, 3, 2)};
        const float gl = sqrtf(g[0] * g[0] + g[1] * g[1] + g[2] * g[2]);
        if (!(gl > 1.0e-12f)) return;
        g[0] /= gl; g[1] /= gl; g[2] /= gl;
        float n[3];
        qrot(P.q, g, n, false);
        if (c.surface == 0) { vb[0] = vb[1] = vb[2] = 0.0f; return; }
        if (c.surface == 1) {   // v = v_s + (v_r - (v_r . n) n)
            const float nb = n[0] * vb[0] + n[1] * vb[1] + n[2] * vb[2];
#pragma unroll
            for (int d = 0; d < 3; ++d) vb[d] -= nb * n[d];
            return;
        }
        const float vs[3] = {c.vel[0] + (c.omega[1] * rel[2] - c.omega[2] * rel[1]),
                             c.vel[1] + (c.omega[2] * rel[0] - c.omega[0] * rel[2]),
                             c.vel[2] + (c.omega[0] * rel[1] - c.omega[1] * rel[0])};
        const float vr[3] = {vin[0] - vs[0], vin[1] - vs[1], vin[2] - vs[2]};
        coulomb_adj(vr, n, c.friction, 1.0e-12f, vb);
        return;
    }
    case GBMPM_COLLIDER_WALLS: {
        const int pad = 3, n = a.ng;
        if ((gx < pad && vin[0] < 0.0f) || (gx >= n - pad && vin[0] > 0.0f)) vb[0] = 0.0f;
        if ((gy < pad && vin[1] < 0.0f) || (gy >= n - pad && vin[1] > 0.0f)) vb[1] = 0.0f;
        if ((gz < pad && vin[2] < 0.0f) || (gz >= n - pad && vin[2] > 0.0f)) vb[2] = 0.0f;
        return;
    }
    default:
        return;
    }
}

__global__ void k_adj_grid_bwd(AdjK a) {
    const size_t N = box_count(a.box);
    const GK gk = adj_gk(a);
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < N; t += (size_t)gridDim.x * blockDim.x) {
        int gx, gy, gz;
        size_t id;
        if (!box_node(a.box, t, a.ng, gx, gy, gz, id)) break;
        const float4 mv = a.gmv[id];
        if (!(mv.w > 1e-15f)) { a.gmb[id] = make_float4(0.f, 0.f, 0.f, 0.f); continue; }
        float vin[kMaxCol][3], v[3], acc[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
        grid_pre(a, mv, v);
        for (int c = 0; c < a.ncol; ++c) {
            vin[c][0] = v[0]; vin[c][1] = v[1]; vin[c][2] = v[2];
            if (a.poses[c].mode != 0) collide(a.cols[c], a.poses[c], gx, gy, gz, mv.w, v, gk, acc);
        }
        const float4 b4 = a.gvb[id];
        float vb[3] = {b4.x, b4.y, b4.z};
        float mb_col = 0.0f;
        for (int c = a.ncol - 1; c >= 0; --c) {
            if (a.poses[c].mode == 0) continue;
            float velb[3] = {0.f, 0.f, 0.f};
            collide_adj(a.cols[c], a.poses[c], gx, gy, gz, vin[c], vb, a, mv.w,
                        a.col_force_b ? a.col_force_b + 3 * c : nullptr, velb, mb_col);
            if (a.col_vel_b && a.cols[c].kind == GBMPM_COLLIDER_BOX &&
                (velb[0] != 0.0f || velb[1] != 0.0f || velb[2] != 0.0f)) {
#pragma unroll
                for (int d = 0; d < 3; ++d) atomicAdd(a.col_vel_b + 3 * c + d, velb[d]);
            }
        }
        if (a.damp < 1.0f) { vb[0] *= a.damp; vb[1] *= a.damp; vb[2] *= a.damp; }
        const float inv = 1.0f / mv.w;
        const float mb = -(vb[0] * mv.x + vb[1] * mv.y + vb[2] * mv.z) * inv * inv + mb_col;
        a.gmb[id] = make_float4(vb[0] * inv, vb[1] * inv, vb[2] * inv, mb);
    }
}

__global__ void __launch_bounds__(128, 4) k_adj_p2g_bwd(AdjK a) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= a.n || (a.sel && a.sel[p] != 0)) return;
    const float x[3] = {a.x[3 * p], a.x[3 * p + 1], a.x[3 * p + 2]};
    const float v[3] = {a.v[3 * p], a.v[3 * p + 1], a.v[3 * p + 2]};
    float C[9], S[9], Fp[9], Ft[9], Fb[9];
#pragma unroll
    for (int i = 0; i < 9; ++i) {
        C[i] = a.C[9 * (size_t)p + i];
        S[i] = a.S[9 * (size_t)p + i];
        Fp[i] = a.Fp[9 * (size_t)p + i];
        Ft[i] = a.Ft[9 * (size_t)p + i];
        Fb[i] = a.Fpb[9 * (size_t)p + i];
    }
    const float m = a.mass[p], vol = a.vol[p], mu = a.mu[p], lam = a.lam[p], ys = a.ys[p];
    const int mat = a.mat[p];
    float xb[3] = {a.xb[3 * p], a.xb[3 * p + 1], a.xb[3 * p + 2]};
    Stencil s;
    stencil(x, a.inv_dx, s);
    if (!stencil_ok(s, a.ng, 0)) return;
    float A[9];
#pragma unroll
    for (int i = 0; i < 9; ++i) A[i] = -vol * S[i];
    float vb[3] = {0.f, 0.f, 0.f}, Cb[9] = {0.f}, Ab[9] = {0.f};
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
            for (int kk = 0; kk < 3; ++kk) {
                const size_t id = ((size_t)(s.b[0] + i) * a.ng + (s.b[1] + j)) * a.ng + (s.b[2] + kk);
                const float4 b4 = a.gmb[id];
                const float mb[3] = {b4.x, b4.y, b4.z};
                float w, g[3], H[9];
                weight_derivs(s, a.inv_dx, i, j, kk, w, g, H);
                const float r[3] = {((float)i - s.fx[0]) * a.dx, ((float)j - s.fx[1]) * a.dx, ((float)kk - s.fx[2]) * a.dx};
                float q[3], CTm[3], ATm[3];
#pragma unroll
                for (int u = 0; u < 3; ++u) {
                    q[u] = v[u] + C[3 * u] * r[0] + C[3 * u + 1] * r[1] + C[3 * u + 2] * r[2];
                    CTm[u] = C[u] * mb[0] + C[3 + u] * mb[1] + C[6 + u] * mb[2];
                    ATm[u] = A[u] * mb[0] + A[3 + u] * mb[1] + A[6 + u] * mb[2];
                    vb[u] += w * m * mb[u];
#pragma unroll
                    for (int t = 0; t < 3; ++t) {
                        Cb[3 * u + t] += w * m * mb[u] * r[t];
                        Ab[3 * u + t] += a.dt * mb[u] * g[t];
                    }
                }
                const float qm = q[0] * mb[0] + q[1] * mb[1] + q[2] * mb[2];
#pragma unroll
                for (int d = 0; d < 3; ++d)
                    xb[d] += m * (qm + b4.w) * g[d] - w * m * CTm[d] +
                             a.dt * (H[3 * d] * ATm[0] + H[3 * d + 1] * ATm[1] + H[3 * d + 2] * ATm[2]);
            }
    // stress adjoint: S = sym(tau), A = -vol S
    float tb[9];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) tb[3 * i + j] = -0.5f * vol * (Ab[3 * i + j] + Ab[3 * j + i]);
    float mub = 0.0f, lamb = 0.0f, pvb = 0.0f;
    float Lb[9] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};   // adjoint of the state's L
    float Ftb[9];
    float ysb_in = a.ysb[p], ysb = ysb_in;
    // the (mu, lam) the stress used, and whether mu and lam are still the
    // parameters (von Mises with softening zeroes them once its yield is used up)
    float mus = mu, lams = lam, ys_next = ys, jp_next = a.Jp[p];
    if (mat != 6 && mat != 10 && mat != 12) {
        float Fq[9];
        solid_return(a, mat, Ft, mu, lam, ys, a.Jp[p], Fq, mus, lams, ys_next, jp_next);
    }
    float jpb_new = a.Jpb[p];   // adjoint of Jp after the substep; the stress adds to it
    const bool params_live = (mu != 0.0f);
    if (mat == 6 || mat == 10 || mat == 12) {
        // tau = J (p I + 2 eta dev D) with J = Jc^3, Jc = det(F_trial)^(1/3), F = Jc I,
        // p = -K (J^-1.1 - 1), D = sym(L), eta = eta_p + tau_y / gd + K_p gd^(n - 1)
        const MatTables &T = *a.tab;
        float L[9], Sx[9], Fq[9];
#pragma unroll
        for (int i = 0; i < 9; ++i) L[i] = a.Lst[9 * (size_t)p + i];
        FluidTerms f;
        fluid_stress(a, p, mat, Ft, L, f, Fq, Sx);
        const float trb = tb[0] + tb[4] + tb[8];
        const float dpr = 1.1f * T.bulk[mat] * powf(f.J, -2.1f);
        float Jb = trb * f.pr + f.J * trb * dpr;
        if (mat == 10 || mat == 12) {
            float tD = 0.0f;
#pragma unroll
            for (int i = 0; i < 9; ++i) tD += tb[i] * f.Dd[i];
            Jb += 2.0f * f.eta * tD;
            const float etab = 2.0f * f.J * tD;
            const float ys_p = a.ys[p], Kp = T.hardening[mat], np_ = T.softening[mat];
            const float detadgd =
                (mat == 12)
                    ? table_slope(a.eta_tab, a.eta_n, a.eta_smin, a.eta_smax, logf(f.gd) * 0.43429448190325176f) *
                          0.43429448190325176f / f.gd
                    : -ys_p / (f.gd * f.gd) + (Kp != 0.0f ? Kp * (np_ - 1.0f) * powf(f.gd, np_ - 2.0f) : 0.0f);
            const float gdb = etab * detadgd;
            float Ddb[9];
#pragma unroll
            for (int i = 0; i < 9; ++i) Ddb[i] = 2.0f * f.J * f.eta * tb[i] + gdb * 2.0f * f.Dd[i] / f.gd;
            // L adjoint: sym(dev(Ddb))
            const float tr3 = (Ddb[0] + Ddb[4] + Ddb[8]) / 3.0f;
#pragma unroll
            for (int i = 0; i < 3; ++i)
#pragma unroll
                for (int j = 0; j < 3; ++j)
                    Lb[3 * i + j] = 0.5f * (Ddb[3 * i + j] + Ddb[3 * j + i]) - ((i == j) ? tr3 : 0.0f);
            if (mat == 10) {
                ysb = ysb_in + etab / f.gd;
                pvb = etab;
            }
        }
        // back through J = Jc^3, F = Jc I and Jc = det(F_trial)^(1/3)
        const float Jcb = 3.0f * f.Jc * f.Jc * Jb + (Fb[0] + Fb[4] + Fb[8]);
        const float Jtb = Jcb * f.Jc / (3.0f * f.Jt);
        float cof[9];
        cofactor(Ft, cof);
#pragma unroll
        for (int i = 0; i < 9; ++i) Ftb[i] = Jtb * cof[i];
    } else {
        float U[9], V[9], sg[3], yd[3];
        svd3(Fp, U, sg, V);
        const float mu = mus, lam = lams;   // the stress's moduli (zero once softened away)
        float mub_s = 0.0f, lamb_s = 0.0f;
        if (mat == 11) {   // tau = G F^T, G = U diag(h / s) V^T, h = 2 mu (e - mean) - pc Jc
            const MatTables &T = *a.tab;
            const float Jr = (jp_next < 0.5f) ? 1.0f : jp_next;
            const float K = T.E[11] / (3.0f * (1.0f - 2.0f * T.nu[11]));
            const float pc = fmaxf(K * (Jr / fmaxf(det3(Fp), 1e-6f) - 1.0f), 0.0f);
            float e[3], de[3], h[3], gg[3], Jg[3][3];
#pragma unroll
            for (int i = 0; i < 3; ++i) {
                e[i] = logf(fmaxf(sg[i], 1e-6f));
                de[i] = (sg[i] > 1e-6f) ? 1.0f / sg[i] : 0.0f;
            }
            const float mean = (e[0] + e[1] + e[2]) / 3.0f;
            const float Jc = fmaxf(sg[0], 1e-6f) * fmaxf(sg[1], 1e-6f) * fmaxf(sg[2], 1e-6f);
            const float kp = (pc > 0.0f) ? K : 0.0f;   // d(pc Jc)/dJr; d(pc Jc)/ds_j = -K Jc / s_j
#pragma unroll
            for (int i = 0; i < 3; ++i) {
                h[i] = 2.0f * mu * (e[i] - mean) - pc * Jc;
                gg[i] = (sg[i] > 1e-6f) ? h[i] / sg[i] : 0.0f;
            }
#pragma unroll
            for (int i = 0; i < 3; ++i)
#pragma unroll
                for (int j = 0; j < 3; ++j) {
                    const float dh = 2.0f * mu * (((i == j) ? 1.0f : 0.0f) - 1.0f / 3.0f) * de[j] + kp * Jc * de[j];
                    Jg[i][j] = (sg[i] > 1e-6f) ? (dh / sg[i] - ((i == j) ? h[i] / (sg[i] * sg[i]) : 0.0f)) : 0.0f;
                }
            float G[9], Gb[9], T1[9];
            udvt(U, gg[0], gg[1], gg[2], V, G);
            mm(tb, Fp, Gb);
            mTm(tb, G, T1);
#pragma unroll
            for (int i = 0; i < 9; ++i) Fb[i] += T1[i];
            iso_adjoint(U, sg, V, gg, Jg, Gb, Fb, yd);
#pragma unroll
            for (int i = 0; i < 3; ++i)
                if (sg[i] > 1e-6f) {
                    mub_s += yd[i] * 2.0f * (e[i] - mean) / sg[i];
                    if (!(jp_next < 0.5f)) jpb_new += yd[i] * (-kp) / sg[i];
                }
        } else if (mat == 0 || mat == 5) {   // tau = 2 mu (F - R) F^T + lam J (J - 1) I
            float R[9], FR[9], T1[9], T2[9], cof[9];
            mmT(U, V, R);
#pragma unroll
            for (int i = 0; i < 9; ++i) FR[i] = Fp[i] - R[i];
            mm(tb, Fp, T1);       // tau_b F
            mTm(tb, FR, T2);      // tau_b^T (F - R)
            float Rb[9];
#pragma unroll
            for (int i = 0; i < 9; ++i) {
                Fb[i] += 2.0f * mu * (T1[i] + T2[i]);
                Rb[i] = -2.0f * mu * T1[i];
            }
            const float one[3] = {1.0f, 1.0f, 1.0f};
            const float J0[3][3] = {{0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}};
            iso_adjoint(U, sg, V, one, J0, Rb, Fb, yd);
            const float J = det3(Fp);
            const float trb = tb[0] + tb[4] + tb[8];
            cofactor(Fp, cof);
#pragma unroll
            for (int i = 0; i < 9; ++i) Fb[i] += lam * (2.0f * J - 1.0f) * trb * cof[i];
            float FRF[9];
            mmT(FR, Fp, FRF);
#pragma unroll
            for (int i = 0; i < 9; ++i) mub_s += 2.0f * tb[i] * FRF[i];
            lamb_s += J * (J - 1.0f) * trb;
        } else {          // Hencky: tau = G F^T, G = U diag(h / s) V^T
            float e[3], de[3], h[3], gg[3], Jg[3][3];
#pragma unroll
            for (int i = 0; i < 3; ++i) {
                e[i] = logf(fmaxf(sg[i], 1e-6f));
                de[i] = (sg[i] > 1e-6f) ? 1.0f / sg[i] : 0.0f;
            }
            const float tr = e[0] + e[1] + e[2];
#pragma unroll
            for (int i = 0; i < 3; ++i) {
                h[i] = 2.0f * mu * e[i] + lam * tr;
                gg[i] = (sg[i] > 1e-6f) ? h[i] / sg[i] : 0.0f;
            }
#pragma unroll
            for (int i = 0; i < 3; ++i)
#pragma unroll
                for (int j = 0; j < 3; ++j) {
                    const float dh = ((i == j) ? 2.0f * mu : 0.0f) * de[j] + lam * de[j];
                    Jg[i][j] = (sg[i] > 1e-6f) ? (dh / sg[i] - ((i == j) ? h[i] / (sg[i] * sg[i]) : 0.0f)) : 0.0f;
                }
            float G[9], Gb[9], T1[9];
            udvt(U, gg[0], gg[1], gg[2], V, G);
            mm(tb, Fp, Gb);
            mTm(tb, G, T1);
#pragma unroll
            for (int i = 0; i < 9; ++i) Fb[i] += T1[i];
            iso_adjoint(U, sg, V, gg, Jg, Gb, Fb, yd);
#pragma unroll
            for (int i = 0; i < 3; ++i)
                if (sg[i] > 1e-6f) {
                    mub_s += yd[i] * 2.0f * e[i] / sg[i];
                    lamb_s += yd[i] * tr / sg[i];
                }
        }
        // the stress used the parameters unless softening zeroed them
        if (params_live && mus != 0.0f) {
            mub += mub_s;
            lamb += lamb_s;
        }
    }
    // return-map adjoint: F (projected) -> F_trial, yield, mu (fluids done above)
    if ((mat == 1 || mat == 5) && !(mat == 5 && ys <= 0.0f)) {
        const MatTables &T = *a.tab;
        float U[9], V[9], sg[3], e[3], Fq[9];
        const bool plastic = vm_return(Ft, mu, lam, ys, U, sg, V, e, Fq);
        if (!plastic) {
#pragma unroll
            for (int i = 0; i < 9; ++i) Ftb[i] = Fb[i];
        } else {
            const float mean = (e[0] + e[1] + e[2]) / 3.0f;
            const float eh[3] = {e[0] - mean, e[1] - mean, e[2] - mean};
            const float nrm = sqrtf(eh[0] * eh[0] + eh[1] * eh[1] + eh[2] * eh[2]);
            const float ehn = nrm + 1e-6f;
            const float kap = ys / (2.0f * mu * ehn);
            float de[3], ep[3], g[3], Jg[3][3];
#pragma unroll
            for (int i = 0; i < 3; ++i) {
                de[i] = (sg[i] > 0.01f) ? 1.0f / sg[i] : 0.0f;
                ep[i] = e[i] - (1.0f - kap) * eh[i];
                g[i] = expf(ep[i]);
            }
#pragma unroll
            for (int i = 0; i < 3; ++i)
#pragma unroll
                for (int j = 0; j < 3; ++j) {
                    const float dep = ((i == j) ? kap : 0.0f) + (1.0f - kap) / 3.0f -
                                      (nrm > 0.0f ? kap / ehn * eh[i] * eh[j] / nrm : 0.0f);
                    Jg[i][j] = g[i] * dep * de[j];
                }
#pragma unroll
            for (int i = 0; i < 9; ++i) Ftb[i] = 0.0f;
            float yd[3];
            iso_adjoint(U, sg, V, g, Jg, Fb, Ftb, yd);
            ysb = 0.0f;
            float mub_r = 0.0f;
#pragma unroll
            for (int i = 0; i < 3; ++i) {
                ysb += yd[i] * g[i] * eh[i] / (2.0f * mu * ehn);
                mub_r += yd[i] * g[i] * (-eh[i] * kap / mu);
            }
            // yield after the substep: y1 = y - soft |r h| (id 5; r h = (1 - kap) h),
            // then + 2 mu' xi (ehn - y / (2 mu)) with hardening (mu' = 0 once softened away)
            const float soft = (mat == 5) ? T.softening[mat] : 0.0f;
            const bool hard = T.hardening[mat] > 0.5f && mus != 0.0f;
            const float xi = T.xi[mat];
            float ydy = 1.0f + soft * nrm / (2.0f * mu * ehn);
            float ydmu = -soft * nrm * ys / (2.0f * mu * mu * ehn);
            float ydn = -soft * (1.0f - ys / (2.0f * mu) * 1e-6f / (ehn * ehn));
            if (hard) {
                ydy += -xi;
                ydmu += 2.0f * xi * ehn;
                ydn += 2.0f * mu * xi;
            }
            ysb += ysb_in * ydy;
            mub_r += ysb_in * ydmu;
            if (nrm > 0.0f && ydn != 0.0f) {
                float sb[3];
#pragma unroll
                for (int i = 0; i < 3; ++i) sb[i] = ysb_in * ydn * eh[i] / nrm * de[i];
                float Tm[9];
                udvt(U, sb[0], sb[1], sb[2], V, Tm);
#pragma unroll
                for (int i = 0; i < 9; ++i) Ftb[i] += Tm[i];
            }
            if (params_live) mub += mub_r;
        }
    } else if (mat == 2) {   // Drucker-Prager: e' = e - (dg / |h|) h, dg = |h| + c tr, c = alpha (3 lam + 2 mu) / (2 mu)
        const MatTables &T = *a.tab;
        float U[9], V[9], sg[3], e[3], h[3], hn, Fq[9];
        const int br = dp_return(Ft, mu, lam, T.alpha[mat], U, sg, V, e, h, hn, Fq);
        if (br == 0) {
#pragma unroll
            for (int i = 0; i < 9; ++i) Ftb[i] = Fb[i];
        } else {
            float g[3], Jg[3][3], yd[3];
            const float alpha = T.alpha[mat];
            const float c = alpha * (3.0f * lam + 2.0f * mu) / (2.0f * mu);
            const float tr = e[0] + e[1] + e[2];
            float hh[3], de[3];
#pragma unroll
            for (int i = 0; i < 3; ++i) {
                hh[i] = (br == 2) ? h[i] / hn : 0.0f;
                de[i] = (fabsf(sg[i]) > 1e-14f) ? 1.0f / sg[i] : 0.0f;
                g[i] = (br == 2) ? expf(e[i] - h[i] * ((hn + c * tr) / hn)) : 1.0f;
            }
#pragma unroll
            for (int i = 0; i < 3; ++i)
#pragma unroll
                for (int j = 0; j < 3; ++j) {
                    const float P = ((i == j) ? 1.0f : 0.0f) - 1.0f / 3.0f;
                    const float dep = 1.0f / 3.0f - c * (hh[i] + tr * (P - hh[i] * hh[j]) / hn);
                    Jg[i][j] = (br == 2) ? g[i] * dep * de[j] : 0.0f;
                }
#pragma unroll
            for (int i = 0; i < 9; ++i) Ftb[i] = 0.0f;
            iso_adjoint(U, sg, V, g, Jg, Fb, Ftb, yd);
            if (br == 2 && params_live) {
                float cb = 0.0f;
#pragma unroll
                for (int i = 0; i < 3; ++i) cb += yd[i] * g[i] * (-tr * hh[i]);
                mub += cb * alpha * (-3.0f * lam / (2.0f * mu * mu));
                lamb += cb * alpha * (3.0f / (2.0f * mu));
            }
        }
    } else if (mat == 9 || mat == 13) {   // mu(I)
        float U[9], V[9], sg[3], Fq[9];
        MuI m;
        const int br = mui_return(a, mat, Ft, mu, lam, U, sg, V, m, Fq);
        if (br == 0) {
#pragma unroll
            for (int i = 0; i < 9; ++i) Ftb[i] = Fb[i];
        } else {
            float g[3], Jg[3][3], yd[3];
#pragma unroll
            for (int i = 0; i < 3; ++i) g[i] = (br == 2) ? expf(m.d[i] * m.sc + m.mean) : 1.0f;
#pragma unroll
            for (int i = 0; i < 3; ++i) {
                float unit[3] = {0.0f, 0.0f, 0.0f}, row[3], dm = 0.0f, dl = 0.0f;
                unit[i] = 1.0f;
                if (br == 2) mui_reverse(a, mat, m, sg, mu, lam, unit, row, dm, dl);
#pragma unroll
                for (int j = 0; j < 3; ++j) Jg[i][j] = (br == 2) ? row[j] : 0.0f;
            }
#pragma unroll
            for (int i = 0; i < 9; ++i) Ftb[i] = 0.0f;
            iso_adjoint(U, sg, V, g, Jg, Fb, Ftb, yd);
            if (br == 2 && params_live) {
                float sbd[3], dm = 0.0f, dl = 0.0f;
                mui_reverse(a, mat, m, sg, mu, lam, yd, sbd, dm, dl);
                mub += dm;
                lamb += dl;
            }
        }
    } else if (mat == 11) {   // mu(I)-Phi(I), with the packing state Jp
        float U[9], V[9], sg[3], Fq[9], jpn;
        MuIPhi m;
        const int br = muiphi_return(a, Ft, mu, a.Jp[p], U, sg, V, m, Fq, jpn);
        float jrb = 0.0f;
        if (br == 1) {
#pragma unroll
            for (int i = 0; i < 9; ++i) Ftb[i] = Fb[i];
            jrb = jpb_new;
        } else {
            float g[3], Jg[3][3], yd[3];
            if (br == 0) {   // g = exp(mean) = (s0 s1 s2)^(1/3)
                const float gi = expf(m.mean);
#pragma unroll
                for (int i = 0; i < 3; ++i) {
                    g[i] = gi;
#pragma unroll
                    for (int j = 0; j < 3; ++j)
                        Jg[i][j] = (fabsf(sg[j]) > 1e-6f) ? gi / (3.0f * sg[j]) : 0.0f;
                }
                jrb = jpb_new;
            } else {
#pragma unroll
                for (int i = 0; i < 3; ++i) g[i] = expf(m.d[i] * m.sc + m.mean);
#pragma unroll
                for (int i = 0; i < 3; ++i) {
                    float unit[3] = {0.0f, 0.0f, 0.0f}, row[3], dm = 0.0f, dj = 0.0f;
                    unit[i] = 1.0f;
                    muiphi_reverse(a, m, sg, mu, unit, 0.0f, row, dm, dj);
#pragma unroll
                    for (int j = 0; j < 3; ++j) Jg[i][j] = row[j];
                }
            }
#pragma unroll
            for (int i = 0; i < 9; ++i) Ftb[i] = 0.0f;
            iso_adjoint(U, sg, V, g, Jg, Fb, Ftb, yd);
            if (br == 2) {
                // mu and the old Jp through both g and the new Jp; the trial singular
                // values through the new Jp (the g part went through iso_adjoint)
                float sbd[3], dm = 0.0f;
                muiphi_reverse(a, m, sg, mu, yd, jpb_new, sbd, dm, jrb);
                float sbj[3], dmx = 0.0f, djx = 0.0f;
                const float z[3] = {0.0f, 0.0f, 0.0f};
                muiphi_reverse(a, m, sg, mu, z, jpb_new, sbj, dmx, djx);
                float Tm[9];
                udvt(U, sbj[0], sbj[1], sbj[2], V, Tm);
#pragma unroll
                for (int i = 0; i < 9; ++i) Ftb[i] += Tm[i];
                if (params_live) mub += dm;
            }
        }
        jpb_new = m.jr_clamped ? 0.0f : jrb;
    } else if (mat != 6 && mat != 10 && mat != 12) {   // jelly, and id 5 once softened away: F = F_trial
#pragma unroll
        for (int i = 0; i < 9; ++i) Ftb[i] = Fb[i];
    }
#pragma unroll
    for (int d = 0; d < 3; ++d) { a.xb[3 * p + d] = xb[d]; a.vb[3 * p + d] = vb[d]; }
#pragma unroll
    for (int i = 0; i < 9; ++i) {
        a.Cb[9 * (size_t)p + i] = Cb[i];
        a.Ftb[9 * (size_t)p + i] = Ftb[i];
        a.Lb[9 * (size_t)p + i] = Lb[i];
    }
    a.ysb[p] = ysb;
    if (mat == 11) a.Jpb[p] = jpb_new;
    a.mub[p] += mub;
    a.lamb[p] += lamb;
    a.pvb[p] += pvb;
}

}  // namespace gbmpm

// ------------------------------------------------------------- host side ----
namespace {

int adjoint_supported(gbmpm_engine *e) {
    if (e->M.periodic_x) return fail(GBMPM_ERR_UNSUPPORTED, "the adjoint does not wrap the periodic x axis");
    if (e->M.rpic_damping != 0.0f) return fail(GBMPM_ERR_UNSUPPORTED, "the adjoint needs rpic_damping == 0");
    const uint32_t covered = (1u << 0) | (1u << 1) | (1u << 2) | (1u << 5) | (1u << 6) | (1u << 9) | (1u << 10) |
                             (1u << 11) | (1u << 12) | (1u << 13);
    if (e->M.material_mask & ~covered)
        return fail(GBMPM_ERR_UNSUPPORTED,
                    "the adjoint covers jelly (0), von Mises (1), sand (2), softening von Mises (5), water (6), "
                    "mu(I) (9, 11, 13), Newtonian (10) and tabulated viscous (12) particles");
    if (e->cdf.n > 0) return fail(GBMPM_ERR_UNSUPPORTED, "the adjoint does not cover CDF colliders");
    if (e->n_bodies > 0 || e->n_mods > 0)
        return fail(GBMPM_ERR_UNSUPPORTED, "the adjoint does not cover rigid bodies or particle modifiers");
    return GBMPM_OK;
}

// The forward part of an adjoint segment on stream s: `substeps` split-schedule
// substeps from the bound state, each substep's starting state kept in `states`
// (x 3, v 3, C 9, F_trial 9, L 9, yield 1, mu 1, lam 1, Jp 1 floats a particle, in
// that order, per substep). Returns the first error of a copy call (kernel launches
// report through cudaGetLastError).
cudaError_t record_adjoint_forward(gbmpm_engine *e, float dtf, int substeps, float *states, cudaStream_t s) {
    const gbmpm_particles &P = e->P;
    const int n = P.n;
    const size_t per = (size_t)37 * n;
    cudaError_t first = cudaSuccess;
    auto keep = [&](cudaError_t err) { if (first == cudaSuccess) first = err; };
    for (int i = 0; i < substeps; ++i) {
        float *st = states + per * i;
        keep(cudaMemcpyAsync(st, P.x, 3 * sizeof(float) * n, cudaMemcpyDeviceToDevice, s));
        keep(cudaMemcpyAsync(st + 3 * (size_t)n, P.v, 3 * sizeof(float) * n, cudaMemcpyDeviceToDevice, s));
        keep(cudaMemcpyAsync(st + 6 * (size_t)n, P.C, 9 * sizeof(float) * n, cudaMemcpyDeviceToDevice, s));
        keep(cudaMemcpyAsync(st + 15 * (size_t)n, P.F_trial, 9 * sizeof(float) * n, cudaMemcpyDeviceToDevice, s));
        keep(cudaMemcpyAsync(st + 24 * (size_t)n, P.L, 9 * sizeof(float) * n, cudaMemcpyDeviceToDevice, s));
        keep(cudaMemcpyAsync(st + 33 * (size_t)n, P.yield_stress, sizeof(float) * n, cudaMemcpyDeviceToDevice, s));
        keep(cudaMemcpyAsync(st + 34 * (size_t)n, P.mu, sizeof(float) * n, cudaMemcpyDeviceToDevice, s));
        keep(cudaMemcpyAsync(st + 35 * (size_t)n, P.lam, sizeof(float) * n, cudaMemcpyDeviceToDevice, s));
        keep(cudaMemcpyAsync(st + 36 * (size_t)n, P.Jp, sizeof(float) * n, cudaMemcpyDeviceToDevice, s));
        record_tick(e, dtf, 1, false, false, s, false, 0.0, 0.0, i);
    }
    return first;
}

// The reverse part of an adjoint segment on stream s, from the states the forward
// part kept: the adjoints in gr carried from the end of the segment to its start.
cudaError_t record_adjoint_reverse(gbmpm_engine *e, float dtf, int substeps, const gbmpm_adj_grads *gr,
                                   const float *states, cudaStream_t s) {
    const gbmpm_particles &P = e->P;
    const int n = P.n, ng = e->G.n_grid, nc = (int)e->cols.size();
    const size_t nn = (size_t)ng * ng * ng;
    const size_t per = (size_t)37 * n;
    float4 *grid = e->adj_grid.ptr;
    const int pb = std::max(1, (n + 127) / 128);
    // the grid kernels stride over the segment's node box; sized for the whole grid
    // at most, so that the scenes of a batch run side by side
    const int gb = (int)std::max<size_t>(1, std::min<size_t>((size_t)e->num_sms * 2, (nn + 255) / 256));
    int *box = e->adj_box.ptr;
    k_adj_box_init<<<1, 32, 0, s>>>(box, ng);
    k_adj_box<<<std::max(1, std::min(e->num_sms * 4, (int)(((size_t)n * substeps + 255) / 256))), 256, 0, s>>>(
        states, per, n, substeps, e->M.inv_dx, ng, box);
    e->launches += 2;
    for (int i = substeps - 1; i >= 0; --i) {
        const float *st = states + per * i;
        AdjK a{};
        a.x = st; a.v = st + 3 * (size_t)n; a.C = st + 6 * (size_t)n; a.Ft = st + 15 * (size_t)n;
        a.Lst = st + 24 * (size_t)n; a.ys = st + 33 * (size_t)n; a.Jp = st + 36 * (size_t)n;
        a.tab = e->d_tab.ptr;
        a.mass = P.mass; a.vol = P.vol; a.mu = st + 34 * (size_t)n; a.lam = st + 35 * (size_t)n;
        a.mat = P.material; a.sel = P.selection;
        a.eta_tab = e->M.eta_table; a.eta_n = e->M.eta_table_n;
        a.eta_smin = e->M.eta_table_smin; a.eta_smax = e->M.eta_table_smax;
        a.n = n;
        a.Fp = e->adj_scratch.ptr; a.S = a.Fp + 9 * (size_t)n; a.Fpb = a.S + 9 * (size_t)n;
        a.gmv = grid; a.gv = grid + nn; a.gvb = grid + 2 * nn; a.gmb = grid + 3 * nn;
        a.ng = ng; a.dx = e->M.dx; a.inv_dx = e->M.inv_dx; a.dt = dtf;
        for (int d = 0; d < 3; ++d) a.grav[d] = e->M.gravity[d];
        a.damp = e->M.grid_v_damping_scale;
        a.hard1 = e->M.hardening[1]; a.xi1 = e->M.xi[1];
        a.xb = gr->x; a.vb = gr->v; a.Cb = gr->C; a.Ftb = gr->F_trial; a.Lb = gr->L; a.ysb = gr->yield_stress;
        a.mub = gr->mu; a.lamb = gr->lam; a.pvb = gr->viscosity; a.Jpb = gr->Jp;
        a.col_force_b = gr->collider_force ? gr->collider_force + (size_t)i * 3 * std::max(1, nc) : nullptr;
        a.col_vel_b = gr->collider_velocity;
        a.ncol = nc; a.cols = e->d_cols.ptr; a.poses = e->d_pose.ptr + (size_t)i * std::max(1, nc);
        a.box = box;
        // the engine's P2G building block reads its inputs through a PK
        gbmpm_particles Ps = P;
        Ps.x = const_cast<float *>(a.x); Ps.v = const_cast<float *>(a.v); Ps.C = const_cast<float *>(a.C);
        PK k = make_pk(e, Ps, dtf, 0);
        k.cdf_on = 0;
        k_adj_zero_box<<<gb, 256, 0, s>>>(a);
        k_adj_stress_fwd<<<pb, 128, 0, s>>>(a);
        k_adj_p2g_fwd<<<pb, 128, 0, s>>>(a, k);
        k_adj_grid_fwd<<<gb, 256, 0, s>>>(a);
        k_adj_g2p_bwd<<<pb, 128, 0, s>>>(a);
        k_adj_grid_bwd<<<gb, 256, 0, s>>>(a);
        k_adj_p2g_bwd<<<pb, 128, 0, s>>>(a);
        e->launches += 7;
    }
    return cudaSuccess;
}

// Argument checks and scratch shared by the adjoint entry points; uploads the
// segment's pose table (the forward and the reverse parts read the same one).
int adjoint_prepare(gbmpm_engine *e, double *time, double dt, int32_t substeps, const gbmpm_adj_grads *gr,
                    bool need_grads, cudaStream_t s, uint64_t &version0) {
    int rc = check_ready(e);
    if (rc) return rc;
    if (!time || substeps < 1 || substeps > GBMPM_MAX_SUBSTEPS || !(dt > 0.0))
        return fail(GBMPM_ERR_ARG, "bad adjoint arguments");
    if (need_grads && (!gr || !gr->x || !gr->v || !gr->C || !gr->F_trial || !gr->yield_stress || !gr->mu ||
                       !gr->lam || !gr->L || !gr->viscosity || !gr->Jp))
        return fail(GBMPM_ERR_ARG, "every adjoint array is required");
    if (!e->P.L) return fail(GBMPM_ERR_ARG, "the adjoint needs particles.L");
    if ((rc = adjoint_supported(e))) return rc;
    const int n = e->P.n, ng = e->G.n_grid;
    const size_t nn = (size_t)ng * ng * ng;
    GB_CUDA(e->adj_states.ensure((size_t)37 * n * substeps));
    GB_CUDA(e->adj_scratch.ensure((size_t)27 * n));
    float4 *old_grid = e->adj_grid.ptr;
    GB_CUDA(e->adj_grid.ensure(4 * nn));   // four float4 grids
    if (e->adj_grid.ptr != old_grid)        // zero once; then each substep zeroes its box
        GB_CUDA(cudaMemsetAsync(e->adj_grid.ptr, 0, 4 * nn * sizeof(float4), s));
    GB_CUDA(e->adj_box.ensure(6));
    // one pose table for the whole segment, uploaded here, outside the captured graph
    bool reorder = false;
    version0 = e->version;
    return prepare_tick(e, time, dt, substeps, 0, s, reorder);
}

// Runs `rec` on stream s through the captured graph cached in `c` (captured anew
// when the segment length, dt, the engine's buffers or the adjoint arrays changed),
// or live after a failed capture, as ticks do.
template <typename Rec>
int run_adjoint_graph(gbmpm_engine *e, AdjGraph &c, int substeps, double dt, const gbmpm_adj_grads *gr,
                      uint64_t version0, cudaStream_t s, Rec rec) {
    gbmpm_adj_grads key{};
    if (gr) key = *gr;
    const bool same = c.g && c.substeps == substeps && c.dt == dt && c.version == e->version &&
                      version0 == e->version && std::memcmp(&c.grads, &key, sizeof key) == 0;
    if (same) {
        GB_CUDA(cudaGraphLaunch(c.g, s));
        e->launches += c.launches;
        return GBMPM_OK;
    }
    c.drop();
    if (!e->graph_failed) {
        cudaStream_t cap;
        GB_CUDA(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));
        cudaError_t be = cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal);
        if (be != cudaSuccess) {
            cudaStreamDestroy(cap);
            return fail(GBMPM_ERR_CUDA, std::string("cudaStreamBeginCapture: ") + cudaGetErrorString(be));
        }
        const int64_t before = e->launches;
        cudaError_t ce = rec(cap);
        c.launches = e->launches - before;
        e->launches = before;
        cudaGraph_t graph = nullptr;
        cudaError_t ee = cudaStreamEndCapture(cap, &graph);
        cudaStreamDestroy(cap);
        if (ce == cudaSuccess) ce = ee;
        if (ce == cudaSuccess) ce = cudaGraphInstantiate(&c.g, graph, 0);
        if (graph) cudaGraphDestroy(graph);
        if (ce == cudaSuccess) {
            c.substeps = substeps;
            c.dt = dt;
            c.version = e->version;
            c.grads = key;
            GB_CUDA(cudaGraphLaunch(c.g, s));
            e->launches += c.launches;
            return GBMPM_OK;
        }
        // as a failed tick capture: launched live from here on
        c.g = nullptr;
        e->graph_failed = true;
        (void)cudaGetLastError();
    }
    GB_CUDA(rec(s));
    GB_CUDA(cudaGetLastError());
    return GBMPM_OK;
}

}  // namespace

extern "C" {

int gbmpm_adjoint_segment(gbmpm_engine *e, double *time, double dt, int32_t substeps, const gbmpm_adj_grads *gr,
                          void *stream) {
    cudaStream_t s = (cudaStream_t)stream;
    uint64_t version0 = 0;
    int rc = adjoint_prepare(e, time, dt, substeps, gr, true, s, version0);
    if (rc) return rc;
    const float dtf = (float)dt;
    return run_adjoint_graph(e, e->adj_seg, substeps, dt, gr, version0, s, [&](cudaStream_t cs) {
        cudaError_t ce = record_adjoint_forward(e, dtf, substeps, e->adj_states.ptr, cs);
        cudaError_t cr = record_adjoint_reverse(e, dtf, substeps, gr, e->adj_states.ptr, cs);
        return ce != cudaSuccess ? ce : cr;
    });
}

int gbmpm_adjoint_forward(gbmpm_engine *e, double *time, double dt, int32_t substeps, float *states, void *stream) {
    if (!states) return fail(GBMPM_ERR_ARG, "null states");
    cudaStream_t s = (cudaStream_t)stream;
    uint64_t version0 = 0;
    int rc = adjoint_prepare(e, time, dt, substeps, nullptr, false, s, version0);
    if (rc) return rc;
    const float dtf = (float)dt;
    // the captured graph writes the engine's segment storage; the copy to the
    // caller's buffer follows it on the stream
    rc = run_adjoint_graph(e, e->adj_fwd, substeps, dt, nullptr, version0, s, [&](cudaStream_t cs) {
        return record_adjoint_forward(e, dtf, substeps, e->adj_states.ptr, cs);
    });
    if (rc) return rc;
    GB_CUDA(cudaMemcpyAsync(states, e->adj_states.ptr, (size_t)37 * e->P.n * substeps * sizeof(float),
                            cudaMemcpyDeviceToDevice, s));
    return GBMPM_OK;
}

int gbmpm_adjoint_reverse(gbmpm_engine *e, double *time, double dt, int32_t substeps, const float *states,
                          const gbmpm_adj_grads *gr, void *stream) {
    if (!states) return fail(GBMPM_ERR_ARG, "null states");
    cudaStream_t s = (cudaStream_t)stream;
    uint64_t version0 = 0;
    int rc = adjoint_prepare(e, time, dt, substeps, gr, true, s, version0);
    if (rc) return rc;
    GB_CUDA(cudaMemcpyAsync(e->adj_states.ptr, states, (size_t)37 * e->P.n * substeps * sizeof(float),
                            cudaMemcpyDeviceToDevice, s));
    const float dtf = (float)dt;
    return run_adjoint_graph(e, e->adj_rev, substeps, dt, gr, version0, s, [&](cudaStream_t cs) {
        return record_adjoint_reverse(e, dtf, substeps, gr, e->adj_states.ptr, cs);
    });
}

}  // extern "C"
