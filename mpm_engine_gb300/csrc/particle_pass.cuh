// The particle pass: stencils and B-spline weights, the G2P and P2G cores, the
// CPIC (CDF) transfer helpers, and the direct and tiled particle kernels.
//
// Included by gbmpm.cu inside namespace gbmpm, after the constants and helpers
// and before the host code; it is not a standalone header.

// ------------------------------------------------------ particle pass ------
struct Stencil {
    int b[3];
    float fx[3];
    float w[3][3], dw[3][3];
};

__device__ __forceinline__ void stencil(const float *x, float inv_dx, Stencil &s) {
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        float gp = x[a] * inv_dx;
        s.b[a] = (int)floorf(gp - 0.5f);
        float fx = gp - (float)s.b[a];
        s.fx[a] = fx;
        float wa = 1.5f - fx, wb = fx - 1.0f, wc = fx - 0.5f;
        s.w[a][0] = 0.5f * (wa * wa);
        s.w[a][1] = 0.75f - wb * wb;
        s.w[a][2] = 0.5f * (wc * wc);
        s.dw[a][0] = fx - 1.5f;
        s.dw[a][1] = -2.0f * wb;
        s.dw[a][2] = wc;
    }
}

// true when the 3x3x3 stencil lies inside the grid (x wraps when periodic)
__device__ __forceinline__ bool stencil_ok(const Stencil &s, int ng, int periodic_x) {
    bool ok = true;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        if (a == 0 && periodic_x) continue;
        ok = ok && s.b[a] >= 0 && s.b[a] + 2 < ng;
    }
    return ok;
}

__device__ __forceinline__ int wrap(int i, int n) { return ((i % n) + n) % n; }

__device__ __forceinline__ void mark_block(const PK &k, int bx, int by, int bz) {
    int b = (bx * k.bd + by) * k.bd + bz;
    if (k.blk_flag[b] == 0 && atomicExch(&k.blk_flag[b], 1) == 0) {
        int i = atomicAdd(k.blk_count, 1);
        k.blk_list[i] = b;
    }
}

// ---- building blocks shared by the direct and the tiled particle kernels ----

// Paired single-precision arithmetic: one FFMA2 / FMUL2 / FADD2 instruction does
// two independent fp32 operations with the rounding of two scalar ones, so the
// (x, y) components of the velocity moments below share an instruction (the pass
// is bound by instruction issue, not by FP32 throughput).
__device__ __forceinline__ float2 f2(float a, float b) { return make_float2(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }

// G2P for one particle (g2p_particle, mpm_utils.py:944-1043) with the grid
// velocity supplied by `fetch(ix, iy, iz)` (global memory or a shared tile).
// The 27-node sums v = sum w g, C = 4/dx sum w g (x_i - x_p)^T / dx and
// L = sum g grad(w)^T are evaluated axis by axis (z, then y, then x): the
// quadratic weights are separable, so the 7 moment sums cost 441 FMAs instead of
// 27 x 21. The x and y components run as pairs (FFMA2), the z component alone.
template <class Fetch>
__device__ __forceinline__ void g2p_core(const PK &k, const Stencil &s, Fetch fetch, float *v, float *C, float *L) {
    float2 zw[3], zd[3], zg[3];   // z weights, each duplicated into a pair
#pragma unroll
    for (int kk = 0; kk < 3; ++kk) {
        const float w = s.w[2][kk], d = s.w[2][kk] * ((float)kk - s.fx[2]), g = s.dw[2][kk];
        zw[kk] = f2(w, w);
        zd[kk] = f2(d, d);
        zg[kk] = f2(g, g);
    }
    const float2 z2 = f2(0.f, 0.f);
    float2 V0 = z2, SX = z2, SY = z2, SZ = z2, GX = z2, GY = z2, GZ = z2;              // x, y components
    float V0z = 0.f, SXz = 0.f, SYz = 0.f, SZz = 0.f, GXz = 0.f, GYz = 0.f, GZz = 0.f;   // z components
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        float2 B0 = z2, BY = z2, BDY = z2, BZ = z2, BDZ = z2;
        float B0z = 0.f, BYz = 0.f, BDYz = 0.f, BZz = 0.f, BDZz = 0.f;
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            float2 A0 = z2, AZ = z2, ADZ = z2;
            float A0z = 0.f, AZz = 0.f, ADZz = 0.f;
#pragma unroll
            for (int kk = 0; kk < 3; ++kk) {
                const float4 g = fetch(i, j, kk);
                const float2 gxy = f2(g.x, g.y);
                A0 = fma2(zw[kk], gxy, A0);
                AZ = fma2(zd[kk], gxy, AZ);
                ADZ = fma2(zg[kk], gxy, ADZ);
                A0z = fmaf(zw[kk].x, g.z, A0z);
                AZz = fmaf(zd[kk].x, g.z, AZz);
                ADZz = fmaf(zg[kk].x, g.z, ADZz);
            }
            const float wy = s.w[1][j], wyd = s.w[1][j] * ((float)j - s.fx[1]), dwy = s.dw[1][j];
            const float2 wy2 = f2(wy, wy), wyd2 = f2(wyd, wyd), dwy2 = f2(dwy, dwy);
            B0 = fma2(wy2, A0, B0);
            BY = fma2(wyd2, A0, BY);
            BDY = fma2(dwy2, A0, BDY);
            BZ = fma2(wy2, AZ, BZ);
            BDZ = fma2(wy2, ADZ, BDZ);
            B0z = fmaf(wy, A0z, B0z);
            BYz = fmaf(wyd, A0z, BYz);
            BDYz = fmaf(dwy, A0z, BDYz);
            BZz = fmaf(wy, AZz, BZz);
            BDZz = fmaf(wy, ADZz, BDZz);
        }
        const float wx = s.w[0][i], wxd = s.w[0][i] * ((float)i - s.fx[0]), dwx = s.dw[0][i];
        const float2 wx2 = f2(wx, wx), wxd2 = f2(wxd, wxd), dwx2 = f2(dwx, dwx);
        V0 = fma2(wx2, B0, V0);
        SX = fma2(wxd2, B0, SX);
        SY = fma2(wx2, BY, SY);
        SZ = fma2(wx2, BZ, SZ);
        GX = fma2(dwx2, B0, GX);
        GY = fma2(wx2, BDY, GY);
        GZ = fma2(wx2, BDZ, GZ);
        V0z = fmaf(wx, B0z, V0z);
        SXz = fmaf(wxd, B0z, SXz);
        SYz = fmaf(wx, BYz, SYz);
        SZz = fmaf(wx, BZz, SZz);
        GXz = fmaf(dwx, B0z, GXz);
        GYz = fmaf(wx, BDYz, GYz);
        GZz = fmaf(wx, BDZz, GZz);
    }
    const float c4 = k.inv_dx * 4.0f;
    const float2 c42 = f2(c4, c4), id2 = f2(k.inv_dx, k.inv_dx);
    const float2 SXs = mul2(SX, c42), SYs = mul2(SY, c42), SZs = mul2(SZ, c42);
    const float2 GXs = mul2(GX, id2), GYs = mul2(GY, id2), GZs = mul2(GZ, id2);
    v[0] = V0.x; v[1] = V0.y; v[2] = V0z;
    C[0] = SXs.x; C[1] = SYs.x; C[2] = SZs.x;
    C[3] = SXs.y; C[4] = SYs.y; C[5] = SZs.y;
    C[6] = SXz * c4; C[7] = SYz * c4; C[8] = SZz * c4;
    L[0] = GXs.x; L[1] = GYs.x; L[2] = GZs.x;
    L[3] = GXs.y; L[4] = GYs.y; L[5] = GZs.y;
    L[6] = GXz * k.inv_dx; L[7] = GYz * k.inv_dx; L[8] = GZz * k.inv_dx;
}

// advection, F_trial and covariance after the gather; Fpre, when given, holds the
// particle's F (already fetched) instead of the field
template <bool SOA>
__device__ __forceinline__ void g2p_finish(const PK &k, int p, float *x, const float *v, const float *L, float *Ft,
                                           const float *Fpre = nullptr) {
    float xn[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) xn[a] = __fadd_rn(x[a], __fmul_rn(v[a], k.dt));   // x + v dt, as the reference rounds it
    if (k.periodic_x) {
        float lx = (float)k.ng * k.dx;
        if (xn[0] < 0.0f) xn[0] += lx;
        if (xn[0] >= lx) xn[0] -= lx;
    }
#pragma unroll
    for (int a = 0; a < 3; ++a) x[a] = xn[a];
    float Fo[9], A[9];
    if (Fpre) {
#pragma unroll
        for (int i = 0; i < 9; ++i) Fo[i] = Fpre[i];
    } else {
        fld_load<SOA, 9>(k.F, k.n, p, Fo);
    }
    // F_trial = (I + dt L) F with the reference's roundings (L dt, then 1 +, then the
    // product): its determinant drives the fluids' stiff pressure
#pragma unroll
    for (int i = 0; i < 9; ++i) {
        const float ld = __fmul_rn(L[i], k.dt);
        A[i] = (i % 4 == 0) ? __fadd_rn(1.0f, ld) : ld;
    }
    mm_rn(A, Fo, Ft);
    if (k.update_cov && k.cov) {
        float c6[6];
        fld_load<SOA, 6>(k.cov, k.n, p, c6);
        float cn[9] = {c6[0], c6[1], c6[2], c6[1], c6[3], c6[4], c6[2], c6[4], c6[5]};
        float a1[9], a2[9];
        mm(L, cn, a1);
        mmT(cn, L, a2);
        c6[0] = cn[0] + k.dt * (a1[0] + a2[0]);
        c6[1] = cn[1] + k.dt * (a1[1] + a2[1]);
        c6[2] = cn[2] + k.dt * (a1[2] + a2[2]);
        c6[3] = cn[4] + k.dt * (a1[4] + a2[4]);
        c6[4] = cn[5] + k.dt * (a1[5] + a2[5]);
        c6[5] = cn[8] + k.dt * (a1[8] + a2[8]);
        fld_store<SOA, 6>(k.cov, k.n, p, c6);
    }
}

// P2G for one particle (p2g_particle, mpm_utils.py:819-916): every node
// contribution {m v_i, m} goes through `deposit(i, j, kk, float4)`.
template <class Deposit>
__device__ __forceinline__ void p2g_core(const PK &k, const Stencil &s, int p, const float *v, const float *Cin,
                                         const float *S, Deposit deposit) {
    float C[9];
#pragma unroll
    for (int i = 0; i < 9; ++i) C[i] = Cin[i];
    if (k.rpic != 0.0f) {
        float Cn[9];
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = 0; j < 3; ++j)
                Cn[3 * i + j] = (1.0f - k.rpic) * C[3 * i + j] + k.rpic / 2.0f * (C[3 * i + j] - C[3 * j + i]);
#pragma unroll
        for (int i = 0; i < 9; ++i) C[i] = (k.rpic < -0.001f) ? 0.0f : Cn[i];
    }
    const float m = k.mass[p];
    const float fs = -k.vol[p] * k.dt * k.inv_dx;
    float A[9];
#pragma unroll
    for (int i = 0; i < 9; ++i) A[i] = fs * S[i];
    float mCdx[9], base[3];
#pragma unroll
    for (int i = 0; i < 9; ++i) mCdx[i] = m * C[i] * k.dx;
#pragma unroll
    for (int a = 0; a < 3; ++a)
        base[a] = m * v[a] - (mCdx[3 * a] * s.fx[0] + mCdx[3 * a + 1] * s.fx[1] + mCdx[3 * a + 2] * s.fx[2]);
#pragma unroll
    for (int i = 0; i < 3; ++i) {
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            float wij = s.w[0][i] * s.w[1][j];
            float dwi_j = s.dw[0][i] * s.w[1][j];
            float wi_dj = s.w[0][i] * s.dw[1][j];
#pragma unroll
            for (int kk = 0; kk < 3; ++kk) {
                float wt = wij * s.w[2][kk];
                float gx = dwi_j * s.w[2][kk], gy = wi_dj * s.w[2][kk], gz = wij * s.dw[2][kk];
                float mom[3];
#pragma unroll
                for (int a = 0; a < 3; ++a) {
                    float aff = base[a] + mCdx[3 * a] * (float)i + mCdx[3 * a + 1] * (float)j + mCdx[3 * a + 2] * (float)kk;
                    mom[a] = wt * aff + (A[3 * a] * gx + A[3 * a + 1] * gy + A[3 * a + 2] * gz);
                }
                deposit(i, j, kk, make_float4(mom[0], mom[1], mom[2], wt * m));
            }
        }
    }
}

__device__ __forceinline__ void mark_stencil_blocks(const PK &k, const Stencil &s) {
    int by0 = s.b[1] >> 2, by1 = (s.b[1] + 2) >> 2;
    int bz0 = s.b[2] >> 2, bz1 = (s.b[2] + 2) >> 2;
    if (k.periodic_x) {
        for (int i = 0; i < 3; ++i) {
            int bxi = wrap(s.b[0] + i, k.ng) >> 2;
            for (int by = by0; by <= by1; ++by)
                for (int bz = bz0; bz <= bz1; ++bz) mark_block(k, bxi, by, bz);
        }
    } else {
        int bx0 = s.b[0] >> 2, bx1 = (s.b[0] + 2) >> 2;
        for (int bx = bx0; bx <= bx1; ++bx)
            for (int by = by0; by <= by1; ++by)
                for (int bz = bz0; bz <= bz1; ++bz) mark_block(k, bx, by, bz);
    }
}

__device__ __forceinline__ void global_deposit_all(const PK &k, const Stencil &s, int p, const float *v,
                                                   const float *C, const float *S) {
    p2g_core(k, s, p, v, C, S, [&](int i, int j, int kk, float4 val) {
        int ix = s.b[0] + i;
        if (k.periodic_x) ix = wrap(ix, k.ng);
        atomicAdd(k.gmv + ((size_t)ix * k.ng + (s.b[1] + j)) * k.ng + (s.b[2] + kk), val);
    });
    mark_stencil_blocks(k, s);
}

__device__ __forceinline__ float4 global_fetch(const PK &k, const Stencil &s, int i, int j, int kk) {
    int ix = s.b[0] + i;
    if (k.periodic_x) ix = wrap(ix, k.ng);
    return __ldg(k.gv + ((size_t)ix * k.ng + (s.b[1] + j)) * k.ng + (s.b[2] + kk));
}

// ---- CPIC (CDF) transfer helpers (mpm_utils.py:648-816) ----------------------
// Node tags: bit 2l = lane l valid here, bit 2l+1 = the node's side of lane l,
// bits 8..9 = the lane nearest the node (owner).
constexpr int kCdfOwnerShift = 8;

// cdf_pair_incompatible: some lane is valid at both ends with opposite sides
__device__ __forceinline__ bool cdf_incompatible(int pc, int nt) {
    return ((pc & nt & 0x55) & ((pc ^ nt) >> 1)) != 0;
}

__device__ __forceinline__ size_t node_id(const PK &k, const Stencil &s, int i, int j, int kk) {
    return ((size_t)(s.b[0] + i) * k.ng + (s.b[1] + j)) * k.ng + (s.b[2] + kk);
}

// cdf_stencil_near: a 4^3 block under the stencil holds tags now or at the last stamp
// k.cblock is null when the early-out is switched off (model.cdf_mask_off,
// mpm_utils.py:856, 980): every particle then takes the full 27-node scan
__device__ __forceinline__ bool cdf_near(const PK &k, const Stencil &s) {
    if (!k.cblock) return true;
    for (int bi = s.b[0] >> 2; bi <= (s.b[0] + 2) >> 2; ++bi)
        for (int bj = s.b[1] >> 2; bj <= (s.b[1] + 2) >> 2; ++bj)
            for (int bk = s.b[2] >> 2; bk <= (s.b[2] + 2) >> 2; ++bk)
                if (__ldg(k.cblock + ((size_t)bi * k.cnb + bj) * k.cnb + bk) != 0) return true;
    return false;
}

// One pass over the 27 stencil nodes of a stamp: caches the node tags (node index
// (i*3 + j)*3 + kk) and forms cdf_particle_tag's lane votes, the weighted signed
// distances of the valid nodes (mpm_utils.py:678-713); with `ghost`, it also forms
// the owner-lane sums of cdf_particle_ghost (:733-771) in the same node order.
struct CdfScan {
    int tag[27];
    float votes[4];
    int side1[4], side0[4];   // per lane: stencil nodes (bit (i*3 + j)*3 + kk) valid on side +, side -
    float d_hat, n_acc[3], best_w;
    int lane_p;
};

template <bool GHOST>
__device__ __forceinline__ void cdf_scan(const PK &k, const Stencil &s, const int *T, const float *D, CdfScan &c) {
    c.votes[0] = c.votes[1] = c.votes[2] = c.votes[3] = 0.f;
#pragma unroll
    for (int l = 0; l < 4; ++l) c.side1[l] = c.side0[l] = 0;
    c.d_hat = 0.f;
    c.n_acc[0] = c.n_acc[1] = c.n_acc[2] = 0.f;
    c.best_w = 0.f;
    c.lane_p = 0;
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j)
#pragma unroll
            for (int kk = 0; kk < 3; ++kk) {
                const size_t id = node_id(k, s, i, j, kk);
                const int t = T[id];
                c.tag[(i * 3 + j) * 3 + kk] = t;
                if (t == 0) continue;
                const float w = s.w[0][i] * s.w[1][j] * s.w[2][kk];
                const float dd = D[id];
                const int nbit = 1 << ((i * 3 + j) * 3 + kk);
#pragma unroll
                for (int l = 0; l < 4; ++l)
                    if ((t >> (2 * l)) & 1) {
                        const bool plus = (t >> (2 * l + 1)) & 1;
                        c.votes[l] += w * dd * (plus ? 1.0f : -1.0f);
                        if (plus) c.side1[l] |= nbit;
                        else c.side0[l] |= nbit;
                    }
                if (GHOST) {
                    const int own = (t >> kCdfOwnerShift) & 3;
                    if (((t >> (2 * own)) & 1) == 0) continue;
                    const float sgn = ((t >> (2 * own + 1)) & 1) ? 1.0f : -1.0f;
                    c.d_hat += w * sgn * dd;
                    const float dw[3] = {s.dw[0][i] * s.w[1][j] * s.w[2][kk], s.w[0][i] * s.dw[1][j] * s.w[2][kk],
                                         s.w[0][i] * s.w[1][j] * s.dw[2][kk]};
#pragma unroll
                    for (int a = 0; a < 3; ++a) c.n_acc[a] += dw[a] * k.inv_dx * sgn * dd;
                    if (w > c.best_w) { c.best_w = w; c.lane_p = own; }
                }
            }
}

// cdf_scan<true> without the node-tag cache, the stencil's x offset taken as a
// rolled loop: the nodes are visited in the same order with the same arithmetic, so
// every vote, mask and sum is the same, in a third of the unrolled body (the tiled
// CPIC pass is bound by instruction fetch; it needs no node tags after the scan).
__device__ __forceinline__ void cdf_scan_rolled(const PK &k, const Stencil &s, const int *T, const float *D,
                                                CdfScan &c) {
    c.votes[0] = c.votes[1] = c.votes[2] = c.votes[3] = 0.f;
#pragma unroll
    for (int l = 0; l < 4; ++l) c.side1[l] = c.side0[l] = 0;
    c.d_hat = 0.f;
    c.n_acc[0] = c.n_acc[1] = c.n_acc[2] = 0.f;
    c.best_w = 0.f;
    c.lane_p = 0;
#pragma unroll 1
    for (int i = 0; i < 3; ++i) {
        const float wx = i == 0 ? s.w[0][0] : (i == 1 ? s.w[0][1] : s.w[0][2]);
        const float dwx = i == 0 ? s.dw[0][0] : (i == 1 ? s.dw[0][1] : s.dw[0][2]);
        const size_t row = (size_t)(s.b[0] + i) * k.ng;
#pragma unroll
        for (int j = 0; j < 3; ++j)
#pragma unroll
            for (int kk = 0; kk < 3; ++kk) {
                const size_t id = (row + (s.b[1] + j)) * k.ng + (s.b[2] + kk);
                const int t = __ldg(T + id);
                if (t == 0) continue;
                const float w = wx * s.w[1][j] * s.w[2][kk];
                const float dd = __ldg(D + id);
                const int nbit = 1 << (9 * i + 3 * j + kk);
#pragma unroll
                for (int l = 0; l < 4; ++l)
                    if ((t >> (2 * l)) & 1) {
                        const bool plus = (t >> (2 * l + 1)) & 1;
                        c.votes[l] += w * dd * (plus ? 1.0f : -1.0f);
                        if (plus) c.side1[l] |= nbit;
                        else c.side0[l] |= nbit;
                    }
                const int own = (t >> kCdfOwnerShift) & 3;
                if (((t >> (2 * own)) & 1) == 0) continue;
                const float sgn = ((t >> (2 * own + 1)) & 1) ? 1.0f : -1.0f;
                c.d_hat += w * sgn * dd;
                const float dw[3] = {dwx * s.w[1][j] * s.w[2][kk], wx * s.dw[1][j] * s.w[2][kk],
                                     wx * s.w[1][j] * s.dw[2][kk]};
#pragma unroll
                for (int a = 0; a < 3; ++a) c.n_acc[a] += dw[a] * k.inv_dx * sgn * dd;
                if (w > c.best_w) { c.best_w = w; c.lane_p = own; }
            }
    }
}

// the particle tag from the votes: valid per lane where a valid node was seen, side
// from the sign of the vote
__device__ __forceinline__ int cdf_vote_tag(const CdfScan &c) {
    int pc = 0;
#pragma unroll
    for (int l = 0; l < 4; ++l)
        if ((c.side1[l] | c.side0[l]) != 0) pc |= (1 << (2 * l)) | ((c.votes[l] >= 0.0f ? 1 : 0) << (2 * l + 1));
    return pc;
}

// the stencil nodes incompatible with tag pc (cdf_incompatible of each node's tag)
__device__ __forceinline__ int cdf_mask(int pc, const CdfScan &c) {
    int m = 0;
#pragma unroll
    for (int l = 0; l < 4; ++l)
        if ((pc >> (2 * l)) & 1) m |= ((pc >> (2 * l + 1)) & 1) ? c.side0[l] : c.side1[l];
    return m;
}

// cdf_persist_tag: a lane the particle already carried keeps its side
__device__ __forceinline__ int cdf_persist(int old, int fresh) {
    int pc = 0;
#pragma unroll
    for (int l = 0; l < 4; ++l)
        if ((fresh >> (2 * l)) & 1) {
            int side_bit = 1 << (2 * l + 1);
            pc |= (1 << (2 * l)) | (((old >> (2 * l)) & 1) ? (old & side_bit) : (fresh & side_bit));
        }
    return pc;
}

// cdf_particle_ghost (mpm_utils.py:733-816): the velocity the particle reads from
// nodes across the surface. Surface normal and distance come from the owner-lane
// sums of the scan; the tangential part follows the surface type (sticky, slip,
// separable Coulomb with a capped impulse) plus a separation push when the
// particle sits within 0.05 dx of the surface.
static __device__ void cdf_ghost(const PK &k, const CdfScan &c, const float *xp, const float *vp, int pc, const float *grav,
                          float *ghost) {
    float vf[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) { vf[a] = vp[a] + grav[a] * k.dt; ghost[a] = vf[a]; }
    const float nl = sqrtf(c.n_acc[0] * c.n_acc[0] + c.n_acc[1] * c.n_acc[1] + c.n_acc[2] * c.n_acc[2]);
    if (!(nl > 1.0e-12f)) return;
    const int lane_p = c.lane_p;
    const float side = ((pc >> (2 * lane_p + 1)) & 1) ? 1.0f : -1.0f;
    float n[3], vs[3], vrel[3];
    const float *cp = k.lanes.c_prev[lane_p], *vl = k.lanes.v_prev[lane_p], *wl = k.lanes.w_prev[lane_p];
    float rel[3] = {xp[0] - cp[0], xp[1] - cp[1], xp[2] - cp[2]};
#pragma unroll
    for (int a = 0; a < 3; ++a) n[a] = c.n_acc[a] / nl * side;
    vs[0] = vl[0] + (wl[1] * rel[2] - wl[2] * rel[1]);
    vs[1] = vl[1] + (wl[2] * rel[0] - wl[0] * rel[2]);
    vs[2] = vl[2] + (wl[0] * rel[1] - wl[1] * rel[0]);
#pragma unroll
    for (int a = 0; a < 3; ++a) vrel[a] = vf[a] - vs[a];
    const float vn = vrel[0] * n[0] + vrel[1] * n[1] + vrel[2] * n[2];
    float vt[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) vt[a] = vrel[a] - n[a] * vn;
    float cc = 0.0f;
    const float d_side = c.d_hat * side, eps = 0.05f * k.dx;
    if (d_side < eps) cc = fminf((eps - d_side) / k.dt, 0.5f * k.dx / k.dt);
    const int stype = k.lanes.type[lane_p];
    if (stype == 0) {
#pragma unroll
        for (int a = 0; a < 3; ++a) ghost[a] = vs[a] + n[a] * cc;
    } else if (stype == 1) {
#pragma unroll
        for (int a = 0; a < 3; ++a) ghost[a] = vs[a] + vt[a] + n[a] * cc;
    } else {
        const float dvn = fmaxf(-vn, 0.0f) + cc;
        const float tl = sqrtf(vt[0] * vt[0] + vt[1] * vt[1] + vt[2] * vt[2]);
        if (tl > 1.0e-12f && dvn > 0.0f) {
            const float sc = fmaxf(0.0f, tl - k.lanes.fric[lane_p] * dvn) / tl;
#pragma unroll
            for (int a = 0; a < 3; ++a) vt[a] *= sc;
        }
        const float vnp = fmaxf(vn, 0.0f);
#pragma unroll
        for (int a = 0; a < 3; ++a) ghost[a] = vs[a] + vt[a] + n[a] * vnp + n[a] * cc;
    }
}

// P2G with the CPIC mask: deposits into nodes incompatible with the particle are
// withheld from the grid and added to the owner lane's reaction (force and torque
// about the lane centre, summed per thread in float64 before one flush per lane).
static __device__ void cdf_deposit_all(const PK &k, const Stencil &s, int p, const float *v, const float *C, const float *S,
                                int pc, const int *tags) {
    double acc[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    int acc_own = -1;
    auto flush = [&]() {
        if (acc_own < 0) return;
        double *w = k.cwrench + ((size_t)blockIdx.x * GBMPM_MAX_CDF + acc_own) * 6;
#pragma unroll
        for (int a = 0; a < 6; ++a) { atomicAdd(w + a, acc[a]); acc[a] = 0.0; }
    };
    p2g_core(k, s, p, v, C, S, [&](int i, int j, int kk, float4 val) {
        size_t id = node_id(k, s, i, j, kk);
        int nt = tags[(i * 3 + j) * 3 + kk];
        if (cdf_incompatible(pc, nt)) {
            int own = (nt >> kCdfOwnerShift) & 3;
            if (own != acc_own) { flush(); acc_own = own; }
            const float *cc = k.lanes.c_cur[own];
            float r[3] = {(float)(s.b[0] + i) * k.dx - cc[0], (float)(s.b[1] + j) * k.dx - cc[1],
                          (float)(s.b[2] + kk) * k.dx - cc[2]};
            acc[0] += (double)val.x;
            acc[1] += (double)val.y;
            acc[2] += (double)val.z;
            acc[3] += (double)(r[1] * val.z - r[2] * val.y);
            acc[4] += (double)(r[2] * val.x - r[0] * val.z);
            acc[5] += (double)(r[0] * val.y - r[1] * val.x);
            return;
        }
        atomicAdd(k.gmv + id, val);
    });
    flush();
    mark_stencil_blocks(k, s);
}

// Particle modifiers before the stress and P2G of a substep (the pre-P2G operations
// and velocity modifiers of p2g2p, mpm_solver_warp.py:1182-1196; kernels
// :2385-2540): impulses first, then velocity overrides, each in list order, on the
// float32 time window [start, end). Returns true when v changed.
static __device__ bool apply_modifiers(const PK &k, int mask, const float *x, float mass, float *v) {
    const float t = (float)k.sub_time[k.sub];
    bool changed = false;
    for (int pass = 0; pass < 2; ++pass)
        for (int m = 0; m < k.n_mods; ++m) {
            if (!((mask >> m) & 1)) continue;
            const gbmpm_modifier &d = k.mods[m];
            if ((d.kind == 0) != (pass == 0)) continue;
            if (!(t >= d.start_time && t < d.end_time)) continue;
            changed = true;
            if (d.kind == 0) {
                const float imp[3] = {d.vec[0] / mass, d.vec[1] / mass, d.vec[2] / mass};
#pragma unroll
                for (int a = 0; a < 3; ++a) v[a] = v[a] + imp[a] * k.dt;
            } else if (d.kind == 1) {
#pragma unroll
                for (int a = 0; a < 3; ++a) v[a] = d.vec[a];
            } else {
                const float off[3] = {x[0] - d.point[0], x[1] - d.point[1], x[2] - d.point[2]};
                const float on = off[0] * d.normal[0] + off[1] * d.normal[1] + off[2] * d.normal[2];
                const float hz[3] = {off[0] - on * d.normal[0], off[1] - on * d.normal[1], off[2] - on * d.normal[2]};
                const float hd = sqrtf(hz[0] * hz[0] + hz[1] * hz[1] + hz[2] * hz[2]);
                const float cosine = (off[0] * d.axis1[0] + off[1] * d.axis1[1] + off[2] * d.axis1[2]) / hd;
                float theta = acosf(fminf(fmaxf(cosine, -1.0f), 1.0f));
                if (!(off[0] * d.axis2[0] + off[1] * d.axis2[1] + off[2] * d.axis2[2] > 0.0f)) theta = -theta;
                const float a1 = -hd * sinf(theta) * d.rotation_scale;
                const float a2 = hd * cosf(theta) * d.rotation_scale;
#pragma unroll
                for (int a = 0; a < 3; ++a)
                    v[a] = a1 * d.axis1[a] + a2 * d.axis2[a] + d.translation_scale * d.normal[a];
            }
        }
    return changed;
}

// ---- direct kernel: one thread per particle, global gather and atomics ------
// One kernel serves every particle pass of the schedule; `mode` selects the
// stages (G2P, STRESS, P2G): the fused interior pass is G2P|STRESS|P2G, the tick
// prologue STRESS|P2G and the epilogue G2P.
template <bool SOLIDS>
__global__ void __launch_bounds__(kParticleThreads, 5) k_particles(PK k, int mode) {
    if ((mode & PASS_RESET_LISTS) && blockIdx.x == 0 && threadIdx.x == 0) {
        k.blk_count[0] = 0;
        k.blk_count[1] = 0;
    }
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= k.n) return;
    if (k.sel && k.sel[p] != 0) return;
    const int mat = k.mat[p];
    float x[3] = {k.x[3 * p], k.x[3 * p + 1], k.x[3 * p + 2]};
    float v[3], C[9], L[9], Ft[9], S[9];
    bool gathered = false;
    int ptag = 0;   // CPIC particle tag carried from G2P into P2G
    if ((mode & PASS_G2P) && mat != 7 && mat != 8) {
        Stencil s;
        stencil(x, k.inv_dx, s);
        if (!stencil_ok(s, k.ng, k.periodic_x)) {
            set_status(k.status, GBMPM_FLAG_STENCIL_OOB);
            return;
        }
        CdfScan cs;
        if (k.cdf_on) {
            int pc = 0;
            if (cdf_near(k, s)) {
                cdf_scan<true>(k, s, k.ctag_prev, k.cd_prev, cs);
                pc = cdf_persist(k.ptag[p], cdf_vote_tag(cs));
            }
            k.ptag[p] = pc;
            ptag = pc;
        }
        if (ptag != 0) {
            const float *vi = k.v + 3 * (size_t)p;
            const float vp[3] = {vi[0], vi[1], vi[2]};
            float gh[3];
            cdf_ghost(k, cs, x, vp, ptag, k.grav, gh);
            const float4 g4 = make_float4(gh[0], gh[1], gh[2], 0.0f);
            g2p_core(k, s, [&](int i, int j, int kk) {
                return cdf_incompatible(ptag, cs.tag[(i * 3 + j) * 3 + kk]) ? g4 : global_fetch(k, s, i, j, kk);
            }, v, C, L);
        } else {
            g2p_core(k, s, [&](int i, int j, int kk) { return global_fetch(k, s, i, j, kk); }, v, C, L);
        }
        g2p_finish<false>(k, p, x, v, L, Ft);
        gathered = true;
    } else if (k.cdf_on && (mode & PASS_P2G)) {
        ptag = k.ptag[p];
    }
    if (gathered) {
        float *xo = k.x + 3 * (size_t)p;
        xo[0] = x[0]; xo[1] = x[1]; xo[2] = x[2];
        if (!(mode & (PASS_STRESS | PASS_P2G)) || (mode & PASS_STORE_VC)) {
            float *vo = k.v + 3 * (size_t)p;
            vo[0] = v[0]; vo[1] = v[1]; vo[2] = v[2];
            mat_store(k.C + 9 * (size_t)p, C);
        }
        if (!(mode & PASS_STRESS)) {
            mat_store(k.L + 9 * (size_t)p, L);
            mat_store(k.Ft + 9 * (size_t)p, Ft);
        }
    }
    if (mode & PASS_STRESS) {
        if (!gathered) {
            mat_load(k.Ft + 9 * (size_t)p, Ft);
            mat_load(k.L + 9 * (size_t)p, L);
        }
        float Fn[9];
        stress_update<SOLIDS>(k, p, mat, Ft, L, Fn, S);
        mat_store(k.F + 9 * (size_t)p, Fn);
        if (mode & PASS_STORE_ALL) mat_store(k.S + 9 * (size_t)p, S);
    }
    if (mode & PASS_P2G) {
        if (!(mode & PASS_STRESS)) mat_load(k.S + 9 * (size_t)p, S);
        if (!gathered) {
            const float *vi = k.v + 3 * (size_t)p;
            v[0] = vi[0]; v[1] = vi[1]; v[2] = vi[2];
            mat_load(k.C + 9 * (size_t)p, C);
        }
        if (k.n_mods && k.mod_mask) {
            const int mm = k.mod_mask[p];
            if (mm && apply_modifiers(k, mm, x, k.mass[p], v)) {
                float *vo = k.v + 3 * (size_t)p;
                vo[0] = v[0]; vo[1] = v[1]; vo[2] = v[2];
            }
        }
        if (k.rigid_defer && mat == 8) return;   // deposits after the rigid update
        Stencil s;
        stencil(x, k.inv_dx, s);
        if (!stencil_ok(s, k.ng, k.periodic_x)) {
            set_status(k.status, GBMPM_FLAG_STENCIL_OOB);
            return;
        }
        int pc = 0;
        CdfScan cs;
        if (k.cdf_on && cdf_near(k, s)) {
            cdf_scan<false>(k, s, k.ctag, k.cd, cs);
            pc = cdf_persist(ptag, cdf_vote_tag(cs));
        }
        if (pc != 0) cdf_deposit_all(k, s, p, v, C, S, pc, cs.tag);
        else global_deposit_all(k, s, p, v, C, S);
    }
}

// ---- tiled kernel: block-sorted particles, shared-memory gather tile, run-wise scatter
// Particles arrive sorted by (4^3 block, cell); a CTA owns Tile<CDF>::threads
// consecutive particles, one per thread.
//  * Gather: the CTA reduces the bounding box of its stencils; when it holds at
//    most Tile<CDF>::gather_cap nodes the grid velocity of that box is copied to
//    shared memory and the 27-node gathers read it there (neighbouring threads
//    share nodes, so most reads are broadcasts).
//  * Scatter: each particle leaves a 40-float record in shared memory. Runs of
//    consecutive particles whose stencils share the same base node (the same
//    cell) are scattered together, three runs per warp: nine lanes take one
//    (i, j) node line each, sum the run's contributions to its three nodes from
//    shared reads, and issue one red.global.add.v4.f32 per node. Global atomics
//    drop from 27 per particle to 27 per run, and no shared-memory atomics are
//    needed.
// The plain pass runs 128-thread CTAs (six per SM); the CPIC pass, whose larger
// body runs best with fewer, wider CTAs, 256 (three per SM).
constexpr int kTileThreads = 128;
constexpr int kTileThreadsCdf = 256;
constexpr int kRec = 40;                  // floats per particle scatter record (10 float4)
// record stride in shared memory: 44 floats = 176 B, so the 16-byte stores of eight
// consecutive lanes land on disjoint bank groups (a 160 B stride pairs them up)
constexpr int kRecStride = 44;
// shared-memory shape of a tile of TH particles
template <int TH>
struct TileShape {
    static constexpr int threads = TH;
    static constexpr int gather_cap = 6 * TH;   // nodes in the shared gather tile (16 B each)
    static constexpr int smem_floats = (gather_cap * 4 > TH * kRecStride) ? gather_cap * 4 : TH * kRecStride;
    static_assert(gather_cap * 4 + 11 * TH <= smem_floats, "prefetch slots fit past the gather tile");
};
template <bool CDF>
struct Tile : TileShape<CDF ? kTileThreadsCdf : kTileThreads> {};
// the CPIC reaction partials are indexed by CTA; they are sized for the narrower of
// the direct and the tiled CPIC launches
constexpr int kCdfCtaThreads = kParticleThreads < kTileThreadsCdf ? kParticleThreads : kTileThreadsCdf;

struct TileBox {
    int lo[3], e[3];
    int vol;
    bool fits;
};

template <int TH>
__device__ __forceinline__ void block_box(const int *b, bool valid, TileBox &box, int (*s_red)[6], int cap) {
    int v[6];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        v[a] = valid ? b[a] : INT_MAX;
        v[3 + a] = valid ? -b[a] : INT_MAX;   // max as min of negatives
    }
#pragma unroll
    for (int a = 0; a < 6; ++a)
        for (int o = 16; o > 0; o >>= 1) v[a] = min(v[a], __shfl_xor_sync(0xffffffffu, v[a], o));
    const int w = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0) {
#pragma unroll
        for (int a = 0; a < 6; ++a) s_red[w][a] = v[a];
    }
    __syncthreads();
    int r[6];
#pragma unroll
    for (int a = 0; a < 6; ++a) r[a] = INT_MAX;
    for (int ww = 0; ww < TH / 32; ++ww)
#pragma unroll
        for (int a = 0; a < 6; ++a) r[a] = min(r[a], s_red[ww][a]);
    __syncthreads();
    bool any = r[0] != INT_MAX;
    long long vol = 1;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        box.lo[a] = any ? r[a] : 0;
        box.e[a] = any ? (-r[3 + a]) - r[a] + 3 : 0;
        vol *= (long long)box.e[a];
    }
    box.vol = any ? (int)min(vol, (long long)INT_MAX) : 0;
    box.fits = any && vol <= cap;
}

// quadratic B-spline weight and its derivative for node offset o of one axis
__device__ __forceinline__ void bspline_o(float fx, int o, float &w, float &dw) {
    float t0 = 1.5f - fx, t1 = fx - 1.0f, t2 = fx - 0.5f;
    float w0 = 0.5f * (t0 * t0), w1 = 0.75f - t1 * t1, w2 = 0.5f * (t2 * t2);
    w = (o == 0) ? w0 : ((o == 1) ? w1 : w2);
    dw = (o == 0) ? -t0 : ((o == 1) ? -2.0f * t1 : t2);
}

// One tile of TH consecutive particles of the sorted working set (`tile` is its
// index; the kernels below map CTAs to tiles). CDF adds the CPIC branches of the
// direct kernel: the gather reads the ghost velocity at nodes incompatible with the
// particle, and scatter runs are keyed by (base cell, particle tag) so each run
// deposits under one mask, its blocked nodes becoming the owner lane's reaction.
template <bool SOLIDS, bool CDF, int TH>
__device__ __forceinline__ void particles_tile(const PK &k, int mode, int tile) {
    constexpr int kTileThreads = TH;
    constexpr int kGatherCap = TileShape<TH>::gather_cap;
    __shared__ __align__(16) float s_mem[TileShape<TH>::smem_floats];
    __shared__ int s_key[kTileThreads];
    __shared__ int s_pc[CDF ? kTileThreads : 1];
    __shared__ int s_mask[CDF ? kTileThreads : 1];
    __shared__ int s_seg[kTileThreads + 1];
    __shared__ int s_wcnt[kTileThreads / 32];
    __shared__ int s_red[kTileThreads / 32][6];
    // F, mass and volume of a gather pass's particle, fetched asynchronously at the
    // start so that their L2 round trip overlaps the tile box, the tile load and the
    // gather (a gather pass starts before its wait: nothing still running writes
    // them). The slots lie past the gather tile, in the record area, and are read
    // into registers before the barrier that ends the gather.
    float(*s_pf)[kTileThreads] = reinterpret_cast<float(*)[kTileThreads]>(s_mem + kGatherCap * 4);
    const int t = threadIdx.x;
    const int lane = t & 31, warp = t >> 5;
    const int p = tile * kTileThreads + t;
    bool live = p < k.n && !(k.sel && k.sel[p] != 0);
    const int mat = live ? k.mat[p] : 0;
    if (!(mode & PASS_G2P)) {   // without a gather, x and the stress inputs are what the previous pass wrote
        pdl_wait();
        pdl_trigger();
    }
    const bool pf = (mode & PASS_G2P) && live;
    if (pf) {
#pragma unroll
        for (int c = 0; c < 9; ++c) cp_async4(&s_pf[c][t], k.F + (size_t)c * k.n + p);
        if (mode & PASS_P2G) {
            cp_async4(&s_pf[9][t], k.mass + p);
            cp_async4(&s_pf[10][t], k.vol + p);
        }
    }
    float x[3] = {0.f, 0.f, 0.f};
    if (live) fld_load<true, 3>(k.x, k.n, p, x);
    float v[3] = {0.f, 0.f, 0.f}, C[9], L[9], Ft[9], S[9];
    float Fpf[9], mpf = 0.f, vpf = 0.f;
    bool gathered = false;
    int ptag = 0;   // CPIC particle tag carried from the gather into the scatter
    if (mode & PASS_G2P) {
        bool want = live && mat != 7 && mat != 8;
        Stencil s;
        stencil(x, k.inv_dx, s);
        if (want && !stencil_ok(s, k.ng, k.periodic_x)) {
            set_status(k.status, GBMPM_FLAG_STENCIL_OOB);
            want = false;
            live = false;
        }
        // CPIC: the gather's scan (previous stamp at this position) is the scan the
        // last scatter made (current stamp then, at the same position), so its
        // result comes from the cache: the tag, the mask of incompatible stencil
        // nodes and the owner-lane sums of the ghost velocity.
        int gmask = 0;
        float4 g4 = make_float4(0.f, 0.f, 0.f, 0.f);
        if (CDF && want) {
            float old;
            fld_load<true, 1>(reinterpret_cast<float *>(k.ptag), k.n, p, &old);
            ptag = __float_as_int(old);
            if (ptag != 0) {
                CdfScan cs;
                float cch[5], vp[3], gh[3];
                fld_load<true, 5>(k.ccache, k.n, p, cch);
                const int mb = __float_as_int(cch[0]);
                gmask = mb & 0x7ffffff;
                cs.lane_p = (mb >> 27) & 3;
                cs.d_hat = cch[1];
                cs.n_acc[0] = cch[2]; cs.n_acc[1] = cch[3]; cs.n_acc[2] = cch[4];
                fld_load<true, 3>(k.v, k.n, p, vp);
                cdf_ghost(k, cs, x, vp, ptag, k.grav, gh);
                g4 = make_float4(gh[0], gh[1], gh[2], 0.0f);
            }
        }
        TileBox box;
        block_box<kTileThreads>(s.b, want, box, s_red, kGatherCap);
        pdl_wait();   // the grid velocities come from the grid pass before this one
        pdl_trigger();
        if ((mode & PASS_RESET_LISTS) && tile == 0 && threadIdx.x == 0) {
            k.blk_count[0] = 0;
            k.blk_count[1] = 0;
        }
        float4 *s_tile = reinterpret_cast<float4 *>(s_mem);
        // the prefetched fields, taken into registers before the record area is reused
        auto take_prefetch = [&]() {
            if (pf) {
                cp_async_wait_all();
#pragma unroll
                for (int c = 0; c < 9; ++c) Fpf[c] = s_pf[c][t];
                mpf = s_pf[9][t];
                vpf = s_pf[10][t];
            }
        };
        if (box.fits) {
            // one thread per (x, y) row of the box: the row's nodes are contiguous in
            // the grid and in the tile, and all its 16-byte copies are in flight at once
            const int rows = box.e[0] * box.e[1];
            for (int r = t; r < rows; r += kTileThreads) {
                const int qx = r / box.e[1], qy = r - qx * box.e[1];
                const float4 *src = k.gv + ((size_t)(box.lo[0] + qx) * k.ng + (box.lo[1] + qy)) * k.ng + box.lo[2];
                float4 *dst = s_tile + r * box.e[2];
                for (int qz = 0; qz < box.e[2]; ++qz) cp_async16(dst + qz, src + qz);
            }
            cp_async_wait_all();
            __syncthreads();
            if (want) {
                const int o0 = s.b[0] - box.lo[0], o1 = s.b[1] - box.lo[1], o2 = s.b[2] - box.lo[2];
                // one copy of the unrolled gather serves masked and unmasked particles
                g2p_core(k, s, [&](int i, int j, int kk) {
                    const float4 t4 = s_tile[((o0 + i) * box.e[1] + (o1 + j)) * box.e[2] + (o2 + kk)];
                    return (CDF && ((gmask >> ((i * 3 + j) * 3 + kk)) & 1)) ? g4 : t4;
                }, v, C, L);
            }
            take_prefetch();
            __syncthreads();
        } else {   // box.fits is uniform over the CTA, so is this branch and its barrier
            if (want)
                g2p_core(k, s, [&](int i, int j, int kk) {
                    const float4 t4 = global_fetch(k, s, i, j, kk);
                    return (CDF && ((gmask >> ((i * 3 + j) * 3 + kk)) & 1)) ? g4 : t4;
                }, v, C, L);
            take_prefetch();
            __syncthreads();
        }
        if (want) {
            g2p_finish<true>(k, p, x, v, L, Ft, Fpf);
            gathered = true;
            fld_store<true, 3>(k.x, k.n, p, x);
            if (!(mode & (PASS_STRESS | PASS_P2G)) || (mode & PASS_STORE_VC)) {
                fld_store<true, 3>(k.v, k.n, p, v);
                fld_store<true, 9>(k.C, k.n, p, C);
            }
            if (!(mode & PASS_STRESS)) {
                fld_store<true, 9>(k.L, k.n, p, L);
                fld_store<true, 9>(k.Ft, k.n, p, Ft);
            }
        }
    }
    if ((mode & PASS_STRESS) && live) {
        if (!gathered) {
            fld_load<true, 9>(k.Ft, k.n, p, Ft);
            fld_load<true, 9>(k.L, k.n, p, L);
        }
        float Fn[9];
        stress_update<SOLIDS>(k, p, mat, Ft, L, Fn, S);
        fld_store<true, 9>(k.F, k.n, p, Fn);
        if (mode & PASS_STORE_ALL) fld_store<true, 9>(k.S, k.n, p, S);
    }
    if (!(mode & PASS_P2G)) return;
    pdl_wait();   // the scatter target and block lists are the grid pass's (no-op after the gather's wait)
    pdl_trigger();
    if (live) {
        if (!(mode & PASS_STRESS)) fld_load<true, 9>(k.S, k.n, p, S);
        if (!gathered) {
            fld_load<true, 3>(k.v, k.n, p, v);
            fld_load<true, 9>(k.C, k.n, p, C);
            if (CDF) {
                float old;
                fld_load<true, 1>(reinterpret_cast<float *>(k.ptag), k.n, p, &old);
                ptag = __float_as_int(old);
            }
        }
    }
    if (live && k.n_mods && k.mod_mask) {
        const int mm = k.mod_mask[p];
        if (mm && apply_modifiers(k, mm, x, k.mass[p], v)) fld_store<true, 3>(k.v, k.n, p, v);
    }
    Stencil s;
    stencil(x, k.inv_dx, s);
    bool want = live && !(k.rigid_defer && mat == 8);   // rigid particles deposit after the rigid update
    if (want && !stencil_ok(s, k.ng, k.periodic_x)) {
        set_status(k.status, GBMPM_FLAG_STENCIL_OOB);
        want = false;
    }
    int pcs = 0, pmask = 0;   // CPIC tag at the current stamp, mask of incompatible nodes
    if (CDF && want) {
        if (cdf_near(k, s)) {
            CdfScan cs;
            cdf_scan_rolled(k, s, k.ctag, k.cd, cs);
            pcs = cdf_persist(ptag, cdf_vote_tag(cs));
            if (pcs != 0) {
                pmask = cdf_mask(pcs, cs);
                const float cch[5] = {__int_as_float(pmask | (cs.lane_p << 27)), cs.d_hat, cs.n_acc[0],
                                      cs.n_acc[1], cs.n_acc[2]};
                fld_store<true, 5>(k.ccache, k.n, p, cch);
            }
        }
        const float pcf = __int_as_float(pcs);
        fld_store<true, 1>(reinterpret_cast<float *>(k.ptag), k.n, p, &pcf);
    }
    if (CDF) { s_pc[t] = pcs; s_mask[t] = pmask; }
    // ---- scatter record (40 floats, 16-byte aligned): [0..11] the x and y weights and
    // derivatives a lane indexes by its node line (wx[3], wy[3], dwx[3], dwy[3]);
    // [12..39] what every lane of a particle reads, packed for seven float4 loads:
    // wz[3], m | dwz[3], b0 | b1, b2, c00, c01 | c02, c10, c11, c12 | c20, c21, c22,
    // A00 | A01, A02, A10, A11 | A12, A20, A21, A22, with b = m v - m C fx dx the
    // affine momentum base, c = m C dx and A = -vol dt/dx stress
    if (want) {
        float Cr[9];
#pragma unroll
        for (int i = 0; i < 9; ++i) Cr[i] = C[i];
        if (k.rpic != 0.0f) {
#pragma unroll
            for (int i = 0; i < 3; ++i)
#pragma unroll
                for (int j = 0; j < 3; ++j)
                    Cr[3 * i + j] = (k.rpic < -0.001f) ? 0.0f
                                    : (1.0f - k.rpic) * C[3 * i + j] + k.rpic / 2.0f * (C[3 * i + j] - C[3 * j + i]);
        }
        const float m = (pf && (mode & PASS_P2G)) ? mpf : k.mass[p];
        const float fs = -((pf && (mode & PASS_P2G)) ? vpf : k.vol[p]) * k.dt * k.inv_dx;
        float rec[kRec];
#pragma unroll
        for (int o = 0; o < 3; ++o) {
            rec[o] = s.w[0][o];
            rec[3 + o] = s.w[1][o];
            rec[6 + o] = s.dw[0][o];
            rec[9 + o] = s.dw[1][o];
            rec[12 + o] = s.w[2][o];
            rec[16 + o] = s.dw[2][o];
        }
        rec[15] = m;
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            float c0 = m * Cr[3 * a] * k.dx, c1 = m * Cr[3 * a + 1] * k.dx, c2 = m * Cr[3 * a + 2] * k.dx;
            rec[19 + a] = m * v[a] - (c0 * s.fx[0] + c1 * s.fx[1] + c2 * s.fx[2]);
            rec[22 + 3 * a] = c0; rec[23 + 3 * a] = c1; rec[24 + 3 * a] = c2;
            rec[31 + 3 * a] = fs * S[3 * a]; rec[32 + 3 * a] = fs * S[3 * a + 1]; rec[33 + 3 * a] = fs * S[3 * a + 2];
        }
        float4 *dst = reinterpret_cast<float4 *>(s_mem + t * kRecStride);
#pragma unroll
        for (int q = 0; q < kRec / 4; ++q) dst[q] = make_float4(rec[4 * q], rec[4 * q + 1], rec[4 * q + 2], rec[4 * q + 3]);
        s_key[t] = (s.b[0] << 20) | (s.b[1] << 10) | s.b[2];   // n_grid <= 1024 on this path
    } else {
        s_key[t] = -1 - t;   // a dead slot forms its own, skipped run
    }
    __syncthreads();
    // ---- runs of equal base node (and CPIC tag): compact the run heads
    const bool head = (t == 0) || (s_key[t] != s_key[t - 1]) || (CDF && s_pc[t] != s_pc[t - 1]);
    const unsigned bal = __ballot_sync(0xffffffffu, head);
    if (lane == 0) s_wcnt[warp] = __popc(bal);
    __syncthreads();
    int off = 0, total = 0;
    for (int w = 0; w < kTileThreads / 32; ++w) {
        int c = s_wcnt[w];
        if (w < warp) off += c;
        total += c;
    }
    if (head) s_seg[off + __popc(bal & ((1u << lane) - 1u))] = t;
    if (t == 0) s_seg[total] = kTileThreads;
    __syncthreads();
    // ---- runs: a warp takes three runs at once, one per 9-lane group; lane
    // (group, node line (i,j)) sums the three nodes k = 0..2 of its line over its
    // run's particles and deposits them itself
    const int g3 = lane / 9, li = (lane % 9) / 3, lj = lane % 3;
    const float fi = (float)li, fj = (float)lj;
    for (int sg0 = warp * 3; sg0 < total; sg0 += 3 * (kTileThreads / 32)) {
        const int sg = sg0 + g3;
        int q0 = 0, q1 = 0, key = -1;
        if (lane < 27 && sg < total) {
            q0 = s_seg[sg];
            q1 = s_seg[sg + 1];
            key = s_key[q0];
        }
        if (key < 0) q1 = q0;   // dead slot or idle lane: no particles
        float acc[3][4];
#pragma unroll
        for (int kk = 0; kk < 3; ++kk) acc[kk][0] = acc[kk][1] = acc[kk][2] = acc[kk][3] = 0.f;
#pragma unroll 1   // unrolling by two measured slower (22.01 against 21.87 ms per pour frame, 56.5 against 54.9 CPIC)
        for (int q = q0; q < q1; ++q) {
            const float *r = s_mem + q * kRecStride;
            const float wxi = r[li], wyj = r[3 + lj], dwxi = r[6 + li], dwyj = r[9 + lj];
            const float4 *r4 = reinterpret_cast<const float4 *>(r);
            float inv[28];
#pragma unroll
            for (int h = 0; h < 7; ++h) {
                const float4 f4 = r4[3 + h];
                inv[4 * h] = f4.x; inv[4 * h + 1] = f4.y; inv[4 * h + 2] = f4.z; inv[4 * h + 3] = f4.w;
            }
            // inv[i] = rec[12 + i]
            const float u = wxi * wyj, ux = dwxi * wyj, uy = wxi * dwyj;
            const float wz0 = inv[0], wz1 = inv[1], wz2 = inv[2], dz0 = inv[4], dz1 = inv[5], dz2 = inv[6];
            const float m = inv[3];
            float P[3], Q[3], R[3];
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                P[a] = u * (inv[7 + a] + inv[10 + 3 * a] * fi + inv[11 + 3 * a] * fj) + inv[19 + 3 * a] * ux +
                       inv[20 + 3 * a] * uy;
                Q[a] = u * inv[12 + 3 * a];
                R[a] = u * inv[21 + 3 * a];
            }
            const float um = u * m;
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                acc[0][a] += wz0 * P[a] + dz0 * R[a];
                acc[1][a] += wz1 * (P[a] + Q[a]) + dz1 * R[a];
                acc[2][a] += wz2 * (P[a] + 2.0f * Q[a]) + dz2 * R[a];
            }
            acc[0][3] += wz0 * um;
            acc[1][3] += wz1 * um;
            acc[2][3] += wz2 * um;
        }
        if (q1 > q0) {
            const int bx = key >> 20, by = (key >> 10) & 1023, bz = key & 1023;
            const int gx = bx + li, gy = by + lj;
            const int lmask = CDF ? (s_mask[q0] >> ((li * 3 + lj) * 3)) & 7 : 0;   // the run's mask, this line
            int marked = -1;   // 4^3 block (z index) this lane marked last
#pragma unroll
            for (int kk = 0; kk < 3; ++kk) {
                if (CDF && lmask != 0) {
                    if ((lmask >> kk) & 1) {   // blocked: the owner lane's reaction
                        const int nt = __ldg(k.ctag + ((size_t)gx * k.ng + gy) * k.ng + (bz + kk));
                        const int own = (nt >> kCdfOwnerShift) & 3;
                        const float *cc = k.lanes.c_cur[own];
                        const float r[3] = {(float)gx * k.dx - cc[0], (float)gy * k.dx - cc[1],
                                            (float)(bz + kk) * k.dx - cc[2]};
                        double *w = k.cwrench + ((size_t)tile * GBMPM_MAX_CDF + own) * 6;
                        atomicAdd(w + 0, (double)acc[kk][0]);
                        atomicAdd(w + 1, (double)acc[kk][1]);
                        atomicAdd(w + 2, (double)acc[kk][2]);
                        atomicAdd(w + 3, (double)(r[1] * acc[kk][2] - r[2] * acc[kk][1]));
                        atomicAdd(w + 4, (double)(r[2] * acc[kk][0] - r[0] * acc[kk][2]));
                        atomicAdd(w + 5, (double)(r[0] * acc[kk][1] - r[1] * acc[kk][0]));
                        continue;
                    }
                }
                if (acc[kk][0] != 0.f || acc[kk][1] != 0.f || acc[kk][2] != 0.f || acc[kk][3] != 0.f) {
                    const int gz = bz + kk;
                    atomicAdd(k.gmv + ((size_t)gx * k.ng + gy) * k.ng + gz,
                              make_float4(acc[kk][0], acc[kk][1], acc[kk][2], acc[kk][3]));
                    if ((gz >> 2) != marked) {
                        mark_block(k, gx >> 2, gy >> 2, gz >> 2);
                        marked = gz >> 2;
                    }
                }
            }
        }
    }
}

// The tiled particle pass of one scene: CTA b takes tile b.
template <bool SOLIDS, int MINB, bool CDF = false>
__global__ void __launch_bounds__(Tile<CDF>::threads, MINB * 256 / Tile<CDF>::threads)
    k_particles_tiled(PK k, int mode) {
    particles_tile<SOLIDS, CDF, Tile<CDF>::threads>(k, mode, blockIdx.x);
}

// ---- batched scenes: one launch runs the same pass over many scenes ---------
// Scene s contributes ceil(n_s / TH) tiles; CTA b takes tile ctas[b].tile of scene
// ctas[b].scene, whose pass record (its working set, grid, block lists, material
// tables) it copies from the per-scene table into shared memory. The record holds
// block list 0 and the tick's first substep; `list` and `sub` select this pass's.
__device__ __forceinline__ void load_scene_pk(PK &dst, const PK *table, int scene, int list, int sub) {
    const int *src = reinterpret_cast<const int *>(table + scene);
    int *d = reinterpret_cast<int *>(&dst);
    for (int i = threadIdx.x; i < (int)(sizeof(PK) / 4); i += blockDim.x) d[i] = src[i];
    __syncthreads();
    if (threadIdx.x == 0) {
        dst.blk_list += (size_t)list * dst.bd * dst.bd * dst.bd;
        dst.blk_count += list;
        dst.sub += sub;
    }
    __syncthreads();
}

template <bool SOLIDS, int MINB, int TH>
__global__ void __launch_bounds__(TH, MINB * 256 / TH)
    k_particles_batch(const PK *table, const BatchCta *ctas, int mode, int list, int sub) {
    __shared__ PK s_k;
    const BatchCta c = ctas[blockIdx.x];
    load_scene_pk(s_k, table, c.scene, list, sub);
    particles_tile<SOLIDS, false, TH>(s_k, mode, c.tile);
}
