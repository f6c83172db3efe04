// Rigid bodies: the per-substep tail of the reference's split pipeline
// (MPM_Simulator_WARP._p2g2p_tail, mpm_solver_warp.py:1338-1367) on the device,
// including the restitution impulses the reference applies in a host numpy loop
// (_apply_rigid_restitution, :887-987).
//
// After the G2P of substep n the bodies gather the grid momentum of their particles
// (k_rigid_gather), integrate (k_rigid_integrate), take one impulse per active
// rigid surface at their deepest particle (k_rigid_contact twice for all surfaces:
// the minimum signed distance, then the lowest particle index at that distance, as
// numpy's argmin picks; then k_rigid_impulse, surface after surface), and write x,
// v, C = skew(omega), F = I back to their particles (k_rigid_update).
//
// In fused ticks the G2P of substep n and the P2G of substep n+1 are one pass, so
// rigid particles sit out that pass's scatter (PK.rigid_defer) and k_rigid_update
// deposits them after their body moved: the same order as the split pipeline,
// where the tail of substep n runs before the P2G of substep n+1.

namespace gbmpm {

struct RigidSurfaces {   // the rigid contact surfaces, by value
    gbmpm_rigid_surface s[GBMPM_MAX_RIGID_SURFACES];
    int n;
};

// The rigid particles of the tick's particle order, compacted once per tick so the
// rigid passes visit them alone (order within the list is arbitrary; nothing the
// passes compute depends on it beyond float summation order).
__global__ void k_rigid_list(const int *mat, const int *sel, int n, int *list, int *count) {
    const int lane = threadIdx.x & 31;
    for (int base = blockIdx.x * blockDim.x + threadIdx.x - lane; base < n; base += gridDim.x * blockDim.x) {
        const int p = base + lane;
        const bool on = p < n && !(sel && sel[p] != 0) && mat[p] == 8;
        const unsigned act = __ballot_sync(0xffffffffu, on);
        if (!act) continue;
        int first = 0;
        if (lane == 0) first = atomicAdd(count, __popc(act));
        first = __shfl_sync(0xffffffffu, first, 0);
        if (on) list[first + __popc(act & ((1u << lane) - 1u))] = p;
    }
}

// A warp whose rigid particles all belong to one body (the usual case: particles
// arrive block-sorted) reduces with shuffles and makes one atomic per warp;
// otherwise each particle makes its own. The loops below step whole warps.
__device__ __forceinline__ bool warp_one_body(bool on, int b, int &b0) {
    const unsigned act = __ballot_sync(0xffffffffu, on);
    if (!act) { b0 = -1; return true; }
    b0 = __shfl_sync(0xffffffffu, b, __ffs(act) - 1);
    return __all_sync(0xffffffffu, !on || b == b0);
}

// grid velocity at a rigid particle's position (the gather of rigid_g2p_accumulate)
__device__ __forceinline__ void rigid_velocity(const PK &k, const Stencil &s, float *vi) {
    vi[0] = vi[1] = vi[2] = 0.0f;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
            for (int kk = 0; kk < 3; ++kk) {
                const float w = s.w[0][i] * s.w[1][j] * s.w[2][kk];
                const float4 g = global_fetch(k, s, i, j, kk);
                vi[0] = vi[0] + g.x * w;
                vi[1] = vi[1] + g.y * w;
                vi[2] = vi[2] + g.z * w;
            }
}

// rigid_g2p_accumulate (mpm_utils.py:1369-1414): each rigid particle's momentum
// and angular momentum about its body's centre of mass, summed per body in float64
template <bool SOA>
__global__ void k_rigid_gather(PK k, const int *rlist, const int *rcount, const int *rid, const gbmpm_rigid_body *B,
                               double *acc) {
    const int lane = threadIdx.x & 31;
    const int stride = gridDim.x * blockDim.x;
    const int cnt = *rcount;
    for (int base = blockIdx.x * blockDim.x + threadIdx.x - lane; base < cnt; base += stride) {
        bool on = base + lane < cnt;
        const int p = on ? rlist[base + lane] : 0;
        const int b = on ? rid[p] : -1;
        double c6[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
        if (on) {
            float x[3], vi[3];
            fld_load<SOA, 3>(k.x, k.n, p, x);
            Stencil s;
            stencil(x, k.inv_dx, s);
            if (stencil_ok(s, k.ng, k.periodic_x)) {
                rigid_velocity(k, s, vi);
                const float m = k.mass[p];
                const float r[3] = {x[0] - B[b].x_cm[0], x[1] - B[b].x_cm[1], x[2] - B[b].x_cm[2]};
                const float pm[3] = {vi[0] * m, vi[1] * m, vi[2] * m};
                c6[0] = pm[0]; c6[1] = pm[1]; c6[2] = pm[2];
                c6[3] = r[1] * pm[2] - r[2] * pm[1];
                c6[4] = r[2] * pm[0] - r[0] * pm[2];
                c6[5] = r[0] * pm[1] - r[1] * pm[0];
            } else {
                set_status(k.status, GBMPM_FLAG_STENCIL_OOB);
                on = false;
            }
        }
        int b0;
        if (warp_one_body(on, b, b0)) {
            if (b0 < 0) continue;
#pragma unroll
            for (int c = 0; c < 6; ++c) {
                double v = c6[c];
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
                if (lane == 0) atomicAdd(acc + 6 * (size_t)b0 + c, v);
            }
        } else if (on) {
#pragma unroll
            for (int c = 0; c < 6; ++c) atomicAdd(acc + 6 * (size_t)b + c, c6[c]);
        }
    }
}

__device__ __forceinline__ void m33(const float *a, const float *b, float *c) { mm(a, b, c); }

// rigid_body_integrate (mpm_utils.py:1417-1460), one thread a body; clears the
// body's momentum sums for the next substep
__global__ void k_rigid_integrate(gbmpm_rigid_body *B, int nb, double *acc, float dt) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nb) return;
    gbmpm_rigid_body r = B[b];
    double *a = acc + 6 * (size_t)b;
    const float P[3] = {(float)a[0], (float)a[1], (float)a[2]};
    const float L[3] = {(float)a[3], (float)a[4], (float)a[5]};
#pragma unroll
    for (int c = 0; c < 6; ++c) a[c] = 0.0;
    const float M = r.mass;
    float v[3], T1[9], Iw[9], w[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) v[c] = P[c] / M;
    m33(r.R, r.inv_inertia, T1);
    mmT(T1, r.R, Iw);   // R I_body^-1 R^T
#pragma unroll
    for (int i = 0; i < 3; ++i) w[i] = Iw[3 * i] * L[0] + Iw[3 * i + 1] * L[1] + Iw[3 * i + 2] * L[2];
#pragma unroll
    for (int c = 0; c < 3; ++c) r.x_cm[c] = r.x_cm[c] + v[c] * dt;
    const float Wk[9] = {0.0f, -w[2], w[1], w[2], 0.0f, -w[0], -w[1], w[0], 0.0f};
    float WR[9], Rn[9], U[9], V[9], sg[3];
    m33(Wk, r.R, WR);
#pragma unroll
    for (int i = 0; i < 9; ++i) Rn[i] = r.R[i] + WR[i] * dt;
    svd3(Rn, U, sg, V);
    mmT(U, V, r.R);
#pragma unroll
    for (int c = 0; c < 3; ++c) { r.v_cm[c] = v[c]; r.omega[c] = w[c]; }
    B[b] = r;
}

// order-preserving map of a float64 onto unsigned 64-bit keys
__device__ __forceinline__ unsigned long long dkey(double d) {
    const unsigned long long u = (unsigned long long)__double_as_longlong(d);
    return (u >> 63) ? ~u : (u | 0x8000000000000000ull);
}
__device__ __forceinline__ double dunkey(unsigned long long k) {
    const unsigned long long u = (k >> 63) ? (k & 0x7fffffffffffffffull) : ~k;
    return __longlong_as_double((long long)u);
}

// signed distance of a rigid particle's world position from the surface plane:
// x_world = x_cm + R x_ref in float32, then (x_world - point) . normal in float64
template <bool SOA>
__device__ __forceinline__ double rigid_plane_dist(const PK &k, int p, const float *x_ref, const gbmpm_rigid_body &r,
                                                   const gbmpm_rigid_surface &sf) {
    float xr[3];
    fld_load<SOA, 3>(x_ref, k.n, p, xr);
    double d = 0.0;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        const float xw = r.x_cm[i] + (r.R[3 * i] * xr[0] + r.R[3 * i + 1] * xr[1] + r.R[3 * i + 2] * xr[2]);
        d += ((double)xw - sf.point[i]) * sf.normal[i];
    }
    return d;
}

__device__ __forceinline__ unsigned long long warp_min_u64(unsigned long long v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long w = __shfl_xor_sync(0xffffffffu, v, o);
        v = w < v ? w : v;
    }
    return v;
}

// Deepest particle of every body under every rigid surface, in two passes over the
// particles for all surfaces at once: stage 0 the smallest signed distance per
// (body, surface), stage 1 the lowest particle index (in the caller's order, through
// perm) at that distance, with the pass row. The distances use the pose after
// integration; the pushes of earlier surfaces move a body's particles together,
// which leaves each surface's deepest particle unchanged (the reference likewise
// shifts its world positions by each push). Keys: [body][surface][2].
template <bool SOA>
__global__ void k_rigid_contact(PK k, const int *rlist, const int *rcount, const int *rid, const float *x_ref,
                                const gbmpm_rigid_body *B, RigidSurfaces sf, unsigned long long *key, int stage,
                                const int *perm) {
    const int lane = threadIdx.x & 31;
    const int stride = gridDim.x * blockDim.x;
    const int cnt = *rcount;
    for (int base = blockIdx.x * blockDim.x + threadIdx.x - lane; base < cnt; base += stride) {
        const bool on = base + lane < cnt;
        const int p = on ? rlist[base + lane] : 0;
        const int b = on ? rid[p] : -1;
        int b0;
        const bool one = warp_one_body(on, b, b0);
        if (b0 < 0) continue;
        for (int q = 0; q < sf.n; ++q) {
            unsigned long long v = ~0ull;
            unsigned long long *kq = nullptr;
            if (on) {
                kq = key + 2 * ((size_t)b * sf.n + q);
                const unsigned long long dk = dkey(rigid_plane_dist<SOA>(k, p, x_ref, B[b], sf.s[q]));
                if (stage == 0) v = dk;
                else if (dk == kq[0])
                    v = ((unsigned long long)(perm ? perm[p] : p) << 32) | (unsigned long long)(unsigned)p;
            }
            if (one) {
                v = warp_min_u64(v);
                if (lane == 0 && v != ~0ull) atomicMin(key + 2 * ((size_t)b0 * sf.n + q) + stage, v);
            } else if (on && v != ~0ull) {
                atomicMin(kq + stage, v);
            }
        }
    }
}

// The restitution contacts of one body, surface after surface
// (_apply_rigid_restitution, mpm_solver_warp.py:915-975): where the deepest
// particle, shifted by the pushes so far, penetrates, push the body out by that
// depth, then apply a normal impulse -(1 + e) v_n / (1/M + ((I^-1 (r x n)) x r) . n)
// and a Coulomb-capped tangential one, in float64 with the body state rounded to
// float32 as the reference stores it. Resets the keys for the next substep.
template <bool SOA>
__global__ void k_rigid_impulse(PK k, gbmpm_rigid_body *B, int nb, const float *x_ref, unsigned long long *key,
                                RigidSurfaces sfs, int tail_sub) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nb) return;
    gbmpm_rigid_body r = B[b];
    const float xc0[3] = {r.x_cm[0], r.x_cm[1], r.x_cm[2]};   // the pose the distances were measured at
    float T1[9], Iwf[9];
    m33(r.R, r.inv_inertia, T1);
    mmT(T1, r.R, Iwf);
    double Iw[9];
#pragma unroll
    for (int i = 0; i < 9; ++i) Iw[i] = (double)Iwf[i];
    auto cross = [](const double *a, const double *c, double *o) {
        o[0] = a[1] * c[2] - a[2] * c[1];
        o[1] = a[2] * c[0] - a[0] * c[2];
        o[2] = a[0] * c[1] - a[1] * c[0];
    };
    auto mv = [&](const double *v, double *o) {
#pragma unroll
        for (int i = 0; i < 3; ++i) o[i] = Iw[3 * i] * v[0] + Iw[3 * i + 1] * v[1] + Iw[3 * i + 2] * v[2];
    };
    const double t = k.sub_time[tail_sub];
    double pacc[3] = {0.0, 0.0, 0.0};   // pushes so far
    for (int q = 0; q < sfs.n; ++q) {
        unsigned long long *kb = key + 2 * ((size_t)b * sfs.n + q);
        const unsigned long long k0 = kb[0], k1 = kb[1];
        kb[0] = ~0ull;
        kb[1] = ~0ull;
        const gbmpm_rigid_surface &sf = sfs.s[q];
        if (!(t >= sf.start_time && t < sf.end_time) || k0 == ~0ull) continue;
        const double n[3] = {sf.normal[0], sf.normal[1], sf.normal[2]};
        const double dmin = dunkey(k0) + (pacc[0] * n[0] + pacc[1] * n[1] + pacc[2] * n[2]);
        if (!(dmin < 0.0)) continue;
        const int p = (int)(unsigned)(k1 & 0xffffffffull);
        float xr[3];
        fld_load<SOA, 3>(x_ref, k.n, p, xr);
        double xc[3];
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            const float xw = xc0[i] + (r.R[3 * i] * xr[0] + r.R[3 * i + 1] * xr[1] + r.R[3 * i + 2] * xr[2]);
            const double push = -dmin * n[i];
            pacc[i] += push;
            xc[i] = (double)xw + pacc[i];
            r.x_cm[i] = (float)((double)r.x_cm[i] + push);
        }
        double rr[3], om[3], vc[3], tmp[3];
#pragma unroll
        for (int i = 0; i < 3; ++i) { rr[i] = xc[i] - (double)r.x_cm[i]; om[i] = (double)r.omega[i]; }
        cross(om, rr, tmp);
#pragma unroll
        for (int i = 0; i < 3; ++i) vc[i] = (double)r.v_cm[i] + tmp[i];
        const double vn = vc[0] * n[0] + vc[1] * n[1] + vc[2] * n[2];
        if (!(vn < 0.0)) continue;
        const double M = (double)r.mass;
        double rxn[3], qv[3], qq[3];
        cross(rr, n, rxn);
        mv(rxn, qv);
        cross(qv, rr, qq);
        const double den = 1.0 / M + (qq[0] * n[0] + qq[1] * n[1] + qq[2] * n[2]);
        const double Jn = -(1.0 + sf.restitution) * vn / den;
        double dw[3];
        const double jr[3] = {Jn * rxn[0], Jn * rxn[1], Jn * rxn[2]};
        mv(jr, dw);
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            r.v_cm[i] = (float)((double)r.v_cm[i] + (Jn / M) * n[i]);
            r.omega[i] = (float)((double)r.omega[i] + dw[i]);
        }
        if (sf.friction > 0.0) {
            double vt[3];
#pragma unroll
            for (int i = 0; i < 3; ++i) vt[i] = vc[i] - vn * n[i];
            const double vtm = sqrt(vt[0] * vt[0] + vt[1] * vt[1] + vt[2] * vt[2]);
            if (vtm > 1e-10) {
                const double th[3] = {vt[0] / vtm, vt[1] / vtm, vt[2] / vtm};
                double rxt[3], q2[3], qq2[3];
                cross(rr, th, rxt);
                mv(rxt, q2);
                cross(q2, rr, qq2);
                const double dent = 1.0 / M + (qq2[0] * th[0] + qq2[1] * th[1] + qq2[2] * th[2]);
                const double Jt = fmin(vtm / dent, sf.friction * Jn);
                const double jt[3] = {Jt * rxt[0], Jt * rxt[1], Jt * rxt[2]};
                mv(jt, dw);
#pragma unroll
                for (int i = 0; i < 3; ++i) {
                    r.v_cm[i] = (float)((double)r.v_cm[i] - (Jt / M) * th[i]);
                    r.omega[i] = (float)((double)r.omega[i] - dw[i]);
                }
            }
        }
    }
    B[b] = r;
}

// rigid_particle_update (mpm_utils.py:1463-1493): x = x_cm + R x_ref, v = v_cm +
// omega x r, C = skew(omega), F = I; with `deposit` the particle's P2G follows
// (a rigid particle carries no stress)
template <bool SOA>
__global__ void k_rigid_update(PK k, const int *rlist, const int *rcount, const int *rid, const float *x_ref,
                               const gbmpm_rigid_body *B, int deposit) {
    const int cnt = *rcount;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < cnt; i += gridDim.x * blockDim.x) {
        const int p = rlist[i];
        const gbmpm_rigid_body &r = B[rid[p]];
        float xr[3], x[3], v[3];
        fld_load<SOA, 3>(x_ref, k.n, p, xr);
#pragma unroll
        for (int i = 0; i < 3; ++i)
            x[i] = r.x_cm[i] + (r.R[3 * i] * xr[0] + r.R[3 * i + 1] * xr[1] + r.R[3 * i + 2] * xr[2]);
        const float rr[3] = {x[0] - r.x_cm[0], x[1] - r.x_cm[1], x[2] - r.x_cm[2]};
        v[0] = r.v_cm[0] + (r.omega[1] * rr[2] - r.omega[2] * rr[1]);
        v[1] = r.v_cm[1] + (r.omega[2] * rr[0] - r.omega[0] * rr[2]);
        v[2] = r.v_cm[2] + (r.omega[0] * rr[1] - r.omega[1] * rr[0]);
        const float C[9] = {0.0f, -r.omega[2], r.omega[1], r.omega[2], 0.0f, -r.omega[0], -r.omega[1], r.omega[0], 0.0f};
        const float I[9] = {1.0f, 0.0f, 0.0f, 0.0f, 1.0f, 0.0f, 0.0f, 0.0f, 1.0f};
        fld_store<SOA, 3>(k.x, k.n, p, x);
        fld_store<SOA, 3>(k.v, k.n, p, v);
        fld_store<SOA, 9>(k.C, k.n, p, C);
        fld_store<SOA, 9>(k.F, k.n, p, I);
        if (deposit) {
            Stencil s;
            stencil(x, k.inv_dx, s);
            if (!stencil_ok(s, k.ng, k.periodic_x)) {
                set_status(k.status, GBMPM_FLAG_STENCIL_OOB);
                continue;
            }
            const float S[9] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
            global_deposit_all(k, s, p, v, C, S);
        }
    }
}

}  // namespace gbmpm
