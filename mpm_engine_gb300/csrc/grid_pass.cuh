// The per-tick working set (block-sorted copy of the particles), the grid pass
// with every collider, and the CPIC (CDF) stamping kernels.
//
// Included by gbmpm.cu inside namespace gbmpm, after the constants and helpers
// and before the host code; it is not a standalone header.

// ---- per-tick working set: block-sorted copy of the particles --------------
// key = (4^3 block of the stencil base, cell within the block); positions are
// clamped into the grid so every particle gets a key. SOA reads the working copy's
// own positions (a re-sort inside a tick), else the caller's records.
template <bool SOA>
__global__ void k_cell_keys(const float *x, int n, float inv_dx, int ng, int bd, unsigned long long *keys,
                            int *idx) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    int b[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        float g = x[SOA ? (size_t)a * n + p : 3 * (size_t)p + a] * inv_dx - 0.5f;
        int c = isfinite(g) ? (int)floorf(fminf(fmaxf(g, 0.0f), (float)(ng - 1))) : 0;
        b[a] = c;
    }
    unsigned blk = (unsigned)(((b[0] >> 2) * bd + (b[1] >> 2)) * bd + (b[2] >> 2));
    unsigned cell = (unsigned)(((b[0] & 3) << 4) | ((b[1] & 3) << 2) | (b[2] & 3));
    keys[p] = ((unsigned long long)blk << 6) | cell;
    idx[p] = p;
}

struct WsField {
    float *ext;
    float *ws;
    int width;
    int back;   // copied back to the caller's buffer at the end of the tick
};
constexpr int kMaxWsFields = 21;   // the 20 particle fields, plus the CPIC scan cache a re-sort carries
struct WsTable {
    WsField f[kMaxWsFields];
    int nf;
};

// caller AoS records -> working-copy SoA components, in block-sorted order
__global__ void k_ws_gather(WsTable T, const int *perm, int n) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const size_t src = (size_t)perm[i];
    for (int f = 0; f < T.nf; ++f) {
        const int w = T.f[f].width;
        const float *a = T.f[f].ext + src * w;
        float *b = T.f[f].ws + i;
        for (int c = 0; c < w; ++c) b[(size_t)c * n] = a[c];
    }
}

// working copy -> the other working copy, re-sorted inside a tick: row i takes row
// idx[i] of every field, and the map from working rows to caller particles follows
__global__ void k_ws_permute(WsTable from, WsTable to, const int *idx, const int *perm_in, int *perm_out, int n) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const size_t src = (size_t)idx[i];
    for (int f = 0; f < from.nf; ++f) {
        const int w = from.f[f].width;
        const float *a = from.f[f].ws + src;
        float *b = to.f[f].ws + i;
        for (int c = 0; c < w; ++c) b[(size_t)c * n] = a[(size_t)c * n];
    }
    perm_out[i] = perm_in[src];
}

__global__ void k_ws_scatter(WsTable T, const int *perm, int n) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const size_t dst = (size_t)perm[i];
    for (int f = 0; f < T.nf; ++f) {
        if (!T.f[f].back) continue;
        const int w = T.f[f].width;
        const float *a = T.f[f].ws + i;
        float *b = T.f[f].ext + dst * w;
        for (int c = 0; c < w; ++c) b[c] = a[(size_t)c * n];
    }
}

// -------------------------------------------------------- grid pass --------
// capped_cylinder_sdf / revolved_glass_sdf (mpm_solver_warp.py:29-57). The cup's
// contact normal is a central difference of this SDF over half a cell, which
// cancels all but about 1e-2 of its value: so every operation here and in the cup
// branch rounds once (no contraction into FMAs), in the order the fp32 statement of
// the collider writes it, and the normal carries no rounding of its own.
__device__ __forceinline__ float dot3_rn(float a0, float b0, float a1, float b1, float a2, float b2) {
    return __fadd_rn(__fadd_rn(__fmul_rn(a0, b0), __fmul_rn(a1, b1)), __fmul_rn(a2, b2));
}
__device__ __forceinline__ float capped_cyl(float r, float z, float rad, float z0, float z1) {
    const float zc = __fmul_rn(0.5f, __fadd_rn(z0, z1)), hh = __fmul_rn(0.5f, __fsub_rn(z1, z0));
    const float dr = __fsub_rn(r, rad), dz = __fsub_rn(fabsf(__fsub_rn(z, zc)), hh);
    const float dro = fmaxf(dr, 0.0f), dzo = fmaxf(dz, 0.0f);
    return __fadd_rn(__fsqrt_rn(__fadd_rn(__fmul_rn(dro, dro), __fmul_rn(dzo, dzo))), fminf(fmaxf(dr, dz), 0.0f));
}
__device__ __forceinline__ float glass_sdf(float l0, float l1, float l2, const ColDev &c) {
    const float r = __fsqrt_rn(__fadd_rn(__fmul_rn(l0, l0), __fmul_rn(l1, l1)));
    const float d_outer = capped_cyl(r, l2, c.outer_r, -c.half_h, c.half_h);
    const float d_cav = __fsub_rn(capped_cyl(r, l2, __fsub_rn(c.inner_r, c.fillet), __fadd_rn(c.floor_z, c.fillet),
                                             __fadd_rn(c.half_h, c.outer_r)),
                                  c.fillet);
    return fmaxf(d_outer, -d_cav);
}
__device__ __forceinline__ float trilerp(const float *vals, int res, float f0, float f1, float f2, int stride,
                                         int comp) {
    float fi = fminf(fmaxf(f0, 0.0f), (float)res - 1.0001f);
    float fj = fminf(fmaxf(f1, 0.0f), (float)res - 1.0001f);
    float fk = fminf(fmaxf(f2, 0.0f), (float)res - 1.0001f);
    int i = (int)floorf(fi), j = (int)floorf(fj), kk = (int)floorf(fk);
    float tx = fi - (float)i, ty = fj - (float)j, tz = fk - (float)kk;
    auto at = [&](int a, int b, int c) { return __ldg(vals + ((((size_t)a * res + b) * res + c) * stride + comp)); };
    float c00 = at(i, j, kk) * (1.0f - tx) + at(i + 1, j, kk) * tx;
    float c01 = at(i, j, kk + 1) * (1.0f - tx) + at(i + 1, j, kk + 1) * tx;
    float c10 = at(i, j + 1, kk) * (1.0f - tx) + at(i + 1, j + 1, kk) * tx;
    float c11 = at(i, j + 1, kk + 1) * (1.0f - tx) + at(i + 1, j + 1, kk + 1) * tx;
    float c0 = c00 * (1.0f - ty) + c10 * ty;
    float c1 = c01 * (1.0f - ty) + c11 * ty;
    return c0 * (1.0f - tz) + c1 * tz;
}
// quaternion rotation x(2w^2-1) +/- 2w (q x x) + 2 q (q . x)
__device__ __forceinline__ void qrot(const float *q, const float *x, float *out, bool inv) {
    float w = q[3];
    float c = 2.0f * w * w - 1.0f;
    float cx = q[1] * x[2] - q[2] * x[1], cy = q[2] * x[0] - q[0] * x[2], cz = q[0] * x[1] - q[1] * x[0];
    float d = q[0] * x[0] + q[1] * x[1] + q[2] * x[2];
    float sgn = inv ? -2.0f * w : 2.0f * w;
    out[0] = x[0] * c + cx * sgn + q[0] * d * 2.0f;
    out[1] = x[1] * c + cy * sgn + q[1] * d * 2.0f;
    out[2] = x[2] * c + cz * sgn + q[2] * d * 2.0f;
}

// ---- CPIC (CDF) stamping (mpm_solver_warp.py:94-183) ---------------------------
// The stamp decides node tags by thresholds on interpolated fields, so its
// arithmetic is spelled out with round-to-nearest intrinsics: no contraction into
// FMAs, every operation rounded once, as in the fp32 statement of the algorithm.
struct CdfBox {
    int lo[3], hi[3];   // node range [lo, hi)
};

__device__ __forceinline__ float trilerp_rn(const float *vals, int res, float f0, float f1, float f2) {
    const float top = (float)res - 1.0001f;
    float fi = fminf(fmaxf(f0, 0.0f), top), fj = fminf(fmaxf(f1, 0.0f), top), fk = fminf(fmaxf(f2, 0.0f), top);
    int i = (int)floorf(fi), j = (int)floorf(fj), kk = (int)floorf(fk);
    float tx = __fsub_rn(fi, (float)i), ty = __fsub_rn(fj, (float)j), tz = __fsub_rn(fk, (float)kk);
    auto at = [&](int a, int b, int c) { return __ldg(vals + (((size_t)a * res + b) * res + c)); };
    auto lerp = [](float a, float b, float t) { return __fadd_rn(__fmul_rn(a, __fsub_rn(1.0f, t)), __fmul_rn(b, t)); };
    float c00 = lerp(at(i, j, kk), at(i + 1, j, kk), tx);
    float c01 = lerp(at(i, j, kk + 1), at(i + 1, j, kk + 1), tx);
    float c10 = lerp(at(i, j + 1, kk), at(i + 1, j + 1, kk), tx);
    float c11 = lerp(at(i, j + 1, kk + 1), at(i + 1, j + 1, kk + 1), tx);
    return lerp(lerp(c00, c10, ty), lerp(c01, c11, ty), tz);
}

// inverse quaternion rotation x(2w^2-1) - 2w (q x x) + 2 q (q . x), rounded per operation
__device__ __forceinline__ void qrot_inv_rn(const float *q, const float *x, float *out) {
    const float w = q[3];
    const float c = __fsub_rn(__fmul_rn(__fmul_rn(2.0f, w), w), 1.0f);
    const float cr[3] = {__fsub_rn(__fmul_rn(q[1], x[2]), __fmul_rn(q[2], x[1])),
                         __fsub_rn(__fmul_rn(q[2], x[0]), __fmul_rn(q[0], x[2])),
                         __fsub_rn(__fmul_rn(q[0], x[1]), __fmul_rn(q[1], x[0]))};
    const float d = __fadd_rn(__fadd_rn(__fmul_rn(q[0], x[0]), __fmul_rn(q[1], x[1])), __fmul_rn(q[2], x[2]));
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        float ta = __fmul_rn(x[a], c);
        float tb = __fmul_rn(__fmul_rn(cr[a], w), 2.0f);
        float td = __fmul_rn(__fmul_rn(q[a], d), 2.0f);
        out[a] = __fadd_rn(__fsub_rn(ta, tb), td);
    }
}

// Folds the per-CTA partial reactions into the per-lane totals and clears them:
// one warp per component.
__global__ void k_cdf_wrench_fold(double *partial, int nctas, double *total) {
    const int comp = blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;   // lane * 6 + axis
    if (comp >= 6 * GBMPM_MAX_CDF) return;
    const int l = threadIdx.x & 31;
    double acc = 0.0;
    for (int c = l; c < nctas; c += 32) {
        double *q = partial + (size_t)c * 6 * GBMPM_MAX_CDF + comp;
        acc += *q;
        *q = 0.0;
    }
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (l == 0) total[comp] += acc;
}

__device__ __forceinline__ bool box_node(const CdfBox &b, long long idx, int &x, int &y, int &z) {
    const long long ny = b.hi[1] - b.lo[1], nz = b.hi[2] - b.lo[2];
    z = b.lo[2] + (int)(idx % nz);
    long long r = idx / nz;
    y = b.lo[1] + (int)(r % ny);
    x = b.lo[0] + (int)(r / ny);
    return x < b.hi[0];
}

__device__ __forceinline__ long long box_volume(const CdfBox &b) {
    return (long long)(b.hi[0] - b.lo[0]) * (b.hi[1] - b.lo[1]) * (b.hi[2] - b.lo[2]);
}

// cdf_zero_tags over a box
__global__ void k_cdf_clear(int *tag, float *d, CdfBox b, int ng) {
    const long long total = box_volume(b);
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total; i += (long long)gridDim.x * blockDim.x) {
        int x, y, z;
        if (!box_node(b, i, x, y, z)) break;
        size_t id = ((size_t)x * ng + y) * ng + z;
        tag[id] = 0;
        d[id] = 1.0e9f;
    }
}

// cdf_copy_prev over a box
__global__ void k_cdf_copy_prev(const int *tag, const float *d, int *tag_prev, float *d_prev, CdfBox b, int ng) {
    const long long total = box_volume(b);
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total; i += (long long)gridDim.x * blockDim.x) {
        int x, y, z;
        if (!box_node(b, i, x, y, z)) break;
        size_t id = ((size_t)x * ng + y) * ng + z;
        tag_prev[id] = tag[id];
        d_prev[id] = d[id];
    }
}

struct CdfStamp {
    const float *values, *valid;
    int res, lane, ng;
    float origin[3], cell, center[3], quat[4], band;
    float dx;
    CdfBox box;
    int *tag;
    float *d;
};

// cdf_stamp for one lane: a node within `band` of the surface, where the field is
// valid, gains the lane's valid bit and side bit; the nearest lane owns the node.
__global__ void k_cdf_stamp(CdfStamp a) {
    const long long total = box_volume(a.box);
    const float rf = (float)a.res - 1.0f;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total; i += (long long)gridDim.x * blockDim.x) {
        int x, y, z;
        if (!box_node(a.box, i, x, y, z)) break;
        const float rel[3] = {__fsub_rn(__fmul_rn((float)x, a.dx), a.center[0]),
                              __fsub_rn(__fmul_rn((float)y, a.dx), a.center[1]),
                              __fsub_rn(__fmul_rn((float)z, a.dx), a.center[2])};
        float body[3];
        qrot_inv_rn(a.quat, rel, body);
        const float f0 = __fdiv_rn(__fsub_rn(body[0], a.origin[0]), a.cell);
        const float f1 = __fdiv_rn(__fsub_rn(body[1], a.origin[1]), a.cell);
        const float f2 = __fdiv_rn(__fsub_rn(body[2], a.origin[2]), a.cell);
        if (f0 < 0.0f || f1 < 0.0f || f2 < 0.0f || f0 > rf || f1 > rf || f2 > rf) continue;
        if (trilerp_rn(a.valid, a.res, f0, f1, f2) < 0.999f) continue;
        const float dd = trilerp_rn(a.values, a.res, f0, f1, f2);
        const float ud = fabsf(dd);
        if (ud > a.band) continue;
        const size_t id = ((size_t)x * a.ng + y) * a.ng + z;
        int t = a.tag[id] | (1 << (2 * a.lane)) | ((dd >= 0.0f ? 1 : 0) << (2 * a.lane + 1));
        if (ud < a.d[id]) {
            a.d[id] = ud;
            t = (t & ~(3 << kCdfOwnerShift)) | (a.lane << kCdfOwnerShift);
        }
        a.tag[id] = t;
    }
}

__device__ __forceinline__ bool in_box(const CdfBox &b, int x, int y, int z) {
    return x >= b.lo[0] && x < b.hi[0] && y >= b.lo[1] && y < b.hi[1] && z >= b.lo[2] && z < b.hi[2];
}

// One lane's stamp of node (x,y,z) into the node's running (tag, distance): the
// arithmetic of k_cdf_stamp on registers.
__device__ __forceinline__ void stamp_node(const CdfStamp &a, int x, int y, int z, int &t, float &d) {
    const float rf = (float)a.res - 1.0f;
    const float rel[3] = {__fsub_rn(__fmul_rn((float)x, a.dx), a.center[0]),
                          __fsub_rn(__fmul_rn((float)y, a.dx), a.center[1]),
                          __fsub_rn(__fmul_rn((float)z, a.dx), a.center[2])};
    float body[3];
    qrot_inv_rn(a.quat, rel, body);
    const float f0 = __fdiv_rn(__fsub_rn(body[0], a.origin[0]), a.cell);
    const float f1 = __fdiv_rn(__fsub_rn(body[1], a.origin[1]), a.cell);
    const float f2 = __fdiv_rn(__fsub_rn(body[2], a.origin[2]), a.cell);
    if (f0 < 0.0f || f1 < 0.0f || f2 < 0.0f || f0 > rf || f1 > rf || f2 > rf) return;
    if (trilerp_rn(a.valid, a.res, f0, f1, f2) < 0.999f) return;
    const float dd = trilerp_rn(a.values, a.res, f0, f1, f2);
    const float ud = fabsf(dd);
    if (ud > a.band) return;
    t |= (1 << (2 * a.lane)) | ((dd >= 0.0f ? 1 : 0) << (2 * a.lane + 1));
    if (ud < d) {
        d = ud;
        t = (t & ~(3 << kCdfOwnerShift)) | (a.lane << kCdfOwnerShift);
    }
}

// The whole restamp of a substep in one launch, one warp per 4^3 block of `bb`
// (two nodes a lane): the previous grids catch up with the current ones over
// `stale`; nodes of `box` are cleared and stamped by every listed lane in lane
// order (the nearest lane owns a node, the first on a tie); with `post_copy` the
// previous grids then take the new stamp over `box`; blocks of `mb` get their
// mask, the OR of current and previous tags over the block's nodes. Equivalent to
// copy_prev(stale), clear(box), stamp(lane) for each lane, [copy_prev(box)],
// block_mask(mb) in sequence, as each node depends on itself alone.
struct CdfRestamp {
    CdfStamp lane[GBMPM_MAX_CDF];   // per lane: field, pose and its clip of `box`
    int nl, post_copy, ng, nb;
    CdfBox box, stale, bb, mb;
    int *tag, *tag_prev, *block;
    float *d, *d_prev;
};

__global__ void k_cdf_restamp(CdfRestamp a) {
    const int lane = threadIdx.x & 31;
    const int wpb = blockDim.x >> 5;
    const int e1 = a.bb.hi[1] - a.bb.lo[1], e2 = a.bb.hi[2] - a.bb.lo[2];
    const long long nblk = (long long)(a.bb.hi[0] - a.bb.lo[0]) * e1 * e2;
    const int ng = a.ng;
    for (long long w = (long long)blockIdx.x * wpb + (threadIdx.x >> 5); w < nblk; w += (long long)gridDim.x * wpb) {
        const int bi = a.bb.lo[0] + (int)(w / ((long long)e1 * e2));
        const int r = (int)(w % ((long long)e1 * e2));
        const int bj = a.bb.lo[1] + r / e2, bk = a.bb.lo[2] + r % e2;
        int occ = 0;
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int n = lane + 32 * h;
            const int x = (bi << 2) + (n >> 4), y = (bj << 2) + ((n >> 2) & 3), z = (bk << 2) + (n & 3);
            if (x >= ng || y >= ng || z >= ng) continue;
            const size_t id = ((size_t)x * ng + y) * ng + z;
            int t = a.tag[id], tp = a.tag_prev[id];
            float d = a.d[id];
            if (in_box(a.stale, x, y, z)) {
                a.tag_prev[id] = t;
                a.d_prev[id] = d;
                tp = t;
            }
            if (in_box(a.box, x, y, z)) {
                t = 0;
                d = 1.0e9f;
                for (int l = 0; l < a.nl; ++l)
                    if (in_box(a.lane[l].box, x, y, z)) stamp_node(a.lane[l], x, y, z, t, d);
                a.tag[id] = t;
                a.d[id] = d;
                if (a.post_copy) {
                    a.tag_prev[id] = t;
                    a.d_prev[id] = d;
                    tp = t;
                }
            }
            occ |= t | tp;
        }
        occ = __reduce_or_sync(0xffffffffu, occ);
        if (lane == 0 && in_box(a.mb, bi, bj, bk)) a.block[((size_t)bi * a.nb + bj) * a.nb + bk] = occ;
    }
}

// cdf_block_mask over a box of 4^3 blocks: OR of the current and previous tags
__global__ void k_cdf_block_mask(const int *tag, const int *tag_prev, int *block, CdfBox bb, int nb, int ng) {
    const long long total = box_volume(bb);
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total; i += (long long)gridDim.x * blockDim.x) {
        int bi, bj, bk;
        if (!box_node(bb, i, bi, bj, bk)) break;
        int occ = 0;
        for (int a = 0; a < 4; ++a)
            for (int b = 0; b < 4; ++b)
                for (int c = 0; c < 4; ++c) {
                    int ci = (bi << 2) + a, cj = (bj << 2) + b, ck = (bk << 2) + c;
                    if (ci < ng && cj < ng && ck < ng) {
                        size_t id = ((size_t)ci * ng + cj) * ng + ck;
                        occ |= tag[id] | tag_prev[id];
                    }
                }
        block[((size_t)bi * nb + bj) * nb + bk] = occ;
    }
}

// Applies collider c to node (gx,gy,gz) of mass m (> 0); adds the reaction
// impulse and torque into acc[6].
__device__ __forceinline__ void collide(const ColDev &c, const PoseRec &P, int gx, int gy, int gz, float m,
                                        float *v, const GK &k, float *acc) {
    const float dx = k.dx;
    switch (c.kind) {
    case GBMPM_COLLIDER_PLANE: {  // mpm_solver_warp.py:1929-1992 (each operation rounded once, as written)
        const float o0 = __fsub_rn(__fmul_rn((float)gx, dx), P.p[0]), o1 = __fsub_rn(__fmul_rn((float)gy, dx), P.p[1]),
                    o2 = __fsub_rn(__fmul_rn((float)gz, dx), P.p[2]);
        const float *n = c.normal;
        const float dp = dot3_rn(o0, n[0], o1, n[1], o2, n[2]);
        if (dp < 0.0f) {
            if (c.surface == 0) {
                v[0] = v[1] = v[2] = 0.0f;
            } else if (c.surface == 11) {
                if ((float)gz * dx < 0.4f || (float)gz * dx > 0.53f) { v[0] = v[1] = v[2] = 0.0f; }
                else { v[0] *= 0.3f; v[1] = 0.0f; v[2] *= 0.3f; }
            } else {
                const float nc = dot3_rn(v[0], n[0], v[1], n[1], v[2], n[2]);
                const float sub = (c.surface == 1) ? nc : fminf(nc, 0.0f);
                float w[3] = {__fsub_rn(v[0], __fmul_rn(n[0], sub)), __fsub_rn(v[1], __fmul_rn(n[1], sub)),
                              __fsub_rn(v[2], __fmul_rn(n[2], sub))};
                const float len = __fsqrt_rn(dot3_rn(w[0], w[0], w[1], w[1], w[2], w[2]));
                if (nc < 0.0f && len > 1e-20f) {   // the unit tangent times the Coulomb-reduced speed
                    const float t = __fadd_rn(len, __fmul_rn(nc, c.friction));
                    const float sp = (0.0f < t) ? t : 0.0f;
#pragma unroll
                    for (int a = 0; a < 3; ++a) w[a] = __fmul_rn(__fdiv_rn(w[a], len), sp);
                }
                v[0] = w[0]; v[1] = w[1]; v[2] = w[2];
            }
        }
        return;
    }
    case GBMPM_COLLIDER_BOX: {  // mpm_solver_warp.py:2053-2088
        if (P.mode == 2) { v[0] = v[1] = v[2] = 0.0f; return; }
        const float o0 = __fsub_rn(__fmul_rn((float)gx, dx), P.p[0]), o1 = __fsub_rn(__fmul_rn((float)gy, dx), P.p[1]),
                    o2 = __fsub_rn(__fmul_rn((float)gz, dx), P.p[2]);
        if (fabsf(o0) < c.size[0] && fabsf(o1) < c.size[1] && fabsf(o2) < c.size[2]) {
#pragma unroll
            for (int a = 0; a < 3; ++a) { acc[a] += m * (v[a] - c.vel[a]); v[a] = c.vel[a]; }
        }
        return;
    }
    case GBMPM_COLLIDER_CUP: {  // mpm_solver_warp.py:2161-2225
        const float rel[3] = {__fsub_rn(__fmul_rn((float)gx, dx), P.p[0]), __fsub_rn(__fmul_rn((float)gy, dx), P.p[1]),
                              __fsub_rn(__fmul_rn((float)gz, dx), P.p[2])};
        const float *R = P.r;
        const float l0 = dot3_rn(R[0], rel[0], R[3], rel[1], R[6], rel[2]);
        const float l1 = dot3_rn(R[1], rel[0], R[4], rel[1], R[7], rel[2]);
        const float l2 = dot3_rn(R[2], rel[0], R[5], rel[1], R[8], rel[2]);
        const float sdf = glass_sdf(l0, l1, l2, c);
        if (sdf < c.band_c) {
            const float *o = c.omega;
            const float vs[3] = {__fadd_rn(c.vel[0], __fsub_rn(__fmul_rn(o[1], rel[2]), __fmul_rn(o[2], rel[1]))),
                                 __fadd_rn(c.vel[1], __fsub_rn(__fmul_rn(o[2], rel[0]), __fmul_rn(o[0], rel[2]))),
                                 __fadd_rn(c.vel[2], __fsub_rn(__fmul_rn(o[0], rel[1]), __fmul_rn(o[1], rel[0])))};
            float vn_[3] = {vs[0], vs[1], vs[2]};
            if (sdf > -c.sticky) {
                vn_[0] = v[0]; vn_[1] = v[1]; vn_[2] = v[2];
                const float h = __fmul_rn(0.25f, dx);
                float n0 = __fsub_rn(glass_sdf(__fadd_rn(l0, h), l1, l2, c), glass_sdf(__fsub_rn(l0, h), l1, l2, c));
                float n1 = __fsub_rn(glass_sdf(l0, __fadd_rn(l1, h), l2, c), glass_sdf(l0, __fsub_rn(l1, h), l2, c));
                float n2 = __fsub_rn(glass_sdf(l0, l1, __fadd_rn(l2, h), c), glass_sdf(l0, l1, __fsub_rn(l2, h), c));
                const float nl = __fsqrt_rn(dot3_rn(n0, n0, n1, n1, n2, n2));
                if (nl > 1.0e-12f) {
                    n0 = __fdiv_rn(n0, nl); n1 = __fdiv_rn(n1, nl); n2 = __fdiv_rn(n2, nl);
                    const float n[3] = {dot3_rn(R[0], n0, R[1], n1, R[2], n2), dot3_rn(R[3], n0, R[4], n1, R[5], n2),
                                        dot3_rn(R[6], n0, R[7], n1, R[8], n2)};
                    const float vr[3] = {__fsub_rn(v[0], vs[0]), __fsub_rn(v[1], vs[1]), __fsub_rn(v[2], vs[2])};
                    const float vn = dot3_rn(vr[0], n[0], vr[1], n[1], vr[2], n[2]);
                    if (vn < 0.0f) {
                        float vt[3] = {__fsub_rn(vr[0], __fmul_rn(n[0], vn)), __fsub_rn(vr[1], __fmul_rn(n[1], vn)),
                                       __fsub_rn(vr[2], __fmul_rn(n[2], vn))};
                        const float vtl = __fsqrt_rn(dot3_rn(vt[0], vt[0], vt[1], vt[1], vt[2], vt[2]));
                        if (vtl > 1.0e-20f) {   // the unit tangent times the Coulomb-reduced speed
                            const float sp = fmaxf(__fadd_rn(vtl, __fmul_rn(c.friction, vn)), 0.0f);
#pragma unroll
                            for (int a = 0; a < 3; ++a) vt[a] = __fmul_rn(__fdiv_rn(vt[a], vtl), sp);
                        }
#pragma unroll
                        for (int a = 0; a < 3; ++a) vn_[a] = __fadd_rn(vs[a], vt[a]);
                    }
                }
            }
            const float imp[3] = {__fmul_rn(__fsub_rn(v[0], vn_[0]), m), __fmul_rn(__fsub_rn(v[1], vn_[1]), m),
                                  __fmul_rn(__fsub_rn(v[2], vn_[2]), m)};
            acc[0] += imp[0]; acc[1] += imp[1]; acc[2] += imp[2];
            acc[3] += rel[1] * imp[2] - rel[2] * imp[1];
            acc[4] += rel[2] * imp[0] - rel[0] * imp[2];
            acc[5] += rel[0] * imp[1] - rel[1] * imp[0];
            v[0] = vn_[0]; v[1] = vn_[1]; v[2] = vn_[2];
        }
        return;
    }
    case GBMPM_COLLIDER_WALLS: {  // mpm_solver_warp.py:2294-2359
        const int pad = 3;
        const int n = k.ng;
        if (gx < pad && v[0] < 0) v[0] = 0.0f;
        if (gx >= n - pad && v[0] > 0) v[0] = 0.0f;
        if (gy < pad && v[1] < 0) v[1] = 0.0f;
        if (gy >= n - pad && v[1] > 0) v[1] = 0.0f;
        if (gz < pad && v[2] < 0) v[2] = 0.0f;
        if (gz >= n - pad && v[2] > 0) v[2] = 0.0f;
        return;
    }
    case GBMPM_COLLIDER_SDF: {  // mpm_solver_warp.py:2680-2736
        float rel[3] = {(float)gx * dx - P.p[0], (float)gy * dx - P.p[1], (float)gz * dx - P.p[2]};
        float body[3];
        qrot(P.q, rel, body, true);
        float f0 = (body[0] - c.origin[0]) / c.cell, f1 = (body[1] - c.origin[1]) / c.cell,
              f2 = (body[2] - c.origin[2]) / c.cell;
        float rf = (float)c.sdf_res - 1.0f;
        if (!(f0 >= 0.0f && f1 >= 0.0f && f2 >= 0.0f && f0 <= rf && f1 <= rf && f2 <= rf)) return;
        float sd = trilerp(c.sdf_val, c.sdf_res, f0, f1, f2, 1, 0);
        if (sd <= c.band) {
            float g[3] = {trilerp(c.sdf_grad, c.sdf_res, f0, f1, f2, 3, 0), trilerp(c.sdf_grad, c.sdf_res, f0, f1, f2, 3, 1),
                          trilerp(c.sdf_grad, c.sdf_res, f0, f1, f2, 3, 2)};
            float gl = sqrtf(g[0] * g[0] + g[1] * g[1] + g[2] * g[2]);
            if (gl > 1.0e-12f) {
                g[0] /= gl; g[1] /= gl; g[2] /= gl;
                float n[3];
                qrot(P.q, g, n, false);
                float vs[3] = {c.vel[0] + (c.omega[1] * rel[2] - c.omega[2] * rel[1]),
                               c.vel[1] + (c.omega[2] * rel[0] - c.omega[0] * rel[2]),
                               c.vel[2] + (c.omega[0] * rel[1] - c.omega[1] * rel[0])};
                float vr[3] = {v[0] - vs[0], v[1] - vs[1], v[2] - vs[2]};
                float vn = vr[0] * n[0] + vr[1] * n[1] + vr[2] * n[2];
                float nv[3] = {v[0], v[1], v[2]};
                if (c.surface == 0) {
                    nv[0] = vs[0]; nv[1] = vs[1]; nv[2] = vs[2];
                } else if (c.surface == 1) {
#pragma unroll
                    for (int a = 0; a < 3; ++a) nv[a] = vs[a] + (vr[a] - vn * n[a]);
                } else if (vn < 0.0f) {
                    float vt[3] = {vr[0] - vn * n[0], vr[1] - vn * n[1], vr[2] - vn * n[2]};
                    float tl = sqrtf(vt[0] * vt[0] + vt[1] * vt[1] + vt[2] * vt[2]);
                    if (tl > 1.0e-12f) {
                        float sc = fmaxf(0.0f, tl + c.friction * vn) / tl;
                        vt[0] *= sc; vt[1] *= sc; vt[2] *= sc;
                    }
#pragma unroll
                    for (int a = 0; a < 3; ++a) nv[a] = vs[a] + vt[a];
                }
                float imp[3] = {m * (v[0] - nv[0]), m * (v[1] - nv[1]), m * (v[2] - nv[2])};
                acc[0] += imp[0]; acc[1] += imp[1]; acc[2] += imp[2];
                acc[3] += rel[1] * imp[2] - rel[2] * imp[1];
                acc[4] += rel[2] * imp[0] - rel[0] * imp[2];
                acc[5] += rel[0] * imp[1] - rel[1] * imp[0];
                v[0] = nv[0]; v[1] = nv[1]; v[2] = nv[2];
            }
        }
        return;
    }
    default: return;
    }
}

// Grid pass over the active-block list: normalize + gravity (mpm_utils.py:927-941),
// damping (:1287-1295), every collider in list order, then clear the scatter
// target and the block flags for the next particle pass.
// The grid update over a scene's active-block list, by CTA `cta` of the `nctas`
// CTAs given to that scene.
__device__ __forceinline__ void grid_update(const GK &k, int cta, int nctas) {
    __shared__ ColDev s_cols[kMaxCol];
    __shared__ PoseRec s_pose[kMaxCol];
    __shared__ float s_acc[kMaxCol][6];
    // a cup's glass lies inside the sphere of radius sqrt(outer_r^2 + half_h^2) about
    // its centre, so its SDF exceeds the contact band at every node of a 4^3 block
    // whose centre is farther than that radius plus the band plus the block's
    // half-diagonal (1.5 sqrt(3) dx < 3 dx): such a block skips the cup, exactly
    __shared__ float s_cull[kMaxCol];
    const int t = threadIdx.x;
    for (int i = t; i < k.ncol; i += blockDim.x) {
        s_cols[i] = k.cols[i];
        s_pose[i] = k.poses[i];
        const ColDev &c = k.cols[i];
        const float rc = sqrtf(c.outer_r * c.outer_r + c.half_h * c.half_h) + c.band_c + 3.0f * k.dx;
        s_cull[i] = (c.kind == GBMPM_COLLIDER_CUP) ? rc * rc : -1.0f;
    }
    for (int i = t; i < k.ncol * 6; i += blockDim.x) s_acc[i / 6][i % 6] = 0.0f;
    pdl_wait();   // the particle pass before this one deposits into gmv and fills the block list
    pdl_trigger();
    const int per = blockDim.x / 64;
    const int stride = nctas * per;
    const int first = cta * per + t / 64;
    // the count and this thread's first list entry are read together: the list holds
    // bd^3 entries, and an entry at or past the count is never used
    const int count = *k.blk_count_read;
    int b_next = (first < k.bd * k.bd * k.bd) ? k.blk_list[first] : 0;
    if (cta == 0 && t == 0) *k.blk_count_reset = 0;
    __syncthreads();
    const int lane = t & 31;
    for (int item = first; item < count; item += stride) {
        bool valid = true;
        int b = b_next;
        if (item + stride < count) b_next = k.blk_list[item + stride];   // next iteration's entry, in flight now
        int bz = b % k.bd, r = b / k.bd, by = r % k.bd, bx = r / k.bd;
        int cell = t & 63;
        int gx = bx * 4 + (cell >> 4), gy = by * 4 + ((cell >> 2) & 3), gz = bz * 4 + (cell & 3);
        valid = valid && gx < k.ng && gy < k.ng && gz < k.ng;
        float m = 0.0f;
        float v[3] = {0.f, 0.f, 0.f};
        size_t id = 0;
        if (valid) {
            id = ((size_t)gx * k.ng + gy) * k.ng + gz;
            float4 mv = k.gmv[id];
            m = mv.w;
            if (m > 1e-15f) {
                // each product and sum rounded once, as the fp32 statement writes it
                const float inv = 1.0f / m;
                v[0] = __fadd_rn(__fmul_rn(mv.x, inv), __fmul_rn(k.dt, k.g[0]));
                v[1] = __fadd_rn(__fmul_rn(mv.y, inv), __fmul_rn(k.dt, k.g[1]));
                v[2] = __fadd_rn(__fmul_rn(mv.z, inv), __fmul_rn(k.dt, k.g[2]));
            }
            if (k.damp < 1.0f) { v[0] *= k.damp; v[1] *= k.damp; v[2] *= k.damp; }
        }
        const float cb[3] = {((float)(bx * 4) + 1.5f) * k.dx, ((float)(by * 4) + 1.5f) * k.dx,
                             ((float)(bz * 4) + 1.5f) * k.dx};
        for (int c = 0; c < k.ncol; ++c) {
            if (s_cull[c] > 0.0f) {   // uniform over the block, so over each warp
                const float d0 = cb[0] - s_pose[c].p[0], d1 = cb[1] - s_pose[c].p[1], d2 = cb[2] - s_pose[c].p[2];
                if (d0 * d0 + d1 * d1 + d2 * d2 > s_cull[c]) continue;
            }
            float acc[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
            if (valid && m > 0.0f && s_pose[c].mode != 0) collide(s_cols[c], s_pose[c], gx, gy, gz, m, v, k, acc);
            int kind = s_cols[c].kind;
            if (kind == GBMPM_COLLIDER_BOX || kind == GBMPM_COLLIDER_CUP || kind == GBMPM_COLLIDER_SDF) {
                bool any = __any_sync(0xffffffffu, acc[0] != 0.f || acc[1] != 0.f || acc[2] != 0.f || acc[3] != 0.f ||
                                                       acc[4] != 0.f || acc[5] != 0.f);
                if (any) {
#pragma unroll
                    for (int a = 0; a < 6; ++a) {
                        float x = acc[a];
#pragma unroll
                        for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
                        if (lane == 0) atomicAdd(&s_acc[c][a], x);
                    }
                }
            }
        }
        if (valid) {
            k.gv[id] = make_float4(v[0], v[1], v[2], 0.0f);
            k.gmv[id] = make_float4(0.f, 0.f, 0.f, 0.f);
            if (cell == 0) k.blk_flag[b] = 0;
        }
    }
    __syncthreads();
    for (int i = t; i < k.ncol * 6; i += blockDim.x) {
        float a = s_acc[i / 6][i % 6];
        if (a != 0.0f) atomicAdd(&k.wrench[i], (double)a);
    }
}

__global__ void __launch_bounds__(kGridThreads) k_grid(GK k) { grid_update(k, blockIdx.x, gridDim.x); }

// Batched scenes: CTA b updates scene ctas[b].x as CTA ctas[b].y of ctas[b].z.
// The per-scene record holds the tick's first pose row, block list 0 and the
// count pair; `substep` and `list` select this pass's.
__global__ void __launch_bounds__(kGridThreads) k_grid_batch(const GK *table, const int4 *ctas, int substep, int list) {
    __shared__ GK s_g;
    const int4 c = ctas[blockIdx.x];
    const int *src = reinterpret_cast<const int *>(table + c.x);
    int *d = reinterpret_cast<int *>(&s_g);
    for (int i = threadIdx.x; i < (int)(sizeof(GK) / 4); i += blockDim.x) d[i] = src[i];
    __syncthreads();
    if (threadIdx.x == 0) {
        int *counts = s_g.blk_count_read;
        s_g.poses += (size_t)substep * (s_g.ncol > 0 ? s_g.ncol : 1);
        s_g.blk_list += (size_t)list * s_g.bd * s_g.bd * s_g.bd;
        s_g.blk_count_read = counts + list;
        s_g.blk_count_reset = counts + (list ^ 1);
    }
    __syncthreads();
    grid_update(s_g, c.y, c.z);
}
