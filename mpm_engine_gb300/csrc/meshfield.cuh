// Mesh -> distance-field builders: the O(points x surface elements) searches of
// warpmpm.geometry.mesh_sdf (src/warpmpm/geometry/mesh_sdf.py) on the device. The
// host composes them into build_sdf / build_surface_cdf (mpm_engine_gb300/meshfield.py).
//
//  * Nearest surface sample: the query the reference makes with scipy's cKDTree
//    (build_sdf :329-364 through _unsigned_distance :314-326, build_surface_cdf
//    :412-480) or, without scipy, by a chunked numpy argmin (:455-466). An exact
//    nearest neighbour: float64 distances formed as numpy's norm forms them,
//    sqrt((dx^2 + dy^2) + dz^2) with every operation rounded once, and ties on the
//    rounded distance going to the lowest sample index, as argmin does. A float32
//    pass over the samples first bounds the nearest distance; the float64 distance
//    is then formed only for samples within that bound plus the float32 rounding
//    error, so the result is the float64 search's.
//  * Generalized winding number (_winding_number :210-233): the signed solid angles
//    2 atan2(num, den) of the faces (Van Oosterom-Strackee) summed and divided by
//    4 pi. Summed in float32; a point whose value lies within the float32 error of
//    the +-0.5 inside threshold, or that lies near a face's plane inside its
//    outline (where one face's angle flips by 4 pi), is summed again in float64,
//    as is every point of a `precise` call.
//  * Exact point-triangle distance (_point_triangle_distance_exact :236-289): the
//    closest point by barycentric region (Ericson), with the reference's override
//    order for degenerate triangles, in float64.
//
// One thread owns one query point; surface elements stream through shared memory
// in tiles, so a CTA reads each element once per tile for 256 points.

namespace gbmpm {
namespace mesh {

constexpr int kThreads = 256;
constexpr int kSampleTile = 1024;   // float4 samples: 16 KB
constexpr int kFaceTile = 256;      // float32 faces (9 floats) 9 KB; float64 faces 18 KB

struct Points {
    const double *pts;   // explicit [n][3], or null: the res^3 nodes of the grid below
    long long n;
    double origin[3], cell;
    int res;
};

// Grid node i (x slowest): origin + cell * index, each product and sum rounded
// once, as numpy forms `origin[d] + cell * np.arange(res)`.
__device__ __forceinline__ void point_at(const Points &P, long long i, double *p) {
    if (P.pts) {
        p[0] = P.pts[3 * i];
        p[1] = P.pts[3 * i + 1];
        p[2] = P.pts[3 * i + 2];
        return;
    }
    const long long rr = (long long)P.res * P.res;
    const int x = (int)(i / rr), y = (int)((i / P.res) % P.res), z = (int)(i % P.res);
    p[0] = __dadd_rn(P.origin[0], __dmul_rn(P.cell, (double)x));
    p[1] = __dadd_rn(P.origin[1], __dmul_rn(P.cell, (double)y));
    p[2] = __dadd_rn(P.origin[2], __dmul_rn(P.cell, (double)z));
}

__global__ void k_samples_f32(const double *s, long long m, float4 *out) {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < m; i += (long long)gridDim.x * blockDim.x)
        out[i] = make_float4((float)s[3 * i], (float)s[3 * i + 1], (float)s[3 * i + 2], 0.0f);
}

__global__ void k_faces_f32(const double *t, long long nf, float *out) {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < 9 * nf; i += (long long)gridDim.x * blockDim.x)
        out[i] = (float)t[i];
}

__global__ void __launch_bounds__(kThreads) k_nearest(Points P, const float4 *s32, const double *s64, long long m,
                                                      double *dist, long long *index) {
    __shared__ float4 tile[kSampleTile];
    const long long i = (long long)blockIdx.x * kThreads + threadIdx.x;
    const bool live = i < P.n;
    double p[3] = {0.0, 0.0, 0.0};
    if (live) point_at(P, i, p);
    const float px = (float)p[0], py = (float)p[1], pz = (float)p[2];
    float best = INFINITY;
    for (long long b = 0; b < m; b += kSampleTile) {
        const int cnt = (int)min((long long)kSampleTile, m - b);
        __syncthreads();
        for (int q = threadIdx.x; q < cnt; q += kThreads) tile[q] = s32[b + q];
        __syncthreads();
        for (int q = 0; q < cnt; ++q) {
            const float4 s = tile[q];
            const float dx = px - s.x, dy = py - s.y, dz = pz - s.z;
            best = fminf(best, dx * dx + dy * dy + dz * dz);
        }
    }
    // float32 error of a distance: coordinate rounding (2^-24 of |p| and of |s| <=
    // |p| + d per axis) and the arithmetic (a few 2^-24 of d); 1e-6 covers both twice
    const float pm = fmaxf(fabsf(px), fmaxf(fabsf(py), fabsf(pz)));
    const float bd32 = sqrtf(best);
    const float lim = bd32 + 1.0e-6f * (pm + bd32) + 1.0e-30f;
    const float lim2 = lim * lim;
    double bd = INFINITY;
    long long bi = -1;
    for (long long b = 0; b < m; b += kSampleTile) {
        const int cnt = (int)min((long long)kSampleTile, m - b);
        __syncthreads();
        for (int q = threadIdx.x; q < cnt; q += kThreads) tile[q] = s32[b + q];
        __syncthreads();
        for (int q = 0; q < cnt; ++q) {
            const float4 s = tile[q];
            const float dx = px - s.x, dy = py - s.y, dz = pz - s.z;
            if (dx * dx + dy * dy + dz * dz <= lim2) {
                const double *e = s64 + 3 * (b + q);
                const double ex = __dsub_rn(p[0], e[0]), ey = __dsub_rn(p[1], e[1]), ez = __dsub_rn(p[2], e[2]);
                const double d = __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(ex, ex), __dmul_rn(ey, ey)), __dmul_rn(ez, ez)));
                if (d < bd) { bd = d; bi = b + q; }
            }
        }
    }
    if (live) {
        dist[i] = bd;
        index[i] = bi;
    }
}

// 2 atan2(num, den) of one face seen from p. `cut` is set when the point lies near
// the face's plane inside its outline (den < 0, num ~ 0): there the angle jumps
// between +2 pi and -2 pi with the sign of num, so a float32 sum is not trusted.
// In float64 an exact zero num counts as +0, as numpy's einsum (which sums from
// +0) forms it for a point in the face's plane: the in-plane face gives +2 pi.
template <class T>
__device__ __forceinline__ T solid_angle(const T *f, T px, T py, T pz, bool &cut) {
    const T A[3] = {f[0] - px, f[1] - py, f[2] - pz};
    const T B[3] = {f[3] - px, f[4] - py, f[5] - pz};
    const T C[3] = {f[6] - px, f[7] - py, f[8] - pz};
    const T la = sqrt(A[0] * A[0] + A[1] * A[1] + A[2] * A[2]);
    const T lb = sqrt(B[0] * B[0] + B[1] * B[1] + B[2] * B[2]);
    const T lc = sqrt(C[0] * C[0] + C[1] * C[1] + C[2] * C[2]);
    const T bc[3] = {B[1] * C[2] - B[2] * C[1], B[2] * C[0] - B[0] * C[2], B[0] * C[1] - B[1] * C[0]};
    T num = A[0] * bc[0] + A[1] * bc[1] + A[2] * bc[2];
    const T den = la * lb * lc + (A[0] * B[0] + A[1] * B[1] + A[2] * B[2]) * lc +
                  (B[0] * C[0] + B[1] * C[1] + B[2] * C[2]) * la + (C[0] * A[0] + C[1] * A[1] + C[2] * A[2]) * lb;
    if (den < T(0) && fabs(num) <= T(1e-4) * fabs(den)) cut = true;
    if (num == T(0)) num = T(0);   // -0 -> +0
    return T(2) * atan2(num, den);
}

__global__ void __launch_bounds__(kThreads) k_winding(Points P, const float *t32, const double *t64, long long nf,
                                                      int precise, float margin, double *wn) {
    __shared__ float tile[kFaceTile * 9];
    const long long i = (long long)blockIdx.x * kThreads + threadIdx.x;
    const bool live = i < P.n;
    double p[3] = {0.0, 0.0, 0.0};
    if (live) point_at(P, i, p);
    const float px = (float)p[0], py = (float)p[1], pz = (float)p[2];
    float sum = 0.0f;
    bool cut = false;
    for (long long b = 0; b < nf; b += kFaceTile) {
        const int cnt = (int)min((long long)kFaceTile, nf - b);
        __syncthreads();
        for (int q = threadIdx.x; q < 9 * cnt; q += kThreads) tile[q] = t32[9 * b + q];
        __syncthreads();
        if (!precise)
            for (int q = 0; q < cnt; ++q) sum += solid_angle<float>(tile + 9 * q, px, py, pz, cut);
    }
    if (!live) return;
    const float w32 = sum / (4.0f * 3.14159265358979f);
    if (!precise && !cut && fabsf(fabsf(w32) - 0.5f) > margin) {
        wn[i] = (double)w32;
        return;
    }
    double s = 0.0;
    for (long long f = 0; f < nf; ++f) s += solid_angle<double>(t64 + 9 * f, p[0], p[1], p[2], cut);
    wn[i] = s / (4.0 * 3.141592653589793);
}

__global__ void __launch_bounds__(kThreads) k_tri_distance(Points P, const double *t64, long long nf, double *dist) {
    __shared__ double tile[kFaceTile * 9];
    const long long i = (long long)blockIdx.x * kThreads + threadIdx.x;
    const bool live = i < P.n;
    double p[3] = {0.0, 0.0, 0.0};
    if (live) point_at(P, i, p);
    double best = INFINITY;
    for (long long b = 0; b < nf; b += kFaceTile) {
        const int cnt = (int)min((long long)kFaceTile, nf - b);
        __syncthreads();
        for (int q = threadIdx.x; q < 9 * cnt; q += kThreads) tile[q] = t64[9 * b + q];
        __syncthreads();
        for (int q = 0; q < cnt; ++q) {
            const double *f = tile + 9 * q;
            double ab[3], ac[3], ap[3], bp[3], cp[3];
            for (int a = 0; a < 3; ++a) {
                ab[a] = f[3 + a] - f[a];
                ac[a] = f[6 + a] - f[a];
                ap[a] = p[a] - f[a];
                bp[a] = p[a] - f[3 + a];
                cp[a] = p[a] - f[6 + a];
            }
            auto dot = [](const double *x, const double *y) { return x[0] * y[0] + x[1] * y[1] + x[2] * y[2]; };
            const double d1 = dot(ap, ab), d2 = dot(ap, ac), d3 = dot(bp, ab), d4 = dot(bp, ac);
            const double d5 = dot(cp, ab), d6 = dot(cp, ac);
            const double va = d3 * d6 - d5 * d4, vb = d5 * d2 - d1 * d6, vc = d1 * d4 - d3 * d2;
            const double den = va + vb + vc;
            const double inv = fabs(den) > 1e-30 ? 1.0 / den : 0.0;
            double v = vb * inv, w = vc * inv;
            // vertex and edge regions override the interior solution, later ones last
            if (d1 <= 0.0 && d2 <= 0.0) { v = 0.0; w = 0.0; }
            if (d3 >= 0.0 && d4 <= d3) { v = 1.0; w = 0.0; }
            if (d6 >= 0.0 && d5 <= d6) { v = 0.0; w = 1.0; }
            if (vc <= 0.0 && d1 >= 0.0 && d3 <= 0.0) { v = fabs(d1 - d3) > 1e-30 ? d1 / (d1 - d3) : 0.0; w = 0.0; }
            if (vb <= 0.0 && d2 >= 0.0 && d6 <= 0.0) { v = 0.0; w = fabs(d2 - d6) > 1e-30 ? d2 / (d2 - d6) : 0.0; }
            if (va <= 0.0 && (d4 - d3) >= 0.0 && (d5 - d6) >= 0.0) {
                const double e = (d4 - d3) + (d5 - d6);
                const double tb = fabs(e) > 1e-30 ? (d4 - d3) / e : 0.0;
                v = 1.0 - tb;
                w = tb;
            }
            double r2 = 0.0;
            for (int a = 0; a < 3; ++a) {
                const double c = f[a] + v * ab[a] + w * ac[a];
                r2 += (p[a] - c) * (p[a] - c);
            }
            best = fmin(best, sqrt(r2));
        }
    }
    if (live) dist[i] = best;
}

// argument checks shared by the three entry points
int points_of(const gbmpm_field_points *pts, Points &P) {
    if (!pts) return fail(GBMPM_ERR_ARG, "null points");
    P.pts = pts->points;
    for (int a = 0; a < 3; ++a) P.origin[a] = pts->origin[a];
    P.cell = pts->cell;
    P.res = pts->res;
    if (pts->points) {
        if (pts->n < 0) return fail(GBMPM_ERR_ARG, "negative point count");
        P.n = pts->n;
    } else {
        if (pts->res < 1 || pts->res > 2048 || !(pts->cell > 0.0))
            return fail(GBMPM_ERR_ARG, "field grid needs 1 <= res <= 2048 and cell > 0");
        P.n = (long long)pts->res * pts->res * pts->res;
    }
    return GBMPM_OK;
}

int point_blocks(long long n) { return (int)std::max<long long>(1, (n + kThreads - 1) / kThreads); }

}  // namespace mesh
}  // namespace gbmpm

extern "C" {

int gbmpm_field_nearest(const gbmpm_field_points *pts, const double *samples, int64_t n_samples, double *dist_out,
                        int64_t *index_out, void *stream) {
    using namespace gbmpm;
    mesh::Points P;
    int rc = mesh::points_of(pts, P);
    if (rc) return rc;
    if (!samples || n_samples < 1 || !dist_out || !index_out) return fail(GBMPM_ERR_ARG, "nearest: needs samples and outputs");
    if (P.n == 0) return GBMPM_OK;
    cudaStream_t s = (cudaStream_t)stream;
    float4 *s32 = nullptr;
    GB_CUDA(cudaMallocAsync(&s32, (size_t)n_samples * sizeof(float4), s));
    mesh::k_samples_f32<<<(int)std::min<long long>((n_samples + 255) / 256, 4096), 256, 0, s>>>(samples, n_samples, s32);
    mesh::k_nearest<<<mesh::point_blocks(P.n), mesh::kThreads, 0, s>>>(P, s32, samples, n_samples, dist_out,
                                                                     reinterpret_cast<long long *>(index_out));
    cudaError_t err = cudaGetLastError();
    cudaFreeAsync(s32, s);
    GB_CUDA(err);
    return GBMPM_OK;
}

int gbmpm_field_winding(const gbmpm_field_points *pts, const double *tri, int64_t n_faces, int32_t precise,
                        double *wn_out, void *stream) {
    using namespace gbmpm;
    mesh::Points P;
    int rc = mesh::points_of(pts, P);
    if (rc) return rc;
    if (!tri || n_faces < 1 || !wn_out) return fail(GBMPM_ERR_ARG, "winding: needs faces and an output");
    if (P.n == 0) return GBMPM_OK;
    cudaStream_t s = (cudaStream_t)stream;
    float *t32 = nullptr;
    GB_CUDA(cudaMallocAsync(&t32, (size_t)n_faces * 9 * sizeof(float), s));
    mesh::k_faces_f32<<<(int)std::min<long long>((9 * n_faces + 255) / 256, 4096), 256, 0, s>>>(tri, n_faces, t32);
    // float32 error of the sum: a few 1e-7 of each face's angle, bounded here by
    // 1e-3 plus 1e-7 a face (the 4 pi division leaves it smaller still)
    const float margin = 1.0e-3f + 1.0e-7f * (float)n_faces;
    mesh::k_winding<<<mesh::point_blocks(P.n), mesh::kThreads, 0, s>>>(P, t32, tri, n_faces, precise ? 1 : 0, margin,
                                                                     wn_out);
    cudaError_t err = cudaGetLastError();
    cudaFreeAsync(t32, s);
    GB_CUDA(err);
    return GBMPM_OK;
}

int gbmpm_field_tri_distance(const gbmpm_field_points *pts, const double *tri, int64_t n_faces, double *dist_out,
                             void *stream) {
    using namespace gbmpm;
    mesh::Points P;
    int rc = mesh::points_of(pts, P);
    if (rc) return rc;
    if (!tri || n_faces < 1 || !dist_out) return fail(GBMPM_ERR_ARG, "tri_distance: needs faces and an output");
    if (P.n == 0) return GBMPM_OK;
    cudaStream_t s = (cudaStream_t)stream;
    mesh::k_tri_distance<<<mesh::point_blocks(P.n), mesh::kThreads, 0, s>>>(P, tri, n_faces, dist_out);
    GB_CUDA(cudaGetLastError());
    return GBMPM_OK;
}

}  // extern "C"
