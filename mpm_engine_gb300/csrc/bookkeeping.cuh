// Bookkeeping around the substep: the edge-guard reductions, the in-place block
// sort, the active-block marks and the R / covariance exports.
//
// Included by gbmpm.cu inside namespace gbmpm, after the constants and helpers
// and before the host code; it is not a standalone header.

// ------------------------------------------------- guard / reductions ------
__device__ __forceinline__ float warp_min(float x) {
    for (int o = 16; o > 0; o >>= 1) x = fminf(x, __shfl_xor_sync(0xffffffffu, x, o));
    return x;
}
__device__ __forceinline__ float warp_max(float x) {
    for (int o = 16; o > 0; o >>= 1) x = fmaxf(x, __shfl_xor_sync(0xffffffffu, x, o));
    return x;
}
__device__ __forceinline__ void atomic_min_f(float *a, float v) {
    if (v >= 0.0f) atomicMin((int *)a, __float_as_int(v));
    else atomicMax((unsigned *)a, __float_as_uint(v));
}
__device__ __forceinline__ void atomic_max_f(float *a, float v) {
    if (v >= 0.0f) atomicMax((int *)a, __float_as_int(v));
    else atomicMin((unsigned *)a, __float_as_uint(v));
}

__global__ void k_guard_init(float *out) {
    if (threadIdx.x < 3) out[threadIdx.x] = INFINITY;
    else if (threadIdx.x < 6) out[threadIdx.x] = -INFINITY;
    else if (threadIdx.x == 6) out[6] = 0.0f;
}

__global__ void k_guard(const float *x, const float *v, int n, float *out, unsigned *status) {
    float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY}, vm = 0.0f;
    bool bad = false;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) {
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            float xa = x[3 * p + a];
            if (!isfinite(xa)) bad = true;
            lo[a] = fminf(lo[a], xa);
            hi[a] = fmaxf(hi[a], xa);
            vm = fmaxf(vm, fabsf(v[3 * p + a]));
        }
    }
    if (__any_sync(0xffffffffu, bad) && (threadIdx.x & 31) == 0) atomicOr(status, GBMPM_FLAG_NONFINITE);
#pragma unroll
    for (int a = 0; a < 3; ++a) { lo[a] = warp_min(lo[a]); hi[a] = warp_max(hi[a]); }
    vm = warp_max(vm);
    if ((threadIdx.x & 31) == 0) {
#pragma unroll
        for (int a = 0; a < 3; ++a) { atomic_min_f(out + a, lo[a]); atomic_max_f(out + 3 + a, hi[a]); }
        atomic_max_f(out + 6, vm);
    }
}

// ------------------------------------------------------- block sort --------
// key = ((bx nb + by) nb + bz), b = floor(x/dx - 0.5) >> 2 in float64
// (core/solver.py:458-465). The pass stores the signed key, flags any descent
// (the reference skips the permutation when keys are already non-decreasing)
// and reduces min/max so the radix sort only walks the bits the keys span.
__global__ void k_sort_keys(const float *x, int n, double dx, long long nb, long long *keys, int *idx,
                            int *unsorted, long long *kminmax) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    long long key = 0;
    bool valid = p < n;
    if (valid) {
        long long b[3];
#pragma unroll
        for (int a = 0; a < 3; ++a) b[a] = ((long long)floor((double)x[3 * p + a] / dx - 0.5)) >> 2;
        key = (b[0] * nb + b[1]) * nb + b[2];
        keys[p] = key;
        idx[p] = p;
        if (p > 0) {
            long long bp[3];
#pragma unroll
            for (int a = 0; a < 3; ++a) bp[a] = ((long long)floor((double)x[3 * (p - 1) + a] / dx - 0.5)) >> 2;
            long long kp = (bp[0] * nb + bp[1]) * nb + bp[2];
            if (kp > key) *unsorted = 1;
        }
    }
    long long lo = valid ? key : LLONG_MAX, hi = valid ? key : LLONG_MIN;
    for (int o = 16; o > 0; o >>= 1) {
        lo = min(lo, __shfl_xor_sync(0xffffffffu, lo, o));
        hi = max(hi, __shfl_xor_sync(0xffffffffu, hi, o));
    }
    if ((threadIdx.x & 31) == 0) { atomicMin(&kminmax[0], lo); atomicMax(&kminmax[1], hi); }
}

__global__ void k_sort_minmax_init(long long *kminmax) {
    kminmax[0] = LLONG_MAX;
    kminmax[1] = LLONG_MIN;
}

// signed key -> unsigned offset from the minimum (order preserving)
__global__ void k_sort_rebase(const long long *keys, int n, const long long *kminmax, unsigned long long *out) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p < n) out[p] = (unsigned long long)(keys[p] - kminmax[0]);
}

constexpr int kRadixBits = 8;
constexpr int kRadixBins = 1 << kRadixBits;
constexpr int kSortTile = 4096;          // elements per tile
constexpr int kSortThreads = 256;        // 16 rounds of 256 elements

// per-tile digit histogram, stored bin-major: hist[bin * ntiles + tile]
__global__ void __launch_bounds__(kSortThreads) k_radix_hist(const unsigned long long *keys, int n, int shift,
                                                             unsigned *hist, int ntiles) {
    __shared__ unsigned h[kRadixBins];
    for (int i = threadIdx.x; i < kRadixBins; i += blockDim.x) h[i] = 0;
    __syncthreads();
    int base = blockIdx.x * kSortTile;
    for (int i = threadIdx.x; i < kSortTile; i += blockDim.x) {
        int e = base + i;
        if (e < n) atomicAdd(&h[(keys[e] >> shift) & (kRadixBins - 1)], 1u);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < kRadixBins; i += blockDim.x) hist[(size_t)i * ntiles + blockIdx.x] = h[i];
}

// exclusive scan of hist in place, one CTA: each thread scans a contiguous
// chunk, the chunk totals are scanned in shared memory, then chunks are rebased
__global__ void __launch_bounds__(1024) k_radix_scan(unsigned *hist, int total) {
    __shared__ unsigned s[1024];
    const int t = threadIdx.x;
    const int chunk = (total + 1023) / 1024;
    const int beg = min(t * chunk, total), end = min(beg + chunk, total);
    unsigned sum = 0;
    for (int i = beg; i < end; ++i) sum += hist[i];
    s[t] = sum;
    __syncthreads();
    for (int off = 1; off < 1024; off <<= 1) {
        unsigned v = t >= off ? s[t - off] : 0;
        __syncthreads();
        s[t] += v;
        __syncthreads();
    }
    unsigned run = s[t] - sum;
    for (int i = beg; i < end; ++i) {
        unsigned v = hist[i];
        hist[i] = run;
        run += v;
    }
}

// stable scatter: elements of a tile are ranked in index order per digit
__global__ void __launch_bounds__(kSortThreads) k_radix_scatter(const unsigned long long *keys_in, const int *idx_in,
                                                                unsigned long long *keys_out, int *idx_out, int n,
                                                                int shift, const unsigned *hist, int ntiles) {
    __shared__ unsigned offs[kRadixBins];
    __shared__ unsigned warp_cnt[kSortThreads / 32][kRadixBins];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int i = threadIdx.x; i < kRadixBins; i += blockDim.x) offs[i] = hist[(size_t)i * ntiles + blockIdx.x];
    int base = blockIdx.x * kSortTile;
    for (int round = 0; round < kSortTile / kSortThreads; ++round) {
        for (int i = threadIdx.x; i < (kSortThreads / 32) * kRadixBins; i += blockDim.x)
            (&warp_cnt[0][0])[i] = 0;
        __syncthreads();
        int e = base + round * kSortThreads + threadIdx.x;
        bool valid = e < n;
        unsigned long long key = valid ? keys_in[e] : 0ull;
        unsigned d = valid ? (unsigned)((key >> shift) & (kRadixBins - 1)) : 0xffffffffu;
        unsigned peers = __match_any_sync(0xffffffffu, d);
        int rank_in_warp = __popc(peers & ((1u << lane) - 1u));
        int leader = 31 - __clz(peers);
        if (valid && lane == leader) warp_cnt[warp][d] = __popc(peers);
        __syncthreads();
        if (valid) {
            unsigned before = 0;
            for (int w = 0; w < warp; ++w) before += warp_cnt[w][d];
            unsigned pos = offs[d] + before + rank_in_warp;
            keys_out[pos] = key;
            idx_out[pos] = idx_in[e];
        }
        __syncthreads();
        for (int b2 = threadIdx.x; b2 < kRadixBins; b2 += blockDim.x) {
            unsigned tot = 0;
            for (int w = 0; w < kSortThreads / 32; ++w) tot += warp_cnt[w][b2];
            offs[b2] += tot;
        }
        __syncthreads();
    }
}

template <int W>
__global__ void k_gather_rows(const float *src, const int *perm, float *dst, int n) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float *s = src + (size_t)perm[i] * W;
    float *d = dst + (size_t)i * W;
#pragma unroll
    for (int a = 0; a < W; ++a) d[a] = s[a];
}

// ------------------------------------------------- active blocks ----------
// blocks_mark / blocks_dilate / blocks_compact (mpm_utils.py:1506-1544)
__global__ void k_blocks_mark(const float *x, int n, float inv_dx, int bd, int *raw) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    int b[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        int v = (int)(x[3 * p + a] * inv_dx - 0.5f);
        b[a] = min(max(v >> 2, 0), bd - 1);
    }
    raw[((size_t)b[0] * bd + b[1]) * bd + b[2]] = 1;
}
__global__ void k_blocks_dilate(const int *raw, int bd, int *cur, const int *prev, int *counts) {
    int id = blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= bd * bd * bd) return;
    int z = id % bd, r = id / bd, y = r % bd, x = r / bd;
    int on = 0;
    for (int i = -1; i <= 1; ++i)
        for (int j = -1; j <= 1; ++j)
            for (int kk = -1; kk <= 1; ++kk) {
                int xi = min(max(x + i, 0), bd - 1), yj = min(max(y + j, 0), bd - 1), zk = min(max(z + kk, 0), bd - 1);
                if (raw[((size_t)xi * bd + yj) * bd + zk] == 1) on = 1;
            }
    cur[id] = on;
    if (on) atomicAdd(&counts[0], 1);
    if (on || prev[id] == 1) atomicAdd(&counts[1], 1);
}

// ----------------------------------------------------------- exports -------
__global__ void k_compute_R(const float *Ft, int n, float *R_out) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    float F[9], U[9], V[9], s[3], R[9];
    mat_load(Ft + 9 * (size_t)p, F);
    svd3(F, U, s, V);
    if (det3(U) < 0.0f) { U[2] = -U[2]; U[5] = -U[5]; U[8] = -U[8]; }
    if (det3(V) < 0.0f) { V[2] = -V[2]; V[5] = -V[5]; V[8] = -V[8]; }
    mmT(U, V, R);
    float *o = R_out + 9 * (size_t)p;
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) o[3 * i + j] = R[3 * j + i];
}
__global__ void k_compute_cov(const float *Ft, const float *c0, int n, float *out) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    float F[9], I0[9], T[9], r[9];
    mat_load(Ft + 9 * (size_t)p, F);
    const float *c = c0 + 6 * (size_t)p;
    I0[0] = c[0]; I0[1] = c[1]; I0[2] = c[2];
    I0[3] = c[1]; I0[4] = c[3]; I0[5] = c[4];
    I0[6] = c[2]; I0[7] = c[4]; I0[8] = c[5];
    mm(F, I0, T);
    mmT(T, F, r);
    float *o = out + 6 * (size_t)p;
    o[0] = r[0]; o[1] = r[1]; o[2] = r[2]; o[3] = r[4]; o[4] = r[5]; o[5] = r[8];
}

// ---- test hook: sums of a deposit over the whole grid ----------------------------
// Sum of m and m v over every node of mv[n^3] in float64 (per-CTA partials folded
// with float64 atomics into out[4] = {m, m vx, m vy, m vz}).
__global__ void __launch_bounds__(256) k_grid_sums(const float4 *mv, long long nodes, double *out) {
    double a[4] = {0.0, 0.0, 0.0, 0.0};
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < nodes; i += (long long)gridDim.x * blockDim.x) {
        const float4 g = mv[i];
        a[0] += (double)g.w; a[1] += (double)g.x; a[2] += (double)g.y; a[3] += (double)g.z;
    }
    __shared__ double s[4][8];
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        for (int o = 16; o > 0; o >>= 1) a[c] += __shfl_xor_sync(0xffffffffu, a[c], o);
        if ((threadIdx.x & 31) == 0) s[c][threadIdx.x >> 5] = a[c];
    }
    __syncthreads();
    if (threadIdx.x < 4) {
        double t = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += s[threadIdx.x][w];
        atomicAdd(out + threadIdx.x, t);
    }
}
