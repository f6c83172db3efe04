// common.cuh - what every translation unit of the engine shares: the records the
// kernels take (particle, grid-pass and collider tables), the per-substep pass
// modes, and the small device helpers (3x3 algebra, programmatic dependent
// launch, asynchronous copies, structure-of-arrays field access).
#pragma once

#include "../../include/gbmpm.h"
#include "svd3.cuh"

#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

namespace gbmpm {

// ------------------------------------------------------------ constants ----
constexpr int kMaxCol = GBMPM_MAX_COLLIDERS;
constexpr int kParticleThreads = 128;
constexpr int kGridThreads = 256;

enum PassMode : int {
    PASS_G2P = 1,        // gather from grid v, advect, C, L, F_trial
    PASS_STRESS = 2,     // return map + Kirchhoff stress
    PASS_P2G = 4,        // scatter into grid mv, mark blocks
    PASS_STORE_ALL = 8,  // also store stress (last stress of the tick)
    PASS_STORE_VC = 16,  // store v and C after the gather
    PASS_RESET_LISTS = 32
};

struct MatTables {
    float E[16], nu[16], bulk[16], hardening[16], xi[16], pv[16], softening[16], alpha[16];
    float mu_s[16], dmu[16], I0[16], d[16], rho_s[16], phi_init[16], phi_chi[16];
};

// CPIC lane state the transfer passes read (the reference's cdf_lane_* arrays):
// poses at the current stamp, and pose/rates/surface at the previous one.
struct CdfLanes {
    float c_cur[4][3], c_prev[4][3], v_prev[4][3], w_prev[4][3];
    float fric[4];
    int type[4];
};

struct PK {
    float *x, *v, *C, *F, *Ft, *L, *S;
    const float *mass, *vol;
    float *Jp, *mu, *lam, *ys;
    const int *mat, *sel;
    float *cov;
    int n;
    const float4 *gv;
    float4 *gmv;
    int ng;
    float dx, inv_dx, dt, rpic;
    int periodic_x, update_cov;
    const MatTables *tab;
    const float *eta;
    int eta_n;
    float eta_smin, eta_smax;
    int *blk_flag, *blk_list, *blk_count;
    int bd;
    unsigned *status;
    // CPIC (CDF) colliders; cdf_on == 0 leaves every branch below unused
    int cdf_on, cnb;
    const int *ctag, *ctag_prev, *cblock;
    const float *cd, *cd_prev;
    int *ptag;
    double *cwrench;   // [CTA][4][6] per-CTA partial sums of the blocked-deposit reaction
    float *ccache;     // tiled kernel: the scatter scan of each particle, SoA x5 (see k_particles_tiled)
    // particle modifiers (bit m of mod_mask selects modifier m) and rigid bodies
    int n_mods;
    const gbmpm_modifier *mods;
    const int *mod_mask;
    const double *sub_time;   // start time of every substep of the tick
    int sub;                  // the substep whose P2G this pass performs
    int rigid_defer;          // material-8 particles leave their P2G to the rigid pass
    float grav[3];
    CdfLanes lanes;
};

// Per-substep collider pose record, built on the host each tick.
struct PoseRec {
    float p[3];
    int mode;     // 0 inactive, 1 live, 2 box reset-zero
    float r[9];   // cup rotation
    float q[4];   // sdf quaternion
    float pad[2];
};

struct ColDev {
    int kind, surface, sdf_res, pad0;
    float normal[3], size[3], vel[3], omega[3];
    float friction, outer_r, inner_r, half_h, floor_z, fillet, sticky, band_c;
    float origin[3], cell, band;
    const float *sdf_val, *sdf_grad;
};

struct GK {
    float4 *gmv;
    float4 *gv;
    int ng;
    float dx, dt;
    float g[3];
    float damp;
    int ncol;
    const ColDev *cols;
    const PoseRec *poses;   // [ncol] for this substep
    double *wrench;         // [ncol][6]
    int *blk_flag, *blk_list, *blk_count_read, *blk_count_reset;
    int bd;
};

// ------------------------------------------------------------- helpers -----
__device__ __forceinline__ void mat_load(const float *p, float (&m)[9]) {
#pragma unroll
    for (int i = 0; i < 9; ++i) m[i] = p[i];
}
__device__ __forceinline__ void mat_store(float *p, const float (&m)[9]) {
#pragma unroll
    for (int i = 0; i < 9; ++i) p[i] = m[i];
}
// Programmatic dependent launch. The particle passes and the grid pass are launched
// with programmatic stream serialization, so a pass may start while the kernel
// before it finishes: pdl_wait() blocks until that kernel has completed and its
// writes are visible, and must come before anything touching its outputs;
// pdl_trigger() lets the next pass start launching. Each pass triggers only after
// its own wait, so the code a pass runs before waiting only ever overlaps a kernel
// that is past its own wait (the grid pass while the particle pass loads its
// particles, or the particle pass's last wave while the grid pass stages its
// collider records), and never reads what that kernel writes. Without the launch
// attribute both are no-ops.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

// 4-byte asynchronous global -> shared copy; cp.async.wait_all makes the calling
// thread's copies complete and visible to that thread
__device__ __forceinline__ void cp_async4(float *dst, const float *src) {
    const unsigned sa = (unsigned)__cvta_generic_to_shared(dst);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(sa), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }
// 16-byte asynchronous global -> shared copy (both addresses 16-byte aligned)
__device__ __forceinline__ void cp_async16(void *dst, const void *src) {
    const unsigned sa = (unsigned)__cvta_generic_to_shared(dst);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(sa), "l"(src) : "memory");
}

// Particle fields are either the caller's records (AoS: W floats per particle)
// or the engine's working copy (SoA: component c of particle p at c*n + p, so a
// warp's access to one component is one coalesced line).
template <bool SOA, int W>
__device__ __forceinline__ void fld_load(const float *base, int n, int p, float *out) {
#pragma unroll
    for (int c = 0; c < W; ++c) out[c] = SOA ? base[(size_t)c * n + p] : base[(size_t)p * W + c];
}
template <bool SOA, int W>
__device__ __forceinline__ void fld_store(float *base, int n, int p, const float *in) {
#pragma unroll
    for (int c = 0; c < W; ++c) {
        if (SOA) base[(size_t)c * n + p] = in[c];
        else base[(size_t)p * W + c] = in[c];
    }
}

__device__ __forceinline__ void mm(const float *a, const float *b, float *c) {
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j)
            c[3 * i + j] = a[3 * i] * b[j] + a[3 * i + 1] * b[3 + j] + a[3 * i + 2] * b[6 + j];
}
// c = a * b^T
__device__ __forceinline__ void mmT(const float *a, const float *b, float *c) {
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j)
            c[3 * i + j] = a[3 * i] * b[3 * j] + a[3 * i + 1] * b[3 * j + 1] + a[3 * i + 2] * b[3 * j + 2];
}
// det(m) as row0 . (row1 x row2), every product and sum rounded on its own in
// that order (the reference's determinant, and the oracle's): the fluid laws feed
// J into a stiff equation of state, K (J^-1.1 - 1) with K ~ 1e6 Pa, where one ulp of
// J is 0.1 Pa, so J is formed exactly as the restatement forms it
__device__ __forceinline__ float det3(const float *m) {
    const float c0 = __fsub_rn(__fmul_rn(m[4], m[8]), __fmul_rn(m[5], m[7]));
    const float c1 = __fsub_rn(__fmul_rn(m[5], m[6]), __fmul_rn(m[3], m[8]));
    const float c2 = __fsub_rn(__fmul_rn(m[3], m[7]), __fmul_rn(m[4], m[6]));
    return __fadd_rn(__fadd_rn(__fmul_rn(m[0], c0), __fmul_rn(m[1], c1)), __fmul_rn(m[2], c2));
}
// c = a b with each product and sum rounded on its own, k ascending (the reference's
// mat33 product): used for F_trial = (I + dt L) F, whose determinant is J
__device__ __forceinline__ void mm_rn(const float *a, const float *b, float *c) {
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j)
            c[3 * i + j] = __fadd_rn(__fadd_rn(__fmul_rn(a[3 * i], b[j]), __fmul_rn(a[3 * i + 1], b[3 + j])),
                                     __fmul_rn(a[3 * i + 2], b[6 + j]));
}
// U diag(d) V^T
__device__ __forceinline__ void udvt(const float *U, float d0, float d1, float d2, const float *V, float *out) {
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j)
            out[3 * i + j] = U[3 * i] * d0 * V[3 * j] + U[3 * i + 1] * d1 * V[3 * j + 1] + U[3 * i + 2] * d2 * V[3 * j + 2];
}

__device__ __forceinline__ void set_status(unsigned *st, unsigned bit) { atomicOr(st, bit); }

// Launch with programmatic stream serialization (see pdl_wait) when `pdl` is set.
template <typename... P, typename... A>
inline void launch_kernel(bool pdl, void (*kern)(P...), int grid, int block, cudaStream_t s, A... args) {
    if (!pdl) {
        kern<<<grid, block, 0, s>>>(args...);
        return;
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(block);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    cudaLaunchKernelEx(&cfg, kern, args...);
}

// The particle-pass launcher (particles.cu): picks the direct or the tiled kernel
// and its specialisation (solids compiled in or out, resident CTAs per SM, CPIC).
struct ParticleLaunch {
    bool tiled;      // block-sorted working set: the tiled kernel
    bool solids;     // SVD-based laws present
    bool pdl;        // programmatic dependent launch
    int tile_occ;    // resident CTAs per SM the plain tiled kernel is compiled for
    int cdf_occ;     // the same for its CPIC variant
};
void launch_particle_pass(const ParticleLaunch &L, const PK &k, int mode, cudaStream_t s);

// Deterministic particle passes (deterministic.cu): every operation rounded once,
// P2G as per-node sums in particle order. det_launch_p2g writes 27 records a
// particle; the caller sorts them by key (stable) and hands them to det_launch_segsum.
void det_launch_g2p(const PK &k, bool reset_lists, cudaStream_t s);
void det_launch_stress(const PK &k, cudaStream_t s);
void det_launch_p2g(const PK &k, unsigned long long *key, int *idx, float4 *val, cudaStream_t s);
void det_launch_segsum(const PK &k, const unsigned long long *key, const int *idx, const float4 *val, int n_rec,
                       cudaStream_t s);

// Batched scenes: one particle pass over many scenes. CTA b of the launch takes
// tile ctas[b].tile of scene ctas[b].scene (particles_batch_*.cu).
struct BatchCta {
    int scene, tile;
};
struct BatchLaunch {
    int threads;     // particles per tile (CTA width): 64, 128 or 256
    int occ;         // resident 256-thread equivalents per SM the kernel is compiled for: 2 or 3
    bool solids;     // SVD-based laws present in some scene
    bool pdl;
};
void launch_particle_batch_fluid(const BatchLaunch &L, const PK *table, const BatchCta *ctas, int nctas, int mode,
                                 int list, int sub, cudaStream_t s);
void launch_particle_batch_solid(const BatchLaunch &L, const PK *table, const BatchCta *ctas, int nctas, int mode,
                                 int list, int sub, cudaStream_t s);
inline void launch_particle_batch(const BatchLaunch &L, const PK *table, const BatchCta *ctas, int nctas, int mode,
                                  int list, int sub, cudaStream_t s) {
    if (L.solids) launch_particle_batch_solid(L, table, ctas, nctas, mode, list, sub, s);
    else launch_particle_batch_fluid(L, table, ctas, nctas, mode, list, sub, s);
}

}  // namespace gbmpm
