// gbmpm.cu - the GB300 MLS/APIC substep: particle kernels, grid kernel, block
// sort, exports, and the C ABI declared in include/gbmpm.h.
//
// Data layout in HBM
//   particles: the reference's per-particle records (x vec3, F mat33 row-major,
//              ...), caller-owned (PyTorch tensors), read and written in place.
//   grid:      mv[n^3] float4 {m vx, m vy, m vz, m}, the scatter target, kept
//              all-zero between substeps; v[n^3] float4 {vx, vy, vz, 0}, the
//              updated grid velocity the gather reads.
//   blocks:    one int flag per 4^3 node block plus two block lists. A particle
//              pass appends each block its stencils touch (first toucher wins the
//              flag); the grid pass that follows visits exactly those blocks,
//              updates, applies the colliders, and clears mv and the flags. The
//              grid update therefore costs O(active nodes), with no host-side
//              box and no per-substep host round trip.
//
// One tick of S substeps is S+1 particle passes and S grid passes (the
// reference's fused schedule, mpm_solver_warp.py:1379-1546), replayed as a
// single CUDA graph. Collider poses for every substep are integrated on the host
// in float64 once per tick (the reference's modify_bc callables) and uploaded as
// one table, so the graph needs no host work between substeps.

#include "common.cuh"

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

namespace gbmpm {

#include "materials.cuh"
#include "particle_pass.cuh"
#include "grid_pass.cuh"
#include "bookkeeping.cuh"

}  // namespace gbmpm

#include "rigid.cuh"

// ====================================================================== host
using namespace gbmpm;

namespace {
thread_local std::string g_err;

int fail(int code, const std::string &msg) {
    g_err = msg;
    return code;
}
#define GB_CUDA(call)                                                                            \
    do {                                                                                         \
        cudaError_t _e = (call);                                                                 \
        if (_e != cudaSuccess)                                                                   \
            return fail(GBMPM_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(_e));     \
    } while (0)

const char *kPhaseNames[GBMPM_NUM_PHASES] = {"compute_stress_from_F_trial", "p2g", "g2p2g_fused",
                                             "grid_update+BC", "g2p", "block_sort+gather"};

template <class T>
struct DevBuf {
    T *ptr = nullptr;
    size_t n = 0;
    cudaError_t ensure(size_t want) {
        if (want <= n && ptr) return cudaSuccess;
        if (ptr) cudaFree(ptr);
        ptr = nullptr;
        n = 0;
        cudaError_t e = cudaMalloc(&ptr, std::max<size_t>(want, 1) * sizeof(T));
        if (e == cudaSuccess) n = want;
        return e;
    }
    void release() { if (ptr) cudaFree(ptr); ptr = nullptr; n = 0; }
};

// Host bookkeeping of the CPIC lanes (the reference keeps the same on the Python
// side of MPM_Simulator_WARP): lane records with poses integrated per substep,
// the lane arrays the transfer passes read, and which boxes need restamping.
struct CdfHost {
    int n = 0;
    gbmpm_cdf rec[GBMPM_MAX_CDF];
    float c_cur[4][3] = {}, v_cur[4][3] = {}, w_cur[4][3] = {};
    float c_prev[4][3] = {}, v_prev[4][3] = {}, w_prev[4][3] = {};
    float fric[4] = {};
    int type[4] = {};
    bool dirty[4] = {}, active[4] = {}, has_prev_box[4] = {};
    int prev_box[4][6] = {};
    bool stale_set = false;     // tag_prev lags tag inside stale_box
    int stale_box[6] = {};
    bool lane_prev_stale = false;
    bool force = false;         // restamp every lane every substep (no dirty-lane skip)
    bool mask_off = false;      // scan every particle's stencil, no block-mask early-out
    int64_t stamps = 0;
    void sync_lane(int l) {    // _sync_cdf_lane (mpm_solver_warp.py:2883-2905)
        for (int a = 0; a < 3; ++a) {
            c_cur[l][a] = rec[l].center[a];
            v_cur[l][a] = rec[l].velocity[a];
            w_cur[l][a] = rec[l].omega[a];
        }
        fric[l] = rec[l].friction;
        type[l] = rec[l].surface_type;
    }
    void copy_lane_prev() {
        std::memcpy(c_prev, c_cur, sizeof c_cur);
        std::memcpy(v_prev, v_cur, sizeof v_cur);
        std::memcpy(w_prev, w_cur, sizeof w_cur);
        lane_prev_stale = false;
    }
};
}  // namespace

constexpr int kStages = 4;
struct Staging {
    PoseRec *pose = nullptr;
    size_t pose_cap = 0;
    double *time = nullptr;
    size_t time_cap = 0;
    ColDev *cols = nullptr;
    cudaEvent_t done = nullptr;
};

// One captured adjoint graph and the arguments it was captured for.
struct AdjGraph {
    cudaGraphExec_t g = nullptr;
    int substeps = -1;
    double dt = 0.0;
    uint64_t version = 0;
    gbmpm_adj_grads grads{};
    int64_t launches = 0;
    void drop() {
        if (g) cudaGraphExecDestroy(g);
        g = nullptr;
    }
};

struct gbmpm_engine {
    int device = 0;
    gbmpm_particles P{};
    gbmpm_grid G{};
    gbmpm_model M{};
    bool bound = false, modeled = false;
    std::vector<gbmpm_collider> cols;
    std::vector<ColDev> h_cols;   // the collider descriptor table (device copy: d_cols)
    bool cols_upload = false;     // h_cols changed since the last upload
    // device scratch
    DevBuf<MatTables> d_tab;
    DevBuf<ColDev> d_cols;
    DevBuf<PoseRec> d_pose;
    DevBuf<double> d_wrench;
    DevBuf<int> d_flag, d_list, d_count;
    DevBuf<unsigned> d_status;
    DevBuf<float> d_guard;
    DevBuf<unsigned long long> d_keys[2];
    DevBuf<long long> d_skeys, d_kminmax;
    DevBuf<int> d_idx[2];
    DevBuf<unsigned> d_hist;
    DevBuf<int> d_flagbuf;
    DevBuf<float> d_tmp;
    DevBuf<int> d_braw, d_bcur, d_bprev, d_bcount;
    // per-tick block-sorted working set
    DevBuf<float> ws_buf;
    DevBuf<unsigned long long> ws_keys[2];
    DevBuf<int> ws_idx[2];
    DevBuf<unsigned> ws_hist;
    gbmpm_particles W{};
    WsTable ws_table{};
    int ws_n = -1;
    // re-sorts inside a fused tick: every resort_every substeps the working copy is
    // sorted again by its current cells into the second copy and back (0: once per
    // tick; GBMPM_RESORT_AUTO: resort_interval's choice)
    int resort_every = GBMPM_RESORT_AUTO;
    DevBuf<float> ws_buf2;
    gbmpm_particles W2{};
    WsTable ws_table2{};
    DevBuf<int> ws_perm[2];   // working row -> caller particle, composed over the re-sorts
    int ws2_n = -1;
    // pinned staging of the per-tick uploads (pose table, substep times, collider
    // table): a ring, so that the host waits on the upload of kStages ticks ago rather
    // than on the last one, which is queued behind the last tick's work
    Staging stage[kStages];
    int stage_i = 0;
    int bd = 0;
    int num_sms = 148;
    bool graph_failed = false;          // a capture failed: live launches for the rest of the run
    bool fake_capture_failure = false;  // test hook: treat the next capture as failed
    int tile_occ = 3;       // resident CTAs per SM the tiled particle kernel is compiled for
    int cdf_occ = 3;        // the same for its CPIC variant
    bool pdl = true;        // programmatic dependent launch of the particle and grid passes
    bool det = false;       // this tick runs the deterministic passes (GBMPM_TICK_DETERMINISTIC)
    DevBuf<unsigned long long> det_key[2];   // P2G records of the deterministic passes, sorted by node
    DevBuf<int> det_idx[2];
    DevBuf<float4> det_val;
    DevBuf<unsigned> det_hist;
    bool cdf_fused_stamp = true;   // one restamp launch a substep (else the five-kernel sequence)
    int grid_ctas = 2;      // grid-update CTAs per SM
    // graph cache
    cudaGraphExec_t graph = nullptr;
    int g_substeps = -1, g_flags = -1;
    int64_t graph_launches = 0;
    double g_dt = 0.0;
    cudaStream_t g_stream = nullptr;
    bool dirty = true;
    uint64_t version = 1;   // bumped with every change a captured graph depends on
    // CPIC (CDF) colliders: lanes, node tag and distance grids (current and as of
    // the previous stamp), 4^3 occupancy mask, per-lane reaction
    CdfHost cdf;
    DevBuf<int> c_tag, c_tag_prev, c_block;
    DevBuf<float> c_d, c_d_prev;
    DevBuf<double> c_wrench;        // [4][6] reaction per lane (float64)
    DevBuf<double> c_partial;       // [CTA][4][6] per-CTA partials the transfer passes add into
    DevBuf<float> c_cache;          // [5][n] the tiled scatter's scan, read by the next gather
    DevBuf<float> c_cache2;   // the scan cache of the second working copy (re-sorts)
    float *c_cache_cur = nullptr;   // the scan cache of the copy the passes run on (null: c_cache)
    size_t c_partial_ctas = 0;
    int c_ng = 0;
    // adjoint segment storage and scratch (allocated by the first adjoint call)
    DevBuf<float> adj_states, adj_scratch;
    DevBuf<float4> adj_grid;
    DevBuf<int> adj_box;     // the adjoint segment's node box
    // the launches of one adjoint segment, captured once and replayed while the
    // segment's shape and buffers stay the same (key: substeps, dt, adjoint arrays,
    // engine version)
    // captured adjoint graphs: replay + reverse, forward with states kept, reverse alone
    AdjGraph adj_seg, adj_fwd, adj_rev;
    // rigid bodies and particle modifiers
    int n_bodies = 0;
    std::vector<gbmpm_rigid_surface> rsurf;
    DevBuf<gbmpm_rigid_body> d_bodies;
    DevBuf<double> d_racc;                  // [body][6] gathered momentum, angular momentum
    DevBuf<unsigned long long> d_rkey;      // [body][surface][2] contact keys (distance, particle)
    DevBuf<int> d_rlist, d_rcount;          // this tick's rigid particles (k_rigid_list) and their count
    int n_rigid = 0;                        // rigid particles when the bodies were set (grid sizing)
    int n_mods = 0;
    DevBuf<gbmpm_modifier> d_mods;
    DevBuf<double> d_time;                  // start time of every substep of the tick
    // profiling
    double prof_ms[GBMPM_NUM_PHASES] = {0};
    int64_t prof_n[GBMPM_NUM_PHASES] = {0};
    int64_t launches = 0;
};

namespace {

void mark_dirty(gbmpm_engine *e) {
    e->dirty = true;
    e->version++;
}

PK make_pk(gbmpm_engine *e, const gbmpm_particles &P, float dt, int list) {
    PK k{};
    k.x = P.x; k.v = P.v; k.C = P.C; k.F = P.F; k.Ft = P.F_trial; k.L = P.L; k.S = P.stress;
    k.mass = P.mass; k.vol = P.vol; k.Jp = P.Jp; k.mu = P.mu; k.lam = P.lam; k.ys = P.yield_stress;
    k.mat = P.material; k.sel = P.selection; k.cov = P.cov; k.n = P.n;
    k.gv = reinterpret_cast<const float4 *>(e->G.v);
    k.gmv = reinterpret_cast<float4 *>(e->G.mv);
    k.ng = e->G.n_grid;
    k.dx = e->M.dx; k.inv_dx = e->M.inv_dx; k.dt = dt; k.rpic = e->M.rpic_damping;
    k.periodic_x = e->M.periodic_x; k.update_cov = e->M.update_cov_with_F && P.cov;
    k.tab = e->d_tab.ptr; k.eta = e->M.eta_table; k.eta_n = e->M.eta_table_n;
    k.eta_smin = e->M.eta_table_smin; k.eta_smax = e->M.eta_table_smax;
    k.blk_flag = e->d_flag.ptr;
    k.bd = e->bd;
    size_t nb = (size_t)e->bd * e->bd * e->bd;
    k.blk_list = e->d_list.ptr + (size_t)list * nb;
    k.blk_count = e->d_count.ptr + list;
    k.status = e->d_status.ptr;
    for (int a = 0; a < 3; ++a) k.grav[a] = e->M.gravity[a];
    k.n_mods = (e->n_mods > 0 && P.mod_mask) ? e->n_mods : 0;
    k.mods = e->d_mods.ptr;
    k.mod_mask = P.mod_mask;
    k.sub_time = e->d_time.ptr;
    k.sub = 0;
    k.rigid_defer = 0;
    if (e->cdf.n > 0 && P.cdf_tag) {
        const CdfHost &H = e->cdf;
        k.cdf_on = 1;
        k.cnb = (e->c_ng + 3) / 4;
        k.ctag = e->c_tag.ptr; k.ctag_prev = e->c_tag_prev.ptr; k.cblock = e->cdf.mask_off ? nullptr : e->c_block.ptr;
        k.cd = e->c_d.ptr; k.cd_prev = e->c_d_prev.ptr;
        k.ptag = P.cdf_tag;
        k.cwrench = e->c_partial.ptr;
        k.ccache = e->c_cache_cur ? e->c_cache_cur : e->c_cache.ptr;
        std::memcpy(k.lanes.c_cur, H.c_cur, sizeof H.c_cur);
        std::memcpy(k.lanes.c_prev, H.c_prev, sizeof H.c_prev);
        std::memcpy(k.lanes.v_prev, H.v_prev, sizeof H.v_prev);
        std::memcpy(k.lanes.w_prev, H.w_prev, sizeof H.w_prev);
        std::memcpy(k.lanes.fric, H.fric, sizeof H.fric);
        std::memcpy(k.lanes.type, H.type, sizeof H.type);
    }
    return k;
}

bool has_solids(const gbmpm_model &m) {
    const uint32_t fluid = (1u << 6) | (1u << 7) | (1u << 8) | (1u << 10) | (1u << 12);
    return (m.material_mask & ~fluid) != 0;
}

// Launch with programmatic stream serialization (see pdl_wait) when enabled.
template <typename... P, typename... A>
void launch_pdl(gbmpm_engine *e, void (*kern)(P...), int grid, int block, cudaStream_t s, A... args) {
    launch_kernel(e->pdl, kern, grid, block, s, args...);
}

// The deterministic passes: G2P, stress, then P2G as 27 records a particle, a stable
// radix sort of the records by node (so each node's records stay in particle
// order) and one in-order sum per node.
void det_pass(gbmpm_engine *e, const PK &k, int mode, cudaStream_t s) {
    if (mode & PASS_G2P) { det_launch_g2p(k, (mode & PASS_RESET_LISTS) != 0, s); e->launches++; }
    if (mode & PASS_STRESS) { det_launch_stress(k, s); e->launches++; }
    if (!(mode & PASS_P2G)) return;
    const int nrec = 27 * k.n;
    det_launch_p2g(k, e->det_key[0].ptr, e->det_idx[0].ptr, e->det_val.ptr, s);
    const unsigned long long none = (unsigned long long)k.ng * k.ng * k.ng;   // key of an empty record
    int bits = 0;
    while (bits < 64 && (none >> bits) != 0ull) ++bits;
    const int ntiles = (nrec + kSortTile - 1) / kSortTile;
    int cur = 0;
    for (int shift = 0; shift < bits; shift += kRadixBits) {
        k_radix_hist<<<ntiles, kSortThreads, 0, s>>>(e->det_key[cur].ptr, nrec, shift, e->det_hist.ptr, ntiles);
        k_radix_scan<<<1, 1024, 0, s>>>(e->det_hist.ptr, ntiles * kRadixBins);
        k_radix_scatter<<<ntiles, kSortThreads, 0, s>>>(e->det_key[cur].ptr, e->det_idx[cur].ptr,
                                                         e->det_key[cur ^ 1].ptr, e->det_idx[cur ^ 1].ptr, nrec,
                                                         shift, e->det_hist.ptr, ntiles);
        e->launches += 3;
        cur ^= 1;
    }
    det_launch_segsum(k, e->det_key[cur].ptr, e->det_idx[cur].ptr, e->det_val.ptr, nrec, s);
    e->launches += 2;
}

void launch_particles(gbmpm_engine *e, const PK &k, int mode, bool tiled, cudaStream_t s) {
    if (e->det) { det_pass(e, k, mode, s); return; }
    ParticleLaunch L{tiled, has_solids(e->M), e->pdl, e->tile_occ, e->cdf_occ};
    launch_particle_pass(L, k, mode, s);
    e->launches++;
}

// Allocates the block-sorted working copy and the table of fields the tick
// gathers into it and scatters back (only fields a tick writes go back). With
// `second`, also the second copy, with the same layout, that re-sorts write.
cudaError_t ensure_ws(gbmpm_engine *e, bool second) {
    const gbmpm_particles &P = e->P;
    const int n = P.n;
    const bool cov = P.cov && e->M.update_cov_with_F;
    struct Spec { float *ext; int w; int back; float **dst; };
    gbmpm_particles &W = e->W;
    W = P;
    Spec spec[] = {
        {P.x, 3, 1, &W.x}, {P.v, 3, 1, &W.v}, {P.C, 9, 1, &W.C}, {P.F, 9, 1, &W.F},
        {P.F_trial, 9, 1, &W.F_trial}, {P.L, 9, 1, &W.L}, {P.stress, 9, 1, &W.stress},
        {P.mass, 1, 0, &W.mass}, {P.vol, 1, 0, &W.vol}, {P.Jp, 1, 1, &W.Jp}, {P.mu, 1, 1, &W.mu},
        {P.lam, 1, 1, &W.lam}, {P.yield_stress, 1, 1, &W.yield_stress},
        {reinterpret_cast<float *>(P.material), 1, 0, reinterpret_cast<float **>(&W.material)},
        {reinterpret_cast<float *>(P.selection), 1, 0, reinterpret_cast<float **>(&W.selection)},
        {cov ? P.cov : nullptr, 6, 1, &W.cov},
        {e->cdf.n > 0 ? reinterpret_cast<float *>(P.cdf_tag) : nullptr, 1, 1, reinterpret_cast<float **>(&W.cdf_tag)},
        {e->n_bodies > 0 ? reinterpret_cast<float *>(P.rigid_id) : nullptr, 1, 0,
         reinterpret_cast<float **>(&W.rigid_id)},
        {e->n_bodies > 0 ? P.x_ref : nullptr, 3, 0, &W.x_ref},
        {e->n_mods > 0 ? reinterpret_cast<float *>(P.mod_mask) : nullptr, 1, 0, reinterpret_cast<float **>(&W.mod_mask)},
    };
    size_t total = 0;
    for (const Spec &sp : spec) if (sp.ext) total += (size_t)sp.w * n;
    cudaError_t err = e->ws_buf.ensure(total);
    if (err != cudaSuccess) return err;
    if (second && (err = e->ws_buf2.ensure(total)) != cudaSuccess) return err;
    size_t off = 0;
    e->ws_table.nf = 0;
    e->ws_table2.nf = 0;
    std::vector<std::pair<size_t, size_t>> rebase;   // (member offset in gbmpm_particles, buffer offset)
    for (const Spec &sp : spec) {
        if (!sp.ext) { *sp.dst = nullptr; continue; }
        float *ws = e->ws_buf.ptr + off;
        *sp.dst = ws;
        e->ws_table.f[e->ws_table.nf++] = WsField{sp.ext, ws, sp.w, sp.back};
        if (second) {
            e->ws_table2.f[e->ws_table2.nf++] = WsField{sp.ext, e->ws_buf2.ptr + off, sp.w, sp.back};
            rebase.push_back({(size_t)(reinterpret_cast<char *>(sp.dst) - reinterpret_cast<char *>(&W)), off});
        }
        off += (size_t)sp.w * n;
    }
    W.density = nullptr;
    W.init_cov = nullptr;
    if (!cov) W.cov = nullptr;
    if (second) {
        e->W2 = W;
        for (const auto &r : rebase)
            *reinterpret_cast<float **>(reinterpret_cast<char *>(&e->W2) + r.first) = e->ws_buf2.ptr + r.second;
        if ((err = e->ws_perm[0].ensure(n)) != cudaSuccess) return err;
        if ((err = e->ws_perm[1].ensure(n)) != cudaSuccess) return err;
    }
    e->ws2_n = second ? n : -1;
    const int ntiles = (n + kSortTile - 1) / kSortTile;
    if ((err = e->ws_keys[0].ensure(n)) != cudaSuccess) return err;
    if ((err = e->ws_keys[1].ensure(n)) != cudaSuccess) return err;
    if ((err = e->ws_idx[0].ensure(n)) != cudaSuccess) return err;
    if ((err = e->ws_idx[1].ensure(n)) != cudaSuccess) return err;
    if ((err = e->ws_hist.ensure((size_t)ntiles * kRadixBins)) != cudaSuccess) return err;
    e->ws_n = n;
    return cudaSuccess;
}

// Records the stable sort of n rows by the cell keys of positions x (the caller's
// records, or with soa the working copy's own components); returns the sorted row
// indices (in ws_idx, which the next sort overwrites).
const int *record_cell_sort(gbmpm_engine *e, const float *x, bool soa, cudaStream_t s) {
    const int n = e->P.n;
    const int ntiles = (n + kSortTile - 1) / kSortTile;
    if (soa)
        k_cell_keys<true><<<(n + 255) / 256, 256, 0, s>>>(x, n, e->M.inv_dx, e->G.n_grid, e->bd, e->ws_keys[0].ptr,
                                                          e->ws_idx[0].ptr);
    else
        k_cell_keys<false><<<(n + 255) / 256, 256, 0, s>>>(x, n, e->M.inv_dx, e->G.n_grid, e->bd, e->ws_keys[0].ptr,
                                                           e->ws_idx[0].ptr);
    e->launches++;
    unsigned long long maxkey = ((unsigned long long)e->bd * e->bd * e->bd << 6) - 1ull;
    int bits = 0;
    while (bits < 64 && (maxkey >> bits) != 0ull) ++bits;
    int cur = 0;
    for (int shift = 0; shift < bits; shift += kRadixBits) {
        k_radix_hist<<<ntiles, kSortThreads, 0, s>>>(e->ws_keys[cur].ptr, n, shift, e->ws_hist.ptr, ntiles);
        k_radix_scan<<<1, 1024, 0, s>>>(e->ws_hist.ptr, ntiles * kRadixBins);
        k_radix_scatter<<<ntiles, kSortThreads, 0, s>>>(e->ws_keys[cur].ptr, e->ws_idx[cur].ptr,
                                                         e->ws_keys[cur ^ 1].ptr, e->ws_idx[cur ^ 1].ptr, n, shift,
                                                         e->ws_hist.ptr, ntiles);
        e->launches += 3;
        cur ^= 1;
    }
    return e->ws_idx[cur].ptr;
}

// Substeps between re-sorts of the working copy inside a tick of S substeps (0: none).
// The automatic choice weighs a re-sort's cost (about 0.15 ms at 340k particles, its
// eleven launches a fixed part of that) against the longer scatter runs it buys:
// scenes of 150,000 particles or more (the 340k pour and the 362k dam break gained;
// 64 scenes of 54k particles stepped one by one, one re-sort in each 100-substep
// tick, ran 5 % slower), ticks of 100 substeps or more, every max(50, S / 3).
constexpr int kResortMinParticles = 150000;
int resort_interval(const gbmpm_engine *e, int S) {
    if (e->resort_every >= 0) return e->resort_every;
    return (S >= 100 && e->P.n >= kResortMinParticles) ? std::max(50, S / 3) : 0;
}

// Records the working-set sort + gather; returns the permutation buffer.
const int *record_ws_begin(gbmpm_engine *e, cudaStream_t s) {
    const int n = e->P.n;
    const int *perm = record_cell_sort(e, e->P.x, false, s);
    k_ws_gather<<<(n + 255) / 256, 256, 0, s>>>(e->ws_table, perm, n);
    e->launches++;
    return perm;
}

// Records a re-sort of the working copy inside a tick: `from` (positions x) is sorted
// again by its current cells into `to`, and the row -> particle map perm_in into
// perm_out.
void record_ws_resort(gbmpm_engine *e, const float *x, const WsTable &from, const WsTable &to, const int *perm_in,
                      int *perm_out, cudaStream_t s) {
    const int n = e->P.n;
    const int *idx = record_cell_sort(e, x, true, s);
    k_ws_permute<<<(n + 255) / 256, 256, 0, s>>>(from, to, idx, perm_in, perm_out, n);
    e->launches++;
}

GK make_gk(gbmpm_engine *e, float dt, int substep, int list) {
    GK g{};
    g.gmv = reinterpret_cast<float4 *>(e->G.mv);
    g.gv = reinterpret_cast<float4 *>(e->G.v);
    g.ng = e->G.n_grid;
    g.dx = e->M.dx; g.dt = dt;
    g.g[0] = e->M.gravity[0]; g.g[1] = e->M.gravity[1]; g.g[2] = e->M.gravity[2];
    g.damp = e->M.grid_v_damping_scale;
    g.ncol = (int)e->cols.size();
    g.cols = e->d_cols.ptr;
    g.poses = e->d_pose.ptr + (size_t)substep * std::max<int>(1, g.ncol);
    g.wrench = e->d_wrench.ptr;
    g.blk_flag = e->d_flag.ptr;
    size_t nb = (size_t)e->bd * e->bd * e->bd;
    g.blk_list = e->d_list.ptr + (size_t)list * nb;
    g.blk_count_read = e->d_count.ptr + list;
    g.blk_count_reset = e->d_count.ptr + (list ^ 1);
    g.bd = e->bd;
    return g;
}

void launch_grid(gbmpm_engine *e, float dt, int substep, int list, cudaStream_t s) {
    GK g = make_gk(e, dt, substep, list);
    // one wave of CTAs looping over the active blocks: the per-CTA setup (collider
    // tables into shared memory, two barriers) is paid once per SM slot, not per item
    int grid = e->num_sms * e->grid_ctas;
    launch_pdl(e, k_grid, grid, kGridThreads, s, g);
    e->launches++;
}

ColDev to_dev(const gbmpm_collider &c) {
    ColDev d{};
    d.kind = c.kind; d.surface = c.surface_type; d.sdf_res = c.sdf_res;
    for (int a = 0; a < 3; ++a) {
        d.normal[a] = c.normal[a]; d.size[a] = c.size[a]; d.vel[a] = c.velocity[a]; d.omega[a] = c.omega[a];
        d.origin[a] = c.sdf_origin[a];
    }
    d.friction = c.friction; d.outer_r = c.outer_radius; d.inner_r = c.inner_radius; d.half_h = c.half_height;
    d.floor_z = c.inner_floor_z; d.fillet = c.fillet_radius; d.sticky = c.sticky_depth; d.band_c = c.contact_band;
    d.cell = c.sdf_cell; d.band = c.band; d.sdf_val = c.sdf_val; d.sdf_grad = c.sdf_grad;
    return d;
}

// Host pose integration for one substep: the reference's modify_bc callables
// (mpm_solver_warp.py:2090-2096, 2227-2254, 2749-2760) on float64 values read
// from the fp32 struct and rounded back.
void integrate_pose(gbmpm_collider &c, double time, double dt) {
    if (!(time >= (double)c.start_time && time < (double)c.end_time)) return;
    if (c.kind == GBMPM_COLLIDER_BOX || c.kind == GBMPM_COLLIDER_CUP || c.kind == GBMPM_COLLIDER_SDF)
        for (int i = 0; i < 3; ++i) c.point[i] = (float)((double)c.point[i] + dt * (double)c.velocity[i]);
    if (c.kind == GBMPM_COLLIDER_CUP) {
        double w[3] = {c.omega[0], c.omega[1], c.omega[2]};
        double wn = std::sqrt(w[0] * w[0] + w[1] * w[1] + w[2] * w[2]);
        double ang = wn * dt;
        if (ang > 1.0e-12) {
            double ax[3] = {w[0] / wn, w[1] / wn, w[2] / wn};
            double K[3][3] = {{0.0, -ax[2], ax[1]}, {ax[2], 0.0, -ax[0]}, {-ax[1], ax[0], 0.0}};
            double s = std::sin(ang), cc = 1.0 - std::cos(ang);
            double Ri[3][3], Rn[3][3];
            for (int i = 0; i < 3; ++i)
                for (int j = 0; j < 3; ++j) {
                    double k2 = K[i][0] * K[0][j] + K[i][1] * K[1][j] + K[i][2] * K[2][j];
                    Ri[i][j] = ((i == j) ? 1.0 : 0.0) + s * K[i][j] + cc * k2;
                }
            for (int i = 0; i < 3; ++i)
                for (int j = 0; j < 3; ++j)
                    Rn[i][j] = Ri[i][0] * c.rot64[j] + Ri[i][1] * c.rot64[3 + j] + Ri[i][2] * c.rot64[6 + j];
            for (int i = 0; i < 3; ++i)
                for (int j = 0; j < 3; ++j) { c.rot64[3 * i + j] = Rn[i][j]; c.rot[3 * i + j] = (float)Rn[i][j]; }
        }
    }
    if (c.kind == GBMPM_COLLIDER_SDF) {
        double w[3] = {c.omega[0], c.omega[1], c.omega[2]};
        double sp = std::sqrt(w[0] * w[0] + w[1] * w[1] + w[2] * w[2]);
        if (!(sp * dt < 1e-12)) {
            double q[4] = {c.quat[0], c.quat[1], c.quat[2], c.quat[3]};
            double half = 0.5 * sp * dt, sh = std::sin(half);
            double d[4] = {w[0] / sp * sh, w[1] / sp * sh, w[2] / sp * sh, std::cos(half)};
            double r[4] = {d[3] * q[0] + d[0] * q[3] + d[1] * q[2] - d[2] * q[1],
                           d[3] * q[1] - d[0] * q[2] + d[1] * q[3] + d[2] * q[0],
                           d[3] * q[2] + d[0] * q[1] - d[1] * q[0] + d[2] * q[3],
                           d[3] * q[3] - d[0] * q[0] - d[1] * q[1] - d[2] * q[2]};
            double nr = std::sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2] + r[3] * r[3]);
            for (int i = 0; i < 4; ++i) c.quat[i] = (float)(r[i] / nr);
        }
    }
}

// A collider's pose record for a substep starting at time tf: live inside its
// window; a cuboid with reset == 1 zeroes its nodes for 15 substeps after it ends.
PoseRec pose_of(const gbmpm_collider &col, float tf, float dtf) {
    PoseRec r;
    std::memset(&r, 0, sizeof r);
    bool live = tf >= col.start_time && tf < col.end_time;
    if (col.kind == GBMPM_COLLIDER_BOX && !live && col.reset == 1)
        r.mode = (tf < col.end_time + 15.0f * dtf) ? 2 : 0;
    else r.mode = live ? 1 : 0;
    for (int a = 0; a < 3; ++a) r.p[a] = col.point[a];
    for (int a = 0; a < 9; ++a) r.r[a] = col.rot[a];
    for (int a = 0; a < 4; ++a) r.q[a] = col.quat[a];
    return r;
}

// Builds the [S][ncol] pose table for a tick and advances the host collider
// records and clock exactly as S calls of _apply_grid_bc + time += dt would.
void build_pose_table(gbmpm_engine *e, PoseRec *out, double &time, double dt, int S) {
    int nc = (int)e->cols.size();
    int stride = std::max(1, nc);
    float dtf = (float)dt;
    for (int s = 0; s < S; ++s) {
        float tf = (float)time;
        for (int c = 0; c < nc; ++c) out[(size_t)s * stride + c] = pose_of(e->cols[c], tf, dtf);
        for (int c = 0; c < nc; ++c) integrate_pose(e->cols[c], time, dt);
        time = time + dt;
    }
}

int check_ready(gbmpm_engine *e) {
    if (!e) return fail(GBMPM_ERR_ARG, "null engine");
    if (!e->bound) return fail(GBMPM_ERR_STATE, "buffers not bound (call gbmpm_bind)");
    if (!e->modeled) return fail(GBMPM_ERR_STATE, "model not set (call gbmpm_set_model)");
    return GBMPM_OK;
}

// ---- CPIC (CDF) host driver ----------------------------------------------------
void fold_cdf_wrench(gbmpm_engine *e, cudaStream_t s) {
    if (!e->c_partial_ctas || !e->c_wrench.ptr) return;
    k_cdf_wrench_fold<<<(6 * GBMPM_MAX_CDF + 7) / 8, 256, 0, s>>>(e->c_partial.ptr, (int)e->c_partial_ctas,
                                                                  e->c_wrench.ptr);
    e->launches++;
}

int cdf_grid_blocks(gbmpm_engine *e, long long work) {
    long long want = (work + 255) / 256;
    return (int)std::max<long long>(1, std::min<long long>(want, (long long)e->num_sms * 8));
}

// The lane's grid box: its field's corners posed by centre and quaternion in
// float64, widened by a 2-node halo and clipped to the grid (cdf_aabb,
// mpm_solver_warp.py:2884-2895, _grid_box).
bool cdf_lane_box(const gbmpm_cdf &r, const gbmpm_model &M, int *box) {
    double qx = r.quat[0], qy = r.quat[1], qz = r.quat[2], qw = r.quat[3];
    double R[3][3] = {{1 - 2 * (qy * qy + qz * qz), 2 * (qx * qy - qz * qw), 2 * (qx * qz + qy * qw)},
                      {2 * (qx * qy + qz * qw), 1 - 2 * (qx * qx + qz * qz), 2 * (qy * qz - qx * qw)},
                      {2 * (qx * qz - qy * qw), 2 * (qy * qz + qx * qw), 1 - 2 * (qx * qx + qy * qy)}};
    double ext = (r.res - 1) * (double)r.cell;
    double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
    for (int a = 0; a < 2; ++a)
        for (int b = 0; b < 2; ++b)
            for (int c = 0; c < 2; ++c) {
                double cr[3] = {(double)r.origin[0] + a * ext, (double)r.origin[1] + b * ext,
                                (double)r.origin[2] + c * ext};
                for (int i = 0; i < 3; ++i) {
                    double p = (double)r.center[i] + R[i][0] * cr[0] + R[i][1] * cr[1] + R[i][2] * cr[2];
                    lo[i] = std::min(lo[i], p);
                    hi[i] = std::max(hi[i], p);
                }
            }
    const double dx = (double)M.grid_lim / M.n_grid;
    for (int i = 0; i < 3; ++i) {
        int l = std::max(0, (int)std::floor(lo[i] / dx) - 2);
        int h = std::min(M.n_grid, (int)std::ceil(hi[i] / dx) + 2 + 1);
        if (h - l <= 0) return false;
        box[i] = l;
        box[3 + i] = h;
    }
    return true;
}

CdfBox to_box(const int *b) {
    CdfBox x;
    for (int i = 0; i < 3; ++i) { x.lo[i] = b[i]; x.hi[i] = b[3 + i]; }
    return x;
}

void cdf_copy_prev_box(gbmpm_engine *e, const int *b, cudaStream_t s) {
    CdfBox box = to_box(b);
    long long vol = (long long)(b[3] - b[0]) * (b[4] - b[1]) * (b[5] - b[2]);
    k_cdf_copy_prev<<<cdf_grid_blocks(e, vol), 256, 0, s>>>(e->c_tag.ptr, e->c_d.ptr, e->c_tag_prev.ptr,
                                                           e->c_d_prev.ptr, box, e->c_ng);
    e->launches++;
}

// Start-of-substep stamp (_stamp_cdf, mpm_solver_warp.py:3040-3098): lanes whose
// activity window flipped or that moved are restamped over the union of their
// current and last boxes; every lane restamps inside that box. With lag_prev
// (fused ticks) the previous grids catch up at the next stamp or before the
// closing G2P, so the G2P inside a fused pass reads the tags its grid velocities
// were computed with.
void cdf_stamp(gbmpm_engine *e, double time, bool lag_prev, cudaStream_t s) {
    CdfHost &H = e->cdf;
    if (H.n == 0) return;
    // a pending catch-up of the previous grids folds into the restamp launch
    int stale[6] = {0, 0, 0, 0, 0, 0};
    const bool had_stale = H.stale_set;
    if (had_stale) { std::memcpy(stale, H.stale_box, sizeof stale); H.stale_set = false; }
    auto flush_stale = [&]() { if (had_stale) cdf_copy_prev_box(e, stale, s); };
    for (int l = 0; l < H.n; ++l) {
        bool act = time >= (double)H.rec[l].start_time && time < (double)H.rec[l].end_time;
        if (act != H.active[l]) { H.active[l] = act; H.dirty[l] = true; }
    }
    if (H.force)
        for (int l = 0; l < H.n; ++l) H.dirty[l] = true;
    bool any = false;
    for (int l = 0; l < H.n; ++l) any = any || H.dirty[l];
    if (!any) { flush_stale(); return; }
    int box[6] = {INT32_MAX, INT32_MAX, INT32_MAX, INT32_MIN, INT32_MIN, INT32_MIN};
    bool have = false;
    auto grow = [&](const int *b) {
        for (int i = 0; i < 3; ++i) { box[i] = std::min(box[i], b[i]); box[3 + i] = std::max(box[3 + i], b[3 + i]); }
        have = true;
    };
    for (int l = 0; l < H.n; ++l) {
        if (!H.dirty[l]) continue;
        int b[6];
        bool ok = cdf_lane_box(H.rec[l], e->M, b);
        if (ok) grow(b);
        if (H.has_prev_box[l]) grow(H.prev_box[l]);
        H.has_prev_box[l] = ok;
        if (ok) std::memcpy(H.prev_box[l], b, sizeof b);
    }
    for (int l = 0; l < H.n; ++l) H.dirty[l] = false;
    if (!have) { flush_stale(); return; }
    H.stamps++;
    const int ng = e->c_ng;
    if (e->cdf_fused_stamp) {
        CdfRestamp a{};
        a.ng = ng;
        a.nb = (ng + 3) / 4;
        a.box = to_box(box);
        a.stale = had_stale ? to_box(stale) : CdfBox{{0, 0, 0}, {0, 0, 0}};
        a.post_copy = lag_prev ? 0 : 1;
        a.tag = e->c_tag.ptr; a.tag_prev = e->c_tag_prev.ptr; a.block = e->c_block.ptr;
        a.d = e->c_d.ptr; a.d_prev = e->c_d_prev.ptr;
        const float tf = (float)time;
        for (int l = 0; l < H.n; ++l) {
            const gbmpm_cdf &r = H.rec[l];
            int lb[6], clip[6];
            if (!cdf_lane_box(r, e->M, lb)) continue;
            bool empty = false;
            for (int i = 0; i < 3; ++i) {
                clip[i] = std::max(box[i], lb[i]);
                clip[3 + i] = std::min(box[3 + i], lb[3 + i]);
                if (clip[3 + i] <= clip[i]) empty = true;
            }
            if (empty || tf < r.start_time || tf >= r.end_time) continue;
            CdfStamp &c = a.lane[a.nl++];
            c.values = r.values; c.valid = r.valid; c.res = r.res; c.lane = l; c.ng = ng;
            for (int i = 0; i < 3; ++i) { c.origin[i] = r.origin[i]; c.center[i] = r.center[i]; }
            for (int i = 0; i < 4; ++i) c.quat[i] = r.quat[i];
            c.cell = r.cell; c.band = r.band; c.dx = e->M.dx;
            c.box = to_box(clip);
        }
        // blocks to visit: those of the stamp box and of the stale box
        int vb[6] = {box[0] >> 2, box[1] >> 2, box[2] >> 2, ((box[3] - 1) >> 2) + 1, ((box[4] - 1) >> 2) + 1,
                     ((box[5] - 1) >> 2) + 1};
        a.mb = to_box(vb);
        if (had_stale && stale[3] > stale[0] && stale[4] > stale[1] && stale[5] > stale[2])
            for (int i = 0; i < 3; ++i) {
                vb[i] = std::min(vb[i], stale[i] >> 2);
                vb[3 + i] = std::max(vb[3 + i], ((stale[3 + i] - 1) >> 2) + 1);
            }
        a.bb = to_box(vb);
        const long long nblk = (long long)(vb[3] - vb[0]) * (vb[4] - vb[1]) * (vb[5] - vb[2]);
        const int ctas = (int)std::max<long long>(1, std::min<long long>((nblk + 7) / 8, (long long)e->num_sms * 8));
        k_cdf_restamp<<<ctas, 256, 0, s>>>(a);
        e->launches++;
        if (lag_prev) { H.stale_set = true; std::memcpy(H.stale_box, box, sizeof box); }
        return;
    }
    flush_stale();
    long long vol = (long long)(box[3] - box[0]) * (box[4] - box[1]) * (box[5] - box[2]);
    k_cdf_clear<<<cdf_grid_blocks(e, vol), 256, 0, s>>>(e->c_tag.ptr, e->c_d.ptr, to_box(box), ng);
    e->launches++;
    const float tf = (float)time;
    for (int l = 0; l < H.n; ++l) {
        const gbmpm_cdf &r = H.rec[l];
        int lb[6], clip[6];
        if (!cdf_lane_box(r, e->M, lb)) continue;
        bool empty = false;
        for (int i = 0; i < 3; ++i) {
            clip[i] = std::max(box[i], lb[i]);
            clip[3 + i] = std::min(box[3 + i], lb[3 + i]);
            if (clip[3 + i] <= clip[i]) empty = true;
        }
        if (empty || tf < r.start_time || tf >= r.end_time) continue;
        CdfStamp a{};
        a.values = r.values; a.valid = r.valid; a.res = r.res; a.lane = l; a.ng = ng;
        for (int i = 0; i < 3; ++i) { a.origin[i] = r.origin[i]; a.center[i] = r.center[i]; }
        for (int i = 0; i < 4; ++i) a.quat[i] = r.quat[i];
        a.cell = r.cell; a.band = r.band; a.dx = e->M.dx;
        a.box = to_box(clip);
        a.tag = e->c_tag.ptr; a.d = e->c_d.ptr;
        long long cv = (long long)(clip[3] - clip[0]) * (clip[4] - clip[1]) * (clip[5] - clip[2]);
        k_cdf_stamp<<<cdf_grid_blocks(e, cv), 256, 0, s>>>(a);
        e->launches++;
    }
    if (lag_prev) { H.stale_set = true; std::memcpy(H.stale_box, box, sizeof box); }
    else cdf_copy_prev_box(e, box, s);
    const int nb = (ng + 3) / 4;
    int bb[6] = {box[0] >> 2, box[1] >> 2, box[2] >> 2, ((box[3] - 1) >> 2) + 1, ((box[4] - 1) >> 2) + 1,
                 ((box[5] - 1) >> 2) + 1};
    long long bv = (long long)(bb[3] - bb[0]) * (bb[4] - bb[1]) * (bb[5] - bb[2]);
    k_cdf_block_mask<<<cdf_grid_blocks(e, bv), 256, 0, s>>>(e->c_tag.ptr, e->c_tag_prev.ptr, e->c_block.ptr,
                                                           to_box(bb), nb, ng);
    e->launches++;
}

// Per-substep lane pose integration (_integrate_cdf_poses, mpm_solver_warp.py:
// 3107-3148): centre += dt v and quaternion composed with exp(dt w / 2), in
// float64 from the fp32 record and rounded back.
void cdf_integrate(gbmpm_engine *e, double time, double dt, bool lag_prev) {
    CdfHost &H = e->cdf;
    if (H.n == 0) return;
    if (lag_prev && H.lane_prev_stale) H.copy_lane_prev();
    for (int l = 0; l < H.n; ++l) {
        gbmpm_cdf &r = H.rec[l];
        if (!(time >= (double)r.start_time && time < (double)r.end_time)) continue;
        if (r.velocity[0] == 0.0f && r.velocity[1] == 0.0f && r.velocity[2] == 0.0f && r.omega[0] == 0.0f &&
            r.omega[1] == 0.0f && r.omega[2] == 0.0f)
            continue;
        for (int a = 0; a < 3; ++a) r.center[a] = (float)((double)r.center[a] + dt * (double)r.velocity[a]);
        double w[3] = {r.omega[0], r.omega[1], r.omega[2]};
        double sp = std::sqrt(w[0] * w[0] + w[1] * w[1] + w[2] * w[2]);
        if (!(sp * dt < 1e-12)) {
            double q[4] = {r.quat[0], r.quat[1], r.quat[2], r.quat[3]};
            double half = 0.5 * sp * dt, sh = std::sin(half);
            double d[4] = {w[0] / sp * sh, w[1] / sp * sh, w[2] / sp * sh, std::cos(half)};
            double o[4] = {d[3] * q[0] + d[0] * q[3] + d[1] * q[2] - d[2] * q[1],
                           d[3] * q[1] - d[0] * q[2] + d[1] * q[3] + d[2] * q[0],
                           d[3] * q[2] + d[0] * q[1] - d[1] * q[0] + d[2] * q[3],
                           d[3] * q[3] - d[0] * q[0] - d[1] * q[1] - d[2] * q[2]};
            double nr = std::sqrt(o[0] * o[0] + o[1] * o[1] + o[2] * o[2] + o[3] * o[3]);
            for (int i = 0; i < 4; ++i) r.quat[i] = (float)(o[i] / nr);
        }
        H.sync_lane(l);
        H.dirty[l] = true;
        H.lane_prev_stale = true;
    }
    if (!lag_prev && H.lane_prev_stale) H.copy_lane_prev();
}

// The rigid tail of substep `tail_sub` (gather, integrate, one contact per active
// rigid surface, write-back); with `deposit` the rigid particles' P2G of substep
// `sub` follows. perm maps working-set rows to the caller's particle order.
void record_rigid(gbmpm_engine *e, const gbmpm_particles &P, float dtf, int tail_sub, int sub, int list, bool deposit,
                  bool soa, const int *perm, cudaStream_t s) {
    if (P.n == 0) return;
    PK k = make_pk(e, P, dtf, list);   // the deposit marks the block list the next grid pass reads
    k.sub = sub;
    const long long nr = std::max(32, e->n_rigid);
    const int pb = (int)std::max<long long>(1, std::min<long long>((nr + 255) / 256, (long long)e->num_sms * 8));
    const int nb = e->n_bodies, bb = (nb + 63) / 64;
    const int *rid = P.rigid_id, *rl = e->d_rlist.ptr, *rc = e->d_rcount.ptr;
    if (soa) k_rigid_gather<true><<<pb, 256, 0, s>>>(k, rl, rc, rid, e->d_bodies.ptr, e->d_racc.ptr);
    else k_rigid_gather<false><<<pb, 256, 0, s>>>(k, rl, rc, rid, e->d_bodies.ptr, e->d_racc.ptr);
    k_rigid_integrate<<<bb, 64, 0, s>>>(e->d_bodies.ptr, nb, e->d_racc.ptr, dtf);
    e->launches += 2;
    if (!e->rsurf.empty()) {
        RigidSurfaces sf{};
        sf.n = (int)e->rsurf.size();
        for (int q = 0; q < sf.n; ++q) sf.s[q] = e->rsurf[q];
        for (int stage = 0; stage < 2; ++stage) {
            if (soa)
                k_rigid_contact<true><<<pb, 256, 0, s>>>(k, rl, rc, rid, P.x_ref, e->d_bodies.ptr, sf, e->d_rkey.ptr,
                                                         stage, perm);
            else
                k_rigid_contact<false><<<pb, 256, 0, s>>>(k, rl, rc, rid, P.x_ref, e->d_bodies.ptr, sf, e->d_rkey.ptr,
                                                          stage, nullptr);
        }
        if (soa) k_rigid_impulse<true><<<bb, 64, 0, s>>>(k, e->d_bodies.ptr, nb, P.x_ref, e->d_rkey.ptr, sf, tail_sub);
        else k_rigid_impulse<false><<<bb, 64, 0, s>>>(k, e->d_bodies.ptr, nb, P.x_ref, e->d_rkey.ptr, sf, tail_sub);
        e->launches += 3;
    }
    if (soa) k_rigid_update<true><<<pb, 256, 0, s>>>(k, rl, rc, rid, P.x_ref, e->d_bodies.ptr, deposit ? 1 : 0);
    else k_rigid_update<false><<<pb, 256, 0, s>>>(k, rl, rc, rid, P.x_ref, e->d_bodies.ptr, deposit ? 1 : 0);
    e->launches++;
}

// Records the launches of one tick on stream s.
// With CPIC lanes the host stamps and integrates lane poses between the
// launches (t0 = the tick's start time, dt its float64 substep), so such ticks
// run live, on the direct kernel.
void record_tick(gbmpm_engine *e, float dtf, int S, bool fused, bool reorder, cudaStream_t s, bool profile,
                 double t0 = 0.0, double dt = 0.0, int pose_offset = 0) {
    // Profiling brackets every phase launch with an event pair and resolves the pairs
    // once at the end of the tick: the host stays ahead of the GPU, so each pair
    // measures the launch itself rather than host submission latency.
    struct Mark { cudaEvent_t a, b; int phase; };
    std::vector<Mark> marks;
    auto timed = [&](int phase, auto fn) {
        if (!profile) { fn(); return; }
        Mark m{nullptr, nullptr, phase};
        cudaEventCreate(&m.a);
        cudaEventCreate(&m.b);
        cudaEventRecord(m.a, s);
        fn();
        cudaEventRecord(m.b, s);
        marks.push_back(m);
    };
    const int *perm = nullptr;
    if (reorder) timed(5, [&] { perm = record_ws_begin(e, s); });
    // the working copy the passes run on: a re-sort moves it to the other copy
    const gbmpm_particles *cur = reorder ? &e->W : &e->P;
    const WsTable *tab = &e->ws_table;
    const gbmpm_particles &P0 = *cur;
    const bool cdf = e->cdf.n > 0;
    const bool rigid = e->n_bodies > 0 && P0.rigid_id && P0.x_ref;
    auto rigid_rows = [&](const gbmpm_particles &P) {   // this tick's rigid particles, in its particle order
        cudaMemsetAsync(e->d_rcount.ptr, 0, sizeof(int), s);
        const int g = (int)std::max<long long>(1, std::min<long long>((P.n + 255) / 256, (long long)e->num_sms * 8));
        k_rigid_list<<<g, 256, 0, s>>>(P.material, P.selection, P.n, e->d_rlist.ptr, e->d_rcount.ptr);
        e->launches++;
    };
    if (rigid && P0.n > 0) rigid_rows(P0);
    // Particles cross cells during a long tick and the scatter's runs of one cell
    // break up; a fused tick sorts its working copy again every `every` substeps
    // (resort_interval), between a grid pass and the next fused pass, except where
    // that would leave less than half an interval of the tick. Every per-particle
    // field moves with the rows (the modifier masks among them); with CPIC lanes the
    // per-row scan cache (written by a scatter, read by the next gather) moves too,
    // and with rigid bodies the list of rigid rows is rebuilt.
    e->c_cache_cur = nullptr;
    const size_t ccache_n = 5 * (size_t)std::max(1, e->P.n);
    const int every = resort_interval(e, S);
    const bool resort = reorder && fused && every > 0 && S > every && e->ws2_n == e->P.n &&
                        (!cdf || (e->c_cache2.ptr && e->c_cache2.n >= ccache_n && e->c_cache.n >= ccache_n));
    int resorts = 0;
    double tc = t0;
    for (int sub = 0; sub < S; ++sub) {
        int list = sub & 1;
        bool resorted = false;
        if (resort && sub > 0 && sub % every == 0 && 2 * (S - sub) >= every) {
            timed(5, [&] {
                if (resorts == 0) {   // the tick's first map is in the sort buffers the re-sort reuses
                    cudaMemcpyAsync(e->ws_perm[0].ptr, perm, (size_t)e->P.n * sizeof(int), cudaMemcpyDeviceToDevice, s);
                }
                const bool to2 = tab == &e->ws_table;
                const WsTable *to = to2 ? &e->ws_table2 : &e->ws_table;
                WsTable from_t = *tab, to_t = *to;
                if (cdf) {   // the scan cache, 5 components a row
                    from_t.f[from_t.nf++] = WsField{nullptr, to2 ? e->c_cache.ptr : e->c_cache2.ptr, 5, 0};
                    to_t.f[to_t.nf++] = WsField{nullptr, to2 ? e->c_cache2.ptr : e->c_cache.ptr, 5, 0};
                    e->c_cache_cur = to2 ? e->c_cache2.ptr : e->c_cache.ptr;
                }
                int *out = e->ws_perm[(resorts + 1) & 1].ptr;
                record_ws_resort(e, cur->x, from_t, to_t, e->ws_perm[resorts & 1].ptr, out, s);
                tab = to;
                cur = to2 ? &e->W2 : &e->W;
                perm = out;
                if (rigid) rigid_rows(*cur);
            });
            ++resorts;
            resorted = true;
        }
        const gbmpm_particles &P = *cur;
        if (cdf) cdf_stamp(e, tc, fused, s);
        PK k = make_pk(e, P, dtf, list);
        k.sub = pose_offset + sub;
        bool last_stress = fused ? (sub == S - 1) : true;
        if (!fused || sub == 0) {
            int mode = PASS_STRESS | PASS_P2G | (last_stress ? PASS_STORE_ALL : 0);
            timed(0, [&] { launch_particles(e, k, mode, reorder, s); });
        } else {
            // a CPIC ghost velocity starts from the particle's previous velocity
            int mode = PASS_G2P | PASS_STRESS | PASS_P2G | (last_stress ? PASS_STORE_ALL : 0) |
                       (cdf ? PASS_STORE_VC : 0);
            k.rigid_defer = rigid ? 1 : 0;
            // after a re-sort the pass waits for the whole permute in stream order: it
            // loads particle rows before its programmatic wait
            const bool pdl = e->pdl;
            if (resorted) e->pdl = false;
            timed(2, [&] { launch_particles(e, k, mode, reorder, s); });
            e->pdl = pdl;
            // the rigid tail of the previous substep, then its rigid particles' P2G
            if (rigid) record_rigid(e, P, dtf, pose_offset + sub - 1, pose_offset + sub, list, true, reorder, perm, s);
        }
        timed(3, [&] { launch_grid(e, dtf, pose_offset + sub, list, s); });
        if (cdf) cdf_integrate(e, tc, dt, fused);
        tc = tc + dt;
        if (!fused) {
            PK kg = make_pk(e, P, dtf, list);
            timed(4, [&] { launch_particles(e, kg, PASS_G2P | PASS_RESET_LISTS, reorder, s); });
            if (rigid) record_rigid(e, P, dtf, pose_offset + sub, pose_offset + sub, list, false, reorder, perm, s);
        }
    }
    if (fused) {
        if (cdf && e->cdf.stale_set) {
            cdf_copy_prev_box(e, e->cdf.stale_box, s);
            e->cdf.stale_set = false;
        }
        PK k = make_pk(e, *cur, dtf, 0);
        timed(4, [&] { launch_particles(e, k, PASS_G2P | PASS_RESET_LISTS, reorder, s); });
        if (rigid) record_rigid(e, *cur, dtf, pose_offset + S - 1, pose_offset + S - 1, 0, false, reorder, perm, s);
    }
    if (reorder) {
        timed(5, [&] {
            k_ws_scatter<<<(e->P.n + 255) / 256, 256, 0, s>>>(*tab, perm, e->P.n);
            e->launches++;
        });
    }
    e->c_cache_cur = nullptr;   // each tick's first pass writes the scan cache afresh
    if (profile) {
        for (Mark &m : marks) {
            cudaEventSynchronize(m.b);
            float ms = 0.f;
            cudaEventElapsedTime(&ms, m.a, m.b);
            e->prof_ms[m.phase] += ms;
            e->prof_n[m.phase] += 1;
            cudaEventDestroy(m.a);
            cudaEventDestroy(m.b);
        }
    }
}

}  // namespace

extern "C" {

const char *gbmpm_last_error(void) { return g_err.c_str(); }

const char *gbmpm_phase_name(int32_t phase) {
    if (phase < 0 || phase >= GBMPM_NUM_PHASES) return "";
    return kPhaseNames[phase];
}

int gbmpm_engine_create(gbmpm_engine **out) {
    if (!out) return fail(GBMPM_ERR_ARG, "null out");
    gbmpm_engine *e = new gbmpm_engine();
    if (cudaGetDevice(&e->device) != cudaSuccess) { delete e; return fail(GBMPM_ERR_CUDA, "no CUDA device"); }
    cudaDeviceGetAttribute(&e->num_sms, cudaDevAttrMultiProcessorCount, e->device);
    if (const char *occ = std::getenv("GBMPM_TILE_OCC")) e->tile_occ = std::atoi(occ);
    if (const char *occ = std::getenv("GBMPM_CDF_OCC")) e->cdf_occ = std::atoi(occ);
    if (const char *pd = std::getenv("GBMPM_NO_PDL")) e->pdl = std::atoi(pd) == 0;
    if (const char *fs = std::getenv("GBMPM_CDF_SPLIT_STAMP")) e->cdf_fused_stamp = std::atoi(fs) == 0;
    if (const char *gc = std::getenv("GBMPM_GRID_CTAS")) e->grid_ctas = std::max(1, std::min(8, std::atoi(gc)));
    for (Staging &st : e->stage) {
        if (cudaEventCreateWithFlags(&st.done, cudaEventDisableTiming) != cudaSuccess) {
            for (Staging &o : e->stage)
                if (o.done) cudaEventDestroy(o.done);
            delete e;
            return fail(GBMPM_ERR_CUDA, "event create failed");
        }
    }
    *out = e;
    return GBMPM_OK;
}

void gbmpm_engine_destroy(gbmpm_engine *e) {
    if (e) { e->adj_seg.drop(); e->adj_fwd.drop(); e->adj_rev.drop(); }
    if (!e) return;
    cudaDeviceSynchronize();
    if (e->graph) cudaGraphExecDestroy(e->graph);
    for (Staging &st : e->stage) {
        if (st.done) cudaEventDestroy(st.done);
        if (st.pose) cudaFreeHost(st.pose);
        if (st.time) cudaFreeHost(st.time);
        if (st.cols) cudaFreeHost(st.cols);
    }
    e->d_bodies.release(); e->d_racc.release(); e->d_rkey.release(); e->d_mods.release(); e->d_time.release();
    e->d_rlist.release(); e->d_rcount.release();
    e->d_tab.release(); e->d_cols.release(); e->d_pose.release(); e->d_wrench.release();
    e->d_flag.release(); e->d_list.release(); e->d_count.release(); e->d_status.release();
    e->d_guard.release(); e->d_keys[0].release(); e->d_keys[1].release(); e->d_skeys.release(); e->d_kminmax.release(); e->d_idx[0].release();
    e->d_idx[1].release(); e->d_hist.release(); e->d_flagbuf.release(); e->d_tmp.release();
    e->d_braw.release(); e->d_bcur.release(); e->d_bprev.release(); e->d_bcount.release();
    e->ws_buf.release(); e->ws_keys[0].release(); e->ws_keys[1].release(); e->ws_idx[0].release();
    e->ws_idx[1].release(); e->ws_hist.release();
    e->c_tag.release(); e->c_tag_prev.release(); e->c_block.release(); e->c_d.release(); e->c_d_prev.release();
    e->c_wrench.release(); e->c_partial.release(); e->c_cache.release(); e->c_cache2.release();
    e->adj_states.release(); e->adj_scratch.release(); e->adj_grid.release(); e->adj_box.release();
    e->det_key[0].release(); e->det_key[1].release(); e->det_idx[0].release(); e->det_idx[1].release();
    e->det_val.release(); e->det_hist.release();
    delete e;
}

int gbmpm_bind(gbmpm_engine *e, const gbmpm_particles *p, const gbmpm_grid *g) {
    if (!e || !p || !g) return fail(GBMPM_ERR_ARG, "null argument");
    if (p->n < 0 || g->n_grid < 4) return fail(GBMPM_ERR_ARG, "bad sizes");
    if (p->n > 0 && (!p->x || !p->v || !p->C || !p->F || !p->F_trial || !p->L || !p->stress || !p->mass ||
                     !p->vol || !p->Jp || !p->mu || !p->lam || !p->yield_stress || !p->material))
        return fail(GBMPM_ERR_ARG, "a required particle buffer is NULL");
    if (!g->mv || !g->v) return fail(GBMPM_ERR_ARG, "grid buffers are NULL");
    e->P = *p;
    e->G = *g;
    e->bd = (g->n_grid + 3) / 4;
    size_t nb = (size_t)e->bd * e->bd * e->bd;
    GB_CUDA(e->d_flag.ensure(nb));
    GB_CUDA(e->d_list.ensure(2 * nb));
    GB_CUDA(e->d_count.ensure(2));
    GB_CUDA(e->d_status.ensure(1));
    GB_CUDA(e->d_guard.ensure(8));
    GB_CUDA(cudaMemset(e->d_flag.ptr, 0, nb * sizeof(int)));
    GB_CUDA(cudaMemset(e->d_count.ptr, 0, 2 * sizeof(int)));
    GB_CUDA(cudaMemset(e->d_status.ptr, 0, sizeof(unsigned)));
    size_t nn = (size_t)g->n_grid * g->n_grid * g->n_grid;
    GB_CUDA(cudaMemset(g->mv, 0, nn * 16));
    GB_CUDA(cudaMemset(g->v, 0, nn * 16));
    e->bound = true;
    mark_dirty(e);
    e->ws_n = -1;
    return GBMPM_OK;
}

int gbmpm_set_model(gbmpm_engine *e, const gbmpm_model *m) {
    if (!e || !m) return fail(GBMPM_ERR_ARG, "null argument");
    if (m->eta_table_n < 2 || !m->eta_table) return fail(GBMPM_ERR_ARG, "eta_table needs >= 2 samples");
    if (e->bound && m->n_grid != e->G.n_grid) return fail(GBMPM_ERR_ARG, "model n_grid differs from bound grid");
    e->M = *m;
    MatTables t;
    std::memcpy(t.E, m->E, sizeof t.E); std::memcpy(t.nu, m->nu, sizeof t.nu);
    std::memcpy(t.bulk, m->bulk, sizeof t.bulk); std::memcpy(t.hardening, m->hardening, sizeof t.hardening);
    std::memcpy(t.xi, m->xi, sizeof t.xi); std::memcpy(t.pv, m->plastic_viscosity, sizeof t.pv);
    std::memcpy(t.softening, m->softening, sizeof t.softening); std::memcpy(t.alpha, m->alpha, sizeof t.alpha);
    std::memcpy(t.mu_s, m->muI_mu_s, sizeof t.mu_s); std::memcpy(t.dmu, m->muI_delta_mu, sizeof t.dmu);
    std::memcpy(t.I0, m->muI_I0, sizeof t.I0); std::memcpy(t.d, m->muI_d, sizeof t.d);
    std::memcpy(t.rho_s, m->muI_rho_s, sizeof t.rho_s); std::memcpy(t.phi_init, m->muI_phi_init, sizeof t.phi_init);
    std::memcpy(t.phi_chi, m->muI_phi_chi, sizeof t.phi_chi);
    GB_CUDA(e->d_tab.ensure(1));
    GB_CUDA(cudaMemcpy(e->d_tab.ptr, &t, sizeof t, cudaMemcpyHostToDevice));
    e->modeled = true;
    e->ws_n = -1;
    mark_dirty(e);
    return GBMPM_OK;
}

int gbmpm_set_colliders(gbmpm_engine *e, const gbmpm_collider *c, int32_t n) {
    if (!e || (n > 0 && !c)) return fail(GBMPM_ERR_ARG, "null argument");
    if (n < 0 || n > kMaxCol) return fail(GBMPM_ERR_ARG, "collider count out of range (max 32)");
    for (int i = 0; i < n; ++i) {
        if (c[i].kind < 0 || c[i].kind > GBMPM_COLLIDER_SDF) return fail(GBMPM_ERR_ARG, "unknown collider kind");
        if (c[i].kind == GBMPM_COLLIDER_SDF && (!c[i].sdf_val || !c[i].sdf_grad || c[i].sdf_res < 2))
            return fail(GBMPM_ERR_ARG, "sdf collider without a field");
    }
    size_t old = e->cols.size();
    e->cols.assign(c, c + n);
    std::vector<ColDev> d(std::max(1, n));
    for (int i = 0; i < n; ++i) d[i] = to_dev(c[i]);
    // The device table (fixed capacity, so its address never changes) is refreshed
    // on the stream of the next tick; a captured tick graph reads it at run time, so
    // only a change of the collider count needs a new capture.
    GB_CUDA(e->d_cols.ensure(kMaxCol));
    if (e->h_cols.size() != d.size() || std::memcmp(e->h_cols.data(), d.data(), d.size() * sizeof(ColDev)) != 0) {
        e->h_cols = d;
        e->cols_upload = true;
    }
    if (e->d_wrench.n < (size_t)kMaxCol * 6) {
        std::vector<double> keep(e->d_wrench.n);
        if (e->d_wrench.ptr && e->d_wrench.n)
            GB_CUDA(cudaMemcpy(keep.data(), e->d_wrench.ptr, keep.size() * sizeof(double), cudaMemcpyDeviceToHost));
        GB_CUDA(e->d_wrench.ensure((size_t)kMaxCol * 6));
        GB_CUDA(cudaMemset(e->d_wrench.ptr, 0, (size_t)kMaxCol * 6 * sizeof(double)));
        if (!keep.empty())
            GB_CUDA(cudaMemcpy(e->d_wrench.ptr, keep.data(), keep.size() * sizeof(double), cudaMemcpyHostToDevice));
    }
    if ((size_t)n > old)
        GB_CUDA(cudaMemset(e->d_wrench.ptr + old * 6, 0, (n - old) * 6 * sizeof(double)));
    if ((size_t)n != old) mark_dirty(e);
    return GBMPM_OK;
}

int gbmpm_get_colliders(gbmpm_engine *e, gbmpm_collider *c, int32_t n) {
    if (!e || (n > 0 && !c)) return fail(GBMPM_ERR_ARG, "null argument");
    if (n != (int)e->cols.size()) return fail(GBMPM_ERR_ARG, "collider count mismatch");
    std::copy(e->cols.begin(), e->cols.end(), c);
    return GBMPM_OK;
}

// add_cdf_collider / set_cdf_pose (mpm_solver_warp.py:2819-2981). The first
// lanes allocate the node grids for the current n_grid; later calls may only
// append lanes or change existing ones. A lane whose centre or quaternion changed
// is restamped at the next substep; any pose or rate change refreshes the lane
// arrays the transfer passes read.
int gbmpm_set_rigid(gbmpm_engine *e, const gbmpm_rigid_body *bodies, int32_t n_bodies,
                    const gbmpm_rigid_surface *surfaces, int32_t n_surfaces) {
    if (!e || n_bodies < 0 || n_surfaces < 0 || (n_bodies > 0 && !bodies) || (n_surfaces > 0 && !surfaces))
        return fail(GBMPM_ERR_ARG, "bad rigid-body arguments");
    if (n_surfaces > GBMPM_MAX_RIGID_SURFACES)
        return fail(GBMPM_ERR_ARG, "at most " + std::to_string(GBMPM_MAX_RIGID_SURFACES) + " rigid surfaces");
    if (!e->bound) return fail(GBMPM_ERR_STATE, "buffers not bound (call gbmpm_bind)");
    if (n_bodies > 0 && e->P.n > 0 && (!e->P.rigid_id || !e->P.x_ref))
        return fail(GBMPM_ERR_ARG, "rigid bodies need particles.rigid_id and particles.x_ref");
    for (int b = 0; b < n_bodies; ++b)
        if (!(bodies[b].mass > 0.0f)) return fail(GBMPM_ERR_ARG, "rigid body " + std::to_string(b) + " has no mass");
    GB_CUDA(cudaDeviceSynchronize());
    if (n_bodies > 0) {
        GB_CUDA(e->d_bodies.ensure(n_bodies));
        GB_CUDA(e->d_racc.ensure(6 * (size_t)n_bodies));
        GB_CUDA(e->d_rkey.ensure(2 * (size_t)n_bodies * GBMPM_MAX_RIGID_SURFACES));
        GB_CUDA(cudaMemcpy(e->d_bodies.ptr, bodies, n_bodies * sizeof(gbmpm_rigid_body), cudaMemcpyHostToDevice));
        GB_CUDA(e->d_rlist.ensure(std::max(1, e->P.n)));
        GB_CUDA(e->d_rcount.ensure(1));
        GB_CUDA(cudaMemset(e->d_rcount.ptr, 0, sizeof(int)));
        if (e->P.n > 0) {   // how many particles are rigid now: sizes the rigid passes' grids
            k_rigid_list<<<std::max(1, std::min((e->P.n + 255) / 256, e->num_sms * 8)), 256>>>(
                e->P.material, e->P.selection, e->P.n, e->d_rlist.ptr, e->d_rcount.ptr);
            GB_CUDA(cudaMemcpy(&e->n_rigid, e->d_rcount.ptr, sizeof(int), cudaMemcpyDeviceToHost));
        }
        GB_CUDA(cudaMemset(e->d_racc.ptr, 0, 6 * (size_t)n_bodies * sizeof(double)));
        GB_CUDA(cudaMemset(e->d_rkey.ptr, 0xff, 2 * (size_t)n_bodies * GBMPM_MAX_RIGID_SURFACES *
                                                   sizeof(unsigned long long)));
    }
    e->rsurf.assign(surfaces, surfaces + n_surfaces);
    if ((e->n_bodies == 0) != (n_bodies == 0)) e->ws_n = -1;   // the working set gains or drops the rigid fields
    e->n_bodies = n_bodies;
    mark_dirty(e);
    return GBMPM_OK;
}

int gbmpm_get_rigid(gbmpm_engine *e, gbmpm_rigid_body *bodies, int32_t n_bodies, void *stream) {
    if (!e || !bodies || n_bodies < 0 || n_bodies > e->n_bodies) return fail(GBMPM_ERR_ARG, "bad rigid-body read");
    if (n_bodies == 0) return GBMPM_OK;
    cudaStream_t s = (cudaStream_t)stream;
    GB_CUDA(cudaMemcpyAsync(bodies, e->d_bodies.ptr, n_bodies * sizeof(gbmpm_rigid_body), cudaMemcpyDeviceToHost, s));
    GB_CUDA(cudaStreamSynchronize(s));
    return GBMPM_OK;
}

int gbmpm_set_modifiers(gbmpm_engine *e, const gbmpm_modifier *mods, int32_t n) {
    if (!e || n < 0 || (n > 0 && !mods)) return fail(GBMPM_ERR_ARG, "bad modifier arguments");
    if (n > GBMPM_MAX_MODIFIERS) return fail(GBMPM_ERR_ARG, "at most 32 particle modifiers");
    if (!e->bound) return fail(GBMPM_ERR_STATE, "buffers not bound (call gbmpm_bind)");
    if (n > 0 && e->P.n > 0 && !e->P.mod_mask) return fail(GBMPM_ERR_ARG, "particle modifiers need particles.mod_mask");
    for (int m = 0; m < n; ++m)
        if (mods[m].kind < 0 || mods[m].kind > 2) return fail(GBMPM_ERR_ARG, "modifier kind must be 0, 1 or 2");
    GB_CUDA(cudaDeviceSynchronize());
    if (n > 0) {
        GB_CUDA(e->d_mods.ensure(n));
        GB_CUDA(cudaMemcpy(e->d_mods.ptr, mods, n * sizeof(gbmpm_modifier), cudaMemcpyHostToDevice));
    }
    if ((e->n_mods == 0) != (n == 0)) e->ws_n = -1;
    e->n_mods = n;
    mark_dirty(e);
    return GBMPM_OK;
}

int gbmpm_set_cdf(gbmpm_engine *e, const gbmpm_cdf *lanes, int32_t n) {
    if (!e || (n > 0 && !lanes)) return fail(GBMPM_ERR_ARG, "null argument");
    if (!e->modeled) return fail(GBMPM_ERR_STATE, "model not set (call gbmpm_set_model)");
    if (e->M.periodic_x) return fail(GBMPM_ERR_UNSUPPORTED, "CDF colliders do not wrap the periodic x axis");
    CdfHost &H = e->cdf;
    if (n < H.n || n > GBMPM_MAX_CDF)
        return fail(GBMPM_ERR_ARG, "CDF lanes can only be added, at most " + std::to_string(GBMPM_MAX_CDF));
    for (int l = 0; l < n; ++l) {
        const gbmpm_cdf &r = lanes[l];
        if (!r.values || !r.valid || r.res < 2 || !(r.cell > 0.0f) || !(r.band > 0.0f))
            return fail(GBMPM_ERR_ARG, "CDF lane " + std::to_string(l) + ": needs values, valid, res >= 2, cell > 0, band > 0");
        if (r.surface_type < 0 || r.surface_type > 2)
            return fail(GBMPM_ERR_ARG, "CDF surface_type must be 0 (sticky), 1 (slip) or 2 (separable)");
    }
    if (n > 0 && e->c_ng == 0) {
        const int ng = e->M.n_grid;
        const size_t N = (size_t)ng * ng * ng;
        const int nb = (ng + 3) / 4;
        GB_CUDA(e->c_tag.ensure(N)); GB_CUDA(e->c_tag_prev.ensure(N));
        GB_CUDA(e->c_d.ensure(N)); GB_CUDA(e->c_d_prev.ensure(N));
        GB_CUDA(e->c_block.ensure((size_t)nb * nb * nb));
        GB_CUDA(e->c_wrench.ensure(6 * GBMPM_MAX_CDF));
        GB_CUDA(cudaMemset(e->c_tag.ptr, 0, N * sizeof(int)));
        GB_CUDA(cudaMemset(e->c_tag_prev.ptr, 0, N * sizeof(int)));
        GB_CUDA(cudaMemset(e->c_block.ptr, 0, (size_t)nb * nb * nb * sizeof(int)));
        GB_CUDA(cudaMemset(e->c_wrench.ptr, 0, 6 * GBMPM_MAX_CDF * sizeof(double)));
        e->c_ng = ng;
        CdfBox all{{0, 0, 0}, {ng, ng, ng}};
        int blocks = cdf_grid_blocks(e, (long long)N);
        k_cdf_clear<<<blocks, 256>>>(e->c_tag.ptr, e->c_d.ptr, all, ng);
        k_cdf_clear<<<blocks, 256>>>(e->c_tag_prev.ptr, e->c_d_prev.ptr, all, ng);
        e->launches += 2;
        GB_CUDA(cudaGetLastError());
        GB_CUDA(cudaDeviceSynchronize());
    }
    for (int l = 0; l < n; ++l) {
        const gbmpm_cdf &r = lanes[l];
        if (l >= H.n) {
            H.rec[l] = r;
            H.dirty[l] = true;
            H.active[l] = false;   // settled by the first stamp, which restamps the lane anyway
            H.has_prev_box[l] = false;
            H.sync_lane(l);
            continue;
        }
        gbmpm_cdf &o = H.rec[l];
        bool moved = std::memcmp(o.center, r.center, sizeof o.center) != 0 ||
                     std::memcmp(o.quat, r.quat, sizeof o.quat) != 0;
        bool synced = std::memcmp(o.velocity, r.velocity, sizeof o.velocity) != 0 ||
                      std::memcmp(o.omega, r.omega, sizeof o.omega) != 0;
        o = r;
        if (moved) H.dirty[l] = true;
        if (moved || synced) { H.sync_lane(l); H.lane_prev_stale = true; }
    }
    if (H.n == 0 && n > 0) e->ws_n = -1;   // the working set gains the particle tag
    H.n = n;
    return GBMPM_OK;
}

int gbmpm_get_cdf(gbmpm_engine *e, gbmpm_cdf *lanes, int32_t n) {
    if (!e || (n > 0 && !lanes)) return fail(GBMPM_ERR_ARG, "null argument");
    if (n > e->cdf.n) return fail(GBMPM_ERR_ARG, "more lanes requested than set");
    for (int l = 0; l < n; ++l) lanes[l] = e->cdf.rec[l];
    return GBMPM_OK;
}

int gbmpm_cdf_wrench(gbmpm_engine *e, int32_t lane, double out[6], void *stream) {
    if (!e || !out) return fail(GBMPM_ERR_ARG, "null argument");
    if (lane < 0 || lane >= e->cdf.n) return fail(GBMPM_ERR_ARG, "CDF lane out of range");
    cudaStream_t s = (cudaStream_t)stream;
    fold_cdf_wrench(e, s);
    GB_CUDA(cudaMemcpyAsync(out, e->c_wrench.ptr + 6 * lane, 6 * sizeof(double), cudaMemcpyDeviceToHost, s));
    GB_CUDA(cudaStreamSynchronize(s));
    return GBMPM_OK;
}

int gbmpm_cdf_grids(gbmpm_engine *e, int32_t *tag_out, float *d_out, int64_t *stamps, void *stream) {
    if (!e) return fail(GBMPM_ERR_ARG, "null argument");
    if (stamps) *stamps = e->cdf.stamps;
    if (e->c_ng == 0) return (tag_out || d_out) ? fail(GBMPM_ERR_STATE, "no CDF collider set") : GBMPM_OK;
    cudaStream_t s = (cudaStream_t)stream;
    const size_t N = (size_t)e->c_ng * e->c_ng * e->c_ng;
    if (tag_out) GB_CUDA(cudaMemcpyAsync(tag_out, e->c_tag.ptr, N * sizeof(int32_t), cudaMemcpyDeviceToDevice, s));
    if (d_out) GB_CUDA(cudaMemcpyAsync(d_out, e->c_d.ptr, N * sizeof(float), cudaMemcpyDeviceToDevice, s));
    return GBMPM_OK;
}

int gbmpm_cdf_restamp(gbmpm_engine *e, double time, void *stream) {
    if (!e) return fail(GBMPM_ERR_ARG, "null argument");
    if (e->cdf.n == 0) return GBMPM_OK;
    for (int l = 0; l < e->cdf.n; ++l) e->cdf.dirty[l] = true;
    cdf_stamp(e, time, false, (cudaStream_t)stream);
    GB_CUDA(cudaGetLastError());
    return GBMPM_OK;
}

int gbmpm_cdf_force_stamp(gbmpm_engine *e, int32_t on) {
    if (!e) return fail(GBMPM_ERR_ARG, "null argument");
    e->cdf.force = on != 0;
    return GBMPM_OK;
}

int gbmpm_cdf_mask_off(gbmpm_engine *e, int32_t off) {
    if (!e) return fail(GBMPM_ERR_ARG, "null argument");
    e->cdf.mask_off = off != 0;   // ticks with CDF lanes launch live, so the next launch sees it
    return GBMPM_OK;
}

int32_t gbmpm_graph_state(gbmpm_engine *e) {
    if (!e) return 0;
    return e->graph_failed ? -1 : (e->graph ? 1 : 0);
}

int gbmpm_debug_fail_next_capture(gbmpm_engine *e) {
    if (!e) return fail(GBMPM_ERR_ARG, "null argument");
    e->fake_capture_failure = true;
    return GBMPM_OK;
}

int gbmpm_reset_cdf_wrench(gbmpm_engine *e, void *stream) {
    if (!e) return fail(GBMPM_ERR_ARG, "null argument");
    if (e->cdf.n == 0) return GBMPM_OK;
    GB_CUDA(cudaMemsetAsync(e->c_wrench.ptr, 0, 6 * GBMPM_MAX_CDF * sizeof(double), (cudaStream_t)stream));
    if (e->c_partial_ctas)
        GB_CUDA(cudaMemsetAsync(e->c_partial.ptr, 0, e->c_partial_ctas * 6 * GBMPM_MAX_CDF * sizeof(double),
                                (cudaStream_t)stream));
    return GBMPM_OK;
}

}  // extern "C"

namespace {
// Everything a tick needs before its launches: argument checks, the float64 pose
// table for every substep (uploaded on stream s) and the working-set buffers.
int prepare_tick(gbmpm_engine *e, double *time, double dt, int32_t substeps, int32_t flags, cudaStream_t s,
                 bool &reorder, bool batched = false) {
    int rc = check_ready(e);
    if (rc) return rc;
    if (!time || substeps < 1 || substeps > GBMPM_MAX_SUBSTEPS || !(dt > 0.0))
        return fail(GBMPM_ERR_ARG, "bad tick arguments");
    const int nc = (int)e->cols.size();
    const size_t need = (size_t)substeps * std::max(1, nc);
    Staging &st = e->stage[e->stage_i];
    e->stage_i = (e->stage_i + 1) % kStages;
    GB_CUDA(cudaEventSynchronize(st.done));   // this slot's last upload (kStages ticks ago) has run
    if (st.pose_cap < need) {
        if (st.pose) cudaFreeHost(st.pose);
        st.pose = nullptr;
        GB_CUDA(cudaMallocHost(&st.pose, need * sizeof(PoseRec)));
        st.pose_cap = need;
    }
    if (!st.cols) GB_CUDA(cudaMallocHost(&st.cols, kMaxCol * sizeof(ColDev)));
    PoseRec *old_dev = e->d_pose.ptr;
    GB_CUDA(e->d_pose.ensure(need));
    if (e->d_pose.ptr != old_dev) mark_dirty(e);
    if (e->cols_upload) {
        std::memcpy(st.cols, e->h_cols.data(), e->h_cols.size() * sizeof(ColDev));
        GB_CUDA(cudaMemcpyAsync(e->d_cols.ptr, st.cols, e->h_cols.size() * sizeof(ColDev), cudaMemcpyHostToDevice,
                                s));
        e->cols_upload = false;
    }
    // substep start times (modifier and rigid-surface windows), as the tick advances them
    if (st.time_cap < (size_t)substeps) {
        if (st.time) cudaFreeHost(st.time);
        st.time = nullptr;
        GB_CUDA(cudaMallocHost(&st.time, (size_t)substeps * sizeof(double)));
        st.time_cap = substeps;
    }
    double *old_time = e->d_time.ptr;
    GB_CUDA(e->d_time.ensure(substeps));
    if (e->d_time.ptr != old_time) mark_dirty(e);
    {
        double t = *time;
        for (int i = 0; i < substeps; ++i) { st.time[i] = t; t = t + dt; }
    }
    GB_CUDA(cudaMemcpyAsync(e->d_time.ptr, st.time, (size_t)substeps * sizeof(double), cudaMemcpyHostToDevice, s));
    build_pose_table(e, st.pose, *time, dt, substeps);
    GB_CUDA(cudaMemcpyAsync(e->d_pose.ptr, st.pose, need * sizeof(PoseRec), cudaMemcpyHostToDevice, s));
    GB_CUDA(cudaEventRecord(st.done, s));
    e->det = (flags & GBMPM_TICK_DETERMINISTIC) != 0;
    if (e->det) {
        // every material law but the rigid bodies' (7, 8); on the caller's particle order
        const uint32_t det_mats = (1u << 0) | (1u << 1) | (1u << 2) | (1u << 5) | (1u << 6) | (1u << 9) |
                                  (1u << 10) | (1u << 11) | (1u << 12) | (1u << 13);
        if (e->M.material_mask & ~det_mats)
            return fail(GBMPM_ERR_UNSUPPORTED, "deterministic ticks do not cover rigid-body materials");
        if (e->cdf.n > 0 || e->n_bodies > 0)
            return fail(GBMPM_ERR_UNSUPPORTED, "deterministic ticks support no CDF colliders or rigid bodies");
        const size_t nrec = (size_t)27 * std::max(1, e->P.n);
        if (nrec > (size_t)INT32_MAX) return fail(GBMPM_ERR_ARG, "too many particles for a deterministic tick");
        const unsigned long long *old_key = e->det_key[0].ptr;
        GB_CUDA(e->det_key[0].ensure(nrec)); GB_CUDA(e->det_key[1].ensure(nrec));
        GB_CUDA(e->det_idx[0].ensure(nrec)); GB_CUDA(e->det_idx[1].ensure(nrec));
        GB_CUDA(e->det_val.ensure(nrec));
        GB_CUDA(e->det_hist.ensure((nrec + kSortTile - 1) / kSortTile * kRadixBins));
        if (e->det_key[0].ptr != old_key) mark_dirty(e);
    }
    reorder = !e->det && (flags & GBMPM_TICK_REORDER) && !e->M.periodic_x && e->P.n > 0 && e->G.n_grid <= 1024;
    // the second working copy, for a tick long enough to re-sort inside (record_tick)
    const int every = resort_interval(e, substeps);
    const bool second = reorder && !batched && (flags & GBMPM_TICK_FUSED) && every > 0 && substeps > every;
    if (reorder && (e->ws_n != e->P.n || (second && e->ws2_n != e->P.n))) {
        GB_CUDA(ensure_ws(e, second || e->ws2_n == e->P.n));
        mark_dirty(e);
    }
    return GBMPM_OK;
}
}  // namespace

extern "C" {

int gbmpm_tick(gbmpm_engine *e, double *time, double dt, int32_t substeps, int32_t flags, void *stream) {
    cudaStream_t s = (cudaStream_t)stream;
    if (e && time && e->bound && e->P.n == 0 && e->cdf.n == 0 && substeps >= 1 && dt > 0.0) {
        for (int i = 0; i < substeps; ++i) *time += dt;
        return GBMPM_OK;
    }
    const bool cdf = e && e->cdf.n > 0;
    if (cdf) {
        int rc = check_ready(e);
        if (rc) return rc;
        const size_t ctas = (size_t)std::max(1, (e->P.n + kCdfCtaThreads - 1) / kCdfCtaThreads);
        if (e->c_partial_ctas < ctas) {
            GB_CUDA(cudaStreamSynchronize(s));
            if (e->c_partial_ctas) fold_cdf_wrench(e, s);
            GB_CUDA(e->c_partial.ensure(ctas * 6 * GBMPM_MAX_CDF));
            GB_CUDA(cudaMemsetAsync(e->c_partial.ptr, 0, ctas * 6 * GBMPM_MAX_CDF * sizeof(double), s));
            e->c_partial_ctas = ctas;
        }
        GB_CUDA(e->c_cache.ensure(5 * (size_t)std::max(1, e->P.n)));
        const int every = resort_interval(e, substeps);
        if (every > 0 && substeps > every && (flags & GBMPM_TICK_FUSED))
            GB_CUDA(e->c_cache2.ensure(5 * (size_t)std::max(1, e->P.n)));
        if (e->c_ng != e->M.n_grid) return fail(GBMPM_ERR_STATE, "CDF grids were sized for another n_grid");
        if (e->M.periodic_x) return fail(GBMPM_ERR_UNSUPPORTED, "CDF colliders do not wrap the periodic x axis");
        if (e->P.n > 0 && !e->P.cdf_tag) return fail(GBMPM_ERR_ARG, "CDF colliders need particles.cdf_tag");
        flags &= ~GBMPM_TICK_GRAPH;
    }
    const double t0 = time ? *time : 0.0;
    bool reorder = false;
    int rc = prepare_tick(e, time, dt, substeps, flags, s, reorder);
    if (rc) return rc;
    const bool fused = (flags & GBMPM_TICK_FUSED) != 0;
    const bool profile = (flags & GBMPM_TICK_PROFILE) != 0;
    const bool use_graph = (flags & GBMPM_TICK_GRAPH) && !profile;
    const float dtf = (float)dt;
    if (!use_graph || e->graph_failed) {
        record_tick(e, dtf, substeps, fused, reorder, s, profile, t0, dt);
        GB_CUDA(cudaGetLastError());
        return GBMPM_OK;
    }
    bool reuse = e->graph && !e->dirty && e->g_substeps == substeps && e->g_flags == flags && e->g_dt == dt &&
                 e->g_stream == s;
    if (!reuse) {
        if (e->graph) { cudaGraphExecDestroy(e->graph); e->graph = nullptr; }
        cudaStream_t cap;
        GB_CUDA(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));
        cudaGraph_t g = nullptr;
        cudaError_t be = cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal);
        if (be != cudaSuccess) {
            cudaStreamDestroy(cap);
            return fail(GBMPM_ERR_CUDA, std::string("cudaStreamBeginCapture: ") + cudaGetErrorString(be));
        }
        int64_t before = e->launches;
        record_tick(e, dtf, substeps, fused, reorder, cap, false);
        e->graph_launches = e->launches - before;
        e->launches = before;
        cudaError_t ce = cudaStreamEndCapture(cap, &g);
        cudaStreamDestroy(cap);
        if (ce == cudaSuccess) ce = cudaGraphInstantiate(&e->graph, g, 0);
        if (g) cudaGraphDestroy(g);
        if (ce == cudaSuccess && e->fake_capture_failure) {   // test hook: this capture counts as failed
            cudaGraphExecDestroy(e->graph);
            ce = cudaErrorStreamCaptureInvalidated;
        }
        e->fake_capture_failure = false;
        if (ce != cudaSuccess) {
            // as the reference does on a failed capture (mpm_solver_warp.py:1118-1125): no
            // graphs for the rest of the run, this tick and the next ones launched live
            e->graph = nullptr;
            e->graph_failed = true;
            (void)cudaGetLastError();
            record_tick(e, dtf, substeps, fused, reorder, s, profile, t0, dt);
            GB_CUDA(cudaGetLastError());
            return GBMPM_OK;
        }
        e->g_substeps = substeps; e->g_flags = flags; e->g_dt = dt; e->g_stream = s;
        e->dirty = false;
    }
    GB_CUDA(cudaGraphLaunch(e->graph, s));
    e->launches += e->graph_launches;
    return GBMPM_OK;
}

int gbmpm_guard(gbmpm_engine *e, float out[7], uint32_t *status, void *stream) {
    if (!e || !out) return fail(GBMPM_ERR_ARG, "null argument");
    if (!e->bound) return fail(GBMPM_ERR_STATE, "buffers not bound");
    cudaStream_t s = (cudaStream_t)stream;
    k_guard_init<<<1, 32, 0, s>>>(e->d_guard.ptr);
    if (e->P.n > 0) {
        int grid = std::min((e->P.n + 255) / 256, e->num_sms * 4);
        k_guard<<<grid, 256, 0, s>>>(e->P.x, e->P.v, e->P.n, e->d_guard.ptr, e->d_status.ptr);
    }
    e->launches += 2;
    float h[8];
    unsigned st = 0;
    GB_CUDA(cudaMemcpyAsync(h, e->d_guard.ptr, 7 * sizeof(float), cudaMemcpyDeviceToHost, s));
    GB_CUDA(cudaMemcpyAsync(&st, e->d_status.ptr, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
    GB_CUDA(cudaMemsetAsync(e->d_status.ptr, 0, sizeof(unsigned), s));
    GB_CUDA(cudaStreamSynchronize(s));
    for (int i = 0; i < 7; ++i) out[i] = h[i];
    if (status) *status = st;
    return GBMPM_OK;
}

int gbmpm_wrench(gbmpm_engine *e, int32_t collider, double out[6], void *stream) {
    if (!e || !out) return fail(GBMPM_ERR_ARG, "null argument");
    if (collider < 0 || collider >= (int)e->cols.size()) return fail(GBMPM_ERR_ARG, "collider index out of range");
    cudaStream_t s = (cudaStream_t)stream;
    GB_CUDA(cudaMemcpyAsync(out, e->d_wrench.ptr + 6 * collider, 6 * sizeof(double), cudaMemcpyDeviceToHost, s));
    GB_CUDA(cudaStreamSynchronize(s));
    return GBMPM_OK;
}

int gbmpm_reset_wrench(gbmpm_engine *e, int32_t collider, void *stream) {
    if (!e) return fail(GBMPM_ERR_ARG, "null argument");
    if (collider < 0 || collider >= (int)e->cols.size()) return fail(GBMPM_ERR_ARG, "collider index out of range");
    GB_CUDA(cudaMemsetAsync(e->d_wrench.ptr + 6 * collider, 0, 6 * sizeof(double), (cudaStream_t)stream));
    return GBMPM_OK;
}

int gbmpm_sort_particles(gbmpm_engine *e, double dx, int32_t *sorted_out, int32_t *perm_out, void *stream) {
    if (!e || !(dx > 0.0)) return fail(GBMPM_ERR_ARG, "bad argument");
    if (!e->bound) return fail(GBMPM_ERR_STATE, "buffers not bound");
    cudaStream_t s = (cudaStream_t)stream;
    const int n = e->P.n;
    if (sorted_out) *sorted_out = 0;
    if (n < 2) return GBMPM_OK;
    GB_CUDA(e->d_keys[0].ensure(n)); GB_CUDA(e->d_keys[1].ensure(n));
    GB_CUDA(e->d_skeys.ensure(n));
    GB_CUDA(e->d_idx[0].ensure(n)); GB_CUDA(e->d_idx[1].ensure(n));
    GB_CUDA(e->d_flagbuf.ensure(1));
    GB_CUDA(e->d_kminmax.ensure(2));
    const int ntiles = (n + kSortTile - 1) / kSortTile;
    GB_CUDA(e->d_hist.ensure((size_t)ntiles * kRadixBins));
    GB_CUDA(cudaMemsetAsync(e->d_flagbuf.ptr, 0, sizeof(int), s));
    k_sort_minmax_init<<<1, 1, 0, s>>>(e->d_kminmax.ptr);
    long long nb = (long long)(e->G.n_grid >> 2) + 2;
    k_sort_keys<<<(n + 255) / 256, 256, 0, s>>>(e->P.x, n, dx, nb, e->d_skeys.ptr, e->d_idx[0].ptr,
                                                  e->d_flagbuf.ptr, e->d_kminmax.ptr);
    e->launches += 2;
    int unsorted = 0;
    long long mm[2];
    GB_CUDA(cudaMemcpyAsync(&unsorted, e->d_flagbuf.ptr, sizeof(int), cudaMemcpyDeviceToHost, s));
    GB_CUDA(cudaMemcpyAsync(mm, e->d_kminmax.ptr, 2 * sizeof(long long), cudaMemcpyDeviceToHost, s));
    GB_CUDA(cudaStreamSynchronize(s));
    if (!unsorted) return GBMPM_OK;
    k_sort_rebase<<<(n + 255) / 256, 256, 0, s>>>(e->d_skeys.ptr, n, e->d_kminmax.ptr, e->d_keys[0].ptr);
    e->launches++;
    unsigned long long span = (unsigned long long)(mm[1] - mm[0]);
    int bits = 0;
    while (bits < 64 && (span >> bits) != 0ull) ++bits;
    int cur = 0;
    for (int shift = 0; shift < bits; shift += kRadixBits) {
        k_radix_hist<<<ntiles, kSortThreads, 0, s>>>(e->d_keys[cur].ptr, n, shift, e->d_hist.ptr, ntiles);
        k_radix_scan<<<1, 1024, 0, s>>>(e->d_hist.ptr, ntiles * kRadixBins);
        k_radix_scatter<<<ntiles, kSortThreads, 0, s>>>(e->d_keys[cur].ptr, e->d_idx[cur].ptr, e->d_keys[cur ^ 1].ptr,
                                                         e->d_idx[cur ^ 1].ptr, n, shift, e->d_hist.ptr, ntiles);
        e->launches += 3;
        cur ^= 1;
    }
    const int *perm = e->d_idx[cur].ptr;
    GB_CUDA(e->d_tmp.ensure((size_t)9 * n));
    float *tmp = e->d_tmp.ptr;
    const gbmpm_particles &P = e->P;
    int g = (n + 255) / 256;
    auto permute = [&](float *a, int w) -> cudaError_t {
        if (!a) return cudaSuccess;
        switch (w) {
        case 1: k_gather_rows<1><<<g, 256, 0, s>>>(a, perm, tmp, n); break;
        case 3: k_gather_rows<3><<<g, 256, 0, s>>>(a, perm, tmp, n); break;
        case 6: k_gather_rows<6><<<g, 256, 0, s>>>(a, perm, tmp, n); break;
        default: k_gather_rows<9><<<g, 256, 0, s>>>(a, perm, tmp, n); break;
        }
        e->launches++;
        return cudaMemcpyAsync(a, tmp, (size_t)w * n * sizeof(float), cudaMemcpyDeviceToDevice, s);
    };
    float *v3[] = {P.x, P.v};
    for (float *a : v3) GB_CUDA(permute(a, 3));
    float *m9[] = {P.F, P.F_trial, P.stress, P.C, P.L};
    for (float *a : m9) GB_CUDA(permute(a, 9));
    float *f1[] = {P.vol, P.mass, P.density, P.Jp, P.mu, P.lam, P.yield_stress};
    for (float *a : f1) GB_CUDA(permute(a, 1));
    float *c6[] = {P.init_cov, P.cov};
    for (float *a : c6) GB_CUDA(permute(a, 6));
    int *i1[] = {P.selection, P.material, P.cdf_tag, P.rigid_id, P.mod_mask};
    for (int *a : i1) GB_CUDA(permute(reinterpret_cast<float *>(a), 1));
    GB_CUDA(permute(P.x_ref, 3));
    if (perm_out) GB_CUDA(cudaMemcpyAsync(perm_out, perm, (size_t)n * sizeof(int), cudaMemcpyDeviceToDevice, s));
    if (sorted_out) *sorted_out = 1;
    return GBMPM_OK;
}

int gbmpm_rebuild_active_blocks(gbmpm_engine *e, int32_t counts[2], void *stream) {
    if (!e || !counts) return fail(GBMPM_ERR_ARG, "null argument");
    if (!e->bound || !e->modeled) return fail(GBMPM_ERR_STATE, "engine not ready");
    cudaStream_t s = (cudaStream_t)stream;
    size_t nb = (size_t)e->bd * e->bd * e->bd;
    bool fresh = e->d_bcur.n < nb;
    GB_CUDA(e->d_braw.ensure(nb)); GB_CUDA(e->d_bcur.ensure(nb)); GB_CUDA(e->d_bprev.ensure(nb));
    GB_CUDA(e->d_bcount.ensure(2));
    if (fresh) {
        GB_CUDA(cudaMemsetAsync(e->d_bcur.ptr, 0, nb * sizeof(int), s));
    }
    std::swap(e->d_bcur, e->d_bprev);
    GB_CUDA(cudaMemsetAsync(e->d_braw.ptr, 0, nb * sizeof(int), s));
    GB_CUDA(cudaMemsetAsync(e->d_bcount.ptr, 0, 2 * sizeof(int), s));
    if (e->P.n > 0)
        k_blocks_mark<<<(e->P.n + 255) / 256, 256, 0, s>>>(e->P.x, e->P.n, e->M.inv_dx, e->bd, e->d_braw.ptr);
    k_blocks_dilate<<<(int)((nb + 255) / 256), 256, 0, s>>>(e->d_braw.ptr, e->bd, e->d_bcur.ptr, e->d_bprev.ptr,
                                                            e->d_bcount.ptr);
    e->launches += 2;
    GB_CUDA(cudaMemcpyAsync(counts, e->d_bcount.ptr, 2 * sizeof(int), cudaMemcpyDeviceToHost, s));
    GB_CUDA(cudaStreamSynchronize(s));
    return GBMPM_OK;
}

int gbmpm_compute_R(gbmpm_engine *e, float *R_out, void *stream) {
    if (!e || !R_out) return fail(GBMPM_ERR_ARG, "null argument");
    if (!e->bound) return fail(GBMPM_ERR_STATE, "buffers not bound");
    if (e->P.n == 0) return GBMPM_OK;
    k_compute_R<<<(e->P.n + 127) / 128, 128, 0, (cudaStream_t)stream>>>(e->P.F_trial, e->P.n, R_out);
    e->launches++;
    GB_CUDA(cudaGetLastError());
    return GBMPM_OK;
}

int gbmpm_compute_cov(gbmpm_engine *e, float *cov_out, void *stream) {
    if (!e || !cov_out) return fail(GBMPM_ERR_ARG, "null argument");
    if (!e->bound || !e->P.init_cov) return fail(GBMPM_ERR_STATE, "no init_cov bound");
    if (e->P.n == 0) return GBMPM_OK;
    k_compute_cov<<<(e->P.n + 127) / 128, 128, 0, (cudaStream_t)stream>>>(e->P.F_trial, e->P.init_cov, e->P.n,
                                                                          cov_out);
    e->launches++;
    GB_CUDA(cudaGetLastError());
    return GBMPM_OK;
}

int gbmpm_profile(gbmpm_engine *e, double ms_out[GBMPM_NUM_PHASES], int64_t count_out[GBMPM_NUM_PHASES],
                  int32_t reset) {
    if (!e) return fail(GBMPM_ERR_ARG, "null engine");
    for (int i = 0; i < GBMPM_NUM_PHASES; ++i) {
        if (ms_out) ms_out[i] = e->prof_ms[i];
        if (count_out) count_out[i] = e->prof_n[i];
        if (reset) { e->prof_ms[i] = 0; e->prof_n[i] = 0; }
    }
    return GBMPM_OK;
}

int64_t gbmpm_launch_count(gbmpm_engine *e) { return e ? e->launches : 0; }

int gbmpm_set_tuning(gbmpm_engine *e, int32_t tile_occ, int32_t grid_ctas) {
    if (!e) return fail(GBMPM_ERR_ARG, "null argument");
    if (tile_occ < 2 || tile_occ > 4 || grid_ctas < 1 || grid_ctas > 8)
        return fail(GBMPM_ERR_ARG, "tile_occ is 2 to 4; grid_ctas 1 to 8");
    e->tile_occ = tile_occ;
    e->grid_ctas = grid_ctas;
    mark_dirty(e);
    return GBMPM_OK;
}

int gbmpm_set_resort(gbmpm_engine *e, int32_t substeps) {
    if (!e) return fail(GBMPM_ERR_ARG, "null argument");
    if (substeps < 0 && substeps != GBMPM_RESORT_AUTO)
        return fail(GBMPM_ERR_ARG, "the re-sort interval is a substep count, 0 (once per tick) or GBMPM_RESORT_AUTO");
    e->resort_every = substeps;
    mark_dirty(e);
    return GBMPM_OK;
}

int32_t gbmpm_get_resort(gbmpm_engine *e) { return e ? e->resort_every : -2; }

int gbmpm_get_tuning(gbmpm_engine *e, int32_t out[2]) {
    if (!e || !out) return fail(GBMPM_ERR_ARG, "null argument");
    out[0] = e->tile_occ;
    out[1] = e->grid_ctas;
    return GBMPM_OK;
}

int gbmpm_debug_deposit_sums(gbmpm_engine *e, double dt, double out[4], void *stream) {
    int rc = check_ready(e);
    if (rc) return rc;
    if (!out || !(dt > 0.0)) return fail(GBMPM_ERR_ARG, "bad argument");
    if (e->cdf.n > 0 || e->n_bodies > 0) return fail(GBMPM_ERR_UNSUPPORTED, "deposit sums cover plain scenes");
    cudaStream_t s = (cudaStream_t)stream;
    const size_t nodes = (size_t)e->G.n_grid * e->G.n_grid * e->G.n_grid;
    const size_t nb = (size_t)e->bd * e->bd * e->bd;
    GB_CUDA(e->d_tmp.ensure(8));
    double *d_out = reinterpret_cast<double *>(e->d_tmp.ptr);
    GB_CUDA(cudaMemsetAsync(d_out, 0, 4 * sizeof(double), s));
    if (e->P.n > 0) {
        // the P2G of the stored stress, velocity and affine velocity (no stress update,
        // so the particle state is left as it is), on the direct path
        PK k = make_pk(e, e->P, (float)dt, 0);
        const bool pdl = e->pdl;
        e->pdl = false;
        launch_particles(e, k, PASS_P2G, false, s);
        e->pdl = pdl;
    }
    k_grid_sums<<<e->num_sms * 4, 256, 0, s>>>(reinterpret_cast<const float4 *>(e->G.mv), (long long)nodes, d_out);
    // undo: the grid and the block bookkeeping return to their between-tick state
    GB_CUDA(cudaMemsetAsync(e->G.mv, 0, nodes * sizeof(float4), s));
    GB_CUDA(cudaMemsetAsync(e->d_flag.ptr, 0, nb * sizeof(int), s));
    GB_CUDA(cudaMemsetAsync(e->d_count.ptr, 0, 2 * sizeof(int), s));
    GB_CUDA(cudaMemcpyAsync(out, d_out, 4 * sizeof(double), cudaMemcpyDeviceToHost, s));
    GB_CUDA(cudaStreamSynchronize(s));
    return GBMPM_OK;
}

}  // extern "C"

// ============================================================ batched scenes
// A batch advances many independent engines (scenes with their own particles,
// grid, materials and colliders) in one CUDA graph whose branches are the
// scenes' tick chains. Small scenes that fill a fraction of the GPU each then run
// concurrently instead of one after another; there is no data exchange between
// branches.
struct gbmpm_batch {
    std::vector<gbmpm_engine *> engines;
    std::vector<uint64_t> versions;
    std::vector<cudaStream_t> streams;
    std::vector<cudaEvent_t> joins;
    cudaEvent_t fork = nullptr, fork2 = nullptr;
    cudaGraphExec_t graph = nullptr;
    int g_substeps = -1, g_flags = -1;
    double g_dt = 0.0;
    int64_t graph_launches = 0;
    int64_t launches = 0;
    bool graph_failed = false;          // a capture failed: live launches from then on
    bool fake_capture_failure = false;  // test hook: treat the next capture as failed
    // The single-launch schedule (fused ticks whose scenes all run the tiled path):
    // every particle pass and every grid pass is one launch over all scenes, each
    // CTA finding its scene and tile in the tables below.
    bool single_launch = true;          // use it when every scene qualifies
    int tile_threads = 128;             // particles per CTA of the batched particle pass
    int tile_occ = 3;                   // its resident 256-thread equivalents per SM
    int grid_ctas = 2;                  // grid-update CTAs per SM, shared out by particle count
    int tuning_version = 0;             // bumped by gbmpm_batch_set_tuning
    bool g_single = false;              // the cached graph runs the single-launch schedule
    int g_tuning = -1;
    DevBuf<PK> d_pk;                    // per-scene particle-pass records
    DevBuf<GK> d_gk;                    // per-scene grid-pass records
    DevBuf<BatchCta> d_pcta;            // particle-pass CTA -> (scene, tile)
    DevBuf<int4> d_gcta;                // grid-pass CTA -> (scene, CTA of the scene, CTAs of the scene)
    int n_pcta = 0, n_gcta = 0;
    bool any_solids = false;
    std::vector<uint64_t> t_versions;   // engine versions the tables were built for
    float t_dt = -1.0f;
    int t_tuning = -1;
    std::vector<const int *> perms;     // each scene's working-set permutation, for the scatter back
};

namespace {

// Every scene of the batch runs the fused schedule on its block-sorted working set,
// with no feature that adds launches between the passes (CPIC lanes, rigid bodies,
// particle modifiers).
bool batch_single_launch_ok(const gbmpm_batch *b, bool fused, const std::vector<char> &reorder) {
    if (!b->single_launch || !fused) return false;
    for (size_t i = 0; i < b->engines.size(); ++i) {
        const gbmpm_engine *e = b->engines[i];
        if (!reorder[i] || e->P.n == 0 || e->cdf.n > 0 || e->n_bodies > 0 || e->n_mods > 0) return false;
    }
    return true;
}

// Builds and uploads the per-scene records and CTA maps when an engine, the
// substep or the tuning changed since the last build. The stream is synchronized
// first: a replay of the previous graph may still be reading the old tables.
int batch_tables(gbmpm_batch *b, float dtf, cudaStream_t s) {
    const int n = (int)b->engines.size();
    bool same = b->t_dt == dtf && b->t_tuning == b->tuning_version && (int)b->t_versions.size() == n;
    for (int i = 0; i < n && same; ++i) same = b->t_versions[i] == b->engines[i]->version;
    if (same) return GBMPM_OK;
    GB_CUDA(cudaStreamSynchronize(s));
    std::vector<PK> pk(n);
    std::vector<GK> gk(n);
    std::vector<BatchCta> pc;
    std::vector<int4> gc;
    long long total = 0;
    for (gbmpm_engine *e : b->engines) total += e->P.n;
    const int th = b->tile_threads;
    const int gtotal = std::max(n, b->engines[0]->num_sms * b->grid_ctas);
    b->any_solids = false;
    for (int i = 0; i < n; ++i) {
        gbmpm_engine *e = b->engines[i];
        pk[i] = make_pk(e, e->W, dtf, 0);
        gk[i] = make_gk(e, dtf, 0, 0);
        b->any_solids = b->any_solids || has_solids(e->M);
        const int tiles = (e->P.n + th - 1) / th;
        for (int t = 0; t < tiles; ++t) pc.push_back(BatchCta{i, t});
        const int g = std::max(1, (int)std::llround((double)gtotal * (double)e->P.n / (double)std::max(1LL, total)));
        for (int c = 0; c < g; ++c) gc.push_back(make_int4(i, c, g, 0));
    }
    GB_CUDA(b->d_pk.ensure(n));
    GB_CUDA(b->d_gk.ensure(n));
    GB_CUDA(b->d_pcta.ensure(pc.size()));
    GB_CUDA(b->d_gcta.ensure(gc.size()));
    GB_CUDA(cudaMemcpy(b->d_pk.ptr, pk.data(), n * sizeof(PK), cudaMemcpyHostToDevice));
    GB_CUDA(cudaMemcpy(b->d_gk.ptr, gk.data(), n * sizeof(GK), cudaMemcpyHostToDevice));
    GB_CUDA(cudaMemcpy(b->d_pcta.ptr, pc.data(), pc.size() * sizeof(BatchCta), cudaMemcpyHostToDevice));
    GB_CUDA(cudaMemcpy(b->d_gcta.ptr, gc.data(), gc.size() * sizeof(int4), cudaMemcpyHostToDevice));
    b->n_pcta = (int)pc.size();
    b->n_gcta = (int)gc.size();
    b->t_versions.resize(n);
    for (int i = 0; i < n; ++i) b->t_versions[i] = b->engines[i]->version;
    b->t_dt = dtf;
    b->t_tuning = b->tuning_version;
    return GBMPM_OK;
}

// Records one fused tick of every scene: each scene's working-set sort and gather on
// its own branch, then per substep one particle pass and one grid pass over all
// scenes on s, then each scene's scatter back on its branch. Returns the first
// error of an event call (the launches report through cudaGetLastError).
cudaError_t batch_record_single_launch(gbmpm_batch *b, float dtf, int S, cudaStream_t s) {
    (void)dtf;
    const int n = (int)b->engines.size();
    cudaError_t first = cudaEventRecord(b->fork, s);
    auto keep = [&](cudaError_t err) { if (first == cudaSuccess) first = err; };
    b->perms.assign(n, nullptr);
    int64_t launches = 0;
    for (int i = 0; i < n; ++i) {
        gbmpm_engine *e = b->engines[i];
        keep(cudaStreamWaitEvent(b->streams[i], b->fork, 0));
        const int64_t before = e->launches;
        b->perms[i] = record_ws_begin(e, b->streams[i]);
        launches += e->launches - before;
        e->launches = before;
        keep(cudaEventRecord(b->joins[i], b->streams[i]));
        keep(cudaStreamWaitEvent(s, b->joins[i], 0));
    }
    const bool pdl = b->engines[0]->pdl;
    const BatchLaunch L{b->tile_threads, b->tile_occ, b->any_solids, pdl};
    for (int sub = 0; sub < S; ++sub) {
        const int list = sub & 1;
        int mode = (sub == 0) ? (PASS_STRESS | PASS_P2G) : (PASS_G2P | PASS_STRESS | PASS_P2G);
        if (sub == S - 1) mode |= PASS_STORE_ALL;
        launch_particle_batch(L, b->d_pk.ptr, b->d_pcta.ptr, b->n_pcta, mode, list, sub, s);
        launch_kernel(pdl, k_grid_batch, b->n_gcta, kGridThreads, s, (const GK *)b->d_gk.ptr,
                      (const int4 *)b->d_gcta.ptr, sub, list);
        launches += 2;
    }
    launch_particle_batch(L, b->d_pk.ptr, b->d_pcta.ptr, b->n_pcta, PASS_G2P | PASS_RESET_LISTS, 0, 0, s);
    launches += 1;
    keep(cudaEventRecord(b->fork2, s));
    for (int i = 0; i < n; ++i) {
        gbmpm_engine *e = b->engines[i];
        keep(cudaStreamWaitEvent(b->streams[i], b->fork2, 0));
        k_ws_scatter<<<(e->P.n + 255) / 256, 256, 0, b->streams[i]>>>(e->ws_table, b->perms[i], e->P.n);
        launches += 1;
        keep(cudaEventRecord(b->joins[i], b->streams[i]));
        keep(cudaStreamWaitEvent(s, b->joins[i], 0));
    }
    b->launches += launches;
    return first;
}

}  // namespace

extern "C" {

int gbmpm_batch_create(gbmpm_engine *const *engines, int32_t n, gbmpm_batch **out) {
    if (!engines || !out || n < 1) return fail(GBMPM_ERR_ARG, "bad batch arguments");
    gbmpm_batch *b = new gbmpm_batch();
    int dev0 = engines[0] ? engines[0]->device : -1;
    for (int i = 0; i < n; ++i) {
        if (!engines[i] || engines[i]->device != dev0) { delete b; return fail(GBMPM_ERR_ARG, "batch engines must be non-null and on one device"); }
        b->engines.push_back(engines[i]);
    }
    b->versions.assign(n, 0);
    b->streams.assign(n, nullptr);
    b->joins.assign(n, nullptr);
    cudaError_t err = cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming);
    if (err == cudaSuccess) err = cudaEventCreateWithFlags(&b->fork2, cudaEventDisableTiming);
    for (int i = 0; i < n && err == cudaSuccess; ++i) {
        err = cudaStreamCreateWithFlags(&b->streams[i], cudaStreamNonBlocking);
        if (err == cudaSuccess) err = cudaEventCreateWithFlags(&b->joins[i], cudaEventDisableTiming);
    }
    if (err != cudaSuccess) { gbmpm_batch_destroy(b); return fail(GBMPM_ERR_CUDA, cudaGetErrorString(err)); }
    *out = b;
    return GBMPM_OK;
}

void gbmpm_batch_destroy(gbmpm_batch *b) {
    if (!b) return;
    if (b->graph) cudaGraphExecDestroy(b->graph);
    for (cudaStream_t st : b->streams) if (st) cudaStreamDestroy(st);
    for (cudaEvent_t ev : b->joins) if (ev) cudaEventDestroy(ev);
    if (b->fork) cudaEventDestroy(b->fork);
    if (b->fork2) cudaEventDestroy(b->fork2);
    b->d_pk.release(); b->d_gk.release(); b->d_pcta.release(); b->d_gcta.release();
    delete b;
}

int gbmpm_batch_tick(gbmpm_batch *b, double *times, double dt, int32_t substeps, int32_t flags, void *stream) {
    if (!b || !times) return fail(GBMPM_ERR_ARG, "bad batch tick arguments");
    if (flags & GBMPM_TICK_PROFILE) return fail(GBMPM_ERR_UNSUPPORTED, "profiling is per engine (gbmpm_tick)");
    if (flags & GBMPM_TICK_DETERMINISTIC)
        return fail(GBMPM_ERR_UNSUPPORTED, "deterministic ticks are per engine (gbmpm_tick)");
    cudaStream_t s = (cudaStream_t)stream;
    const int n = (int)b->engines.size();
    for (int i = 0; i < n; ++i)
        if (b->engines[i]->cdf.n > 0)
            return fail(GBMPM_ERR_UNSUPPORTED, "scenes with CDF colliders tick alone (gbmpm_tick)");
    std::vector<char> reorder(n, 0);
    for (int i = 0; i < n; ++i) {
        bool r = false;
        int rc = prepare_tick(b->engines[i], &times[i], dt, substeps, flags, s, r, true);
        if (rc) return rc;
        reorder[i] = r;
    }
    const bool fused = (flags & GBMPM_TICK_FUSED) != 0;
    const float dtf = (float)dt;
    const bool single = batch_single_launch_ok(b, fused, reorder);
    if (single) {
        int rt = batch_tables(b, dtf, s);
        if (rt) return rt;
    }
    auto live = [&]() -> int {
        if (single) {
            GB_CUDA(batch_record_single_launch(b, dtf, substeps, s));
        } else {
            for (int i = 0; i < n; ++i)
                if (b->engines[i]->P.n > 0) record_tick(b->engines[i], dtf, substeps, fused, reorder[i], s, false);
        }
        return GBMPM_OK;
    };
    if (!(flags & GBMPM_TICK_GRAPH) || b->graph_failed) {
        int rl = live();
        if (rl) return rl;
        GB_CUDA(cudaGetLastError());
        return GBMPM_OK;
    }
    bool reuse = b->graph && b->g_substeps == substeps && b->g_flags == flags && b->g_dt == dt &&
                 b->g_single == single && b->g_tuning == b->tuning_version;
    for (int i = 0; i < n && reuse; ++i) reuse = b->versions[i] == b->engines[i]->version;
    if (!reuse) {
        if (b->graph) { cudaGraphExecDestroy(b->graph); b->graph = nullptr; }
        cudaStream_t cap;
        GB_CUDA(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));
        cudaGraph_t g = nullptr;
        cudaError_t be = cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal);
        if (be != cudaSuccess) {
            cudaStreamDestroy(cap);
            return fail(GBMPM_ERR_CUDA, std::string("cudaStreamBeginCapture: ") + cudaGetErrorString(be));
        }
        // inside the capture the first error is kept rather than returned at once, so
        // the capture is always ended and its stream released; a failed capture then
        // takes the live fallback below
        cudaError_t first = cudaSuccess;
        auto keep = [&](cudaError_t err) { if (first == cudaSuccess) first = err; };
        int64_t total = 0;
        if (single) {
            const int64_t before = b->launches;
            keep(batch_record_single_launch(b, dtf, substeps, cap));
            total = b->launches - before;
            b->launches = before;
        } else {
            keep(cudaEventRecord(b->fork, cap));
        }
        for (int i = 0; i < n && first == cudaSuccess && !single; ++i) {
            gbmpm_engine *e = b->engines[i];
            keep(cudaStreamWaitEvent(b->streams[i], b->fork, 0));
            if (e->P.n > 0 && first == cudaSuccess) {
                int64_t before = e->launches;
                record_tick(e, dtf, substeps, fused, reorder[i], b->streams[i], false);
                total += e->launches - before;
                e->launches = before;
            }
            keep(cudaEventRecord(b->joins[i], b->streams[i]));
            keep(cudaStreamWaitEvent(cap, b->joins[i], 0));
        }
        cudaError_t ce = cudaStreamEndCapture(cap, &g);
        cudaStreamDestroy(cap);
        if (ce == cudaSuccess && first != cudaSuccess) ce = first;
        if (ce == cudaSuccess) ce = cudaGraphInstantiate(&b->graph, g, 0);
        if (g) cudaGraphDestroy(g);
        if (ce == cudaSuccess && b->fake_capture_failure) {   // test hook: this capture counts as failed
            cudaGraphExecDestroy(b->graph);
            ce = cudaErrorStreamCaptureInvalidated;
        }
        b->fake_capture_failure = false;
        if (ce != cudaSuccess) {
            // as a single scene does: this tick and the following ones run live, scene
            // after scene on the caller's stream
            b->graph = nullptr;
            b->graph_failed = true;
            (void)cudaGetLastError();
            int rl = live();
            if (rl) return rl;
            GB_CUDA(cudaGetLastError());
            return GBMPM_OK;
        }
        for (int i = 0; i < n; ++i) b->versions[i] = b->engines[i]->version;
        b->g_substeps = substeps; b->g_flags = flags; b->g_dt = dt;
        b->g_single = single; b->g_tuning = b->tuning_version;
        b->graph_launches = total;
    }
    GB_CUDA(cudaGraphLaunch(b->graph, s));
    b->launches += b->graph_launches;
    return GBMPM_OK;
}

int32_t gbmpm_batch_graph_state(gbmpm_batch *b) {
    if (!b) return 0;
    return b->graph_failed ? -1 : (b->graph ? 1 : 0);
}

int gbmpm_batch_debug_fail_next_capture(gbmpm_batch *b) {
    if (!b) return fail(GBMPM_ERR_ARG, "null argument");
    b->fake_capture_failure = true;
    return GBMPM_OK;
}

int gbmpm_batch_guard(gbmpm_batch *b, float *out, uint32_t *status, void *stream) {
    if (!b || !out || !status) return fail(GBMPM_ERR_ARG, "null argument");
    cudaStream_t s = (cudaStream_t)stream;
    const int n = (int)b->engines.size();
    std::vector<float> h(8 * (size_t)n);
    std::vector<unsigned> st(n);
    for (int i = 0; i < n; ++i) {
        gbmpm_engine *e = b->engines[i];
        if (!e->bound) return fail(GBMPM_ERR_STATE, "batch engine not bound");
        k_guard_init<<<1, 32, 0, s>>>(e->d_guard.ptr);
        if (e->P.n > 0) {
            int grid = std::min((e->P.n + 255) / 256, e->num_sms * 4);
            k_guard<<<grid, 256, 0, s>>>(e->P.x, e->P.v, e->P.n, e->d_guard.ptr, e->d_status.ptr);
        }
        GB_CUDA(cudaMemcpyAsync(&h[8 * (size_t)i], e->d_guard.ptr, 7 * sizeof(float), cudaMemcpyDeviceToHost, s));
        GB_CUDA(cudaMemcpyAsync(&st[i], e->d_status.ptr, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
        GB_CUDA(cudaMemsetAsync(e->d_status.ptr, 0, sizeof(unsigned), s));
        b->launches += 2;
    }
    GB_CUDA(cudaStreamSynchronize(s));
    for (int i = 0; i < n; ++i) {
        for (int a = 0; a < 7; ++a) out[7 * i + a] = h[8 * (size_t)i + a];
        status[i] = st[i];
    }
    return GBMPM_OK;
}

int64_t gbmpm_batch_launch_count(gbmpm_batch *b) { return b ? b->launches : 0; }

int gbmpm_batch_set_tuning(gbmpm_batch *b, int32_t single_launch, int32_t tile_threads, int32_t tile_occ,
                           int32_t grid_ctas) {
    if (!b) return fail(GBMPM_ERR_ARG, "null argument");
    if (!(tile_threads == 64 || tile_threads == 128 || tile_threads == 256) || tile_occ < 2 || tile_occ > 3 ||
        grid_ctas < 1 || grid_ctas > 8)
        return fail(GBMPM_ERR_ARG, "tile_threads is 64, 128 or 256; tile_occ 2 or 3; grid_ctas 1 to 8");
    b->single_launch = single_launch != 0;
    b->tile_threads = tile_threads;
    b->tile_occ = tile_occ;
    b->grid_ctas = grid_ctas;
    b->tuning_version++;
    return GBMPM_OK;
}

int gbmpm_batch_get_tuning(gbmpm_batch *b, int32_t out[5]) {
    if (!b || !out) return fail(GBMPM_ERR_ARG, "null argument");
    out[0] = b->single_launch ? 1 : 0;
    out[1] = b->tile_threads;
    out[2] = b->tile_occ;
    out[3] = b->grid_ctas;
    out[4] = b->g_single ? 1 : 0;
    return GBMPM_OK;
}

}  // extern "C"

// ======================= gbmpm_guard_noalloc: the edge-guard reduction for callers that cannot allocate
//
// gbmpm_guard (above) reduces min/max of the particle positions and max |v|
// into scratch that the engine allocated with cudaMalloc. Some callers cannot
// allow that: a process whose device memory is entirely owned by another
// allocator (a framework that reserves the device up front), or a control loop
// that must never hit cudaMalloc's implicit device synchronization between
// ticks. gbmpm_guard_noalloc computes the same seven numbers with no engine and
// no allocation: its scratch is the file-scope array below, reserved when the
// library is loaded and held by every GPU that loads it until the process exits.
//
// Limits and sharing:
//  * at most kMaxParticles particles per call (larger n is rejected with
//    GBMPM_ERR_ARG);
//  * every call uses the same array; calls that overlap on the GPU (two streams,
//    two threads) race on it and must be serialized by the caller;
//  * nothing in the array needs to start at zero: each call writes every slot
//    it later reads.
//  * every call looks up the array's device address in the current context
//    (cudaGetSymbolAddress, which allocates nothing). The address is not cached:
//    after cudaDeviceReset, or on another context of the same device, the module
//    can load at another address, and a cached pointer would be stale.

namespace noalloc {

constexpr int kThreads = 256;
constexpr int kPerThread = 16;
constexpr int kMaxBlocks = 1024;
constexpr int kSlot = 8;  // min xyz, max xyz, max |v|, non-finite flag
constexpr long long kMaxParticles = (long long)kMaxBlocks * kThreads * kPerThread;   // 4,194,304

// per-block partial results, then the final record at slot kMaxBlocks (33 KB)
static __device__ __align__(256) float g_guard_scratch[(kMaxBlocks + 1) * kSlot];

__device__ __forceinline__ float wmin(float x) {
    for (int o = 16; o > 0; o >>= 1) x = fminf(x, __shfl_xor_sync(0xffffffffu, x, o));
    return x;
}
__device__ __forceinline__ float wmax(float x) {
    for (int o = 16; o > 0; o >>= 1) x = fmaxf(x, __shfl_xor_sync(0xffffffffu, x, o));
    return x;
}

// one block reduces its contiguous slice of at most kThreads * kPerThread particles
__global__ void __launch_bounds__(kThreads) k_guard_partials(const float *x, const float *v, int n, float *scratch) {
    __shared__ float s[kThreads / 32][kSlot];
    float r[kSlot] = {INFINITY, INFINITY, INFINITY, -INFINITY, -INFINITY, -INFINITY, 0.0f, 0.0f};
    const long long begin = (long long)blockIdx.x * kThreads * kPerThread;
    for (int i = 0; i < kPerThread; ++i) {
        long long p = begin + (long long)i * kThreads + threadIdx.x;
        if (p >= n) break;
        for (int a = 0; a < 3; ++a) {
            float xa = x[3 * p + a];
            if (!isfinite(xa)) r[7] = 1.0f;
            r[a] = fminf(r[a], xa);
            r[3 + a] = fmaxf(r[3 + a], xa);
            r[6] = fmaxf(r[6], fabsf(v[3 * p + a]));
        }
    }
    for (int a = 0; a < 3; ++a) { r[a] = wmin(r[a]); r[3 + a] = wmax(r[3 + a]); }
    r[6] = wmax(r[6]);
    r[7] = wmax(r[7]);
    const int w = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0)
        for (int a = 0; a < kSlot; ++a) s[w][a] = r[a];
    __syncthreads();
    if (threadIdx.x < kSlot) {
        const int a = threadIdx.x;
        float acc = s[0][a];
        for (int ww = 1; ww < kThreads / 32; ++ww)
            acc = (a < 3) ? fminf(acc, s[ww][a]) : fmaxf(acc, s[ww][a]);
        scratch[blockIdx.x * kSlot + a] = acc;
    }
}

// one block folds the per-block partials into the final record
__global__ void __launch_bounds__(32) k_guard_final(float *scratch, int nblocks) {
    const int a = threadIdx.x;
    if (a >= kSlot) return;
    float acc = (a < 3) ? INFINITY : ((a < 6) ? -INFINITY : 0.0f);
    for (int b = 0; b < nblocks; ++b) {
        float val = scratch[b * kSlot + a];
        acc = (a < 3) ? fminf(acc, val) : fmaxf(acc, val);
    }
    scratch[kMaxBlocks * kSlot + a] = acc;
}

// device address of the scratch array in the current context, looked up on every
// call (the lookup allocates nothing)
int scratch_for_current_device(float **out) {
    float *ptr = nullptr;
    cudaError_t e = cudaGetSymbolAddress((void **)&ptr, g_guard_scratch);
    if (e != cudaSuccess || !ptr) return fail(GBMPM_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
    *out = ptr;
    return GBMPM_OK;
}

}  // namespace noalloc

extern "C" {

// out = {min x, min y, min z, max x, max y, max z, max |v_i|} over n particles
// (device pointers x, v of [n][3] floats), *nonfinite = 1 when any position is
// not finite. Host out; synchronizes the stream. No allocation of any kind.
int gbmpm_guard_noalloc(const float *x, const float *v, int32_t n, float out[7], int32_t *nonfinite,
                        void *stream) {
    using namespace noalloc;
    if ((long long)n > kMaxParticles)
        return fail(GBMPM_ERR_ARG, "gbmpm_guard_noalloc handles at most 4194304 particles per call");
    if (!out || n < 0 || (n > 0 && (!x || !v))) return fail(GBMPM_ERR_ARG, "bad argument");
    float *scratch = nullptr;
    int rc = noalloc::scratch_for_current_device(&scratch);
    if (rc != GBMPM_OK) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    const int nblocks = n > 0 ? (int)((n + (long long)kThreads * kPerThread - 1) / ((long long)kThreads * kPerThread)) : 0;
    if (nblocks > 0) k_guard_partials<<<nblocks, kThreads, 0, s>>>(x, v, n, scratch);
    k_guard_final<<<1, 32, 0, s>>>(scratch, nblocks);
    // a launch that failed leaves the previous call's record in the array: report
    // the failure instead of copying that record back
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(GBMPM_ERR_CUDA, std::string("gbmpm_guard_noalloc launch: ") + cudaGetErrorString(e));
    float h[kSlot];
    e = cudaMemcpyAsync(h, scratch + kMaxBlocks * kSlot, kSlot * sizeof(float), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return fail(GBMPM_ERR_CUDA, std::string("gbmpm_guard_noalloc: ") + cudaGetErrorString(e));
    for (int i = 0; i < 7; ++i) out[i] = h[i];
    if (nonfinite) *nonfinite = h[7] != 0.0f ? 1 : 0;
    return GBMPM_OK;
}

}  // extern "C"

// ================================================ stress-integral contact wrench
// box_contact_wrench (coupling/wrench.py:15-46) on the device: the reaction on a
// kinematic box from the Cauchy traction of the particles in a layer of thickness T
// under its bottom face, F = -sum sigma.e_z vol / T, torque about the box centre.
// Current volume and Cauchy stress follow the inversion policy of
// Solver.vol() / Solver.cauchy() (core/solver.py:559-598).
namespace gbmpm {

struct CWArgs {
    const float *x, *F, *S, *vol0;
    const int *sel;
    int n;
    double c[3], h[3];
    double layer;        // > 0: given thickness; otherwise 3 mean(vol)^(1/3)
    int compressive, policy;   // policy 0 warn (|J|), 1 nan, 2 raise
    double *acc;         // [0..5] force, torque; [6] contacts; [7] sum vol; [8] invalid count
};

__device__ __forceinline__ void cw_jacobian(const CWArgs &a, int p, double &Jv, double &Jc, bool &bad) {
    float F[9];
#pragma unroll
    for (int i = 0; i < 9; ++i) F[i] = a.F[9 * (size_t)p + i];
    const float J = det3(F);
    bad = !isfinite(J) || J <= 0.0f;
    if (a.policy == 1) Jv = bad ? (double)NAN : (double)J;
    else Jv = isfinite(J) ? (double)fabsf(J) : (double)NAN;
    Jc = (a.policy == 0) ? (Jv < 1e-9 ? 1e-9 : Jv) : Jv;   // NaN stays NaN
}

__device__ __forceinline__ double warp_sum_d(double v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

__global__ void k_cw_volume(CWArgs a) {
    double sv = 0.0, nb = 0.0;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < a.n; p += gridDim.x * blockDim.x) {
        double Jv, Jc;
        bool bad;
        cw_jacobian(a, p, Jv, Jc, bad);
        sv += (double)a.vol0[p] * Jv;
        nb += bad ? 1.0 : 0.0;
    }
    sv = warp_sum_d(sv);
    nb = warp_sum_d(nb);
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(a.acc + 7, sv);
        atomicAdd(a.acc + 8, nb);
    }
}

__global__ void k_cw_layer(CWArgs a) {
    const double T = a.layer > 0.0 ? a.layer : 3.0 * cbrt(a.acc[7] / (double)a.n);
    const double bottom = a.c[2] - a.h[2];
    double f[7] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < a.n; p += gridDim.x * blockDim.x) {
        const double x0 = a.x[3 * (size_t)p], x1 = a.x[3 * (size_t)p + 1], x2 = a.x[3 * (size_t)p + 2];
        if (!(fabs(x0 - a.c[0]) < a.h[0] && fabs(x1 - a.c[1]) < a.h[1] && x2 > bottom - T && x2 < bottom + 0.5 * T))
            continue;
        double Jv, Jc;
        bool bad;
        cw_jacobian(a, p, Jv, Jc, bad);
        const float *S = a.S + 9 * (size_t)p;
        const double s02 = (double)S[2] / Jc, s12 = (double)S[5] / Jc, s22 = (double)S[8] / Jc;
        if (a.compressive && !(s22 < 0.0)) continue;
        const double w = (double)a.vol0[p] * Jv / T;
        const double fp[3] = {-s02 * w, -s12 * w, -s22 * w};
        const double r[3] = {x0 - a.c[0], x1 - a.c[1], x2 - a.c[2]};
        f[0] += fp[0]; f[1] += fp[1]; f[2] += fp[2];
        f[3] += r[1] * fp[2] - r[2] * fp[1];
        f[4] += r[2] * fp[0] - r[0] * fp[2];
        f[5] += r[0] * fp[1] - r[1] * fp[0];
        f[6] += 1.0;
    }
#pragma unroll
    for (int i = 0; i < 7; ++i) {
        const double v = warp_sum_d(f[i]);
        if ((threadIdx.x & 31) == 0 && v != 0.0) atomicAdd(a.acc + i, v);
    }
}

}  // namespace gbmpm

namespace gbmpm {
// Current volume, Cauchy stress and det(F) per particle (Solver.vol / cauchy,
// core/solver.py:559-598): policy 0 warn (|J|, Cauchy divides by max(|J|, 1e-9)),
// 1 nan and 2 raise (NaN for inverted particles); counts the inverted ones.
__global__ void k_export_cauchy(const float *F, const float *S, const float *vol0, int n, int policy, float *cauchy,
                                float *vol, float *Jout, int *bad_count) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    float Fp[9];
#pragma unroll
    for (int i = 0; i < 9; ++i) Fp[i] = F[9 * (size_t)p + i];
    const float J = det3(Fp);
    const bool bad = !isfinite(J) || J <= 0.0f;
    if (bad) atomicAdd(bad_count, 1);
    float Jv = (policy == 0) ? (isfinite(J) ? fabsf(J) : NAN) : (bad ? NAN : J);
    float Jc = (policy == 0 && Jv < 1e-9f) ? 1e-9f : Jv;
    if (Jout) Jout[p] = J;
    if (vol) vol[p] = vol0[p] * Jv;
    if (cauchy) {
#pragma unroll
        for (int i = 0; i < 9; ++i) cauchy[9 * (size_t)p + i] = S[9 * (size_t)p + i] / Jc;
    }
}
}  // namespace gbmpm

extern "C" int gbmpm_compute_cauchy(gbmpm_engine *e, float *cauchy_out, float *vol_out, float *J_out, int32_t policy,
                                    int32_t *n_inverted, void *stream) {
    if (!e) return fail(GBMPM_ERR_ARG, "null engine");
    if (!e->bound) return fail(GBMPM_ERR_STATE, "buffers not bound");
    if (policy < 0 || policy > 2) return fail(GBMPM_ERR_ARG, "policy must be 0 (warn), 1 (nan) or 2 (raise)");
    cudaStream_t s = (cudaStream_t)stream;
    GB_CUDA(e->d_flagbuf.ensure(1));
    GB_CUDA(cudaMemsetAsync(e->d_flagbuf.ptr, 0, sizeof(int), s));
    if (e->P.n > 0) {
        k_export_cauchy<<<(e->P.n + 255) / 256, 256, 0, s>>>(e->P.F, e->P.stress, e->P.vol, e->P.n, policy, cauchy_out,
                                                             vol_out, J_out, e->d_flagbuf.ptr);
        e->launches++;
    }
    if (n_inverted) {
        GB_CUDA(cudaMemcpyAsync(n_inverted, e->d_flagbuf.ptr, sizeof(int), cudaMemcpyDeviceToHost, s));
        GB_CUDA(cudaStreamSynchronize(s));
    }
    return GBMPM_OK;
}

extern "C" int gbmpm_contact_wrench(gbmpm_engine *e, const double box_center[3], const double box_half[3],
                                    double layer, int32_t compressive_only, int32_t policy, double out[9],
                                    void *stream) {
    if (!e || !box_center || !box_half || !out) return fail(GBMPM_ERR_ARG, "null argument");
    if (!e->bound) return fail(GBMPM_ERR_STATE, "buffers not bound");
    if (policy < 0 || policy > 2) return fail(GBMPM_ERR_ARG, "policy must be 0 (warn), 1 (nan) or 2 (raise)");
    cudaStream_t s = (cudaStream_t)stream;
    GB_CUDA(e->d_tmp.ensure(18));   // nine doubles
    CWArgs a{};
    a.x = e->P.x; a.F = e->P.F; a.S = e->P.stress; a.vol0 = e->P.vol; a.sel = e->P.selection; a.n = e->P.n;
    for (int i = 0; i < 3; ++i) { a.c[i] = box_center[i]; a.h[i] = box_half[i]; }
    a.layer = layer;
    a.compressive = compressive_only ? 1 : 0;
    a.policy = policy;
    a.acc = reinterpret_cast<double *>(e->d_tmp.ptr);
    GB_CUDA(cudaMemsetAsync(a.acc, 0, 9 * sizeof(double), s));
    if (a.n > 0) {
        const int grid = std::min((a.n + 255) / 256, e->num_sms * 4);
        k_cw_volume<<<grid, 256, 0, s>>>(a);
        k_cw_layer<<<grid, 256, 0, s>>>(a);
        e->launches += 2;
    }
    GB_CUDA(cudaMemcpyAsync(out, a.acc, 9 * sizeof(double), cudaMemcpyDeviceToHost, s));
    GB_CUDA(cudaStreamSynchronize(s));
    if (policy == 2 && out[8] > 0.0)
        return fail(GBMPM_ERR_STATE, std::to_string((long long)out[8]) +
                                         " particles have non-finite or non-positive det(F); current volume and "
                                         "Cauchy stress are undefined for an inverted configuration");
    return GBMPM_OK;
}

#include "adjoint.cuh"
#include "meshfield.cuh"
