// particles.cu - the particle-pass kernels (k_particles, the direct path, and
// k_particles_tiled, the block-sorted path) with their launcher. They are compiled
// apart from the engine so that the two translation units build in parallel; the
// engine reaches them only through launch_particle_pass.

#include "common.cuh"

#include <climits>

namespace gbmpm {

#include "materials.cuh"
#include "particle_pass.cuh"

namespace {
// launch with programmatic stream serialization (see pdl_wait) when enabled
template <typename... P, typename... A>
void launch_maybe_pdl(bool pdl, void (*kern)(P...), int grid, int block, cudaStream_t s, A... args) {
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
}  // namespace

void launch_particle_pass(const ParticleLaunch &L, const PK &k, int mode, cudaStream_t s) {
    const bool solids = L.solids;
    if (L.tiled && k.cdf_on) {
        constexpr int th = Tile<true>::threads;
        int grid = (k.n + th - 1) / th;
        if (grid < 1) grid = 1;
        if (L.cdf_occ >= 3) {
            if (solids) launch_maybe_pdl(L.pdl, k_particles_tiled<true, 3, true>, grid, th, s, k, mode);
            else launch_maybe_pdl(L.pdl, k_particles_tiled<false, 3, true>, grid, th, s, k, mode);
        } else {
            if (solids) launch_maybe_pdl(L.pdl, k_particles_tiled<true, 2, true>, grid, th, s, k, mode);
            else launch_maybe_pdl(L.pdl, k_particles_tiled<false, 2, true>, grid, th, s, k, mode);
        }
        return;
    }
    if (L.tiled) {
        constexpr int th = Tile<false>::threads;
        int grid = (k.n + th - 1) / th;
        if (grid < 1) grid = 1;
        if (solids && L.tile_occ >= 3) launch_maybe_pdl(L.pdl, k_particles_tiled<true, 3>, grid, th, s, k, mode);
        else if (solids) launch_maybe_pdl(L.pdl, k_particles_tiled<true, 2>, grid, th, s, k, mode);
        else if (L.tile_occ >= 4) launch_maybe_pdl(L.pdl, k_particles_tiled<false, 4>, grid, th, s, k, mode);
        else if (L.tile_occ == 3) launch_maybe_pdl(L.pdl, k_particles_tiled<false, 3>, grid, th, s, k, mode);
        else launch_maybe_pdl(L.pdl, k_particles_tiled<false, 2>, grid, th, s, k, mode);
        return;
    }
    int grid = (k.n + kParticleThreads - 1) / kParticleThreads;
    if (grid < 1) grid = 1;
    if (solids) k_particles<true><<<grid, kParticleThreads, 0, s>>>(k, mode);
    else k_particles<false><<<grid, kParticleThreads, 0, s>>>(k, mode);
}

}  // namespace gbmpm
