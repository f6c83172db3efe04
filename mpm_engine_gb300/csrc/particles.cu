// particles.cu - the particle-pass kernels (k_particles, the direct path, and
// k_particles_tiled, the block-sorted path) with their launcher. They are compiled
// apart from the engine so that the two translation units build in parallel; the
// engine reaches them only through launch_particle_pass.

#include "common.cuh"

#include <climits>

namespace gbmpm {

#include "materials.cuh"
#include "particle_pass.cuh"

void launch_particle_pass(const ParticleLaunch &L, const PK &k, int mode, cudaStream_t s) {
    const bool solids = L.solids;
    if (L.tiled && k.cdf_on) {
        constexpr int th = Tile<true>::threads;
        int grid = (k.n + th - 1) / th;
        if (grid < 1) grid = 1;
        if (L.cdf_occ >= 3) {
            if (solids) launch_kernel(L.pdl, k_particles_tiled<true, 3, true>, grid, th, s, k, mode);
            else launch_kernel(L.pdl, k_particles_tiled<false, 3, true>, grid, th, s, k, mode);
        } else {
            if (solids) launch_kernel(L.pdl, k_particles_tiled<true, 2, true>, grid, th, s, k, mode);
            else launch_kernel(L.pdl, k_particles_tiled<false, 2, true>, grid, th, s, k, mode);
        }
        return;
    }
    if (L.tiled) {
        constexpr int th = Tile<false>::threads;
        int grid = (k.n + th - 1) / th;
        if (grid < 1) grid = 1;
        if (solids && L.tile_occ >= 3) launch_kernel(L.pdl, k_particles_tiled<true, 3>, grid, th, s, k, mode);
        else if (solids) launch_kernel(L.pdl, k_particles_tiled<true, 2>, grid, th, s, k, mode);
        else if (L.tile_occ >= 4) launch_kernel(L.pdl, k_particles_tiled<false, 4>, grid, th, s, k, mode);
        else if (L.tile_occ == 3) launch_kernel(L.pdl, k_particles_tiled<false, 3>, grid, th, s, k, mode);
        else launch_kernel(L.pdl, k_particles_tiled<false, 2>, grid, th, s, k, mode);
        return;
    }
    int grid = (k.n + kParticleThreads - 1) / kParticleThreads;
    if (grid < 1) grid = 1;
    if (solids) k_particles<true><<<grid, kParticleThreads, 0, s>>>(k, mode);
    else k_particles<false><<<grid, kParticleThreads, 0, s>>>(k, mode);
}

}  // namespace gbmpm
