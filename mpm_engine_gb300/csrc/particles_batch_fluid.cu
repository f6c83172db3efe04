// particles_batch_fluid.cu - the batched tiled particle pass (k_particles_batch) with
// the SVD-based solid laws compiled out, in its own translation unit so the
// variants build in parallel. One instantiation per tile width (64, 128, 256
// particles) and occupancy (2 or 3 resident 256-thread equivalents per SM); the
// autotuner picks among them.

#include "common.cuh"

#include <climits>

namespace gbmpm {

#include "materials.cuh"
#include "particle_pass.cuh"

void launch_particle_batch_fluid(const BatchLaunch &L, const PK *table, const BatchCta *ctas, int nctas, int mode,
                                 int list, int sub, cudaStream_t s) {
    if (nctas < 1) return;
    const bool o3 = L.occ >= 3;
    if (L.threads <= 64) {
        if (o3) launch_kernel(L.pdl, k_particles_batch<false, 3, 64>, nctas, 64, s, table, ctas, mode, list, sub);
        else launch_kernel(L.pdl, k_particles_batch<false, 2, 64>, nctas, 64, s, table, ctas, mode, list, sub);
    } else if (L.threads <= 128) {
        if (o3) launch_kernel(L.pdl, k_particles_batch<false, 3, 128>, nctas, 128, s, table, ctas, mode, list, sub);
        else launch_kernel(L.pdl, k_particles_batch<false, 2, 128>, nctas, 128, s, table, ctas, mode, list, sub);
    } else {
        if (o3) launch_kernel(L.pdl, k_particles_batch<false, 3, 256>, nctas, 256, s, table, ctas, mode, list, sub);
        else launch_kernel(L.pdl, k_particles_batch<false, 2, 256>, nctas, 256, s, table, ctas, mode, list, sub);
    }
}

}  // namespace gbmpm
