// sph_abi.cu -- compile-time layout checks of the reference structs as the
// library sees them (fluid.h:56-106, hash.h:35-48, geometry.h:33-40), and
// the runtime size query used by the host-side tests.
#include <cstddef>

#include "sph_cuda.h"

static_assert(sizeof(fluid_particle) == 52, "fluid_particle is 12 floats + int (fluid.h:56-70)");
static_assert(offsetof(fluid_particle, x_prev) == 0, "fluid.h:57");
static_assert(offsetof(fluid_particle, x) == 8, "fluid.h:59");
static_assert(offsetof(fluid_particle, v_x) == 16, "fluid.h:61");
static_assert(offsetof(fluid_particle, density) == 32, "fluid.h:65");
static_assert(offsetof(fluid_particle, pressure) == 40, "fluid.h:67");
static_assert(offsetof(fluid_particle, id) == 48, "fluid.h:69");
static_assert(sizeof(tunable_parameters) == 64, "15 floats + 3 chars, padded (fluid.h:78-97)");
static_assert(offsetof(tunable_parameters, time_step) == 32, "fluid.h:87");
static_assert(offsetof(tunable_parameters, mover_center_x) == 44, "fluid.h:90");
static_assert(offsetof(tunable_parameters, mover_type) == 60, "fluid.h:94");
static_assert(offsetof(tunable_parameters, active) == 62, "fluid.h:96");
static_assert(sizeof(param) == 80, "fluid.h:100-106");
static_assert(offsetof(param, number_halo_particles) == 76, "fluid.h:105");
static_assert(sizeof(AABB_t) == 24, "geometry.h:33-40");
static_assert(sizeof(neighbor) == 2 * sizeof(void *), "fluid.h:72-75");
static_assert(sizeof(bucket_t) == 2 * sizeof(void *), "hash.h:35-38");
static_assert(offsetof(neighbor_grid_t, neighbors) == 16, "hash.h:44");
static_assert(offsetof(neighbor_grid_t, max_neighbors) == 32, "hash.h:46");
static_assert(sizeof(neighbor_grid_t) == 40, "hash.h:40-48");

extern "C" int sph_cuda_abi_sizes(int *sizes, int n)
{
    const int s[7] = {(int)sizeof(fluid_particle), (int)sizeof(neighbor),
                      (int)sizeof(tunable_parameters), (int)sizeof(param), (int)sizeof(bucket_t),
                      (int)sizeof(neighbor_grid_t), (int)sizeof(AABB_t)};
    if (!sizes || n < 7) return 1;
    for (int i = 0; i < 7; ++i) sizes[i] = s[i];
    return 0;
}
