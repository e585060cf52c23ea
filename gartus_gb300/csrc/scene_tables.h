// scene_tables.h — host-side tables derived from a scene description.
#pragma once

#include <cstdint>

namespace gt {

// The state of Perlin::new(seed) (gmath/perlin.rs:19-31), in f64.
struct PerlinTables {
    double grad[256][3];
    uint16_t perm[3][256];
};

// 256 gradients from SampleRng::random_unit_vector (the spherical-inversion form,
// gmath/random.rs:88-115), then the x, y and z permutations, each the identity shuffled
// by one pass from the last index down with target = floor(u * (index + 1))
// (perlin.rs:83-101).
void make_perlin_tables(uint64_t seed, PerlinTables& out);

} // namespace gt
