// scene_tables.cpp — Perlin tables for NoiseTexture materials.
#include "scene_tables.h"

#include <cmath>
#include <utility>

namespace gt {
namespace {

// SampleRng (gmath/random.rs:16-59): SplitMix64 with the (30, 27, 31) finaliser.
struct HostRng {
    uint64_t state;
    uint64_t next() {
        state += 0x9e3779b97f4a7c15ULL;
        uint64_t v = state;
        v = (v ^ (v >> 30)) * 0xbf58476d1ce4e5b9ULL;
        v = (v ^ (v >> 27)) * 0x94d049bb133111ebULL;
        return v ^ (v >> 31);
    }
    double unit() { return double(next() >> 11) * (1.0 / 9007199254740992.0); }
};

} // namespace

void make_perlin_tables(uint64_t seed, PerlinTables& out) {
    HostRng rng{seed};
    const double tau = 6.283185307179586;
    for (int i = 0; i < 256; ++i) {
        const double r1 = rng.unit();
        const double r2 = rng.unit();
        const double z = 1.0 - 2.0 * r2;
        const double radius = std::sqrt(1.0 - z * z);
        const double phi = tau * r1;
        out.grad[i][0] = std::cos(phi) * radius;
        out.grad[i][1] = std::sin(phi) * radius;
        out.grad[i][2] = z;
    }
    for (int axis = 0; axis < 3; ++axis) {
        uint16_t* p = out.perm[axis];
        for (int i = 0; i < 256; ++i) p[i] = uint16_t(i);
        for (int i = 255; i >= 1; --i) {
            const int target = int(rng.unit() * (double(i) + 1.0));
            std::swap(p[i], p[target]);
        }
    }
}

} // namespace gt
