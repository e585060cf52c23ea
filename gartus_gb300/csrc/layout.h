// layout.h — device data layout shared by the host library and the kernels.
//
// Everything a render touches lives in HBM as flat arrays in BVH leaf order:
//   prims  : PrimRec<R>[n]   16 scalars per primitive (64 B in f32, 128 B in f64)
//   meta   : uint2[n]        x = kind | material << 3, y = original primitive index
//   nodes  : Node<R>[m]      internal BVH nodes in pre-order, both child boxes inline
// plus small tables for materials, light targets and the environment distribution.
#pragma once

#include <stdint.h>

#include "../../include/gartus_gpu.h"
#include "wide_bvh.h"

#if defined(__CUDACC__)
#define GT_HD __host__ __device__
#else
#define GT_HD
#endif

namespace gt {

// Primitive kinds in PrimRec/meta (the ABI's gt_geometry_kind plus a never-hit kind for
// degenerate quads/triangles, which the reference rejects on every query:
// geometry.rs:394-397, object.rs:192-203).
enum : uint32_t { K_SPHERE = 0, K_MOVING = 1, K_TRIANGLE = 2, K_QUAD = 3, K_NEVER = 7 };

// PrimRec layout (scalars):
//   sphere   : [0..3) centre, [3] radius
//   moving   : [0..3) centre at t=0, [3] radius, [4..7) centre(1) - centre(0)
//   triangle : [0..3) p0, [4..7) p1 - p0, [8..11) p2 - p0, [12..15) unit geometric normal
//   quad     : [0..3) corner, [3] plane D, [4..7) u, [7] n.x, [8..11) v, [11] n.y, [12..15) w, [15] n.z
template <class R> struct alignas(16) PrimRec {
    R v[16];
};

// Internal node with both child boxes (min xyz, max xyz for left then right) and links:
// link[0]/link[2] = child node index (>= 0) or ~first_primitive (< 0) for a leaf child,
// link[1]/link[3] = leaf primitive count (0 for an internal child).
template <class R> struct alignas(16) Node {
    R box[12];
    int32_t link[4];
};

// Materials (raytracing/material.rs) with a solid or checker colour source.
// Perlin tables of one NoiseTexture (gmath/perlin.rs:8-31): 256 unit gradients (made in
// f64 on the host, stored as R) and the three 256-entry permutations.
template <class R> struct PerlinDev {
    R gx[256], gy[256], gz[256];
    uint16_t perm[3][256];
};

// One bitmap texture on the device (gt_image): 8-bit texels, row 0 at the top.
struct ImageDev {
    const uint8_t* rgb;
    uint32_t w, h, filter, wrap_s, wrap_t, pad;
};

template <class R> struct MatDev {
    int32_t kind;
    int32_t tex;
    R color[3];
    R param;
    R inv_scale; // checker: 1 / |scale|; noise: scale
    R even[3];
    R odd[3];
    int32_t noise_variant;
    int32_t noise_depth;
    const PerlinDev<R>* noise; // this material's tables (GT_TEX_NOISE)
    const ImageDev* image;     // this material's bitmap (GT_TEX_IMAGE)
    const ImageDev* normal_map; // tangent-space normal map, or null
    R normal_strength;
    int32_t normal_neg_y;       // 1 = -Y green channel
};

// Weighted sampling target (raytracing/scene.rs:423-497) with the geometry's derived
// quantities precomputed in f64 on the host.
template <class R> struct LightDev {
    int32_t kind;
    int32_t pad;
    R weight;
    R radius;
    R a[3]; // centre / corner / p0
    R b[3]; // centre(1) - centre(0) / u / p1
    R c[3]; // v / p2
    R n[3]; // quad unit normal / triangle unit normal
    R w[3]; // quad w
    R plane_d;
    R area_sq; // quad |u x v|^2
    R area;    // quad sqrt(area_sq), triangle 0.5 |e1 x e2|
};

// EnvironmentLight (raytracing/environment.rs:22-31): texels plus the luminance x sin
// distribution over texels and its running sum.
template <class R> struct EnvDev {
    int32_t format; // gt_environment_format
    uint32_t width, height;
    const uint8_t* px8;
    const float* px32;
    const R* weights;
    const R* cdf;
    R total;
};

// Camera and integrator constants for one render (camera.rs:613-643 after initialize()).
template <class R> struct CamDev {
    R center[3], pixel00[3], du[3], dv[3], ddu[3], ddv[3];
    R p00_rel[3]; // pixel00 - center, computed in f64 (the f32 camera's cancellation-free form)
    R shutter0, shutter1;
    R light_pdf_weight;
    R adaptive_threshold;
    R bg[9];
    uint64_t seed;
    uint32_t width, height;
    uint32_t spp;        // samples per pixel loop count (effective)
    uint32_t mode;       // gt_pixel_sample_mode
    uint32_t grid;       // stratified grid width
    uint32_t adaptive;   // 1 = Welford stopping rule
    uint32_t adaptive_min, adaptive_max;
    uint32_t max_depth;
    int32_t rr_min_depth; // < 0 = off
    uint32_t defocus;     // defocus_angle > 0
    uint32_t bg_kind;
    uint32_t nee;         // next-event estimation
    uint32_t use_lights, use_env;
};

// ConstantMedium (raytracing/volume/medium.rs:13-187): its boundary (one sphere, or the six
// quads of box_object, object.rs:930-976, in PrimRec layout with derived quantities from
// f64), the RotateY sine and cosine and the Translate offset (instance.rs), and -1/density.
template <class R> struct MediumDev {
    uint32_t parts;     // 1 (sphere) or 6 (box quads)
    uint32_t mat;       // phase-function material
    uint32_t transform; // gt_medium_transform bits
    uint32_t pad;
    R neg_inv_density;
    R sin_t, cos_t;
    R off[3];
    PrimRec<R> part[6]; // K_SPHERE or K_QUAD records (a degenerate quad is never hit)
    uint32_t kind[6];
};

template <class R> struct SceneDev;

// One mesh (TriangleMesh, raytracing/mesh.rs) in object space: a scene view of its own
// primitives and BVH (sharing the scene's material table) and its per-primitive texture
// coordinates (6) and vertex normals (9) in its leaf order, with presence bits
// (bit 0 texture coordinates, bit 1 normals).
template <class R> struct MeshDev;

// A world object: a mesh, or MatrixInstance(mesh) with its object-to-world and
// world-to-object matrices (row-major 4x4; the normal transform is the inverse transposed).
template <class R> struct ObjectDev {
    uint32_t mesh;
    uint32_t transformed;
    R xf[16];
    R inv[16];
};

// Scene view handed to kernels.
template <class R> struct SceneDev {
    const PrimRec<R>* prims;
    const uint2* meta;
    const Node<R>* nodes;
    const MatDev<R>* mats;
    const MediumDev<R>* media; // tested after the surfaces, in order
    uint32_t num_media;
    uint32_t num_objects;       // world objects, tested after the RayScene's surfaces
    const MeshDev<R>* meshes;
    const ObjectDev<R>* objects;
    const Node<R>* tlas;        // BVH over the objects' world boxes (leaves index objects)
    R tlas_box[6];
    int32_t tlas_link;
    int32_t tlas_count;
    R root_box[6];
    int32_t root_link; // >= 0 internal root node, < 0 ~first of a leaf root
    int32_t root_count;
    uint32_t num_prims;
    uint32_t num_nodes;
    // f32 only: the eight-wide compressed tree over the same leaves (leaf slots are the
    // primitive order above), or null to traverse `nodes`.
    const WideNode* wnodes;
};

template <class R> struct MeshDev {
    SceneDev<R> view;
    const R* uv;
    const R* vn;
    const uint8_t* attr;
};

template <class R> struct LightsDev {
    const LightDev<R>* t;
    uint32_t count;
    R total;
};

// Four-wide vector of R used for the path-state arrays (16 B in f32, 32 B in f64).
template <class R> struct alignas(4 * sizeof(R) > 16 ? 16 : 4 * sizeof(R)) R4 {
    R x, y, z, w;
};

// Wavefront path state, one slot per pixel (the reference draws every sample of a pixel
// from one sequential stream, camera.rs:2669, so a pixel's samples run in order).
template <class R> struct PathState {
    R4<R>* ray_o;   // origin xyz, time
    R4<R>* ray_d;   // direction xyz, miss-radiance weight
    R4<R>* att;     // attenuation xyz
    R4<R>* col;     // sample radiance xyz
    uint4* st;      // rng lo, rng hi, flags, samples started
    R* hit_t;       // closest-hit distance
    int32_t* hit_prim; // leaf-order primitive slot or -1 (an object hit: the mesh's leaf)
    int32_t* hit_obj;  // leaf-order object hit or -1 (worlds with objects; else null)
    R4<R>* acc;     // running sum (or Welford mean)
    R4<R>* comp;    // Kahan compensation (or Welford M2)
    uint32_t* accepted;
    R4<R>* sh_o;    // shadow origin xyz, time   [2 per slot]
    R4<R>* sh_d;    // shadow direction xyz, kind (1 area, 2 env)
    R4<R>* sh_a;    // attenuation before the bounce xyz, ratio
    R4<R>* sh_s;    // scatter attenuation (x radiance for env) xyz
    // queues
    uint32_t* q_trace[2];
    uint32_t* q_mat; // 8 queues of capacity n (key = material kind, 7 = miss)
    uint32_t* q_shadow;
    uint32_t* q_migrate; // slots handed to the concurrent persistent kernel
    uint32_t* q_handoff; // slots the side launch hands to its cooperative launch
    uint32_t* counters; // [0,1] trace, [2..10) mat keys, [10] shadow, [11] done, [12] error,
                        // [13] migrated slots, [14] their pull counter, [15] tail slots,
                        // [16..22) hand-over counters
    unsigned long long* totals; // [0] rays, [1] shadow rays, [2] accepted samples, [3] started samples,
                                // [6] queries traced by k_persistent
    unsigned long long* mstat;  // migration: samples started by unfinished slots, their number
    uint32_t n;
    // Stripes: the frame's rows are dealt to `stripes` independent wavefronts (row r to
    // stripe r % stripes), each with its own queues, counters and streams; this one owns
    // `local_n` slots, and its queues hold up to `qcap` entries per key.
    uint32_t stripe, stripes, row, local_n, qcap;
};

// Global slot of this stripe's j-th slot.
template <class R> __host__ __device__ inline uint32_t stripe_slot(const PathState<R>& ps, uint32_t j) {
    if (ps.stripes <= 1) return j;
    const uint32_t r = j / ps.row, x = j - r * ps.row;
    return (r * ps.stripes + ps.stripe) * ps.row + x;
}

enum : uint32_t {
    C_TRACE0 = 0,
    C_TRACE1 = 1,
    C_MAT = 2, // 8 entries
    C_SHADOW = 10,
    C_DONE = 11,
    C_ERROR = 12,
    C_MIGRATED = 13,
    C_MIGRATE_NEXT = 14,
    C_TAIL = 15, // slots finished by the tail launch
    // hand-over of the tail and side launches to cooperative launches (one warp per slot)
    C_TAIL_DONE = 16,
    C_TAIL_COOP = 17,
    C_TAIL_COOP_NEXT = 18,
    C_SIDE_DONE = 19,
    C_SIDE_COOP = 20,
    C_SIDE_COOP_NEXT = 21,
    C_COUNT = 24
};

enum : uint32_t { KEY_MISS = 7, NUM_KEYS = 8 };

// Path flags in st.z.
enum : uint32_t {
    F_BOUNCE_MASK = 0xffffu,
    F_ALLOW_EMIT = 1u << 16,
    F_NEWSAMPLE = 1u << 17, // finalize previous sample (if any) and start the next
    F_TRACE = 1u << 18,
    F_DONE = 1u << 19,
    F_SHADOW0 = 1u << 20, // pending area-light shadow query
    F_SHADOW1 = 1u << 21, // pending environment shadow query
    F_MIGRATED = 1u << 22, // finished by the concurrent persistent kernel, not the wavefront
    F_FRESH = 1u << 23     // resumed from an accumulator: no finished sample to fold in
};

// Error bits in counters[C_ERROR].
enum : uint32_t { E_STACK_OVERFLOW = 1u };

} // namespace gt
