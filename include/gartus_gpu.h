/*
 * gartus_gpu.h — C ABI of the GB300 (sm_103a) path tracer that drops in for the
 * gartus `PathTracer` render path over a compiled `RayScene`.
 *
 * Every entry point here replaces one piece of the reference's Rust surface; the
 * reference interface is cited beside each declaration (paths are relative to the
 * gartus crate root).  The boundary is plain C: POD structs, raw pointers and sizes,
 * status codes instead of panics.  Nothing here exposes CUDA or torch types.
 *
 * Ownership: the library copies every input array it is given.  Handles are opaque
 * and are released by their matching *_destroy call.  Output buffers belong to the
 * caller.
 *
 * Errors: every fallible call returns a gt_status.  The reference panics through
 * `assert!` on invalid input (e.g. graphics/camera.rs:1161-1201,
 * raytracing/scene.rs:1158-1161); here those cases return GT_ERR_INVALID_ARG and the
 * message is available from gt_last_error() on the calling thread.
 *
 * Threading: a gt_context owns one CUDA stream.  Calls on one context (and on the
 * scenes, light lists and environments created from it) are serialised by an
 * internal mutex, so a scene may be shared between threads the way the reference's
 * `RayScene: Send + Sync` is (raytracing/object.rs:594).
 */
#ifndef GARTUS_GPU_H
#define GARTUS_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GT_ABI_VERSION 2u

typedef enum gt_status {
    GT_OK = 0,
    GT_ERR_INVALID_ARG = 1,
    GT_ERR_OOM = 2,
    GT_ERR_CUDA = 3,
    GT_ERR_TIMEOUT = 4,
    GT_ERR_CANCELLED = 5,
    GT_ERR_UNSUPPORTED = 6,
    GT_ERR_NO_DEVICE = 7,
    GT_ERR_INTERNAL = 8
} gt_status;

/* ---------------------------------------------------------------- geometry */

/* RayGeometry (raytracing/object.rs:252-258). */
typedef enum gt_geometry_kind {
    GT_GEOM_SPHERE = 0,        /* p[0..3] centre, p[3] radius (geometry.rs:419-431)        */
    GT_GEOM_MOVING_SPHERE = 1, /* p[0..3] centre at t=0, p[3..6] centre at t=1, p[6] radius */
    GT_GEOM_TRIANGLE = 2,      /* p[0..3] p0, p[3..6] p1, p[6..9] p2 (geometry.rs:129-133)  */
    GT_GEOM_QUAD = 3           /* p[0..3] corner, p[3..6] u, p[6..9] v (geometry.rs:271-301) */
} gt_geometry_kind;

typedef struct gt_geometry {
    uint32_t kind; /* gt_geometry_kind */
    uint32_t reserved;
    double p[9];
} gt_geometry;

/* RayPrimitive { geometry, material } (raytracing/scene.rs:876-880). */
typedef struct gt_primitive {
    gt_geometry geometry;
    uint32_t material; /* index into gt_scene_desc.materials */
    uint32_t reserved;
} gt_primitive;

/* ---------------------------------------------------------------- materials */

/* RayMaterial variants on the path (raytracing/material.rs:2355-2363). */
typedef enum gt_material_kind {
    GT_MAT_LAMBERTIAN = 0,    /* color = albedo                         (material.rs:508-537)   */
    GT_MAT_DIFFUSE_LIGHT = 1, /* color = emission                       (material.rs:1008-1028) */
    GT_MAT_ISOTROPIC = 2,     /* color = albedo                         (material.rs:1124-1147) */
    GT_MAT_GGX = 3,           /* color = specular colour, param = roughness (material.rs:1583-1622) */
    GT_MAT_METAL = 4,         /* color = albedo, param = fuzz           (material.rs:2087-2112) */
    GT_MAT_DIELECTRIC = 5,    /* param = refraction index               (material.rs:2264-2351) */
    GT_MAT_HENYEY_GREENSTEIN = 6 /* color = albedo, param = anisotropy g in (-1, 1): phase function
                                    around the incoming direction (material.rs:1175-1333,
                                    HenyeyGreensteinPdf gmath/sampling.rs:86-165)          */
} gt_material_kind;

/* Colour source of a material (graphics/raytracing/texture.rs SolidColor, CheckerTexture,
 * NoiseTexture). */
typedef enum gt_texture_kind {
    GT_TEX_SOLID = 0,   /* the material's color                                           */
    GT_TEX_CHECKER = 1, /* tex[0] = scale, tex[1..4] = even colour, tex[4..7] = odd colour  */
    GT_TEX_NOISE = 2,   /* Perlin: tex[0] = scale, tex[1] = variant (gt_noise_variant),
                           tex[2] = octave depth, tex[3] / tex[4] = seed bits 0-31 / 32-63  */
    GT_TEX_IMAGE = 3    /* ImageTexture (raytracing/texture.rs:110-156): tex[0] = index into
                           gt_scene_desc.images, sampled at the hit's (u, v)               */
} gt_texture_kind;

/* A bitmap texture (graphics/texture.rs Texture, sampled by Texture::sample 202-208):
 * 8-bit sRGB texels, decoded to linear as (c / 255)^2 (LinearRgb::from_rgb_srgb). */
typedef enum gt_texture_filter {
    GT_FILTER_NEAREST = 0, /* sample_nearest, texture.rs:716-722 */
    GT_FILTER_LINEAR = 1   /* sample_linear with u8 lerps, texture.rs:724-735 */
} gt_texture_filter;
typedef enum gt_texture_wrap {
    GT_WRAP_CLAMP = 0,
    GT_WRAP_REPEAT = 1
} gt_texture_wrap;
typedef struct gt_image {
    uint32_t width;
    uint32_t height;      /* an empty image (0 texels) samples as cyan (texture.rs:150-152) */
    const uint8_t* rgb;   /* width * height * 3 bytes, row 0 at the top (t = 1) */
    uint32_t filter;      /* gt_texture_filter */
    uint32_t wrap_s;      /* gt_texture_wrap */
    uint32_t wrap_t;
    uint32_t reserved;
} gt_image;

/* NoiseTexture kinds (graphics/raytracing/texture.rs:287-291). */
typedef enum gt_noise_variant {
    GT_NOISE_PLAIN = 0,      /* 0.5 (1 + noise(scale p))                         */
    GT_NOISE_TURBULENCE = 1, /* turbulence(scale p, depth)                      */
    GT_NOISE_MARBLE = 2      /* 0.5 (1 + sin(q.z + 10 turbulence(q, depth))), q = scale p */
} gt_noise_variant;

typedef struct gt_material {
    uint32_t kind;         /* gt_material_kind */
    uint32_t texture_kind; /* gt_texture_kind  */
    double color[3];
    double param;
    double tex[7];
    /* Tangent-space normal map (NormalMap, raytracing/texture.rs:160-276; Lambertian and
     * GgxMicrofacet only, material.rs:456-460, 1663-1684): 1 + index into
     * gt_scene_desc.images, 0 = none.  Applied at mesh triangles with texture coordinates
     * (their tangent frame, mesh.rs:94-101). */
    uint32_t normal_map;
    uint32_t normal_map_flags; /* GT_NORMAL_MAP_NEGATIVE_Y: DirectX-style green channel */
    double normal_map_strength;
} gt_material;

enum { GT_NORMAL_MAP_NEGATIVE_Y = 1 };

/* ------------------------------------------------------------------- scene */

/* A compiled RayScene (raytracing/scene.rs:1102-1106) with its BVH build options
 * (BvhBuildOptions, raytracing/bvh.rs:55-89). */
/* Which tree the f32 throughput path traverses. */
typedef enum gt_bvh_builder {
    GT_BVH_REFERENCE_SAH = 0, /* the reference's binary SAH tree, built on the host at creation */
    GT_BVH_GPU_LBVH = 1       /* a linear BVH built on the GPU when the scene is uploaded (Morton
                                 order, Karras 2012): for large scenes whose host build would
                                 dominate; f64 rendering and the traversal statistics still use
                                 the reference tree, built on the host when first needed.  No
                                 reference counterpart.                                        */
} gt_bvh_builder;

/* The tree the f32 path traverses (no reference counterpart; the f64 path and the
 * traversal statistics always walk the reference's binary tree).  GT_F32_TREE_WIDE: an
 * eight-wide tree with byte-quantised child boxes, collapsed from the reference SAH tree
 * (same leaves, same hits; the binary walk is kept where a scene has no wide form: a
 * single leaf, leaves of more than four primitives, or a GT_BVH_GPU_LBVH scene).  The
 * meshes of world objects get their own wide trees the same way, walked by the wavefront
 * schedules (the persistent kernel walks their binary trees).
 * GT_F32_TREE_BINARY: the reference's binary tree, for the RayScene and the meshes. */
typedef enum gt_f32_tree {
    GT_F32_TREE_WIDE = 0,
    GT_F32_TREE_BINARY = 1
} gt_f32_tree;

/* A constant-density participating medium (ConstantMedium, raytracing/volume/medium.rs:13-187)
 * whose boundary is a sphere or a box_object (object.rs:930-976), optionally wrapped as
 * Translate(RotateY(shape, rotate_y), translate) (instance.rs).  A scene with media renders as
 * the reference's HittableList [the RayScene's surfaces, media[0], media[1], ...]
 * (scene.rs:177-197): each ray's media are tested in order after the surfaces, and a medium
 * whose boundary interval, clipped to the closest hit so far, is not empty draws one sample
 * from the pixel's stream (path, shadow and AOV rays alike).  The ray queries
 * gt_trace_rays / gt_trace_primary see the surfaces only, as RayScene::hit does. */
typedef enum gt_medium_shape {
    GT_MEDIUM_SPHERE = 0, /* p[0..3) centre, p[3] radius */
    GT_MEDIUM_BOX = 1     /* p[0..3) / p[3..6) two opposite corners */
} gt_medium_shape;
typedef enum gt_medium_transform {
    GT_MEDIUM_ROTATE_Y = 1, /* RotateY::new(shape, rotate_y degrees)              */
    GT_MEDIUM_TRANSLATE = 2 /* Translate::new(.., translate), outside the rotation */
} gt_medium_transform;
typedef struct gt_medium {
    uint32_t shape;       /* gt_medium_shape */
    uint32_t material;    /* phase function (ConstantMedium::new uses Isotropic(albedo)) */
    double p[6];
    double rotate_y;      /* degrees */
    double translate[3];
    double density;       /* positive and finite (medium.rs:93-96) */
    uint32_t transform;   /* gt_medium_transform bits */
    uint32_t reserved;
} gt_medium;

/* A triangle mesh in object space (TriangleMesh, raytracing/mesh.rs:149-360, with its own
 * BVH, mesh.rs:640-668): primitives (triangles; spheres and quads are accepted too, for
 * instancing any RayScene-like object) with optional per-triangle texture coordinates and
 * vertex normals (MeshTriangle, mesh.rs:22-141). */
typedef struct gt_mesh {
    uint32_t num_primitives;
    uint32_t bvh_leaf_size;           /* 0 = 4 (BvhBuildOptions::default) */
    const gt_primitive* primitives;   /* geometry and material per primitive */
    const double* texcoords;          /* 6 per primitive (u0 v0 u1 v1 u2 v2) or NULL */
    const double* normals;            /* 9 per primitive (n0 n1 n2) or NULL */
    const uint8_t* attribute_flags;   /* per primitive: bit 0 texcoords, bit 1 normals present;
                                         NULL = present wherever the array is given */
} gt_mesh;

/* One world object after the RayScene's surfaces: a mesh, or MatrixInstance(mesh,
 * transform) (raytracing/instance.rs:205-317).  `inverse` is the instance's world-to-object
 * matrix as MatrixInstance::inverse returns it; the normal transform is its transpose. */
typedef struct gt_object {
    uint32_t mesh;       /* index into gt_scene_desc.meshes */
    uint32_t transformed; /* 0 = the mesh as it is, 1 = MatrixInstance */
    double transform[16]; /* row-major object to world */
    double inverse[16];   /* row-major world to object */
} gt_object;

typedef struct gt_scene_desc {
    uint32_t struct_size; /* sizeof(gt_scene_desc) */
    uint32_t num_primitives;
    const gt_primitive* primitives;
    uint32_t num_materials;
    uint32_t bvh_leaf_size; /* 0 selects the reference default of 4 */
    const gt_material* materials;
    uint32_t bvh_builder;   /* gt_bvh_builder */
    uint32_t num_images;
    const gt_image* images; /* textures referenced by GT_TEX_IMAGE materials (copied) */
    uint32_t num_media;
    uint32_t num_meshes;
    const gt_medium* media; /* participating media after the surfaces, in list order (copied) */
    const gt_mesh* meshes;  /* meshes that objects place (copied) */
    uint32_t num_objects;
    uint32_t f32_tree;        /* gt_f32_tree: the tree the f32 path traverses (0 = wide) */
    const gt_object* objects; /* world objects tested after the RayScene's surfaces and before
                                 the media (copied) */
} gt_scene_desc;

/* One weighted sampling target (WeightedSamplingTargetList, raytracing/scene.rs:423-497).
 * SamplingTargetList::add_* uses weight 1.0 (scene.rs:381-391). */
typedef struct gt_light_target {
    gt_geometry geometry;
    double weight;
} gt_light_target;

/* EnvironmentLight texels (raytracing/environment.rs:22-31).  GT_ENV_SRGB8 is the
 * reference's 8-bit gamma-2 canvas; GT_ENV_RGB32F is the linear f32 extension whose
 * radiance is not limited to 1.0.  Texel (x, y) is at y*width + x, row 0 = zenith. */
typedef enum gt_environment_format {
    GT_ENV_SRGB8 = 0,
    GT_ENV_RGB32F = 1
} gt_environment_format;

typedef struct gt_environment_desc {
    uint32_t struct_size;
    uint32_t format; /* gt_environment_format */
    uint32_t width;
    uint32_t height;
    const void* texels; /* width*height*3 bytes (SRGB8) or floats (RGB32F) */
} gt_environment_desc;

/* ------------------------------------------------------------------ camera */

/* PixelSampleMode (graphics/camera.rs:43-56). */
typedef enum gt_pixel_sample_mode {
    GT_SAMPLE_RANDOM = 0,
    GT_SAMPLE_STRATIFIED = 1,
    GT_SAMPLE_STRATIFIED_GRID = 2
} gt_pixel_sample_mode;

/* DirectLightingMode (graphics/camera.rs:58-64). */
typedef enum gt_direct_lighting_mode {
    GT_DIRECT_CURRENT_PATH_CONTINUATION = 0,
    GT_DIRECT_NEXT_EVENT_ESTIMATION = 1
} gt_direct_lighting_mode;

/* RayBackground (graphics/camera.rs:203-215); the Function variant cannot cross the ABI. */
typedef enum gt_background_kind {
    GT_BG_CONSTANT = 0,         /* background[0..3] */
    GT_BG_VERTICAL_GRADIENT = 1 /* background[0..3] nadir, [3..6] horizon, [6..9] zenith */
} gt_background_kind;

/* RayCameraParams (graphics/camera.rs:646-669) plus the builder state of RayCamera
 * (camera.rs:613-643).  gt_camera_default() fills the values of RayCamera::new
 * (camera.rs:1034-1065). */
typedef struct gt_camera_desc {
    uint32_t struct_size;
    uint32_t image_width;
    double aspect_ratio;
    uint32_t samples_per_pixel;
    uint32_t pixel_sample_mode; /* gt_pixel_sample_mode */
    uint32_t grid_width;        /* used by GT_SAMPLE_STRATIFIED_GRID */
    uint32_t adaptive;          /* 1 = AdaptiveSampling enabled (camera.rs:367-396) */
    uint32_t adaptive_min_samples;
    uint32_t adaptive_max_samples;
    double adaptive_error_threshold;
    uint32_t direct_lighting_mode; /* gt_direct_lighting_mode */
    uint32_t max_depth;
    double light_pdf_weight;
    int32_t russian_roulette_min_depth; /* negative = None (without_russian_roulette) */
    uint32_t reserved0;
    uint64_t rng_seed;
    double vertical_fov;
    double lookfrom[3];
    double lookat[3];
    double view_up[3];
    double defocus_angle;
    double focus_distance;
    double shutter_start;
    double shutter_end;
    uint32_t background_kind; /* gt_background_kind */
    uint32_t reserved1;
    double background[9];
} gt_camera_desc;

/* ------------------------------------------------------------------ render */

typedef enum gt_precision {
    GT_PRECISION_F32 = 0, /* throughput path: f32 arithmetic, Kahan-compensated accumulation */
    GT_PRECISION_F64 = 1  /* reference-exact path: the reference's f64 arithmetic, op for op  */
} gt_precision;

/* Progress callback between wavefront batches; a nonzero return cancels the render
 * (the reference cancels remaining tiles when its progress callback returns Err,
 * graphics/camera.rs:3195-3243). */
typedef int (*gt_progress_fn)(void* user, uint64_t samples_done, uint64_t samples_total);

/* Per-render measurements (no reference counterpart: the reference's bench only prints
 * wall-clock milliseconds, benches/render_performance.rs:52-61). */
typedef enum gt_kernel_id {
    GT_KERNEL_GENERATE = 0, /* finish samples, start camera rays          */
    GT_KERNEL_TRACE = 1,    /* closest-hit traversal + material binning    */
    GT_KERNEL_SHADE = 2,    /* one bounce of the integrator per path       */
    GT_KERNEL_SHADOW = 3,   /* deferred next-event shadow queries          */
    GT_KERNEL_OTHER = 4,    /* init, resolve, AOVs                         */
    GT_KERNEL_PERSISTENT = 5, /* the persistent schedule's single kernel   */
    GT_KERNEL_COUNT = 6
} gt_kernel_id;

typedef struct gt_render_stats {
    double gpu_ms;          /* device time of the whole render (CUDA events on the library's stream) */
    uint64_t iterations;    /* wavefront iterations launched                                          */
    uint64_t rays;          /* closest-hit queries (camera + bounce rays)                             */
    uint64_t shadow_rays;   /* next-event shadow queries                                              */
    uint64_t samples;       /* accepted camera samples summed over pixels                             */
    uint64_t samples_started;
    double kernel_ms[GT_KERNEL_COUNT];     /* filled when gt_render_opts.profile = 1 */
    uint64_t kernel_launches[GT_KERNEL_COUNT]; /* always filled: this library's kernel launches */
    uint64_t migrated_pixels; /* GT_SCHEDULE_AUTO: slow pixels moved early to the concurrent persistent kernel */
    uint64_t tail_pixels;     /* GT_SCHEDULE_AUTO: pixels the persistent kernel finished after the wavefront */
    uint64_t persistent_rays; /* closest-hit + shadow queries traced inside k_persistent launches           */
} gt_render_stats;

/* How the frame is scheduled on the GPU.  All give identical images.  A scene with media
 * (gt_scene_desc.media) always runs the persistent kernel, whose hits draw the media's
 * random numbers in the reference's order; a scene with objects and no media runs every
 * schedule. */
typedef enum gt_schedule {
    GT_SCHEDULE_AUTO = 0,       /* wavefront until few pixels are left, then the persistent kernel
                                   finishes them (gt_render_opts.tail_slots)                      */
    GT_SCHEDULE_WAVEFRONT = 1,  /* per-bounce kernels over material-binned queues, graph-replayed */
    GT_SCHEDULE_PERSISTENT = 2  /* one launch; threads pull pixels and run their paths in registers */
} gt_schedule;

typedef struct gt_render_opts {
    uint32_t struct_size;
    uint32_t precision;   /* gt_precision */
    uint32_t aovs;        /* 1 = also produce albedo and normal AOVs (camera.rs:3064-3116) */
    uint32_t profile;     /* 1 = launch kernels one by one with CUDA events around each (slower) */
    gt_progress_fn progress;
    void* progress_user;
    gt_render_stats* stats; /* optional output */
    uint32_t schedule;      /* gt_schedule */
    uint32_t tail_slots;    /* GT_SCHEDULE_AUTO: hand over to the persistent kernel once at most
                               this many pixels are unfinished; 0 = as many as one persistent
                               launch keeps resident */
    uint32_t stripes;       /* wavefront schedules: the frame's rows are dealt to this many
                               independent wavefronts on their own streams, whose kernels
                               overlap on the GPU; 0 = 4 (2 for the sample rows of the
                               substream mode), at most 8; images do not depend on it */
    /* Optional host buffer of width*height*3 floats.  Before each progress call the library
     * writes the image as far as it is known: finished pixels hold their final value, the
     * others 0 (the partially filled `pixels` of ProgressiveRenderUpdate,
     * camera.rs:3172-3270).  Pixels still being written by a running persistent launch
     * may show a partial value; in the substream mode (rng) every pixel holds the estimate of
     * the samples folded so far. */
    float* progress_rgb;
    /* Wavefront launch shapes, in resident 256-thread blocks per SM (0 = the library's
     * choice: 8 for the generate kernel, 6 for trace, shade and shadow); gt_autotune
     * picks them per workload. */
    uint32_t generate_blocks_per_sm;
    uint32_t trace_blocks_per_sm;
    /* GT_SCHEDULE_AUTO: once per stripe, early in the frame, the pixels progressing at less
     * than half the stripe's mean sample rate (long sample chains: glass, adaptive pixels at
     * their cap) move to a persistent kernel that runs them concurrently with the wavefront.
     * gt_migrate; f64 images do not depend on it.  Never in a world with objects. */
    uint32_t migrate;
    /* Per-sample random streams, gt_rng.  GT_RNG_PIXEL (the reference, camera.rs:2669):
     * each pixel's samples continue one stream.  GT_RNG_SUBSTREAMS (throughput mode, no
     * reference counterpart): sample s of pixel (x, y) draws from its own SplitMix64 stream
     * started at pixel_seed(seed, x, y) ^ sample_key(s), where sample_key(s) is SplitMix64's
     * output for state (s + 1) * 0x9E3779B97F4A7C15; the samples of a pixel are then
     * independent and run in parallel.  The estimator is the reference's (adaptive
     * sampling stops at the same sample for the same sample values), the streams are not.
     * The schedule is ignored; accumulation, worlds with media, batches of worlds with
     * objects, and f64 batches return GT_ERR_UNSUPPORTED. */
    uint32_t rng;
} gt_render_opts;

typedef enum gt_rng { GT_RNG_PIXEL = 0, GT_RNG_SUBSTREAMS = 1 } gt_rng;

typedef enum gt_migrate {
    GT_MIGRATE_DEFAULT = 0, /* on for scenes of at most 65,536 primitives, off above: there the
                               persistent kernel's unsorted walks of the large tree run slower
                               than the wavefront's */
    GT_MIGRATE_ON = 1,
    GT_MIGRATE_OFF = 2
} gt_migrate;

/* Caller-owned output images, row-major, 3 channels, y = 0 is the top row
 * (HdrImage, graphics/display.rs:282-295).  Any pointer may be NULL except rgb. */
typedef struct gt_frame {
    uint32_t struct_size;
    uint32_t width;
    uint32_t height;
    uint32_t device_buffers; /* 0: host pointers, 1: pointers into device memory */
    float* rgb;
    float* albedo;
    float* normal;
    double* rgb64;      /* host or device, f64 copy of rgb (useful with GT_PRECISION_F64) */
    uint32_t* accepted; /* accepted (finite) samples per pixel */
} gt_frame;

/* BvhTraversalStats (raytracing/bvh.rs:9-17). */
typedef struct gt_bvh_stats {
    uint64_t rays;
    uint64_t node_bounds_tests;
    uint64_t node_bounds_hits;
    uint64_t leaf_visits;
    uint64_t primitive_candidates;
    uint64_t leaf_hit_results;
    uint64_t max_stack_depth;
} gt_bvh_stats;

/* What gt_trace_rays_f32 / gt_trace_primary_f32 did. */
typedef struct gt_trace_report {
    uint32_t struct_size; /* sizeof(gt_trace_report) */
    uint32_t tree;        /* gt_f32_tree the f32 walk traversed */
    uint64_t rays;
    uint64_t refined;     /* rays re-traced in f64: near ties, near edges, near t_min */
    uint64_t changed;     /* of those, rays whose primitive the f64 re-trace changed */
    uint32_t wide_nodes;  /* nodes of the scene's wide tree (0 without one) */
    uint32_t wide_depth;  /* its levels */
} gt_trace_report;

/* Opaque handles. */
typedef struct gt_context gt_context;
typedef struct gt_scene gt_scene;
typedef struct gt_lights gt_lights;
typedef struct gt_environment gt_environment;

/* ------------------------------------------------------------ entry points */

/* ABI version of the loaded library (GT_ABI_VERSION). */
uint32_t gt_abi_version(void);

/* Message of the last failed call on this thread ("" if none). */
const char* gt_last_error(void);

/* Fills *camera with RayCamera::new(image_width, aspect_ratio) defaults
 * (graphics/camera.rs:1034-1065). */
gt_status gt_camera_default(uint32_t image_width, double aspect_ratio, gt_camera_desc* camera);

/* Image height of RayCamera::initialized (graphics/camera.rs:1071) and the
 * effective samples per pixel (camera.rs:1547-1556). */
gt_status gt_camera_image_size(const gt_camera_desc* camera, uint32_t* width, uint32_t* height,
                               uint32_t* samples_per_pixel);

/* Creates a context on CUDA device `device` with its own streams. */
gt_status gt_context_create(int device, gt_context** out);
/* Destroy every scene, light list, environment and accumulator made on a context before
 * the context itself. */
void gt_context_destroy(gt_context* context);

/* Copies a RayScene to the device and builds its BVH on the host with the
 * reference's binary SAH builder (RayScene::build_bvh_with_options,
 * raytracing/scene.rs:1562-1565; FlatBvh::build, raytracing/bvh.rs:233-288). */
gt_status gt_scene_create(gt_context* context, const gt_scene_desc* desc, gt_scene** out);
void gt_scene_destroy(gt_scene* scene);

/* Replaces primitives [first, first + count) in place (same scene, same materials table):
 * the per-frame update of an animation's moving geometry.  The reference rebuilds such a
 * dynamic layer's BVH every frame (RayScene::build_bvh on the layer of a HittableLayers
 * static + dynamic split, raytracing/scene.rs:227-351).  Here a scene created with
 * GT_BVH_GPU_LBVH that is resident in f32 has its GPU-built tree refitted on the device
 * (the updated records scattered to their leaves, every internal box recomputed bottom-up;
 * the topology stays, so a refitted tree may be slower than a rebuilt one); the reference
 * SAH tree, which the f64 path, the traversal statistics and GT_BVH_REFERENCE_SAH scenes
 * use, is rebuilt on the host.  Waits for the context's stream first. */
gt_status gt_scene_update_primitives(gt_scene* scene, uint32_t first, uint32_t count, const gt_primitive* primitives);

/* RayScene::bvh_node_count (raytracing/scene.rs:1432-1437). */
gt_status gt_scene_bvh_node_count(const gt_scene* scene, uint32_t* count);

/* RayScene::emissive_targets (raytracing/scene.rs:1401-1423): one weight-1 target per
 * primitive whose material is a DiffuseLight, in primitive order.  Writes at most
 * `capacity` targets and the total count to *count. */
gt_status gt_scene_emissive_targets(const gt_scene* scene, gt_light_target* targets,
                                    uint32_t capacity, uint32_t* count);

/* A SamplingTargetList / WeightedSamplingTargetList (raytracing/scene.rs:355-497). */
gt_status gt_lights_create(gt_context* context, const gt_light_target* targets, uint32_t count,
                           gt_lights** out);
void gt_lights_destroy(gt_lights* lights);

/* EnvironmentLight::new (raytracing/environment.rs:36-51) and its f32 extension. */
gt_status gt_environment_create(gt_context* context, const gt_environment_desc* desc,
                                gt_environment** out);
void gt_environment_destroy(gt_environment* environment);

/* Renders one frame.  Replaces, by which handles are passed:
 *   lights = NULL, environment = NULL : PathTracer::render_hdr_image (renderer.rs:112-117)
 *   lights != NULL                    : PathTracer::render_with_lights_hdr_image (renderer.rs:391-406)
 *   environment != NULL               : PathTracer::render_with_environment_hdr_image (renderer.rs:431-449),
 *                                       which forces next-event estimation (camera.rs:4171-4173)
 *   both                              : render_with_lights_and_environment_hdr_image (renderer.rs:588-609)
 * With opts->aovs = 1 it also fills frame->albedo / frame->normal like
 * PathTracer::render_denoising_aovs (renderer.rs:121-129). */
gt_status gt_render(gt_scene* scene, const gt_lights* lights, const gt_environment* environment,
                    const gt_camera_desc* camera, const gt_render_opts* opts, gt_frame* frame);

/* Accumulation state of one frame across calls (resumable rendering): per pixel the
 * position in its sample stream, the running radiance sums and the accepted count —
 * what the reference's pixel loop keeps in locals (camera.rs:2660-2723).  No reference
 * counterpart: the reference's progressive rendering (PathTracer::render_progressive,
 * renderer.rs:136-146) reports tiles as they finish; this is the GPU form of pausing
 * and resuming a render, in memory or through a host checkpoint. */
typedef struct gt_accumulator gt_accumulator;

/* An empty accumulator for width x height pixels of the given precision (gt_precision). */
gt_status gt_accumulator_create(gt_context* ctx, uint32_t width, uint32_t height, uint32_t precision,
                                gt_accumulator** out);
void gt_accumulator_destroy(gt_accumulator* acc);
/* Samples per pixel accumulated so far. */
gt_status gt_accumulator_samples(const gt_accumulator* acc, uint32_t* samples);
/* Checkpoint: the state as an opaque host blob.  With host = NULL only *size is set. */
gt_status gt_accumulator_save(const gt_accumulator* acc, void* host, uint64_t capacity, uint64_t* size);
/* Restores a checkpoint made by gt_accumulator_save for the same size and precision. */
gt_status gt_accumulator_load(gt_accumulator* acc, const void* host, uint64_t size);

/* Renders `samples` more samples per pixel onto `acc` and writes the image of everything
 * accumulated into `frame`.  The camera must use random pixel sampling without adaptive
 * stopping (its samples_per_pixel is ignored) and keep the same rng_seed across calls;
 * the image after k calls equals one gt_render with the summed sample count.  The
 * precision is the accumulator's; opts.schedule PERSISTENT is not available here. */
gt_status gt_render_accumulate(gt_scene* scene, const gt_lights* lights, const gt_environment* environment,
                               const gt_camera_desc* camera, uint32_t samples, gt_accumulator* acc,
                               const gt_render_opts* opts, gt_frame* frame);

/* One frame of a batched render: its camera and its caller-owned outputs. */
typedef struct gt_frame_job {
    const gt_camera_desc* camera;
    gt_frame* frame;
} gt_frame_job;

/* Renders `count` frames of one scene — each with its own camera, pose, shutter, sample
 * count and adaptive settings — together: the per-frame loop a caller would write around
 * PathTracer::render_with_*_hdr_image (renderer.rs:101-117, 391-449) for an animation or
 * a camera sweep.  In f32 with schedule AUTO or WAVEFRONT, frames of one width run
 * through the striped wavefront as one image of their stacked rows (every slot rendered
 * with its frame's camera, graphs replayed, slow slots migrated, the tail finished in the
 * persistent kernel; no migration in a world with objects); in f64, with schedule
 * PERSISTENT, with frames of different widths, or for a scene with media, all pixels go
 * through one persistent launch.  Every frame's image and accepted
 * counts equal what gt_render gives for that frame alone (bit for bit in f64).  opts:
 * precision, schedule, tail_slots, stripes, stats (summed over the batch), profile,
 * progress and cancellation; `progress_rgb` is not written; `aovs` is GT_ERR_UNSUPPORTED. */
gt_status gt_render_batch(gt_scene* scene, const gt_lights* lights, const gt_environment* environment,
                          const gt_frame_job* jobs, uint32_t count, const gt_render_opts* opts);

/* Autotuner (no reference counterpart: the reference has no launch parameters to tune).
 * Renders the given jobs (count = 1: one gt_render of jobs[0]; count > 1: gt_render_batch)
 * under candidate settings and writes the fastest into *opts: wavefront stripes, tail
 * size, the wavefront kernels' blocks per SM and (schedule AUTO) slow-pixel migration on
 * or off, chosen one after another (coordinate descent), and last (schedule AUTO only) the
 * persistent schedule, which wins for small frames.  Each candidate is timed by the device time of its second render (the first
 * captures its graphs).  A candidate replaces the current best only when at least 1%
 * faster.  The jobs' frames receive the last render.  *opts supplies everything else
 * (precision; schedule AUTO or WAVEFRONT, and PERSISTENT, the outcome of an earlier tune, is
 * tuned as AUTO); report (optional) receives the trial count and the device times with the
 * given and the chosen options.  Launch shapes never change an image.  Choosing the
 * PERSISTENT schedule or another migration setting can change f32 pixels: other kernels
 * finish them and fuse f32 operations differently (f64 images and accepted-sample counts
 * stay identical).  The rng mode of *opts is kept. */
typedef struct gt_autotune_report {
    uint32_t struct_size;
    uint32_t trials;   /* renders timed */
    double given_ms;   /* device time with the options as given */
    double best_ms;    /* device time with the options written back */
} gt_autotune_report;

gt_status gt_autotune(gt_scene* scene, const gt_lights* lights, const gt_environment* environment,
                      const gt_frame_job* jobs, uint32_t count, gt_render_opts* opts, gt_autotune_report* report);

/* Closest-hit queries with traversal statistics on the reference-layout BVH in f64:
 * RayScene::hit (raytracing/scene.rs:1639-1657) and
 * RayScene::bvh_traversal_stats_for_rays (scene.rs:1478-1492).
 * rays: count * 7 doubles (origin xyz, direction xyz, time), host memory.
 * prim_ids[i] = primitive index or -1 on a miss; t may be NULL. */
gt_status gt_trace_rays(gt_scene* scene, const double* rays, uint32_t count, double t_min,
                        double t_max, int32_t* prim_ids, double* t, gt_bvh_stats* stats);

/* Primary probe rays RayCamera::ray_for_pixel (graphics/camera.rs:1641-1653) for every
 * `stride`-th pixel in x and y (the reference bench uses 4,
 * benches/render_performance.rs:42-50), traced as gt_trace_rays does with
 * Interval(0.001, inf).  prim_ids receives ceil(w/stride)*ceil(h/stride) entries in
 * row-major probe order. */
gt_status gt_trace_primary(gt_scene* scene, const gt_camera_desc* camera, uint32_t stride,
                           int32_t* prim_ids, double* t, gt_bvh_stats* stats);

/* The same closest-hit queries as gt_trace_rays (RayScene::hit, raytracing/scene.rs:
 * 1639-1657; the traversal of raytracing/bvh.rs:306-399) through the f32 walk the renderer
 * uses: the wide tree (gt_f32_tree) or the binary one, f32 primitive tests.  Rays whose
 * f32 decision may differ from f64 — a second candidate whose distance lies within the
 * two distances' estimated f32 errors of the closest, a hit point within a few dozen f32
 * ulps (scaled at grazing angles) of an edge, a distance near t_min — are re-traced by
 * the f64 walk; their ids are then the
 * reference's.  refined (may be NULL): per ray 0 = f32 result, 1 = re-traced (same
 * primitive), 2 = re-traced (the f64 walk chose another primitive).  report may be NULL. */
gt_status gt_trace_rays_f32(gt_scene* scene, const double* rays, uint32_t count, double t_min,
                            double t_max, int32_t* prim_ids, double* t, uint8_t* refined,
                            gt_trace_report* report);

/* gt_trace_primary's probe rays (f64 camera, RayCamera::ray_for_pixel, camera.rs:
 * 1641-1653) through gt_trace_rays_f32. */
gt_status gt_trace_primary_f32(gt_scene* scene, const gt_camera_desc* camera, uint32_t stride,
                               int32_t* prim_ids, double* t, uint8_t* refined, gt_trace_report* report);

/* ---------------------------------------------------------------- denoiser */

/* A learned denoiser over the AOVs of PathTracer::render_denoising_aovs
 * (renderer.rs:121-129; DenoisingAovs, camera.rs:491-526).  No reference counterpart: the
 * reference produces the AOVs and stops there.  The network is a 5-level U-Net of 3x3
 * convolutions (32/48/64/80/96 channels, ReLU, 2x2 average pooling, nearest upsampling
 * concatenated with the skip) from log(1 + beauty), albedo and normal to log(1 + radiance),
 * predicted as a residual over log(1 + beauty).  Weights and activations are BF16 with FP32
 * accumulation on the tensor cores; training keeps FP32 master weights and uses Adam on an
 * L1 loss in log(1 + x).
 *
 * Flat parameter layout (FP32), layer by layer: weights [cout][3][3][cin] then bias [cout].
 * Layers: enc0a 9->32, enc0b 32->32, then per level l = 1..4 enc(l)a c(l-1)->c(l), enc(l)b
 * c(l)->c(l); per level l = 3..0 dec(l)a c(l+1)+c(l)->c(l) (upsampled input first, then the
 * skip), dec(l)b c(l)->c(l); out 32->3 (no ReLU). */
typedef struct gt_denoiser gt_denoiser;

/* A network with seeded He-normal weights (the output layer scaled by 0.1) and zero biases. */
gt_status gt_denoiser_create(gt_context* ctx, uint64_t seed, gt_denoiser** out);
void gt_denoiser_destroy(gt_denoiser* denoiser);
gt_status gt_denoiser_param_count(const gt_denoiser* denoiser, uint64_t* count);
/* Copies the FP32 parameters to / from host memory (`count` must equal the network's).
 * Setting them resets the optimiser state. */
gt_status gt_denoiser_get_params(const gt_denoiser* denoiser, float* host, uint64_t count);
gt_status gt_denoiser_set_params(gt_denoiser* denoiser, const float* host, uint64_t count);

/* One training step on a batch of n images of h x w pixels (h, w multiples of 16).  All
 * image pointers are DEVICE memory, [n][h][w][3] floats: beauty (a low-sample render),
 * albedo and normal (may be NULL: zeros), target (a high-sample render).  Runs the forward
 * pass, the mean L1 loss on log(1 + max(x, 0)), the backward pass and, when lr > 0, one
 * Adam step (beta 0.9 / 0.999, eps 1e-8).  *loss (optional) receives the loss before the
 * step; grad (optional, host, param_count floats) the gradient in the flat layout. */
gt_status gt_denoiser_train_step(gt_denoiser* denoiser, const float* beauty, const float* albedo,
                                 const float* normal, const float* target, uint32_t n, uint32_t h,
                                 uint32_t w, float lr, float* loss, float* grad);

/* One frame to denoise.  Images are [height][width][3] floats, in host memory
 * (device_buffers = 0) or device memory (1). */
typedef struct gt_denoise_input {
    uint32_t struct_size;
    uint32_t width;
    uint32_t height;
    uint32_t device_buffers;
    const float* beauty;      /* the render: mean of all its samples (required)                  */
    const float* beauty_half; /* optional: mean of the first half of the same samples (the split
                                 buffer); enables the per-tile fallback                          */
    const float* albedo;      /* optional (zeros) */
    const float* normal;      /* optional (zeros) */
} gt_denoise_input;

/* Denoises one frame into `out` (same memory kind and shape as the beauty image).
 *
 * Per-tile fallback (split-buffer residual test): with beauty_half given, p = beauty and
 * a = beauty_half, each tile of tile x tile pixels (0 = 16) of N pixels compares, per
 * channel, the mean of the denoised tile m_d with the render's mean m_p.  The variance of
 * m_p is estimated from the split as v = sum((a - p)^2) / N^2.  When
 *     sum_c (m_d - m_p)^2 > threshold^2 * sum_c (v + (0.01 m_p)^2)
 * (the denoiser moved the tile's mean by more than `threshold` standard errors, 0 = 3.0,
 * with 1% of the mean as a floor) the tile keeps the plain render p.
 * tile_fallback (optional, host, ceil(h/tile) * ceil(w/tile) bytes, row-major) receives 1
 * for each tile that fell back; *fallback_count (optional) their number. */
gt_status gt_denoise(gt_denoiser* denoiser, const gt_denoise_input* input, uint32_t tile, float threshold,
                     float* out, uint8_t* tile_fallback, uint32_t* fallback_count);

/* Largest image gt_render_noalloc accepts (1024 x 1024 pixels). */
#define GT_NOALLOC_MAX_PIXELS 1048576u

/* Renders one f32 frame without allocating any memory.  It has no counterpart in the
 * reference; it exists for callers that cannot allocate device memory while they render:
 * a real-time loop that must not pay cudaMalloc's latency and synchronisation, a host
 * runtime whose own allocator owns all device memory, or code running where allocation
 * is not allowed.
 *
 * Same image as gt_render with GT_PRECISION_F32 and GT_SCHEDULE_PERSISTENT.  Its scratch
 * is one fixed array in the library's device code (about 20 MiB, enough for
 * GT_NOALLOC_MAX_PIXELS pixels); every GPU that loads the library holds that array until
 * the process exits.  Images larger than GT_NOALLOC_MAX_PIXELS return GT_ERR_INVALID_ARG.
 *
 * - rgb (width*height*3 floats, required) and accepted (width*height, optional) are
 *   DEVICE pointers on the context's device; the call returns when they are complete.
 * - The scene, lights and environment must already be resident on the device in f32:
 *   render them once with gt_render during set-up, otherwise GT_ERR_INVALID_ARG.
 * - The first call on a device looks up the array's device address (and may load the
 *   library's device code); make that first call during set-up, before any stream
 *   capture.
 * - All calls share the one array: calls whose work overlaps on the GPU (from different
 *   contexts on the same device) race and must be serialised by the caller.
 * - No progress callback, no cancellation, no statistics. */
gt_status gt_render_noalloc(gt_scene* scene, const gt_lights* lights, const gt_environment* environment,
                            const gt_camera_desc* camera, float* rgb, uint32_t* accepted);

#ifdef __cplusplus
}
#endif

#endif /* GARTUS_GPU_H */
