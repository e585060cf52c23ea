"""ctypes mirror of the POD structs and enums in include/gartus_gpu.h.

The layouts here must match the header byte for byte; tests/test_abi_layout.py checks
the sizes and offsets against a C compile of the header.
"""
from __future__ import annotations

import ctypes as C

GT_ABI_VERSION = 2

# gt_status
GT_OK = 0
GT_ERR_INVALID_ARG = 1
GT_ERR_OOM = 2
GT_ERR_CUDA = 3
GT_ERR_TIMEOUT = 4
GT_ERR_CANCELLED = 5
GT_ERR_UNSUPPORTED = 6
GT_ERR_NO_DEVICE = 7
GT_ERR_INTERNAL = 8
STATUS_NAMES = {
    0: "GT_OK", 1: "GT_ERR_INVALID_ARG", 2: "GT_ERR_OOM", 3: "GT_ERR_CUDA", 4: "GT_ERR_TIMEOUT",
    5: "GT_ERR_CANCELLED", 6: "GT_ERR_UNSUPPORTED", 7: "GT_ERR_NO_DEVICE", 8: "GT_ERR_INTERNAL",
}

# gt_geometry_kind
GT_GEOM_SPHERE = 0
GT_GEOM_MOVING_SPHERE = 1
GT_GEOM_TRIANGLE = 2
GT_GEOM_QUAD = 3

# gt_material_kind
GT_MAT_LAMBERTIAN = 0
GT_MAT_DIFFUSE_LIGHT = 1
GT_MAT_ISOTROPIC = 2
GT_MAT_GGX = 3
GT_MAT_METAL = 4
GT_MAT_DIELECTRIC = 5
GT_MAT_HENYEY_GREENSTEIN = 6

GT_BVH_REFERENCE_SAH = 0
GT_BVH_GPU_LBVH = 1
GT_F32_TREE_WIDE = 0
GT_F32_TREE_BINARY = 1

# gt_texture_kind
GT_TEX_SOLID = 0
GT_TEX_CHECKER = 1
GT_TEX_NOISE = 2
GT_TEX_IMAGE = 3
# gt_texture_filter / gt_texture_wrap
GT_FILTER_NEAREST = 0
GT_FILTER_LINEAR = 1
GT_WRAP_CLAMP = 0
GT_WRAP_REPEAT = 1
# gt_medium_shape / gt_medium_transform
GT_MEDIUM_SPHERE = 0
GT_MEDIUM_BOX = 1
GT_MEDIUM_ROTATE_Y = 1
GT_MEDIUM_TRANSLATE = 2
GT_NORMAL_MAP_NEGATIVE_Y = 1
# gt_noise_variant
GT_NOISE_PLAIN = 0
GT_NOISE_TURBULENCE = 1
GT_NOISE_MARBLE = 2

# gt_environment_format
GT_ENV_SRGB8 = 0
GT_ENV_RGB32F = 1

# gt_pixel_sample_mode
GT_SAMPLE_RANDOM = 0
GT_SAMPLE_STRATIFIED = 1
GT_SAMPLE_STRATIFIED_GRID = 2

# gt_direct_lighting_mode
GT_DIRECT_CURRENT_PATH_CONTINUATION = 0
GT_DIRECT_NEXT_EVENT_ESTIMATION = 1

# gt_background_kind
GT_BG_CONSTANT = 0
GT_BG_VERTICAL_GRADIENT = 1

# gt_precision
GT_PRECISION_F32 = 0
GT_PRECISION_F64 = 1


class gt_geometry(C.Structure):
    _fields_ = [("kind", C.c_uint32), ("reserved", C.c_uint32), ("p", C.c_double * 9)]


class gt_primitive(C.Structure):
    _fields_ = [("geometry", gt_geometry), ("material", C.c_uint32), ("reserved", C.c_uint32)]


class gt_material(C.Structure):
    _fields_ = [
        ("kind", C.c_uint32),
        ("texture_kind", C.c_uint32),
        ("color", C.c_double * 3),
        ("param", C.c_double),
        ("tex", C.c_double * 7),
        ("normal_map", C.c_uint32),
        ("normal_map_flags", C.c_uint32),
        ("normal_map_strength", C.c_double),
    ]


class gt_image(C.Structure):
    _fields_ = [
        ("width", C.c_uint32),
        ("height", C.c_uint32),
        ("rgb", C.c_void_p),
        ("filter", C.c_uint32),
        ("wrap_s", C.c_uint32),
        ("wrap_t", C.c_uint32),
        ("reserved", C.c_uint32),
    ]


class gt_medium(C.Structure):
    _fields_ = [
        ("shape", C.c_uint32),
        ("material", C.c_uint32),
        ("p", C.c_double * 6),
        ("rotate_y", C.c_double),
        ("translate", C.c_double * 3),
        ("density", C.c_double),
        ("transform", C.c_uint32),
        ("reserved", C.c_uint32),
    ]


class gt_mesh(C.Structure):
    _fields_ = [
        ("num_primitives", C.c_uint32),
        ("bvh_leaf_size", C.c_uint32),
        ("primitives", C.c_void_p),
        ("texcoords", C.c_void_p),
        ("normals", C.c_void_p),
        ("attribute_flags", C.c_void_p),
    ]


class gt_object(C.Structure):
    _fields_ = [
        ("mesh", C.c_uint32),
        ("transformed", C.c_uint32),
        ("transform", C.c_double * 16),
        ("inverse", C.c_double * 16),
    ]


class gt_scene_desc(C.Structure):
    _fields_ = [
        ("struct_size", C.c_uint32),
        ("num_primitives", C.c_uint32),
        ("primitives", C.POINTER(gt_primitive)),
        ("num_materials", C.c_uint32),
        ("bvh_leaf_size", C.c_uint32),
        ("materials", C.POINTER(gt_material)),
        ("bvh_builder", C.c_uint32),
        ("num_images", C.c_uint32),
        ("images", C.POINTER(gt_image)),
        ("num_media", C.c_uint32),
        ("num_meshes", C.c_uint32),
        ("media", C.POINTER(gt_medium)),
        ("meshes", C.POINTER(gt_mesh)),
        ("num_objects", C.c_uint32),
        ("f32_tree", C.c_uint32),
        ("objects", C.POINTER(gt_object)),
    ]


class gt_light_target(C.Structure):
    _fields_ = [("geometry", gt_geometry), ("weight", C.c_double)]


class gt_environment_desc(C.Structure):
    _fields_ = [
        ("struct_size", C.c_uint32),
        ("format", C.c_uint32),
        ("width", C.c_uint32),
        ("height", C.c_uint32),
        ("texels", C.c_void_p),
    ]


class gt_camera_desc(C.Structure):
    _fields_ = [
        ("struct_size", C.c_uint32),
        ("image_width", C.c_uint32),
        ("aspect_ratio", C.c_double),
        ("samples_per_pixel", C.c_uint32),
        ("pixel_sample_mode", C.c_uint32),
        ("grid_width", C.c_uint32),
        ("adaptive", C.c_uint32),
        ("adaptive_min_samples", C.c_uint32),
        ("adaptive_max_samples", C.c_uint32),
        ("adaptive_error_threshold", C.c_double),
        ("direct_lighting_mode", C.c_uint32),
        ("max_depth", C.c_uint32),
        ("light_pdf_weight", C.c_double),
        ("russian_roulette_min_depth", C.c_int32),
        ("reserved0", C.c_uint32),
        ("rng_seed", C.c_uint64),
        ("vertical_fov", C.c_double),
        ("lookfrom", C.c_double * 3),
        ("lookat", C.c_double * 3),
        ("view_up", C.c_double * 3),
        ("defocus_angle", C.c_double),
        ("focus_distance", C.c_double),
        ("shutter_start", C.c_double),
        ("shutter_end", C.c_double),
        ("background_kind", C.c_uint32),
        ("reserved1", C.c_uint32),
        ("background", C.c_double * 9),
    ]


GT_PROGRESS_FN = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_uint64, C.c_uint64)

GT_NOALLOC_MAX_PIXELS = 1048576

# gt_schedule
GT_SCHEDULE_AUTO = 0
GT_SCHEDULE_WAVEFRONT = 1
GT_SCHEDULE_PERSISTENT = 2
GT_MIGRATE_DEFAULT = 0
GT_MIGRATE_ON = 1
GT_MIGRATE_OFF = 2
GT_RNG_PIXEL = 0
GT_RNG_SUBSTREAMS = 1

# gt_kernel_id
GT_KERNEL_GENERATE = 0
GT_KERNEL_TRACE = 1
GT_KERNEL_SHADE = 2
GT_KERNEL_SHADOW = 3
GT_KERNEL_OTHER = 4
GT_KERNEL_PERSISTENT = 5
GT_KERNEL_COUNT = 6
KERNEL_NAMES = ["generate", "trace", "shade", "shadow", "other", "persistent"]


class gt_render_stats(C.Structure):
    _fields_ = [
        ("gpu_ms", C.c_double),
        ("iterations", C.c_uint64),
        ("rays", C.c_uint64),
        ("shadow_rays", C.c_uint64),
        ("samples", C.c_uint64),
        ("samples_started", C.c_uint64),
        ("kernel_ms", C.c_double * GT_KERNEL_COUNT),
        ("kernel_launches", C.c_uint64 * GT_KERNEL_COUNT),
        ("migrated_pixels", C.c_uint64),
        ("tail_pixels", C.c_uint64),
        ("persistent_rays", C.c_uint64),
    ]

    def as_dict(self) -> dict:
        return {
            "gpu_ms": self.gpu_ms, "iterations": self.iterations, "rays": self.rays,
            "shadow_rays": self.shadow_rays, "samples": self.samples, "samples_started": self.samples_started,
            "kernel_ms": {KERNEL_NAMES[i]: self.kernel_ms[i] for i in range(GT_KERNEL_COUNT)},
            "kernel_launches": {KERNEL_NAMES[i]: int(self.kernel_launches[i]) for i in range(GT_KERNEL_COUNT)},
            "migrated_pixels": int(self.migrated_pixels), "tail_pixels": int(self.tail_pixels),
            "persistent_rays": int(self.persistent_rays),
        }


class gt_render_opts(C.Structure):
    _fields_ = [
        ("struct_size", C.c_uint32),
        ("precision", C.c_uint32),
        ("aovs", C.c_uint32),
        ("profile", C.c_uint32),
        ("progress", GT_PROGRESS_FN),
        ("progress_user", C.c_void_p),
        ("stats", C.POINTER(gt_render_stats)),
        ("schedule", C.c_uint32),
        ("tail_slots", C.c_uint32),
        ("stripes", C.c_uint32),
        ("progress_rgb", C.c_void_p),
        ("generate_blocks_per_sm", C.c_uint32),
        ("trace_blocks_per_sm", C.c_uint32),
        ("migrate", C.c_uint32),
        ("rng", C.c_uint32),
    ]


class gt_frame(C.Structure):
    _fields_ = [
        ("struct_size", C.c_uint32),
        ("width", C.c_uint32),
        ("height", C.c_uint32),
        ("device_buffers", C.c_uint32),
        ("rgb", C.c_void_p),
        ("albedo", C.c_void_p),
        ("normal", C.c_void_p),
        ("rgb64", C.c_void_p),
        ("accepted", C.c_void_p),
    ]


class gt_frame_job(C.Structure):
    _fields_ = [("camera", C.POINTER(gt_camera_desc)), ("frame", C.POINTER(gt_frame))]


class gt_bvh_stats(C.Structure):
    _fields_ = [
        ("rays", C.c_uint64),
        ("node_bounds_tests", C.c_uint64),
        ("node_bounds_hits", C.c_uint64),
        ("leaf_visits", C.c_uint64),
        ("primitive_candidates", C.c_uint64),
        ("leaf_hit_results", C.c_uint64),
        ("max_stack_depth", C.c_uint64),
    ]

    def as_dict(self) -> dict:
        return {name: int(getattr(self, name)) for name, _ in self._fields_}


class gt_trace_report(C.Structure):
    _fields_ = [
        ("struct_size", C.c_uint32),
        ("tree", C.c_uint32),
        ("rays", C.c_uint64),
        ("refined", C.c_uint64),
        ("changed", C.c_uint64),
        ("wide_nodes", C.c_uint32),
        ("wide_depth", C.c_uint32),
    ]

    def as_dict(self) -> dict:
        return {name: int(getattr(self, name)) for name, _ in self._fields_ if name != "struct_size"}


class gt_autotune_report(C.Structure):
    _fields_ = [
        ("struct_size", C.c_uint32),
        ("trials", C.c_uint32),
        ("given_ms", C.c_double),
        ("best_ms", C.c_double),
    ]


class gt_denoise_input(C.Structure):
    _fields_ = [
        ("struct_size", C.c_uint32),
        ("width", C.c_uint32),
        ("height", C.c_uint32),
        ("device_buffers", C.c_uint32),
        ("beauty", C.c_void_p),
        ("beauty_half", C.c_void_p),
        ("albedo", C.c_void_p),
        ("normal", C.c_void_p),
    ]


STRUCTS = [
    gt_geometry, gt_primitive, gt_material, gt_image, gt_medium, gt_mesh, gt_object, gt_scene_desc, gt_light_target, gt_environment_desc,
    gt_camera_desc, gt_render_opts, gt_frame, gt_frame_job, gt_bvh_stats, gt_render_stats, gt_denoise_input,
    gt_autotune_report, gt_trace_report,
]
