"""ctypes mirror of include/asuna_rt.h and the loader of the native library.

The structs below are byte-identical to the C ABI (and hence to the
reference's device ABI structs in src/shared/).  numpy dtypes are given for the
large arrays (vertices, path records) so they can be passed without copies.
"""
import ctypes as C
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "libasuna_rt.so")

# ---- status codes and enums (asuna_rt.h) -----------------------------------
ABI_VERSION = 2
OK, ERR_INVALID, ERR_CUDA, ERR_OOM, ERR_IO, ERR_PARSE, ERR_TIMEOUT, ERR_UNSUPPORTED, ERR_NO_DEVICE, ERR_BUSY, \
    ERR_TRAVERSAL = range(11)
CAMERA_PERSPECTIVE, CAMERA_OPENCV = 0, 1
LIGHT_DIRECTIONAL, LIGHT_RECT, LIGHT_TRIANGLE, LIGHT_POINT = 0, 1, 2, 3
MAT_LAMBERTIAN, MAT_EMISSIVE, MAT_PLASTIC, MAT_ROUGH_PLASTIC, MAT_MIRROR, MAT_DIELECTRIC = 0, 2, 4, 5, 8, 10
MAT_CONDUCTOR, MAT_ROUGH_CONDUCTOR, MAT_PHONG, MAT_PBR_METALNESS_ROUGHNESS, MAT_DISNEY, MAT_KANG18 = 6, 7, 11, 3, 9, 1
CH_DIFFUSE, CH_NORMAL, CH_SPECULAR, CH_TANGENT, CH_ROUGHNESS, CH_POSITION, CH_UV, CH_DEPTH = range(8)
SHOT_RR = 1
NUM_OUTPUT_IMAGES = 9
MAX_CHANNELS = 7

VERTEX_DTYPE = np.dtype([("pos", "<f4", 3), ("uv", "<f4", 2), ("normal", "<f4", 3), ("tangent", "<f4", 3)])
assert VERTEX_DTYPE.itemsize == 44
PATH_RECORD_DTYPE = np.dtype([("radiance", "<f4", 3), ("filter_weight", "<f4"), ("depth", "<u4"),
                              ("signature", "<u4"), ("events", "<u4"), ("shadows", "<u4")])
assert PATH_RECORD_DTYPE.itemsize == 32

f3 = C.c_float * 3


class Material(C.Structure):
    """GpuMaterial (src/shared/material.h:24-49)."""
    _fields_ = [("diffuse", f3), ("rho_spec", f3), ("aniso_alpha", C.c_float * 2), ("ior", C.c_float),
                ("roughness", C.c_float), ("subsurface", C.c_float), ("specular", C.c_float),
                ("specular_tint", C.c_float), ("anisotropic", C.c_float), ("sheen", C.c_float),
                ("sheen_tint", C.c_float), ("clearcoat", C.c_float), ("clearcoat_gloss", C.c_float),
                ("radiance", f3), ("metalness", C.c_float), ("radiance_factor", f3),
                ("diffuse_texture_id", C.c_int32), ("roughness_texture_id", C.c_int32),
                ("metalness_texture_id", C.c_int32), ("radiance_texture_id", C.c_int32),
                ("normal_texture_id", C.c_int32), ("tangent_texture_id", C.c_int32),
                ("opacity_texture_id", C.c_int32), ("type", C.c_uint32)]


class Light(C.Structure):
    """GpuLight (src/shared/light.h:16-25)."""
    _fields_ = [("type", C.c_int32), ("position", f3), ("direction", f3), ("radiance", f3), ("u", f3), ("v", f3),
                ("radius", C.c_float), ("area", C.c_float), ("double_side", C.c_uint32)]


class Camera(C.Structure):
    """GpuCamera (src/shared/camera.h:15-24), column-major matrices."""
    _fields_ = [("raster_to_camera", C.c_float * 16), ("camera_to_world", C.c_float * 16),
                ("env_transform", C.c_float * 16), ("fxfycxcy", C.c_float * 4), ("type", C.c_uint32),
                ("aperture", C.c_float), ("focal_distance", C.c_float), ("padding", C.c_float)]


class RtState(C.Structure):
    """GpuPushConstantRaytrace (src/shared/pushconstant.h:10-34)."""
    _fields_ = [("spp", C.c_int32), ("cur_frame", C.c_int32), ("max_path_depth", C.c_int32),
                ("num_lights", C.c_int32), ("bg_color", f3), ("use_face_normal", C.c_uint32),
                ("ignore_emissive", C.c_uint32), ("has_env_map", C.c_uint32),
                ("env_map_resolution", C.c_float * 2), ("env_map_intensity", C.c_float),
                ("n_multi_channel", C.c_uint32), ("diffuse_out_channel", C.c_int32),
                ("specular_out_channel", C.c_int32), ("roughness_out_channel", C.c_int32),
                ("normal_out_channel", C.c_int32), ("position_out_channel", C.c_int32),
                ("tangent_out_channel", C.c_int32), ("uv_out_channel", C.c_int32)]


class MeshDesc(C.Structure):
    _fields_ = [("num_vertices", C.c_uint32), ("num_triangles", C.c_uint32), ("vertices", C.c_void_p),
                ("indices", C.c_void_p)]


class InstanceDesc(C.Structure):
    _fields_ = [("transform", C.c_float * 12), ("mesh_id", C.c_uint32), ("material_id", C.c_int32),
                ("light_id", C.c_int32), ("reserved", C.c_uint32)]


class EnvmapDesc(C.Structure):
    _fields_ = [("width", C.c_uint32), ("height", C.c_uint32), ("rgba", C.c_void_p)]


class TextureDesc(C.Structure):
    _fields_ = [("width", C.c_uint32), ("height", C.c_uint32), ("rgba", C.c_void_p)]


class SunAndSky(C.Structure):
    """GpuSunAndSky (src/shared/sun_and_sky.h:6-27), 96 bytes."""
    _fields_ = [("rgb_unit_conversion", C.c_float * 3), ("multiplier", C.c_float), ("haze", C.c_float),
                ("redblueshift", C.c_float), ("saturation", C.c_float), ("horizon_height", C.c_float),
                ("ground_color", C.c_float * 3), ("horizon_blur", C.c_float), ("night_color", C.c_float * 3),
                ("sun_disk_intensity", C.c_float), ("sun_direction", C.c_float * 3), ("sun_disk_scale", C.c_float),
                ("sun_glow_intensity", C.c_float), ("y_is_up", C.c_int32), ("physically_scaled_sun", C.c_int32),
                ("in_use", C.c_int32)]


assert C.sizeof(SunAndSky) == 96


class SceneDesc(C.Structure):
    _fields_ = [("num_meshes", C.c_uint32), ("meshes", C.POINTER(MeshDesc)), ("num_instances", C.c_uint32),
                ("instances", C.POINTER(InstanceDesc)), ("num_materials", C.c_uint32),
                ("materials", C.POINTER(Material)), ("num_lights", C.c_uint32), ("lights", C.POINTER(Light)),
                ("envmap", EnvmapDesc), ("num_textures", C.c_uint32), ("textures", C.POINTER(TextureDesc)),
                ("sun_and_sky", C.POINTER(SunAndSky))]


class Shot(C.Structure):
    _fields_ = [("camera", Camera), ("state", RtState), ("width", C.c_uint32), ("height", C.c_uint32),
                ("frames", C.c_uint32), ("frame0", C.c_uint32), ("seed", C.c_uint32), ("flags", C.c_uint32),
                ("rr_depth", C.c_uint32), ("depth_out_channel", C.c_int32)]


class RenderStats(C.Structure):
    _fields_ = [("paths", C.c_uint64), ("extend_rays", C.c_uint64), ("shadow_rays", C.c_uint64),
                ("nodes_visited", C.c_uint64), ("tris_tested", C.c_uint64),
                ("shadow_nodes_visited", C.c_uint64), ("shadow_tris_tested", C.c_uint64), ("ms_total", C.c_double),
                ("ms_extend", C.c_double), ("ms_connect", C.c_double), ("ms_shade", C.c_double),
                ("extend_launches", C.c_uint64), ("connect_launches", C.c_uint64),
                ("kernel_launches", C.c_uint64), ("ms_sort", C.c_double)]


class PostState(C.Structure):
    """asuna_post_state = GpuPushConstantPost (src/shared/pushconstant.h:50-62)."""
    _fields_ = [("brightness", C.c_float), ("contrast", C.c_float), ("saturation", C.c_float),
                ("vignette", C.c_float), ("avg_lum", C.c_float), ("zoom", C.c_float),
                ("rendering_ratio", C.c_float * 2), ("auto_exposure", C.c_int32), ("y_white", C.c_float),
                ("key", C.c_float), ("tm_type", C.c_uint32)]


TONEMAP_NONE, TONEMAP_GAMMA, TONEMAP_REINHARD, TONEMAP_ACES, TONEMAP_FILMIC, TONEMAP_PBRT, TONEMAP_CUSTOM = range(7)


class DenoiserOpts(C.Structure):
    _fields_ = [("levels", C.c_uint32), ("channels", C.c_uint32 * 6), ("seed", C.c_uint64),
                ("max_pixels", C.c_uint64), ("training", C.c_uint32), ("tensor_memory", C.c_uint32),
                ("loss", C.c_uint32)]


DENOISER_LOSS_L1_LOG, DENOISER_LOSS_RELMSE = 0, 1


class SceneStats(C.Structure):
    _fields_ = [("triangles", C.c_uint64), ("instances", C.c_uint64), ("blas_nodes", C.c_uint64),
                ("tlas_nodes", C.c_uint64), ("device_bytes", C.c_uint64), ("build_ms", C.c_double)]


assert C.sizeof(Material) == 132 and C.sizeof(Light) == 76 and C.sizeof(Camera) == 224
assert C.sizeof(RtState) == 84 and C.sizeof(InstanceDesc) == 64

# (name, restype, argtypes) of every exported entry point of asuna_rt.h
P = C.c_void_p
SIGNATURES = [
    ("asuna_abi_version", C.c_int, []),
    ("asuna_last_error", C.c_char_p, []),
    ("asuna_ctx_create", C.c_int, [C.c_int, C.POINTER(P)]),
    ("asuna_ctx_destroy", C.c_int, [P]),
    ("asuna_ctx_sync", C.c_int, [P]),
    ("asuna_ctx_stream", P, [P]),
    ("asuna_ctx_set_counters", C.c_int, [P, C.c_int]),
    ("asuna_ctx_set_path_budget", C.c_int, [P, C.c_uint64]),
    ("asuna_ctx_set_launch", C.c_int, [P, C.c_int, C.c_int]),
    ("asuna_ctx_set_graphs", C.c_int, [P, C.c_int]),
    ("asuna_ctx_set_traversal", C.c_int, [P, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int]),
    ("asuna_ctx_set_ray_sort", C.c_int, [P, C.c_int]),
    ("asuna_ctx_set_traversal_stack", C.c_int, [P, C.c_int]),
    ("asuna_ctx_set_bvh_build", C.c_int, [P, C.c_int]),
    ("asuna_ctx_set_traversal_shape", C.c_int, [P, C.c_int, C.c_int]),
    ("asuna_ctx_set_traversal_occupancy", C.c_int, [P, C.c_int, C.c_int]),
    ("asuna_scene_create", C.c_int, [P, C.POINTER(SceneDesc), C.POINTER(P)]),
    ("asuna_sun_and_sky_default", None, [C.POINTER(SunAndSky)]),
    ("asuna_scene_validate", C.c_int, [C.POINTER(SceneDesc)]),
    ("asuna_scene_destroy", C.c_int, [P]),
    ("asuna_scene_get_stats", C.c_int, [P, C.POINTER(SceneStats)]),
    ("asuna_film_create", C.c_int, [P, C.c_uint32, C.c_uint32, C.POINTER(P)]),
    ("asuna_film_destroy", C.c_int, [P]),
    ("asuna_film_read", C.c_int, [P, P, C.c_int, P]),
    ("asuna_film_image", C.c_int, [P, C.c_int, C.POINTER(C.c_void_p)]),
    ("asuna_film_clear", C.c_int, [P, P]),
    ("asuna_render", C.c_int, [P, P, C.POINTER(Shot), P, C.POINTER(RenderStats)]),
    ("asuna_render_batch", C.c_int, [P, P, C.POINTER(Shot), C.POINTER(P), C.c_uint32, C.POINTER(RenderStats)]),
    ("asuna_render_paths", C.c_int, [P, P, C.POINTER(Shot), P, P]),
    ("asuna_scene_trace", C.c_int, [P, P, P, C.c_uint32, C.c_int, P, P]),
    ("asuna_json_load", C.c_int, [C.c_char_p, C.POINTER(P)]),
    ("asuna_json_load_string", C.c_int, [C.c_char_p, C.c_char_p, C.POINTER(P)]),
    ("asuna_json_free", C.c_int, [P]),
    ("asuna_json_scene_desc", C.c_int, [P, C.POINTER(SceneDesc)]),
    ("asuna_json_num_shots", C.c_int, [P, C.POINTER(C.c_uint32)]),
    ("asuna_json_get_shot", C.c_int, [P, C.c_uint32, C.POINTER(Shot)]),
    ("asuna_json_channels", C.c_int, [P, C.POINTER(C.c_uint32), P]),
    ("asuna_camera_perspective", C.c_int, [C.POINTER(C.c_float)] * 3 + [C.c_float, C.c_float, C.c_float,
                                                                        C.c_uint32, C.c_uint32,
                                                                        C.POINTER(Camera)]),
    ("asuna_camera_opencv", C.c_int, [C.POINTER(C.c_float)] * 4 + [C.POINTER(Camera)]),
    ("asuna_envmap_tables", C.c_int, [C.c_uint32, C.c_uint32, P, P, P]),
    ("asuna_diffuse_fresnel", C.c_float, [C.c_float, C.c_int]),
    ("asuna_complex_ior", C.c_int, [C.c_char_p, C.POINTER(C.c_float), C.POINTER(C.c_float)]),
    ("asuna_tracer_run_offline", C.c_int, [P, C.c_char_p, C.c_char_p]),
    ("asuna_tracer_run_offline_scanline", C.c_int, [P, C.c_char_p, C.c_char_p, C.c_int]),
    ("asuna_post_default", None, [C.POINTER(PostState)]),
    ("asuna_tonemap", C.c_int, [P, P, C.c_int, C.POINTER(PostState), P]),
    ("asuna_json_post_state", C.c_int, [P, C.POINTER(PostState)]),
    ("asuna_image_write", C.c_int, [C.c_char_p, C.c_uint32, C.c_uint32, P]),
    ("asuna_image_read", C.c_int, [C.c_char_p, C.POINTER(C.c_uint32), C.POINTER(C.c_uint32), P, C.c_uint64]),
    # include/asuna_denoise.h
    ("asuna_denoiser_create", C.c_int, [P, C.POINTER(DenoiserOpts), C.POINTER(P)]),
    ("asuna_denoiser_destroy", C.c_int, [P]),
    ("asuna_denoiser_num_params", C.c_uint64, [P]),
    ("asuna_denoiser_get_params", C.c_int, [P, P, C.c_uint64]),
    ("asuna_denoiser_set_params", C.c_int, [P, P, C.c_uint64]),
    ("asuna_denoiser_get_grads", C.c_int, [P, P, C.c_uint64]),
    ("asuna_denoiser_forward", C.c_int, [P, P, P, P, P, P, C.c_uint32, C.c_uint32, C.c_uint32, P]),
    ("asuna_denoiser_loss_grad", C.c_int, [P, P, P, P, P, P, P, C.c_uint32, C.c_uint32, C.c_uint32,
                                            C.POINTER(C.c_float)]),
    ("asuna_denoiser_adam", C.c_int, [P, C.c_float, C.c_float, C.c_float, C.c_float]),
    ("asuna_denoise", C.c_int, [P, P, P, C.c_int, C.c_int, P]),
    ("asuna_denoise_estimate", C.c_int, [P, P, P, P, C.c_int, C.c_int, P, C.POINTER(C.c_double),
                                          C.POINTER(C.c_double)]),
    ("asuna_denoise_combined", C.c_int, [P, P, P, P, C.c_int, C.c_int, P, C.POINTER(C.c_double),
                                          C.POINTER(C.c_double)]),
    ("asuna_denoise_blended", C.c_int, [P, P, P, P, C.c_int, C.c_int, P, C.POINTER(C.c_double), C.POINTER(C.c_double),
                                        C.POINTER(C.c_double)]),
    ("asuna_nn_conv3x3", C.c_int, [P, P, C.c_int, C.c_int, C.c_int, C.c_int, P, P, C.c_int, C.c_int, P, P,
                                    C.c_int]),
    ("asuna_nn_conv3x3_wgrad", C.c_int, [P, P, P, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, P]),
    ("asuna_nn_bias_grad", C.c_int, [P, P, C.c_int, C.c_int, P]),
    ("asuna_nn_flip_weights", C.c_int, [P, P, P, C.c_int, C.c_int]),
    ("asuna_nn_avgpool2", C.c_int, [P, P, P, C.c_int, C.c_int, C.c_int, C.c_int]),
    ("asuna_nn_avgpool2_bwd", C.c_int, [P, P, P, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int]),
    ("asuna_nn_upsample2", C.c_int, [P, P, P, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int]),
    ("asuna_nn_upsample2_bwd", C.c_int, [P, P, P, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int]),
    ("asuna_nn_copy_channels", C.c_int, [P, P, C.c_int, C.c_int, P, C.c_int, C.c_int, C.c_int, C.c_uint64,
                                          C.c_int]),
    ("asuna_nn_relu_mask", C.c_int, [P, P, P, C.c_uint64]),
    ("asuna_nn_weights_tc", C.c_int, [P, P, P, C.c_int, C.c_int]),
    ("asuna_nn_conv3x3_tc", C.c_int, [P, P, C.c_int, C.c_int, C.c_int, C.c_int, P, P, C.c_int, C.c_int, P, P,
                                       C.c_int]),
    ("asuna_nn_tc_status", C.c_int, [C.POINTER(C.c_int)]),
    ("asuna_nn_f32_to_bf16", C.c_int, [P, P, P, C.c_uint64]),
]


class AsunaError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"asuna error {code}: {msg}")
        self.code = code


_lib = None


def lib():
    """The loaded native library (built in-tree on first use if absent)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            from . import build as _build
            _build.build()
        L = C.CDLL(LIB_PATH)
        for name, res, args in SIGNATURES:
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        if L.asuna_abi_version() != ABI_VERSION:
            raise AsunaError(ERR_INVALID, "ABI version mismatch")
        _lib = L
    return _lib


def check(rc):
    if rc != OK:
        msg = lib().asuna_last_error()
        raise AsunaError(rc, msg.decode() if msg else "")
    return rc


def fptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_float))
