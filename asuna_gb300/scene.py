"""Scene assembly and the render context (Python mirror of the C ABI).

``SceneBuilder`` assembles the device-ABI arrays the way the reference's
``Scene`` class does (src/scene/scene.cpp:87-316): material 0 and light 0 are
the reference's dummies, rect lights become two-triangle emitter instances,
triangle (mesh-facet) lights one-triangle emitter instances.  ``Context`` owns
one CUDA device + stream of the native library; scenes, films and renders go
through the C ABI in include/asuna_rt.h.
"""
import contextlib
import ctypes as C

import numpy as np

from . import _abi as A
from ._abi import check, lib


def default_material():
    """Material() of src/core/material.h:9-35."""
    m = A.Material()
    m.ior = 1.5
    m.roughness = 0.5
    m.radiance_factor = A.f3(1.0, 1.0, 1.0)
    for f in ("diffuse", "radiance", "metalness", "normal", "roughness", "tangent", "opacity"):
        setattr(m, f + "_texture_id", -1)
    m.type = A.MAT_LAMBERTIAN
    return m


def default_post(tm_type=None):
    """PipelineState's post-pass defaults (src/core/state.h:46-58)."""
    p = A.PostState()
    lib().asuna_post_default(C.byref(p))
    if tm_type is not None:
        p.tm_type = tm_type
    return p


def default_state():
    """State() of src/core/state.h:15-63 (ray-tracing part)."""
    s = A.RtState()
    s.cur_frame = -1
    s.spp = 1
    s.max_path_depth = 3
    s.env_map_intensity = 1.0
    for f in ("diffuse", "specular", "roughness", "normal", "position", "tangent", "uv"):
        setattr(s, f + "_out_channel", -1)
    return s


CHANNEL_NAMES = {"diffuse": A.CH_DIFFUSE, "albedo": A.CH_DIFFUSE, "normal": A.CH_NORMAL,
                 "specular": A.CH_SPECULAR, "tangent": A.CH_TANGENT, "roughness": A.CH_ROUGHNESS,
                 "position": A.CH_POSITION, "uv": A.CH_UV, "depth": A.CH_DEPTH}
_FIELD = {A.CH_DIFFUSE: "diffuse", A.CH_NORMAL: "normal", A.CH_SPECULAR: "specular", A.CH_TANGENT: "tangent",
          A.CH_ROUGHNESS: "roughness", A.CH_POSITION: "position", A.CH_UV: "uv"}


def set_channels(state, names):
    """multi_channel list -> out-channel slots (src/loader/loader.cpp:163-185).
    Returns the slot of the depth channel (an addition; -1 if absent)."""
    if len(names) > A.MAX_CHANNELS:
        raise ValueError(f"channel numbers can not exceed {A.MAX_CHANNELS}")
    state.n_multi_channel = len(names)
    depth = -1
    for i, n in enumerate(names):
        kind = CHANNEL_NAMES[n]
        if kind == A.CH_DEPTH:
            depth = i
        else:
            setattr(state, _FIELD[kind] + "_out_channel", i)
    return depth


class _LibraryHelpers:
    """Host preprocessing of a scene description through the library: the
    diffuse-Fresnel integral of the plastics' substrate and the perspective
    camera's matrices."""

    @staticmethod
    def diffuse_fresnel(ior):
        return lib().asuna_diffuse_fresnel(C.c_float(ior), 1000)

    @staticmethod
    def camera_perspective(e, l, u, fov, aperture, focal_distance, width, height, cam):
        check(lib().asuna_camera_perspective(A.fptr(e), A.fptr(l), A.fptr(u), fov, aperture, focal_distance, width,
                                             height, C.byref(cam)))


_helpers = _LibraryHelpers()


def _default_sky(s):
    """Scene::reset's sun & sky (src/scene/scene.cpp:112-129); equal to the
    library's asuna_sun_and_sky_default (tested), set here so scene
    descriptions build without the library."""
    s.rgb_unit_conversion = (C.c_float * 3)(1, 1, 1)
    s.multiplier = 0.0000101320
    s.haze, s.redblueshift, s.saturation, s.horizon_height = 0.0, 0.0, 1.0, 0.0
    s.ground_color = (C.c_float * 3)(0.4, 0.4, 0.4)
    s.horizon_blur = 0.1
    s.night_color = (C.c_float * 3)(0.0, 0.0, 0.01)
    s.sun_disk_intensity = 0.8
    s.sun_direction = (C.c_float * 3)(0.00, 0.78, 0.62)
    s.sun_disk_scale, s.sun_glow_intensity = 5.0, 1.0
    s.y_is_up, s.physically_scaled_sun, s.in_use = 1, 1, 0


@contextlib.contextmanager
def host_helpers(provider):
    """Builds scene descriptions with another provider of the host
    preprocessing (an object with diffuse_fresnel and camera_perspective like
    _LibraryHelpers), e.g. for a process that must not load the library."""
    global _helpers
    old, _helpers = _helpers, provider
    try:
        yield
    finally:
        _helpers = old


def _length(v):
    # float32 length as the reference's host code computes it (no BLAS reduction)
    v = np.asarray(v, np.float32)
    return np.sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2], dtype=np.float32)


def _identity34():
    return np.array([[1, 0, 0, 0], [0, 1, 0, 0], [0, 0, 1, 0]], np.float32)


class SceneBuilder:
    """Host scene in the reference's device-ABI form."""

    def __init__(self):
        self.meshes = []  # (vertices[VERTEX_DTYPE], indices uint32 [3n])
        self.mesh_names = []
        self.materials = [default_material()]
        self.material_names = ["add_by_default_dummy_material"]
        self.lights = []
        self.instances = []  # (transform 3x4, mesh, material, light)
        self.env = None
        self.sky = None
        # textures[0] is the reference's dummy texture (src/scene/scene.cpp:87-130)
        self.textures = [np.zeros((1, 1, 4), np.float32)]
        self.texture_names = ["add_by_default_dummy_texture"]
        dummy = A.Light()
        dummy.type = A.LIGHT_DIRECTIONAL
        dummy.double_side = 1
        self.lights.append(dummy)

    # -- textures (src/loader/loader.cpp:334-347; decoded RGBA32F) --
    def add_texture(self, name, rgba):
        """An [h, w, 3|4] float image (row 0 = v 0); returns its texture id
        for the materials' *_texture_id fields."""
        a = np.asarray(rgba, np.float32)
        if a.ndim != 3 or a.shape[2] not in (3, 4):
            raise ValueError("texture must be [h, w, 3] or [h, w, 4]")
        if a.shape[2] == 3:
            a = np.concatenate([a, np.ones(a.shape[:2] + (1,), np.float32)], 2)
        if name in self.texture_names:
            raise ValueError(f"texture [{name}] defined twice")
        self.textures.append(np.ascontiguousarray(a))
        self.texture_names.append(name)
        return len(self.textures) - 1

    # -- materials (src/loader/material.cpp:104-231) --
    def add_lambertian(self, name, diffuse):
        m = default_material()
        m.type = A.MAT_LAMBERTIAN
        m.diffuse = A.f3(*diffuse)
        return self._add_material(name, m)

    def add_rough_plastic(self, name, diffuse, alpha, ior=1.5):
        m = default_material()
        m.type = A.MAT_ROUGH_PLASTIC
        m.diffuse = A.f3(*diffuse)
        m.aniso_alpha = (C.c_float * 2)(*alpha)
        m.ior = ior
        m.radiance[0] = _helpers.diffuse_fresnel(ior)
        return self._add_material(name, m)

    def add_plastic(self, name, diffuse, ior=1.5):
        """brdf_plastic (src/loader/material.cpp:197-210): smooth coating over a diffuse base."""
        m = default_material()
        m.type = A.MAT_PLASTIC
        m.diffuse = A.f3(*diffuse)
        m.ior = ior
        m.radiance[0] = _helpers.diffuse_fresnel(ior)
        return self._add_material(name, m)

    def add_mirror(self, name, reflectance=(1.0, 1.0, 1.0)):
        """brdf_mirror (src/loader/material.cpp:233-243)."""
        m = default_material()
        m.type = A.MAT_MIRROR
        m.diffuse = A.f3(*reflectance)
        return self._add_material(name, m)

    def add_conductor(self, name, metal="Cu", reflectance=(0.0, 0.0, 0.0), alpha=None):
        """brdf_conductor, or brdf_rough_conductor with `alpha` (src/loader/material.cpp:306-347):
        the complex index of refraction of the named metal in radiance / radiance_factor.
        The reflectance scale defaults to the reference's default albedo, 0
        (a scene file without diffuse_reflectance renders the metal black)."""
        m = default_material()
        m.type = A.MAT_CONDUCTOR if alpha is None else A.MAT_ROUGH_CONDUCTOR
        m.diffuse = A.f3(*reflectance)
        check(lib().asuna_complex_ior(metal.encode(), m.radiance, m.radiance_factor))
        if alpha is not None:
            m.aniso_alpha = (C.c_float * 2)(*alpha)
        return self._add_material(name, m)

    def add_phong(self, name, diffuse, specular, shininess):
        """brdf_phong (src/loader/material.cpp:391-405): a Lambertian lobe and a
        normalised Phong lobe (reflectance `specular`, exponent `shininess`),
        mixed by the luminances of the two reflectances."""
        m = default_material()
        m.type = A.MAT_PHONG
        m.diffuse = A.f3(*diffuse)
        m.rho_spec = A.f3(*specular)
        m.specular = float(shininess)
        return self._add_material(name, m)

    def add_pbr(self, name, albedo, metalness=0.0, roughness=0.5, ior=1.5):
        """brdf_pbr_metalness_roughness (src/loader/material.cpp:116-143):
        GGX specular with Schlick Fresnel (f0 from ior, tinted by albedo with
        metalness) over a Lambertian base weighted by 1 - metalness."""
        m = default_material()
        m.type = A.MAT_PBR_METALNESS_ROUGHNESS
        m.diffuse = A.f3(*albedo)
        m.metalness = float(metalness)
        m.roughness = float(roughness)
        m.ior = float(ior)
        return self._add_material(name, m)

    def add_disney(self, name, base_color, metallic=0.0, roughness=0.5, subsurface=0.0, specular_tint=0.0,
                   sheen=0.0, sheen_tint=0.0, clearcoat=0.0, clearcoat_gloss=0.0, anisotropic=0.0, ior=1.5):
        """brdf_disney (src/loader/material.cpp:359-389; the JSON path sets
        base colour, metallic and roughness, the others stay 0): diffuse with
        retro-reflection, fake subsurface and sheen, anisotropic GGX
        specular and a GTR1 clearcoat."""
        m = default_material()
        m.type = A.MAT_DISNEY
        m.diffuse = A.f3(*base_color)
        m.metalness = float(metallic)
        m.roughness = float(roughness)
        m.subsurface = float(subsurface)
        m.specular_tint = float(specular_tint)
        m.sheen = float(sheen)
        m.sheen_tint = float(sheen_tint)
        m.clearcoat = float(clearcoat)
        m.clearcoat_gloss = float(clearcoat_gloss)
        m.anisotropic = float(anisotropic)
        m.ior = float(ior)
        return self._add_material(name, m)

    def add_kang18(self, name, diffuse, specular, alpha, ior=1.5):
        """brdf_kang18 (src/loader/material.cpp:156-187): anisotropic GGX
        (alpha = (ax, ay)) with Schlick Fresnel over a Lambertian base; the
        shading frame is rebuilt from the normal and the tangent."""
        m = default_material()
        m.type = A.MAT_KANG18
        m.diffuse = A.f3(*diffuse)
        m.rho_spec = A.f3(*specular)
        m.aniso_alpha = (C.c_float * 2)(*alpha)
        m.ior = float(ior)
        return self._add_material(name, m)

    def add_dielectric(self, name, ior=1.5):
        m = default_material()
        m.type = A.MAT_DIELECTRIC
        m.ior = ior
        return self._add_material(name, m)

    def add_emissive(self, name, radiance, radiance_factor=(1.0, 1.0, 1.0)):
        m = default_material()
        m.type = A.MAT_EMISSIVE
        m.radiance = A.f3(*radiance)
        m.radiance_factor = A.f3(*radiance_factor)
        return self._add_material(name, m)

    def _add_material(self, name, m):
        if name in self.material_names:
            raise ValueError(f"material [{name}] defined twice")
        self.material_names.append(name)
        self.materials.append(m)
        return len(self.materials) - 1

    # -- meshes / instances --
    def add_mesh(self, name, vertices, indices):
        v = np.ascontiguousarray(vertices, dtype=A.VERTEX_DTYPE)
        i = np.ascontiguousarray(indices, dtype=np.uint32).reshape(-1)
        if i.size % 3:
            raise ValueError("indices must hold whole triangles")
        self.meshes.append((v, i))
        self.mesh_names.append(name)
        return len(self.meshes) - 1

    def add_instance(self, mesh, material, transform=None):
        m = self.mesh_names.index(mesh) if isinstance(mesh, str) else int(mesh)
        mat = self.material_names.index(material) if isinstance(material, str) else int(material)
        t = _identity34() if transform is None else np.asarray(transform, np.float32).reshape(3, 4)
        self.instances.append((t, m, mat, -1))
        return len(self.instances) - 1

    # -- lights (src/scene/scene.cpp:220-283, src/loader/loader.cpp:270-332) --
    def add_rect_light(self, position, v1, v2, radiance, double_side=False, triangle=False):
        """JSON "rect" / "triangle" light: LightTypeRect, half area for "triangle"."""
        p = np.asarray(position, np.float32)
        u = np.asarray(v1, np.float32) - p
        v = np.asarray(v2, np.float32) - p
        l = A.Light()
        l.type = A.LIGHT_RECT
        l.position = A.f3(*p)
        l.u = A.f3(*u)
        l.v = A.f3(*v)
        l.radiance = A.f3(*radiance)
        area = np.float32(_length(np.cross(u, v)))
        l.area = area * np.float32(0.5) if triangle else area
        l.double_side = 1 if double_side else 0
        light_id = len(self.lights)
        verts = np.zeros(4, A.VERTEX_DTYPE)
        verts["pos"] = [p, p + u, p + u + v, p + v]
        self.meshes.append((verts, np.array([0, 1, 2, 0, 2, 3], np.uint32)))
        self.mesh_names.append(f"__rectLight:{light_id}")
        self.instances.append((_identity34(), len(self.meshes) - 1, 0, light_id))
        self.lights.append(l)
        return light_id

    def add_triangle_light(self, p0, p1, p2, radiance):
        """One facet of a JSON "mesh" light: LightTypeTriangle, single sided."""
        p0 = np.asarray(p0, np.float32)
        u = np.asarray(p1, np.float32) - p0
        v = np.asarray(p2, np.float32) - p0
        l = A.Light()
        l.type = A.LIGHT_TRIANGLE
        l.position = A.f3(*p0)
        l.u = A.f3(*u)
        l.v = A.f3(*v)
        l.radiance = A.f3(*radiance)
        l.area = np.float32(_length(np.cross(u, v))) * np.float32(0.5)
        light_id = len(self.lights)
        verts = np.zeros(3, A.VERTEX_DTYPE)
        verts["pos"] = [p0, p0 + u, p0 + v]
        self.meshes.append((verts, np.array([0, 1, 2], np.uint32)))
        self.mesh_names.append(f"__meshLight:{light_id}")
        self.instances.append((_identity34(), len(self.meshes) - 1, 0, light_id))
        self.lights.append(l)
        return light_id

    def add_point_light(self, position, radiance):
        l = A.Light()
        l.type = A.LIGHT_POINT
        l.position = A.f3(*position)
        l.radiance = A.f3(*radiance)
        self.lights.append(l)
        return len(self.lights) - 1

    def add_distant_light(self, direction, radiance):
        l = A.Light()
        l.type = A.LIGHT_DIRECTIONAL
        l.direction = A.f3(*direction)
        l.radiance = A.f3(*radiance)
        self.lights.append(l)
        return len(self.lights) - 1

    def set_envmap(self, rgba):
        rgba = np.ascontiguousarray(rgba, np.float32)
        if rgba.ndim != 3 or rgba.shape[2] not in (3, 4):
            raise ValueError("envmap must be HxWx3 or HxWx4")
        if rgba.shape[2] == 3:
            rgba = np.concatenate([rgba, np.ones(rgba.shape[:2] + (1,), np.float32)], axis=2)
        self.env = np.ascontiguousarray(rgba)

    def set_sun_and_sky(self, **fields):
        """Turns the sun & sky environment on (GpuSunAndSky, in_use = 1):
        the reference's defaults (Scene::reset, scene.cpp:112-129) with the
        given fields replaced, e.g. sun_direction=(0.3, 0.8, 0.5)."""
        s = A.SunAndSky()
        _default_sky(s)
        for k, v in fields.items():
            f = getattr(s, k)
            if hasattr(f, "__len__"):
                setattr(s, k, type(f)(*v))
            else:
                setattr(s, k, v)
        s.in_use = 1
        self.sky = s
        return s

    @property
    def num_lights(self):
        return len(self.lights) - 1  # Scene::submit, scene.cpp:33

    def state(self, spp=1, max_path_depth=3, channels=(), bg_color=(0, 0, 0), env_intensity=1.0):
        s = default_state()
        s.spp = spp
        s.max_path_depth = max_path_depth
        s.num_lights = self.num_lights
        s.bg_color = A.f3(*bg_color)
        s.env_map_intensity = env_intensity
        if self.env is not None:
            s.has_env_map = 1
            s.env_map_resolution = (C.c_float * 2)(self.env.shape[1], self.env.shape[0])
        depth = set_channels(s, list(channels))
        return s, depth

    def desc(self):
        return SceneDescHandle(self)


class SceneDescHandle:
    """An asuna_scene_desc whose arrays stay alive with this object."""

    def __init__(self, b):
        self._keep = []
        nm = len(b.meshes)
        self.meshes = (A.MeshDesc * max(nm, 1))()
        for k, (v, i) in enumerate(b.meshes):
            self.meshes[k] = A.MeshDesc(len(v), i.size // 3, v.ctypes.data, i.ctypes.data)
            self._keep += [v, i]
        ni = len(b.instances)
        self.instances = (A.InstanceDesc * max(ni, 1))()
        for k, (t, m, mat, light) in enumerate(b.instances):
            d = self.instances[k]
            d.transform = (C.c_float * 12)(*np.asarray(t, np.float32).reshape(-1))
            d.mesh_id = m
            d.material_id = mat
            d.light_id = light
        self.materials = (A.Material * len(b.materials))(*b.materials)
        self.lights = (A.Light * len(b.lights))(*b.lights)
        d = A.SceneDesc()
        d.num_meshes = nm
        d.meshes = self.meshes
        d.num_instances = ni
        d.instances = self.instances
        d.num_materials = len(b.materials)
        d.materials = self.materials
        d.num_lights = len(b.lights)
        d.lights = self.lights
        if b.env is not None:
            d.envmap.width = b.env.shape[1]
            d.envmap.height = b.env.shape[0]
            d.envmap.rgba = b.env.ctypes.data
            self._keep.append(b.env)
        self.textures = (A.TextureDesc * len(b.textures))()
        for k, t in enumerate(b.textures):
            self.textures[k] = A.TextureDesc(t.shape[1], t.shape[0], t.ctypes.data)
            self._keep.append(t)
        d.num_textures = len(b.textures)
        d.textures = self.textures
        if b.sky is not None:
            self.sky = A.SunAndSky.from_buffer_copy(b.sky)
            d.sun_and_sky = C.pointer(self.sky)
        self.desc = d

    @property
    def ptr(self):
        return C.byref(self.desc)


def perspective_camera(eye, lookat, up, fov, width, height, aperture=0.0, focal_distance=0.1):
    """GpuCamera of CameraPerspective::toGpuStruct (src/core/camera.cpp:87-99);
    fov in degrees is horizontal."""
    cam = A.Camera()
    e, l, u = (np.asarray(x, np.float32) for x in (eye, lookat, up))
    _helpers.camera_perspective(e, l, u, fov, aperture, focal_distance, width, height, cam)
    return cam


def opencv_camera(eye, lookat, up, fxfycxcy):
    cam = A.Camera()
    e, l, u, f = (np.asarray(x, np.float32) for x in (eye, lookat, up, fxfycxcy))
    check(lib().asuna_camera_opencv(A.fptr(e), A.fptr(l), A.fptr(u), A.fptr(f), C.byref(cam)))
    return cam


def make_shot(camera, state, width, height, frames, frame0=0, seed=0, depth_channel=-1, rr_depth=None):
    s = A.Shot()
    s.camera = camera
    s.state = state
    s.width, s.height = width, height
    s.frames = frames
    s.frame0 = frame0
    s.seed = seed
    s.depth_out_channel = depth_channel
    if rr_depth is not None:
        s.flags |= A.SHOT_RR
        s.rr_depth = rr_depth
    return s


class Film:
    def __init__(self, ctx, width, height):
        self.ctx = ctx
        self.width, self.height = width, height
        h = C.c_void_p()
        check(lib().asuna_film_create(ctx.handle, width, height, C.byref(h)))
        self.handle = h

    def read(self, image=0, out=None):
        if out is None:
            out = np.empty((self.height, self.width, 4), np.float32)
        check(lib().asuna_film_read(self.ctx.handle, self.handle, image, out.ctypes.data))
        return out

    def tensor(self, image=0):
        """Film image `image` as a CUDA [h, w, 4] float32 tensor sharing the
        film's memory (no copy; valid while the film lives)."""
        import torch

        ptr = C.c_void_p()
        check(lib().asuna_film_image(self.handle, int(image), C.byref(ptr)))

        class _View:
            __cuda_array_interface__ = {"shape": (self.height, self.width, 4), "typestr": "<f4",
                                        "data": (int(ptr.value), False), "version": 2, "strides": None}

        return torch.as_tensor(_View(), device=f"cuda:{self.ctx.device}")

    def clear(self):
        check(lib().asuna_film_clear(self.ctx.handle, self.handle))

    def close(self):
        if getattr(self, "handle", None):
            lib().asuna_film_destroy(self.handle)
            self.handle = None

    __del__ = close


class DeviceScene:
    def __init__(self, ctx, desc):
        self.ctx = ctx
        h = C.c_void_p()
        check(lib().asuna_scene_create(ctx.handle, desc.ptr, C.byref(h)))
        self.handle = h

    def stats(self):
        s = A.SceneStats()
        check(lib().asuna_scene_get_stats(self.handle, C.byref(s)))
        return {k: getattr(s, k) for k, _ in A.SceneStats._fields_}

    def trace(self, origins, dirs, tmin=1e-5, tmax=1e10, any_hit=False):
        n = len(origins)
        rays = np.zeros((n, 8), np.float32)
        rays[:, 0:3] = origins
        rays[:, 3] = tmin
        rays[:, 4:7] = dirs
        rays[:, 7] = tmax
        hits = np.zeros((n, 4), np.float32)
        inst = np.zeros(n, np.uint32)
        check(lib().asuna_scene_trace(self.ctx.handle, self.handle, rays.ctypes.data, n, 1 if any_hit else 0,
                                      hits.ctypes.data, inst.ctypes.data))
        return hits, inst

    def close(self):
        if getattr(self, "handle", None):
            lib().asuna_scene_destroy(self.handle)
            self.handle = None

    __del__ = close


def _stats_dict(s):
    return {k: getattr(s, k) for k, _ in A.RenderStats._fields_}


class Context:
    """One CUDA device + stream of the native library (asuna_ctx)."""

    def __init__(self, device=0):
        h = C.c_void_p()
        check(lib().asuna_ctx_create(device, C.byref(h)))
        self.handle = h
        self.device = device

    def set_counters(self, on):
        check(lib().asuna_ctx_set_counters(self.handle, 1 if on else 0))

    def set_path_budget(self, nbytes):
        check(lib().asuna_ctx_set_path_budget(self.handle, int(nbytes)))

    def set_graphs(self, on):
        check(lib().asuna_ctx_set_graphs(self.handle, 1 if on else 0))

    def set_traversal(self, refill_extend=0, refill_shadow=0, speculate_extend=-1, speculate_shadow=-1,
                      blocks_per_sm=0):
        """Traversal settings (results do not depend on them): refill thresholds,
        speculative walking (-1 default on) and the kernel variant's resident
        blocks per SM."""
        check(lib().asuna_ctx_set_traversal(self.handle, int(refill_extend), int(refill_shadow),
                                            int(speculate_extend), int(speculate_shadow), int(blocks_per_sm)))

    def set_ray_sort(self, mode=1):
        """Sort the extend queue by direction octant and origin cell before
        secondary passes: 0 off, 1 octant x 4^3 cells, 2 octant x 8^3 cells
        in Morton order, 3 the same with the origin cell major (True = 1).  Results
        do not depend on it."""
        check(lib().asuna_ctx_set_ray_sort(self.handle, int(mode)))

    def set_bvh_build(self, on_device=True):
        """Build the bottom-level BVHs of new scenes on the device (default)
        or on host threads (the same binned-SAH algorithm)."""
        check(lib().asuna_ctx_set_bvh_build(self.handle, 0 if on_device else 1))

    def set_traversal_shape(self, threads_per_block=0, shared_stack=0):
        """Traversal kernel variant: threads per block (64, 128, 256) and
        stack entries in shared memory (16, 24, 32); 0 = defaults.  Results
        do not depend on them."""
        check(lib().asuna_ctx_set_traversal_shape(self.handle, int(threads_per_block), int(shared_stack)))

    def set_traversal_occupancy(self, extend_blocks_per_sm=0, shadow_blocks_per_sm=0):
        """Traversal kernel variant (resident blocks per SM: 8, 10, 12; 0 = 8)
        of the extend and occlusion passes separately.  Results do not depend
        on them."""
        check(lib().asuna_ctx_set_traversal_occupancy(self.handle, int(extend_blocks_per_sm),
                                                      int(shadow_blocks_per_sm)))

    def set_traversal_stack(self, entries=0):
        """Caps the traversal stack per ray (0 = the full 64 entries); a
        traversal needing more is cut short and reported as ERR_TRAVERSAL."""
        check(lib().asuna_ctx_set_traversal_stack(self.handle, int(entries)))

    def set_launch(self, trace_blocks_per_sm=0, shade_blocks_per_sm=0):
        check(lib().asuna_ctx_set_launch(self.handle, int(trace_blocks_per_sm), int(shade_blocks_per_sm)))

    def create_scene(self, desc):
        return DeviceScene(self, desc)

    def create_film(self, width, height):
        return Film(self, width, height)

    def render(self, scene, shot, film, stats=False):
        st = A.RenderStats() if stats else None
        check(lib().asuna_render(self.handle, scene.handle, C.byref(shot), film.handle,
                                 C.byref(st) if st is not None else None))
        return _stats_dict(st) if st is not None else None

    def render_batch(self, scene, shots, films, stats=False):
        n = len(shots)
        sh = (A.Shot * n)(*shots)
        fh = (C.c_void_p * n)(*[f.handle for f in films])
        st = A.RenderStats() if stats else None
        check(lib().asuna_render_batch(self.handle, scene.handle, sh, fh, n, C.byref(st) if st is not None else None))
        return _stats_dict(st) if st is not None else None

    def render_paths(self, scene, shot, film):
        rec = np.zeros(shot.frames * shot.width * shot.height, A.PATH_RECORD_DTYPE)
        check(lib().asuna_render_paths(self.handle, scene.handle, C.byref(shot), film.handle, rec.ctypes.data))
        return rec

    def sync(self):
        check(lib().asuna_ctx_sync(self.handle))

    def tonemap(self, film, image=0, post=None):
        """Post pass (tone mapping) of a film image; returns host RGBA float32."""
        import torch

        if post is None:
            post = default_post()
        out = torch.empty((film.height, film.width, 4), dtype=torch.float32, device=f"cuda:{self.device}")
        torch.cuda.synchronize()
        check(lib().asuna_tonemap(self.handle, film.handle, image, C.byref(post), C.c_void_p(out.data_ptr())))
        self.sync()
        return out.cpu().numpy()

    def run_offline(self, scene_json, out_prefix, output_scanline=False):
        """The offline tracer on a scene file; `output_scanline` is the CLI's
        --output_scanline (AOV channels as [n, 3] .npy arrays of hit pixels)."""
        check(lib().asuna_tracer_run_offline_scanline(self.handle, scene_json.encode(), out_prefix.encode(),
                                                      1 if output_scanline else 0))

    def close(self):
        if getattr(self, "handle", None):
            lib().asuna_ctx_destroy(self.handle)
            self.handle = None

    __del__ = close


class JsonScene:
    """A scene file parsed and assembled by the native host code
    (Loader::parse + Scene, src/loader/loader.cpp:91-144)."""

    def __init__(self, path=None, text=None, base_dir="."):
        h = C.c_void_p()
        if path is not None:
            check(lib().asuna_json_load(path.encode(), C.byref(h)))
        else:
            check(lib().asuna_json_load_string(text.encode(), base_dir.encode(), C.byref(h)))
        self.handle = h

    def desc(self):
        d = A.SceneDesc()
        check(lib().asuna_json_scene_desc(self.handle, C.byref(d)))
        return _DescView(d, self)

    def shots(self):
        n = C.c_uint32()
        check(lib().asuna_json_num_shots(self.handle, C.byref(n)))
        out = []
        for i in range(n.value):
            s = A.Shot()
            check(lib().asuna_json_get_shot(self.handle, i, C.byref(s)))
            out.append(s)
        return out

    def channels(self):
        n = C.c_uint32()
        kinds = (C.c_int32 * A.MAX_CHANNELS)()
        check(lib().asuna_json_channels(self.handle, C.byref(n), kinds))
        return list(kinds[: n.value])

    def close(self):
        if getattr(self, "handle", None):
            lib().asuna_json_free(self.handle)
            self.handle = None

    __del__ = close


class _DescView:
    def __init__(self, d, owner):
        self.desc = d
        self._owner = owner

    @property
    def ptr(self):
        return C.byref(self.desc)


def envmap_tables(rgba):
    rgba = np.ascontiguousarray(rgba, np.float32)
    h, w = rgba.shape[:2]
    marg = np.zeros((h, w, 2), np.float32)
    cond = np.zeros((h, w, 2), np.float32)
    check(lib().asuna_envmap_tables(w, h, rgba.ctypes.data, marg.ctypes.data, cond.ctypes.data))
    return marg, cond
