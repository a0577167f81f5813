"""Drop-in replacement for the reference's native module `dtrt` (src/dtrt.cpp:24-155).

Every class and constructor overload of the pybind module exists here with the same
argument order and meaning. Constructors copy their inputs from the raw addresses
they are given (float_ptr / int_ptr wrap `tensor.data_ptr()` of CPU tensors), as the
reference's constructors do (src/shape.cpp:14-31, src/camera.cpp:13-27); `Scene`
uploads everything to the GPU through the C ABI and `VolPathTracerAD.render` runs the
CUDA path tracer.

`nder` (derivative images per render) is read from the DTRT_NDER environment variable
at import (default 4, the reference's compile-time constant, include/config.h:5) and can
be changed with set_nder() to any of 1, 3, 4, 8.
"""
import ctypes
import os

import numpy as np

from . import _abi

nder = int(os.environ.get("DTRT_NDER", "4"))
angleEps = float(np.float32(1e-4))  # config.h:7 (float literal)


def set_nder(n):
    """Select the derivative width for scenes built afterwards (1, 3, 4 or 8)."""
    global nder
    if n not in (1, 3, 4, 8):
        raise ValueError("nder must be 1, 3, 4 or 8")
    nder = int(n)
    from . import pydtrt
    pydtrt._sync_nder(nder)


if nder not in (1, 3, 4, 8):
    raise ImportError("DTRT_NDER must be 1, 3, 4 or 8")


class _Ptr:
    __slots__ = ("addr",)

    def __init__(self, addr=0):
        self.addr = int(addr)

    def is_null(self):
        return self.addr == 0


class float_ptr(_Ptr):
    """Raw float* address (ptr<float>, include/ptr.h)."""


class int_ptr(_Ptr):
    """Raw int* address (ptr<int>)."""


def _addr(p):
    if p is None:
        return 0
    if isinstance(p, _Ptr):
        return p.addr
    return int(p)


def _read(p, n, ctype=ctypes.c_float, dtype=np.float32):
    a = _addr(p)
    if a == 0:
        return None
    return np.frombuffer((ctype * n).from_address(a), dtype=dtype).copy()


class Spectrum3f:
    def __init__(self, r, g, b):
        self.v = np.array([r, g, b], np.float32)


# --------------------------------------------------------------------------- scene objects
class Camera:
    """Camera(width, height, cam_to_world*, cam_to_ndc*, clip_near, med_id, velocities*)."""

    def __init__(self, width, height, cam_to_world, cam_to_ndc, clip_near, med_id, velocities=0):
        self.width, self.height = int(width), int(height)
        self.cam_to_world = _read(cam_to_world, 16)
        self.cam_to_ndc = _read(cam_to_ndc, 9)
        if abs(self.cam_to_ndc[0] - self.cam_to_ndc[4]) > 0:
            raise ValueError("cam_to_ndc(0,0) must equal cam_to_ndc(1,1) (camera.cpp:21)")
        self.clip_near = float(clip_near)
        self.med_id = int(med_id)
        self.velocities = _read(velocities, 6 * nder)
        self.rect = (0, 0, -1, -1)
        self._nder = nder

    def set_rect(self, offset_x, offset_y, crop_width, crop_height):
        self.rect = (int(offset_x), int(offset_y), int(crop_width), int(crop_height))


class Shape:
    """Shape(V*, F*, UV*, N*, nV, nT, light_id, bsdf_id, med_int_id, med_ext_id, velocities*)."""

    def __init__(self, vertices, indices, uvs, normals, num_vertices, num_triangles, light_id, bsdf_id,
                 med_int_id, med_ext_id, velocities=0):
        nv, nt = int(num_vertices), int(num_triangles)
        self.vertices = _read(vertices, 3 * nv).reshape(nv, 3)
        self.indices = _read(indices, 3 * nt, ctypes.c_int, np.int32).reshape(nt, 3)
        uv = _read(uvs, 2 * nv)
        self.uvs = uv.reshape(nv, 2) if uv is not None else None
        nrm = _read(normals, 3 * nv)
        self.normals = nrm.reshape(nv, 3) if nrm is not None else None
        nvel = nder * nv * 3 * (2 if self.normals is not None else 1)
        vel = _read(velocities, nvel)
        self.velocities = vel.reshape(-1, 3) if vel is not None else None
        self.num_vertices, self.num_triangles = nv, nt
        self.light_id, self.bsdf_id = int(light_id), int(bsdf_id)
        self.med_int_id, self.med_ext_id = int(med_int_id), int(med_ext_id)

    def has_uvs(self):
        return self.uvs is not None

    def has_normals(self):
        return self.normals is not None


class BSDF:
    pass


class BSDF_diffuse(BSDF):
    def __init__(self, reflectance, d_reflectance=None):
        self.type = _abi.BSDF_DIFFUSE
        self.diffuse = reflectance.v
        self.d_diffuse = _read(d_reflectance, 3 * nder)


class BSDF_null(BSDF):
    def __init__(self):
        self.type = _abi.BSDF_NULL


class BSDF_Phong(BSDF):
    def __init__(self, diffuse, specular, exponent, d_diffuse=None, d_specular=None, d_exponent=None):
        self.type = _abi.BSDF_PHONG
        self.diffuse, self.specular, self.exponent = diffuse.v, specular.v, float(exponent)
        self.d_diffuse = _read(d_diffuse, 3 * nder)
        self.d_specular = _read(d_specular, 3 * nder)
        self.d_exponent = _read(d_exponent, nder)


class BSDF_roughdielectric(BSDF):
    def __init__(self, alpha, int_ior, ext_ior, d_alpha=None, d_eta=None):
        self.type = _abi.BSDF_ROUGHDIELECTRIC
        self.alpha, self.int_ior, self.ext_ior = float(alpha), float(int_ior), float(ext_ior)
        self.d_alpha = _read(d_alpha, nder)
        self.d_eta = _read(d_eta, nder)


class Phase:
    pass


class HG(Phase):
    def __init__(self, g, d_g=None):
        self.type = _abi.PHASE_HG
        self.g = float(g)
        self.d_g = _read(d_g, nder)


class Isotropic(Phase):
    def __init__(self):
        self.type = _abi.PHASE_ISOTROPIC
        self.g = 0.0
        self.d_g = None


class Emitter:
    pass


class AreaLight(Emitter):
    """AreaLight(shape_id, intensity*, two_sided) (area.h:13-18)."""

    def __init__(self, shape_id, intensity, two_sided=False):
        self.type = _abi.EMITTER_AREA
        self.shape_id = int(shape_id)
        self.intensity = _read(intensity, 3)
        self.two_sided = bool(two_sided)
        self.kappa, self.d_intensity, self.d_kappa = 0.0, None, None


class AreaLightEx(Emitter):
    """AreaLightEx(shape_id, Spectrum3f intensity, kappa[, dI*, dKappa*]) (area2.h:11-17)."""

    def __init__(self, shape_id, intensity, kappa, d_intensity=None, d_kappa=None):
        self.type = _abi.EMITTER_AREA_EX
        self.shape_id = int(shape_id)
        self.intensity = intensity.v
        self.kappa = float(kappa)
        self.two_sided = False
        self.d_intensity = _read(d_intensity, 3 * nder)
        self.d_kappa = _read(d_kappa, nder)


class Medium:
    pass


class Homogeneous(Medium):
    def __init__(self, sigma_t, albedo, phase_id, d_sigma_t=None, d_albedo=None):
        self.type = _abi.MEDIUM_HOMOGENEOUS
        self.sigma_t, self.albedo, self.phase_id = float(sigma_t), albedo.v, int(phase_id)
        self.d_sigma_t = _read(d_sigma_t, nder)
        self.d_albedo = _read(d_albedo, 3 * nder)


class Heterogeneous(Medium):
    """Heterogeneous(file, toWorld*, scale, albedo (Spectrum3f | albedo file), phase_id
    [, trans_vel*, rot_vel*, d_scale*[, d_albedo*]]) (heterogeneous.h:28-75)."""

    def __init__(self, density_file, to_world, scale, albedo, phase_id, trans_velocities=None,
                 rot_velocities=None, d_scale=None, d_albedo=None):
        self.type = _abi.MEDIUM_HETEROGENEOUS
        self.density_file = str(density_file)
        self.to_world = _read(to_world, 16)
        self.scale = float(scale)
        if isinstance(albedo, str):
            self.albedo_file, self.albedo = albedo, np.zeros(3, np.float32)
        else:
            self.albedo_file, self.albedo = None, albedo.v
        self.phase_id = int(phase_id)
        self.trans_velocities = _read(trans_velocities, 3 * nder)
        self.rot_velocities = _read(rot_velocities, 3 * nder)
        self.d_scale = _read(d_scale, nder)
        self.d_albedo = _read(d_albedo, 3 * nder) if self.albedo_file is None else None


def scene_spec(camera, shapes, bsdfs, emitters, phases, media):
    """The scene description (dtrt_gb300.scenes.SceneSpec) of the dtrt objects a Scene
    is constructed from: what the C ABI's dtrt_scene_create consumes."""
    from . import scenes as S
    cam = S.CameraSpec(camera.width, camera.height, camera.cam_to_world.reshape(4, 4),
                       camera.cam_to_ndc.reshape(3, 3), camera.clip_near, camera.med_id,
                       camera.velocities.reshape(-1, 3) if camera.velocities is not None else None, camera.rect)
    spec = S.SceneSpec(camera._nder, cam, [], [])
    for s in shapes:
        spec.shapes.append(S.ShapeSpec(s.vertices, s.indices, s.bsdf_id, s.light_id, s.med_int_id, s.med_ext_id,
                                       s.normals, s.uvs, s.velocities))
    for b in bsdfs:
        spec.bsdfs.append(S.BsdfSpec(b.type, diffuse=tuple(getattr(b, "diffuse", (0, 0, 0))),
                                     specular=tuple(getattr(b, "specular", (0, 0, 0))),
                                     exponent=getattr(b, "exponent", 0.0), alpha=getattr(b, "alpha", 0.1),
                                     int_ior=getattr(b, "int_ior", 1.5), ext_ior=getattr(b, "ext_ior", 1.0),
                                     d_diffuse=getattr(b, "d_diffuse", None),
                                     d_specular=getattr(b, "d_specular", None),
                                     d_exponent=getattr(b, "d_exponent", None),
                                     d_alpha=getattr(b, "d_alpha", None), d_eta=getattr(b, "d_eta", None)))
    for e in emitters:
        spec.emitters.append(S.EmitterSpec(e.shape_id, tuple(e.intensity), e.type, e.two_sided, e.kappa,
                                           e.d_intensity, e.d_kappa))
    for p in phases:
        spec.phases.append(S.PhaseSpec(p.type, p.g, p.d_g))
    for m in media:
        if m.type == _abi.MEDIUM_HOMOGENEOUS:
            spec.media.append(S.MediumSpec(m.type, m.phase_id, m.sigma_t, tuple(m.albedo), m.d_sigma_t, m.d_albedo))
        else:
            spec.media.append(S.MediumSpec(m.type, m.phase_id, albedo=tuple(m.albedo), d_albedo=m.d_albedo,
                                           density_file=m.density_file, albedo_file=m.albedo_file,
                                           to_world=m.to_world.reshape(4, 4), density_scale=m.scale,
                                           d_density_scale=m.d_scale, trans_velocities=m.trans_velocities,
                                           rot_velocities=m.rot_velocities))
    return spec


class Scene:
    """Scene(camera, shapes, bsdfs, emitters, phases, media) (scene.cpp:9-136): the
    device scene (BVH, light and edge distributions) is built here."""

    def __init__(self, camera, shapes, bsdfs, emitters, phases, media):
        self._nder = camera._nder
        self.spec = self._spec(camera, shapes, bsdfs, emitters, phases, media)
        from .native import NativeScene
        self.native = NativeScene(self.spec)

    @classmethod
    def from_spec(cls, spec):
        """A Scene built directly from a dtrt_gb300.scenes.SceneSpec (same device scene as
        the constructor would build from the equivalent dtrt objects)."""
        from .native import NativeScene
        self = cls.__new__(cls)
        self._nder = spec.nder
        self.spec = spec
        self.native = NativeScene(spec)
        return self

    def update(self, camera, shapes, bsdfs, emitters, phases, media, rebuild_bvh=False):
        """Rebuild this scene in place from objects with the same triangles (same shapes,
        vertex and triangle counts, index lists; same media types and grid sizes): the BVH
        is refit and the edge adjacency reused (dtrt_scene_update). The reference builds a
        new Scene for every render instead (scene_renderer.py:313). Returns the update
        stats; raises DtrtError (status DTRT_ERR_INVALID) when the triangles differ."""
        if camera._nder != self._nder:
            raise _abi.DtrtError(_abi.DTRT_ERR_INVALID, "scene update: nder differs from the scene's")
        spec = self._spec(camera, shapes, bsdfs, emitters, phases, media)
        st = self.native.update(spec, rebuild_bvh=rebuild_bvh)
        self.spec = spec
        return st

    def _spec(self, camera, shapes, bsdfs, emitters, phases, media):
        return scene_spec(camera, shapes, bsdfs, emitters, phases, media)

    def initEdges(self, weights):
        """Secondary-edge sampling weight per shape (scene.h:37-39)."""
        w = _read(weights, len(self.spec.shapes))
        self.native.set_edge_weights(w)

    def close(self):
        self.native.close()


class RenderOptions:
    """RenderOptions(seed, spp, max_bounces, sppe, sppse, quiet[, mode[, ddistCoeff]])."""

    def __init__(self, seed, spp, max_bounces, sppe, sppse, quiet, mode=-1, ddistCoeff=0.0):
        self.seed, self.spp, self.max_bounces = int(seed), int(spp), int(max_bounces)
        self.sppe, self.sppse, self.quiet = int(sppe), int(sppse), bool(quiet)
        self.mode, self.ddistCoeff = int(mode), float(ddistCoeff)

    def _c(self):
        return _abi.RenderOptions(self.seed & ((1 << 64) - 1), self.spp, self.max_bounces, self.sppe, self.sppse,
                                  int(self.quiet), self.mode, self.ddistCoeff)


def _stream():
    """torch's current CUDA stream (the render runs and blocks on it), or the default stream."""
    try:
        import torch
        if torch.cuda.is_available():
            return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    except ImportError:
        pass
    return None


class Integrator:
    name = "Integrator"

    def render(self, scene, options, rendered_image):
        raise NotImplementedError(f"{self.name} is not provided by dtrt_gb300 (only VolPathTracerAD and "
                                  "VolPathTracer render)")


class VolPathTracerAD(Integrator):
    """Forward-mode volumetric path tracer (volpathAD.cpp) on the GPU: writes the image
    and nder derivative images into the float[(nder+1)][H][W][3] buffer at `rendered_image`."""
    name = "VolPathTracerAD"

    def render(self, scene, options, rendered_image):
        lib = _abi.load()
        o = options._c()
        _abi.check(lib.dtrt_render_fwd(scene.native.handle, ctypes.byref(o), ctypes.c_void_p(_addr(rendered_image)),
                                       0, _stream()))


class VolPathTracer(Integrator):
    """Primal volumetric path tracer (volpath.cpp:105-140 through dtrt_render_primal):
    writes the [H, W, 3] image at the start of `rendered_image`."""
    name = "VolPathTracer"

    def render(self, scene, options, rendered_image):
        spec = scene.spec
        n = spec.height * spec.width * 3
        o = options._c()
        lib = _abi.load()
        dst = (ctypes.c_float * n).from_address(_addr(rendered_image))
        _abi.check(lib.dtrt_render_primal(scene.native.handle, ctypes.byref(o), ctypes.cast(dst, ctypes.c_void_p), 0,
                                          _stream()))


class DirectIntegrator(Integrator):
    name = "DirectIntegrator"


class PathTracer(Integrator):
    name = "PathTracer"


class ParticleTracer(Integrator):
    name = "ParticleTracer"


class VolPathTracerSimple(Integrator):
    name = "VolPathTracerSimple"


def _require_surface_scene(scene, name):
    """The reference's surface integrators trace no media, test light visibility with one
    occlusion query (scene.cpp:150-175, 302-392: a null-BSDF surface blocks light) and
    sample lights only in front of the shading normal (scene.cpp:316), so lights behind a
    transmissive surface are reached by BSDF sampling alone while still MIS-weighted
    against light sampling. The volumetric estimator has the same expectation only
    without media, null BSDFs and transmissive BSDFs; other scenes are refused."""
    spec = scene.spec
    if spec.media or spec.camera.med_id >= 0:
        raise NotImplementedError(f"{name} ignores participating media in the reference; dtrt_gb300 renders it "
                                  "for surface scenes only (use VolPathTracerAD)")
    for b in spec.bsdfs:
        if b.type == _abi.BSDF_NULL:
            raise NotImplementedError(f"{name}: a null-BSDF surface blocks light in the reference's visibility test "
                                      "but is crossed by the volumetric estimator (use VolPathTracerAD)")
        if b.type == _abi.BSDF_ROUGHDIELECTRIC:
            raise NotImplementedError(f"{name}: the reference's light sampling skips lights behind a transmissive "
                                      "surface, which changes its expectation (use VolPathTracerAD)")


class PathTracerAD(VolPathTracerAD):
    """Surface forward-mode path tracer (pathAD.cpp) as the surface specialisation of the
    volumetric estimator: for scenes without media both estimate the same image and
    derivatives (interior term, edge-sampled boundary term, primary edges). The reference's
    variant differs in random-number use and in tracing visibility instead of
    transmittance, which changes the noise, not the expectation."""
    name = "PathTracerAD"

    def render(self, scene, options, rendered_image):
        _require_surface_scene(scene, self.name)
        super().render(scene, options, rendered_image)


class DirectAD(VolPathTracerAD):
    """Direct-illumination forward mode (directAD.cpp): emission at the camera hit, light
    sampling and BSDF sampling of the emitters, and the edge term of the camera hit, i.e. the
    volumetric estimator with one bounce on a surface scene. The reference weighs its two
    light strategies with the balance heuristic instead of the power heuristic: a different
    noise, the same expectation."""
    name = "DirectAD"

    def render(self, scene, options, rendered_image):
        _require_surface_scene(scene, self.name)
        o = options._c()
        o.max_bounces = 1
        lib = _abi.load()
        _abi.check(lib.dtrt_render_fwd(scene.native.handle, ctypes.byref(o), ctypes.c_void_p(_addr(rendered_image)),
                                       0, _stream()))
