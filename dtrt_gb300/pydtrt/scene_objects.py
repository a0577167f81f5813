"""Plain scene description classes of the pydtrt API (reference pydtrt/camera.py,
shape.py, bsdf.py, medium.py, phase.py, area_light.py, scene.py)."""
import math

import torch

from . import transform


class Camera:
    """Perspective look-at camera. `resolution` is (width, height); cam_to_ndc maps
    camera space to NDC (diag(1/tan(fov/2), 1/tan(fov/2), 1) when built from fov)."""

    def __init__(self, position, look_at, up, fov, clip_near, resolution, cam_to_ndc=None, med_id=-1,
                 crop_rect=(0, 0, -1, -1)):
        assert position.dtype == torch.float32 and position.shape == (3,)
        assert look_at.dtype == torch.float32 and look_at.shape == (3,)
        assert up.dtype == torch.float32 and up.shape == (3,)
        if fov is not None:
            assert fov.dtype == torch.float32 and fov.shape == (1,)
        assert isinstance(clip_near, float)
        self._position, self._look_at, self._up, self._fov = position, look_at, up, fov
        self._update_world()
        if cam_to_ndc is None:
            self._set_ndc_from_fov()
        else:
            self.cam_to_ndc = cam_to_ndc
        self.clip_near = clip_near
        self.resolution = resolution
        self.med_id = med_id
        self.crop_rect = list(crop_rect)

    def _update_world(self):
        self.cam_to_world = transform.gen_look_at_matrix(self._position, self._look_at, self._up)
        self.world_to_cam = torch.inverse(self.cam_to_world).contiguous()

    def _set_ndc_from_fov(self):
        f = 1.0 / torch.tan(transform.radians(0.5 * self._fov))
        self._cam_to_ndc = torch.diag(torch.cat([f, f, torch.ones(1)], 0)).contiguous()
        self.ndc_to_cam = torch.inverse(self._cam_to_ndc)

    @property
    def position(self):
        return self._position

    @position.setter
    def position(self, v):
        self._position = v
        self._update_world()

    @property
    def look_at(self):
        return self._look_at

    @look_at.setter
    def look_at(self, v):
        self._look_at = v
        self._update_world()

    @property
    def up(self):
        return self._up

    @up.setter
    def up(self, v):
        self._up = v
        self._update_world()

    @property
    def fov(self):
        return self._fov

    @fov.setter
    def fov(self, v):
        self._fov = v
        self._set_ndc_from_fov()

    @property
    def cam_to_ndc(self):
        return self._cam_to_ndc

    @cam_to_ndc.setter
    def cam_to_ndc(self, v):
        self._cam_to_ndc = v.contiguous()
        self.ndc_to_cam = torch.inverse(self._cam_to_ndc)


def compute_vertex_normal(vertices, indices):
    """Angle-weighted vertex normals (Max 1999), as pydtrt/shape.py:4-40."""
    def length(v):
        return torch.sqrt(torch.sum(v * v, dim=1))

    normals = torch.zeros(vertices.shape, dtype=torch.float32, device=vertices.device)
    v = [vertices[indices[:, k].long(), :] for k in range(3)]
    n = None
    for i in range(3):
        e1, e2 = v[(i + 1) % 3] - v[i], v[(i + 2) % 3] - v[i]
        l1, l2 = length(e1), length(e2)
        a, b = e1 / l1[:, None], e2 / l2[:, None]
        if i == 0:
            n = torch.cross(a, b, dim=1)
            n = n / length(n)[:, None]
        angle = torch.where(torch.sum(a * b, 1) < 0, math.pi - 2.0 * torch.asin(0.5 * length(a + b)),
                            2.0 * torch.asin(0.5 * length(b - a)))
        contrib = n * (torch.sin(angle) / (l1 * l2))[:, None]
        normals.scatter_add_(0, indices[:, i].long()[:, None].expand(-1, 3), contrib)
    return (normals / length(normals)[:, None]).contiguous()


class Shape:
    def __init__(self, vertices, indices, uvs, normals, bsdf_id=-1, med_ext_id=-1, med_int_id=-1):
        assert vertices.dtype == torch.float32 and vertices.is_contiguous()
        assert indices.dtype == torch.int32 and indices.is_contiguous()
        if uvs is not None:
            assert uvs.dtype == torch.float32 and uvs.is_contiguous()
        if normals is not None:
            assert normals.dtype == torch.float32 and normals.is_contiguous()
        self.vertices, self.indices, self.uvs, self.normals = vertices, indices, uvs, normals
        self.bsdf_id, self.light_id = bsdf_id, -1
        self.med_ext_id, self.med_int_id = med_ext_id, med_int_id


class BSDF_diffuse:
    def __init__(self, diffuse_reflectance):
        self.diffuse_reflectance = diffuse_reflectance
        self.type = "diffuse"


class BSDF_null:
    def __init__(self):
        self.type = "null"


class BSDF_Phong:
    def __init__(self, diffuse_reflectance, specular_reflectance, exponent):
        self.diffuse_reflectance = diffuse_reflectance
        self.specular_reflectance = specular_reflectance
        self.exponent = exponent
        self.type = "phong"


class BSDF_roughdielectric:
    def __init__(self, alpha, intIOR, extIOR):
        self.alpha, self.intIOR, self.extIOR = alpha, intIOR, extIOR
        self.type = "roughdielectric"


class Homogeneous:
    def __init__(self, sigma_t, albedo, phase_id):
        self.type = "homogeneous"
        self.sigma_t, self.albedo, self.phase_id = sigma_t, albedo, phase_id


class Heterogeneous:
    def __init__(self, fn_density, albedo, to_world, scalar, phase_id):
        self.type = "heterogeneous"
        self.fn_density, self.albedo, self.to_world = fn_density, albedo, to_world
        self.scalar, self.phase_id = scalar, phase_id


class Isotropic:
    def __init__(self):
        self.type = "isotropic"


class HG:
    def __init__(self, g):
        self.g = g
        self.type = "hg"


class AreaLight:
    def __init__(self, shape_id, intensity, two_sided=False):
        self.type = "area_light"
        self.shape_id, self.intensity, self.two_sided = shape_id, intensity, two_sided


class AreaLightEx:
    def __init__(self, shape_id, intensity, kappa):
        self.type = "area_lightEx"
        self.shape_id, self.intensity, self.kappa = shape_id, intensity, kappa


class Scene:
    """Note the argument order (camera, shapes, bsdfs, mediums, phases, area_lights),
    as pydtrt/scene.py."""

    def __init__(self, camera, shapes, bsdfs, mediums, phases, area_lights):
        self.camera, self.shapes, self.bsdfs = camera, shapes, bsdfs
        self.area_lights, self.mediums, self.phases = area_lights, mediums, phases
