"""SceneTransform / SceneManager of the pydtrt API (reference pydtrt/scene_manager.py).

SceneManager owns a copy of the flat argument list and, for a vector of nder
parameter values, (1) applies each transform to the positions/parameters and
(2) writes the matching velocity tensors, which seed the derivative slots of the
next render. Layout of the flat list (serialize_scene):

  num_shapes, num_bsdfs, num_lights, num_mediums, num_phases,
  [camera] cam_to_world (4x4), cam_to_ndc (3x3), clip_near, resolution, medium_id,
           velocities (2*nder x 3: translations then rotation axes), crop rect,
  per shape:   vertices, indices, uvs, normals, bsdf_id, light_id, med_ext, med_int,
               vertex velocities (nder*nV x 3, or 2*nder*nV x 3 with normals),
  per bsdf:    type, then diffuse: reflectance, d_reflectance (nder x 3)
                           phong: kd, ks, exponent, d_kd, d_ks (nder x 3), d_exponent (nder x 1)
                           roughdielectric: alpha, intIOR, extIOR, d_alpha, d_eta (nder x 1)
  per emitter: type, area_light: shape_id, intensity, two_sided
                     area_lightEx: shape_id, intensity, kappa, d_intensity, d_kappa
  per medium:  type, homogeneous: sigma_t, albedo, phase_id, d_sigmaT, d_albedo
                     heterogeneous: file, albedo, to_world, scale, phase_id, d_albedo, d_scale,
                                    translate velocity, rotate velocity (nder x 3 each)
  per phase:   type, hg: g, d_g
  edge sampling weights (or None)
"""
import copy
import math
import struct

import numpy as np
import torch

from .. import dtrt
from . import transform

_KINDS = {"CAMERA_TRANSLATE", "SHAPE_TRANSLATE", "VERTEX_TRANSLATE", "CAMERA_ROTATE", "SHAPE_ROTATE",
          "SHAPE_GLOBAL_ROTATE", "BSDF_VARY", "MEDIUM_VARY", "PHASE_VARY", "EMITTER_VARY"}


class SceneTransform:
    """One parameter direction (scene_manager.py:11-67)."""

    def __init__(self, type_name, *args):
        if type_name not in _KINDS:
            raise ValueError(f"Transform type [{type_name}] not supported")
        self.type_name = type_name
        if type_name in ("CAMERA_TRANSLATE", "CAMERA_ROTATE"):
            self.vec_vel = args[0]
        elif type_name in ("SHAPE_TRANSLATE", "SHAPE_ROTATE", "SHAPE_GLOBAL_ROTATE"):
            self.vec_vel, self.shape_id = args[0], args[1]
        elif type_name == "VERTEX_TRANSLATE":
            self.vec_vel, self.shape_id, self.vert_id = args[0], args[1], args[2]
        elif type_name == "BSDF_VARY":
            self.bsdf_type, self.bsdf_id = args[0], args[1]
            if self.bsdf_type == "diffuse":
                self.d_reflectance = args[2]
            elif self.bsdf_type == "phong":
                self.d_diffuse, self.d_specular, self.d_exponent = args[2], args[3], args[4]
            elif self.bsdf_type == "roughdielectric":
                self.d_alpha, self.d_eta = args[2], args[3]
        elif type_name == "MEDIUM_VARY":
            self.med_type, self.med_id = args[0], args[1]
            if self.med_type == "homogeneous":
                self.d_sigmaT, self.d_albedo = args[2], args[3]
            elif self.med_type == "heterogeneous":
                self.vec_translate, self.vec_rotate, self.d_albedo, self.d_scalar = args[2], args[3], args[4], args[5]
        elif type_name == "PHASE_VARY":
            self.phase_type, self.phase_id, self.d_g = args[0], args[1], args[2]
            assert self.phase_type == "hg"
        elif type_name == "EMITTER_VARY":
            self.emitter_type, self.emitter_id, self.d_intensity, self.d_kappa = args[0], args[1], args[2], args[3]
            assert self.emitter_type == "area_lightEx"

    def determine_range(self, init_val, tmin, tmax):
        """Parameter interval keeping reflectances in [0,1] etc. (scene_manager.py:69-144)."""
        def clamp_unit(vals, dv, lo, hi):
            for ch in range(3):
                if float(dv[ch]) == 0.0:
                    continue
                a = -float(vals[ch]) / float(dv[ch])
                b = (1.0 - float(vals[ch])) / float(dv[ch])
                lo = max(lo, a if dv[ch] > 0 else b)
                hi = min(hi, b if dv[ch] > 0 else a)
            return lo, hi

        if self.type_name == "BSDF_VARY":
            if self.bsdf_type == "diffuse":
                tmin, tmax = clamp_unit(init_val, self.d_reflectance, tmin, tmax)
            elif self.bsdf_type == "phong":
                kd, ks, e = init_val
                for ch in range(3):
                    for val, dv in ((kd[ch], self.d_diffuse[ch]), (ks[ch], self.d_specular[ch])):
                        if dv > 0:
                            tmin = max(tmin, -float(val) / float(dv))
                        elif dv < 0:
                            tmax = min(tmax, -float(val) / float(dv))
                if self.d_exponent > 0.0:
                    tmin = max(tmin, -float(e) / float(self.d_exponent))
                elif self.d_exponent < 0.0:
                    tmax = min(tmin, -float(e) / float(self.d_exponent))  # as in the reference (line 97)
            elif self.bsdf_type == "roughdielectric":
                a = (0.01 - float(init_val[0])) / self.d_alpha if self.d_alpha else 0.0
                b = (0.1 - float(init_val[0])) / self.d_alpha if self.d_alpha else 0.0
                if self.d_alpha > 0.0:
                    tmin = max(tmin, a)
                    tmax = min(tmin, b)  # as in the reference (line 105)
                elif self.d_alpha < 0.0:
                    tmin, tmax = max(tmin, b), min(tmax, a)
                if self.d_eta > 0.0:
                    tmin = max(tmin, -float(init_val[1]) / self.d_eta)
                elif self.d_eta < 0.0:
                    tmax = min(tmax, -float(init_val[1]) / self.d_eta)
        elif self.type_name == "MEDIUM_VARY":
            if self.med_type == "homogeneous":
                sigma_t, albedo = init_val
                tmin, tmax = clamp_unit(albedo, self.d_albedo, tmin, tmax)
                if self.d_sigmaT > 0.0:
                    tmin = max(tmin, -float(sigma_t) / self.d_sigmaT)
                elif self.d_sigmaT < 0.0:
                    tmax = min(tmax, -float(sigma_t) / self.d_sigmaT)
            elif self.med_type == "heterogeneous":
                albedo, scalar = init_val
                tmin, tmax = clamp_unit(albedo, self.d_albedo, tmin, tmax)
                if self.d_scalar > 0.0:
                    tmin = max(tmin, -float(scalar) / self.d_scalar)
                elif self.d_scalar < 0.0:
                    tmax = min(tmax, -float(scalar) / self.d_scalar)
        assert tmax > tmin
        return tmin, tmax


def _vol_center(fn, to_world):
    with open(fn, "rb") as fh:
        assert fh.read(3) == b"VOL" and fh.read(1) == b"\x03"
        assert struct.unpack("I", fh.read(4)) == (1,)
        fh.read(16)
        pmin = np.array(struct.unpack("3f", fh.read(12)))
        pmax = np.array(struct.unpack("3f", fh.read(12)))
    c = torch.tensor([*(0.5 * (pmin + pmax)), 1.0], dtype=torch.float)
    return torch.mm(to_world, c.unsqueeze(1)).squeeze(1)[0:3]


class SceneManager:
    """Applies parameter values and writes derivative seeds (scene_manager.py:227-632)."""

    def __init__(self, args, transforms, check_range=False):
        self.nder = dtrt.nder
        self.offsets = {"camera": 5, "shape": [], "bsdf": [], "medium": [], "phase": [], "emitter": []}
        self.num_shapes, self.num_bsdfs, self.num_lights, self.num_medium, self.num_phases = args[0:5]
        i = 12
        for _ in range(self.num_shapes):
            self.offsets["shape"].append(i)
            i += 9
        sizes_bsdf = {"null": 1, "diffuse": 3, "phong": 7, "roughdielectric": 6}
        for _ in range(self.num_bsdfs):
            self.offsets["bsdf"].append(i)
            i += sizes_bsdf[args[i]]
        for _ in range(self.num_lights):
            self.offsets["emitter"].append(i)
            i += 4 if args[i] == "area_light" else 6
        for _ in range(self.num_medium):
            self.offsets["medium"].append(i)
            i += 6 if args[i] == "homogeneous" else 10
        for _ in range(self.num_phases):
            self.offsets["phase"].append(i)
            i += 1 if args[i] == "isotropic" else 3
        self.offsets["weight"] = i
        self.args_0 = copy.deepcopy(args)
        self.shape_centers_0 = [self.args_0[o].sum(0) / self.args_0[o].size(0) for o in self.offsets["shape"]]
        self.volume_centers_0 = []
        for o in self.offsets["medium"]:
            if self.args_0[o] == "heterogeneous":
                self.volume_centers_0.append(_vol_center(self.args_0[o + 1], self.args_0[o + 3]))
            else:
                self.volume_centers_0.append(None)
        self.transforms = transforms
        self.ranges = []
        if not check_range:
            self.ranges = [[-math.inf, math.inf] for _ in range(self.nder)]
        else:
            self.determine_range()
        assert self.nder == len(transforms)
        self.args = copy.deepcopy(self.args_0)
        self.set_arguments(torch.zeros(self.nder))

    def set_edge_weight(self, weights):
        assert weights.numel() == self.num_shapes
        self.args[self.offsets["weight"]] = weights.contiguous()

    def clean_up(self):
        """Positions/parameters back to the initial state, velocities zeroed (lines 355-411)."""
        n = self.nder
        o = self.offsets["camera"]
        self.args[o] = copy.deepcopy(self.args_0[o])
        self.args[o + 5] = torch.zeros(n * 2, 3)
        for o in self.offsets["shape"]:
            nv = self.args_0[o].size(0)
            has_n = self.args_0[o + 3] is not None
            self.args[o] = self.args_0[o].clone()
            if has_n:
                self.args[o + 3] = self.args_0[o + 3].clone()
            self.args[o + 8] = torch.zeros((2 if has_n else 1) * n * nv, 3)
        for o in self.offsets["bsdf"]:
            t = self.args_0[o]
            if t == "diffuse":
                self.args[o + 1] = copy.deepcopy(self.args_0[o + 1])
                self.args[o + 2] = torch.zeros(n, 3)
            elif t == "phong":
                self.args[o + 1:o + 4] = copy.deepcopy(self.args_0[o + 1:o + 4])
                self.args[o + 4], self.args[o + 5], self.args[o + 6] = torch.zeros(n, 3), torch.zeros(n, 3), torch.zeros(n, 1)
            elif t == "roughdielectric":
                self.args[o + 1] = copy.deepcopy(self.args_0[o + 1])
                self.args[o + 4], self.args[o + 5] = torch.zeros(n, 1), torch.zeros(n, 1)
        for o in self.offsets["medium"]:
            t = self.args_0[o]
            if t == "homogeneous":
                self.args[o + 1:o + 3] = copy.deepcopy(self.args_0[o + 1:o + 3])
                self.args[o + 4], self.args[o + 5] = torch.zeros(n, 1), torch.zeros(n, 3)
            elif t == "heterogeneous":
                self.args[o + 2:o + 5] = copy.deepcopy(self.args_0[o + 2:o + 5])
                self.args[o + 6], self.args[o + 7] = torch.zeros(n, 3), torch.zeros(n, 1)
                self.args[o + 8], self.args[o + 9] = torch.zeros(n, 3), torch.zeros(n, 3)
        for o in self.offsets["phase"]:
            if self.args_0[o] == "hg":
                self.args[o + 1] = copy.deepcopy(self.args_0[o + 1])
                self.args[o + 2] = torch.zeros(n, 1)
        for o in self.offsets["emitter"]:
            if self.args_0[o] == "area_lightEx":
                self.args[o + 2] = copy.deepcopy(self.args_0[o + 2])
                self.args[o + 3] = copy.deepcopy(self.args_0[o + 3])
                self.args[o + 4], self.args[o + 5] = torch.zeros(n, 3), torch.zeros(n, 1)

    def reset(self):
        self.set_arguments(torch.zeros(self.nder))

    def determine_range(self):
        for ivar, Tset in enumerate(self.transforms):
            tmin, tmax = -math.inf, math.inf
            for T in Tset:
                if T.type_name == "BSDF_VARY":
                    o = self.offsets["bsdf"][T.bsdf_id] + 1
                    span = {"diffuse": None, "phong": 3, "roughdielectric": 2}[T.bsdf_type]
                    iv = self.args_0[o] if span is None else self.args_0[o:o + span]
                    tmin, tmax = T.determine_range(iv, tmin, tmax)
                elif T.type_name == "MEDIUM_VARY":
                    o = self.offsets["medium"][T.med_id] + 1
                    if T.med_type == "homogeneous":
                        tmin, tmax = T.determine_range(self.args_0[o:o + 2], tmin, tmax)
                    else:
                        tmin, tmax = T.determine_range([self.args_0[o + 1], self.args_0[o + 3]], tmin, tmax)
            self.ranges.append([tmin, tmax])

    def set_arguments(self, var_list):
        """Apply parameter values; seed velocities for unclamped parameters; return the
        out-of-range penalty gradient (lines 439-632)."""
        n = self.nder
        var_grad = torch.zeros(n)
        var = var_list.detach().clone().float()
        clamped = [False] * n
        for k in range(n):
            lo, hi = self.ranges[k]
            if var[k] < lo or var[k] > hi:
                clamped[k] = True
                edge = lo if var[k] < lo else hi
                var_grad[k] = 2 * (var_list[k].item() - edge) * (hi - lo)
                var[k] = edge
        self.clean_up()
        centers = copy.deepcopy(self.shape_centers_0)
        centers_vol = copy.deepcopy(self.volume_centers_0)
        A = self.args
        for k, Tset in enumerate(self.transforms):
            x = var[k]
            for T in Tset:
                t = T.type_name
                if t == "CAMERA_TRANSLATE":
                    A[self.offsets["camera"]][0:3, 3] += T.vec_vel * x
                elif t == "CAMERA_ROTATE":
                    o = self.offsets["camera"]
                    axis = torch.mv(self.args_0[o][0:3, 0:3], T.vec_vel)
                    A[o][0:3, 0:3] = torch.mm(transform.gen_rotation_matrix3x3(axis, x), A[o][0:3, 0:3])
                elif t == "SHAPE_TRANSLATE":
                    A[self.offsets["shape"][T.shape_id]][:] += T.vec_vel * x
                    centers[T.shape_id] = centers[T.shape_id] + T.vec_vel * x
                elif t == "VERTEX_TRANSLATE":
                    A[self.offsets["shape"][T.shape_id]][T.vert_id] += T.vec_vel * x
                elif t in ("SHAPE_ROTATE", "SHAPE_GLOBAL_ROTATE"):
                    o = self.offsets["shape"][T.shape_id]
                    R = transform.gen_rotation_matrix3x3(T.vec_vel, x)
                    c = centers[T.shape_id] if t == "SHAPE_ROTATE" else torch.zeros(3)
                    A[o] = ((A[o] - c) @ R.T + c).contiguous()
                    if t == "SHAPE_GLOBAL_ROTATE":
                        centers[T.shape_id] = R @ centers[T.shape_id]
                    if self.args_0[o + 3] is not None:
                        A[o + 3] = (A[o + 3] @ R.T).contiguous()
                elif t == "BSDF_VARY":
                    o = self.offsets["bsdf"][T.bsdf_id]
                    assert A[o] == T.bsdf_type
                    if T.bsdf_type == "diffuse":
                        A[o + 1] = A[o + 1] + T.d_reflectance * x
                    elif T.bsdf_type == "phong":
                        A[o + 1] = A[o + 1] + T.d_diffuse * x
                        A[o + 2] = A[o + 2] + T.d_specular * x
                        A[o + 3] = A[o + 3] + T.d_exponent * x
                    elif T.bsdf_type == "roughdielectric":
                        A[o + 1] = A[o + 1] + T.d_alpha * x
                        eta = self.args_0[o + 2] / self.args_0[o + 3] + T.d_eta * x
                        A[o + 2] = eta * A[o + 3]
                elif t == "MEDIUM_VARY":
                    o = self.offsets["medium"][T.med_id]
                    assert A[o] == T.med_type
                    if T.med_type == "homogeneous":
                        A[o + 1] = A[o + 1] + T.d_sigmaT * x
                        A[o + 2] = A[o + 2] + T.d_albedo * x
                    else:
                        if not isinstance(self.args_0[o + 2], str):
                            A[o + 2] = A[o + 2] + T.d_albedo * x
                        A[o + 4] = A[o + 4] + T.d_scalar * x
                        R = transform.gen_rotation_matrix4x4(T.vec_rotate, x)
                        c = centers_vol[T.med_id]
                        M = transform.gen_translate_matrix(c) @ R @ transform.gen_translate_matrix(-c) @ A[o + 3]
                        M = transform.gen_translate_matrix(T.vec_translate * x) @ M
                        A[o + 3] = M.clone().contiguous()
                        centers_vol[T.med_id] = centers_vol[T.med_id] + T.vec_translate * x
                elif t == "PHASE_VARY":
                    o = self.offsets["phase"][T.phase_id]
                    assert A[o] == T.phase_type
                    A[o + 1] = A[o + 1] + T.d_g * x
                elif t == "EMITTER_VARY":
                    o = self.offsets["emitter"][T.emitter_id]
                    assert A[o] == T.emitter_type
                    A[o + 2] = A[o + 2] + T.d_intensity * x
                    A[o + 3] = A[o + 3] + T.d_kappa * x
            if clamped[k]:
                continue
            for T in Tset:
                t = T.type_name
                if t == "CAMERA_TRANSLATE":
                    A[self.offsets["camera"] + 5][k] += T.vec_vel
                elif t == "CAMERA_ROTATE":
                    o = self.offsets["camera"]
                    A[o + 5][n + k] = torch.mv(self.args_0[o][0:3, 0:3], T.vec_vel)
                elif t == "SHAPE_TRANSLATE":
                    o = self.offsets["shape"][T.shape_id]
                    nv = self.args_0[o].size(0)
                    A[o + 8][k * nv:(k + 1) * nv] += T.vec_vel
                elif t == "VERTEX_TRANSLATE":
                    o = self.offsets["shape"][T.shape_id]
                    nv = self.args_0[o].size(0)
                    A[o + 8][k * nv + T.vert_id] += T.vec_vel
                elif t in ("SHAPE_ROTATE", "SHAPE_GLOBAL_ROTATE"):
                    o = self.offsets["shape"][T.shape_id]
                    nv = self.args_0[o].size(0)
                    c = centers[T.shape_id] if t == "SHAPE_ROTATE" else torch.zeros(3)
                    w = T.vec_vel.expand(nv, 3)
                    A[o + 8][k * nv:(k + 1) * nv] += torch.cross(w, A[o] - c, dim=1)
                    if self.args_0[o + 3] is not None:
                        A[o + 8][(k + n) * nv:(k + n + 1) * nv] += torch.cross(w, A[o + 3], dim=1)
                elif t == "BSDF_VARY":
                    o = self.offsets["bsdf"][T.bsdf_id] + 1
                    if T.bsdf_type == "diffuse":
                        A[o + 1][k] += T.d_reflectance
                    elif T.bsdf_type == "phong":
                        A[o + 3][k] += T.d_diffuse
                        A[o + 4][k] += T.d_specular
                        A[o + 5][k] += T.d_exponent
                    elif T.bsdf_type == "roughdielectric":
                        A[o + 3][k] += T.d_alpha
                        A[o + 4][k] += T.d_eta
                elif t == "MEDIUM_VARY":
                    o = self.offsets["medium"][T.med_id] + 1
                    if T.med_type == "homogeneous":
                        A[o + 3][k] += T.d_sigmaT
                        A[o + 4][k] += T.d_albedo
                    else:
                        A[o + 5][k] += T.d_albedo
                        A[o + 6][k] += T.d_scalar
                        A[o + 7][k] += T.vec_translate
                        A[o + 8][k] = T.vec_rotate
                elif t == "PHASE_VARY":
                    o = self.offsets["phase"][T.phase_id] + 1
                    A[o + 1][k] += T.d_g
                elif t == "EMITTER_VARY":
                    o = self.offsets["emitter"][T.emitter_id] + 4
                    A[o][k] += T.d_intensity
                    A[o + 1][k] += T.d_kappa
        return var_grad
