"""Matrix helpers of the pydtrt API (reference pydtrt/transform.py:6-127), over torch."""
import math
from math import cos, sin

import torch


def radians(deg):
    return (math.pi / 180.0) * deg


def normalize(v):
    return v / torch.norm(v)


def gen_look_at_matrix(pos, look, up):
    """Camera-to-world with columns (right, up, dir, pos); right = dir x up."""
    d = normalize(look - pos)
    right = normalize(torch.cross(d, normalize(up), dim=0))
    new_up = normalize(torch.cross(right, d, dim=0))
    m = torch.eye(4, dtype=torch.float32)
    m[0:3, 0], m[0:3, 1], m[0:3, 2], m[0:3, 3] = right, new_up, d, pos
    return m.contiguous()


def gen_scale_matrix(scale):
    return torch.diag(torch.cat([scale.float(), torch.ones(1)], 0))


def gen_translate_matrix(translate):
    m = torch.eye(4, dtype=torch.float32)
    m[0:3, 3] = torch.as_tensor(translate, dtype=torch.float32)[0:3]
    return m


def gen_perspective_matrix(fov, clip_near, clip_far):
    clip_dist = clip_far - clip_near
    cot = 1 / torch.tan(torch.as_tensor(radians(fov / 2.0)))
    m = torch.zeros(4, 4)
    m[0, 0], m[1, 1] = cot, cot
    m[2, 2], m[2, 3] = 1 / clip_dist, -clip_near / clip_dist
    m[3, 2] = 1.0
    return m


def _axis_angle3(ux, uy, uz, theta):
    c, s, C = cos(theta), sin(theta), 1 - cos(theta)
    return [[c + ux * ux * C, ux * uy * C - uz * s, ux * uz * C + uy * s],
            [uy * ux * C + uz * s, c + uy * uy * C, uy * uz * C - ux * s],
            [uz * ux * C - uy * s, uz * uy * C + ux * s, c + uz * uz * C]]


def gen_rotate_matrix(axis, angle):
    """4x4 rotation of `angle` degrees about `axis` (identity for a near-zero axis).
    The reference module defines gen_rotate_matrix twice; this axis-angle form is the
    one its callers see (pydtrt/transform.py:84-97)."""
    d = math.sqrt(float(axis[0]) ** 2 + float(axis[1]) ** 2 + float(axis[2]) ** 2)
    if d <= 1e-4:
        return torch.eye(4)
    r = _axis_angle3(float(axis[0]) / d, float(axis[1]) / d, float(axis[2]) / d, radians(angle))
    m = torch.eye(4)
    m[0:3, 0:3] = torch.tensor(r)
    return m


def gen_rotation_matrix3x3(ang_vel, t):
    """Rotation by |ang_vel|*t about ang_vel (radians)."""
    v = math.sqrt(float(ang_vel[0]) ** 2 + float(ang_vel[1]) ** 2 + float(ang_vel[2]) ** 2)
    if v <= 1e-4:
        return torch.eye(3)
    return torch.tensor(_axis_angle3(float(ang_vel[0]) / v, float(ang_vel[1]) / v, float(ang_vel[2]) / v, v * float(t)))


def gen_rotation_matrix4x4(ang_vel, t):
    m = torch.eye(4)
    m[0:3, 0:3] = gen_rotation_matrix3x3(ang_vel, t)
    return m
