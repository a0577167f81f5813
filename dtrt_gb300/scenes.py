"""Seeded synthetic scenes with the shapes, sizes and value distributions of the
five benchmark configurations, plus Mitsuba VOL v3 grid I/O.

No public dataset is involved; every scene is generated from a seed. The
`SceneSpec` container holds numpy arrays and converts to the C description of
include/dtrt_gb300.h (`to_desc`), which both the CUDA library and the CPU oracle
consume.

Configurations (sizes as in the benchmark definition):
  C0  256x256, 32 spp, depth 5, nder 1: null-bounded homogeneous icosphere (1280 tris)
      over a diffuse ground under a 1x1 area light; derivative = sphere x-translation.
  C1  512x512, 64 spp, depth 10, nder 3: smooth-dielectric unit cube around a 64^3
      Gaussian-blob grid (scale 5, albedo 0.9, HG g=0.3); derivatives = scale, albedo, g.
  C2  256x256, 64 spp, depth 4: diffuse icosphere with 20480 tris, 8 seeded vertex
      displacement directions (forward mode nder 8).
  C3  512x512, 128 spp, depth 16: 128^3 grid of 32 blobs in a null-bounded cube.
  C4  64 seeded scenes of uneven sizes.
"""
import ctypes
import math
import os
import struct
from dataclasses import dataclass, field
from typing import List, Optional

import numpy as np

from . import _abi


# ----------------------------------------------------------------------------- geometry
def icosphere(subdiv: int, radius: float = 1.0, center=(0.0, 0.0, 0.0)):
    """Outward-wound icosphere: 10*4^s+2 vertices, 20*4^s triangles."""
    t = (1.0 + math.sqrt(5.0)) / 2.0
    verts = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t), (0, -1, -t), (0, 1, -t),
             (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    verts = [np.array(v, dtype=np.float64) / np.linalg.norm(v) for v in verts]
    faces = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4), (11, 10, 2),
             (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5), (2, 4, 11),
             (6, 2, 10), (8, 6, 7), (9, 8, 1)]
    for _ in range(subdiv):
        cache = {}

        def mid(a, b):
            key = (min(a, b), max(a, b))
            if key not in cache:
                m = verts[a] + verts[b]
                verts.append(m / np.linalg.norm(m))
                cache[key] = len(verts) - 1
            return cache[key]

        nf = []
        for a, b, c in faces:
            ab, bc, ca = mid(a, b), mid(b, c), mid(c, a)
            nf += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
        faces = nf
    v = np.array(verts) * radius + np.asarray(center, dtype=np.float64)
    f = np.array(faces, dtype=np.int32)
    # enforce outward winding
    c0 = v[f[:, 0]]
    n = np.cross(v[f[:, 1]] - c0, v[f[:, 2]] - c0)
    flip = np.einsum("ij,ij->i", n, c0 - np.asarray(center)) < 0
    f[flip] = f[flip][:, [0, 2, 1]]
    return v.astype(np.float32), f


def quad(center, half_x, half_z, y_normal_sign: float):
    """Axis-aligned quad in the xz-plane at height center[1], wound so that its
    geometric normal (v1-v0)x(v2-v0) points to sign(y_normal_sign)*y."""
    cx, cy, cz = center
    v = np.array([[cx - half_x, cy, cz - half_z], [cx + half_x, cy, cz - half_z],
                  [cx + half_x, cy, cz + half_z], [cx - half_x, cy, cz + half_z]], dtype=np.float32)
    f = np.array([[0, 2, 1], [0, 3, 2]], dtype=np.int32)  # normal +y
    if y_normal_sign < 0:
        f = f[:, [0, 2, 1]]
    return v, f


def box(lo, hi):
    """Closed axis-aligned box, 8 vertices, 12 outward-wound triangles."""
    lo, hi = np.asarray(lo, np.float32), np.asarray(hi, np.float32)
    v = np.array([[lo[0] if i & 1 == 0 else hi[0], lo[1] if i & 2 == 0 else hi[1], lo[2] if i & 4 == 0 else hi[2]]
                  for i in range(8)], dtype=np.float32)
    quads = [(0, 2, 3, 1), (4, 5, 7, 6), (0, 1, 5, 4), (2, 6, 7, 3), (0, 4, 6, 2), (1, 3, 7, 5)]
    f = []
    for a, b, c, d in quads:
        f += [(a, b, c), (a, c, d)]
    f = np.array(f, dtype=np.int32)
    ctr = (lo + hi) / 2
    c0 = v[f[:, 0]]
    n = np.cross(v[f[:, 1]] - c0, v[f[:, 2]] - c0)
    flip = np.einsum("ij,ij->i", n, c0 - ctr) < 0
    f[flip] = f[flip][:, [0, 2, 1]]
    return v, f


def vertex_normals(v, f):
    n = np.zeros_like(v, dtype=np.float64)
    fn = np.cross(v[f[:, 1]] - v[f[:, 0]], v[f[:, 2]] - v[f[:, 0]])
    for k in range(3):
        np.add.at(n, f[:, k], fn)
    n /= np.linalg.norm(n, axis=1, keepdims=True)
    return n.astype(np.float32)


def look_at(pos, target, up):
    """Camera-to-world matrix with columns (right, up, dir, pos), as pydtrt's
    gen_look_at_matrix (pydtrt/transform.py:12-21)."""
    pos, target, up = (np.asarray(a, np.float64) for a in (pos, target, up))
    d = target - pos
    d /= np.linalg.norm(d)
    right = np.cross(d, up / np.linalg.norm(up))
    right /= np.linalg.norm(right)
    nup = np.cross(right, d)
    nup /= np.linalg.norm(nup)
    m = np.eye(4)
    m[:3, 0], m[:3, 1], m[:3, 2], m[:3, 3] = right, nup, d, pos
    return m.astype(np.float32)


def blob_grid(res, nblobs, seed, amp_range=(0.5, 1.0), sigma_range=(0.05, 0.15), amp_jitter=None):
    """Sum of isotropic Gaussian blobs on [0,1]^3 sampled at res^3 vertices
    (x fastest). Returns float32 [res][res][res] and the blob parameters."""
    rng = np.random.default_rng(seed)
    centres = rng.uniform(0.2, 0.8, size=(nblobs, 3))
    sigmas = rng.uniform(*sigma_range, size=nblobs)
    amps = rng.uniform(*amp_range, size=nblobs)
    if amp_jitter is not None:
        amps = amps * (1.0 + rng.uniform(-amp_jitter, amp_jitter, size=nblobs))
    x = np.linspace(0.0, 1.0, res)
    grid = np.zeros((res, res, res), np.float64)
    zz, yy, xx = np.meshgrid(x, x, x, indexing="ij")
    for c, s, a in zip(centres, sigmas, amps):
        grid += a * np.exp(-((xx - c[0]) ** 2 + (yy - c[1]) ** 2 + (zz - c[2]) ** 2) / (2 * s * s))
    return grid.astype(np.float32), (centres, sigmas, amps)


def blob_field(res, centre, sigma):
    """One unit-amplitude Gaussian blob of blob_grid on the same vertices: the derivative
    of the grid with respect to that blob's amplitude."""
    x = np.linspace(0.0, 1.0, res)
    gz = np.exp(-((x - centre[2]) ** 2) / (2 * sigma * sigma))
    gy = np.exp(-((x - centre[1]) ** 2) / (2 * sigma * sigma))
    gx = np.exp(-((x - centre[0]) ** 2) / (2 * sigma * sigma))
    return (gz[:, None, None] * gy[None, :, None] * gx[None, None, :]).astype(np.float32)


def write_vol(path, grid, vmin, vmax):
    """Mitsuba VOL v3: 'VOL', version 3, type 1 (float32), res xyz, channels,
    bounds min/max, data z-major with x fastest (gridvolume.h:88-132)."""
    g = np.ascontiguousarray(grid, dtype=np.float32)
    ch = 1 if g.ndim == 3 else g.shape[3]
    rz, ry, rx = g.shape[:3]
    with open(path, "wb") as fh:
        fh.write(b"VOL")
        fh.write(struct.pack("<B", 3))
        fh.write(struct.pack("<i", 1))
        fh.write(struct.pack("<3i", rx, ry, rz))
        fh.write(struct.pack("<i", ch))
        fh.write(struct.pack("<3f", *vmin))
        fh.write(struct.pack("<3f", *vmax))
        fh.write(g.tobytes())


def read_vol(path):
    with open(path, "rb") as fh:
        if fh.read(3) != b"VOL" or fh.read(1) != b"\x03":
            raise ValueError("not a VOL v3 file")
        (typ,) = struct.unpack("<i", fh.read(4))
        rx, ry, rz = struct.unpack("<3i", fh.read(12))
        (ch,) = struct.unpack("<i", fh.read(4))
        vmin = struct.unpack("<3f", fh.read(12))
        vmax = struct.unpack("<3f", fh.read(12))
        if typ != 1:
            raise ValueError("only float32 VOL grids are supported")
        data = np.frombuffer(fh.read(rx * ry * rz * ch * 4), dtype=np.float32)
    shape = (rz, ry, rx) if ch == 1 else (rz, ry, rx, ch)
    return data.reshape(shape).copy(), vmin, vmax


# ----------------------------------------------------------------------------- scene spec
def _f32(a, shape=None):
    if a is None:
        return None
    a = np.ascontiguousarray(np.asarray(a, dtype=np.float32))
    if shape is not None:
        a = a.reshape(shape)
    return a


@dataclass
class CameraSpec:
    width: int
    height: int
    cam_to_world: np.ndarray
    cam_to_ndc: np.ndarray
    clip_near: float = 1e-2
    med_id: int = -1
    velocities: Optional[np.ndarray] = None  # [2*nder, 3]
    crop: tuple = (0, 0, -1, -1)


@dataclass
class ShapeSpec:
    vertices: np.ndarray
    indices: np.ndarray
    bsdf_id: int
    light_id: int = -1
    med_int_id: int = -1
    med_ext_id: int = -1
    normals: Optional[np.ndarray] = None
    uvs: Optional[np.ndarray] = None
    velocities: Optional[np.ndarray] = None  # [nder*nv, 3] (+ [nv,3] normal velocities)


@dataclass
class BsdfSpec:
    type: int
    diffuse: tuple = (0.5, 0.5, 0.5)
    specular: tuple = (0.2, 0.2, 0.2)
    exponent: float = 30.0
    alpha: float = 0.1
    int_ior: float = 1.5
    ext_ior: float = 1.0
    d_diffuse: Optional[np.ndarray] = None
    d_specular: Optional[np.ndarray] = None
    d_exponent: Optional[np.ndarray] = None
    d_alpha: Optional[np.ndarray] = None
    d_eta: Optional[np.ndarray] = None


@dataclass
class EmitterSpec:
    shape_id: int
    intensity: tuple = (10.0, 10.0, 10.0)
    type: int = _abi.EMITTER_AREA
    two_sided: bool = False
    kappa: float = 0.0
    d_intensity: Optional[np.ndarray] = None
    d_kappa: Optional[np.ndarray] = None


@dataclass
class PhaseSpec:
    type: int = _abi.PHASE_ISOTROPIC
    g: float = 0.0
    d_g: Optional[np.ndarray] = None


@dataclass
class MediumSpec:
    type: int
    phase_id: int = 0
    sigma_t: float = 1.0
    albedo: tuple = (0.8, 0.8, 0.8)
    d_sigma_t: Optional[np.ndarray] = None
    d_albedo: Optional[np.ndarray] = None
    density_file: Optional[str] = None
    density: Optional[np.ndarray] = None  # [rz, ry, rx]
    vol_min: tuple = (0.0, 0.0, 0.0)
    vol_max: tuple = (1.0, 1.0, 1.0)
    albedo_file: Optional[str] = None
    albedo_grid: Optional[np.ndarray] = None
    albedo_min: tuple = (0.0, 0.0, 0.0)
    albedo_max: tuple = (1.0, 1.0, 1.0)
    to_world: np.ndarray = field(default_factory=lambda: np.eye(4, dtype=np.float32))
    density_scale: float = 1.0
    d_density_scale: Optional[np.ndarray] = None
    trans_velocities: Optional[np.ndarray] = None
    rot_velocities: Optional[np.ndarray] = None


@dataclass
class SceneSpec:
    nder: int
    camera: CameraSpec
    shapes: List[ShapeSpec]
    bsdfs: List[BsdfSpec]
    emitters: List[EmitterSpec] = field(default_factory=list)
    phases: List[PhaseSpec] = field(default_factory=list)
    media: List[MediumSpec] = field(default_factory=list)
    edge_weights: Optional[np.ndarray] = None
    name: str = "scene"

    @property
    def width(self):
        c = self.camera
        return c.crop[2] if c.crop[2] > 0 else c.width

    @property
    def height(self):
        c = self.camera
        return c.crop[3] if c.crop[3] > 0 else c.height

    def out_shape(self):
        return (self.nder + 1, self.height, self.width, 3)

    def num_triangles(self):
        return sum(int(s.indices.shape[0]) for s in self.shapes)

    # -------------------------------------------------------------- C description
    def to_desc(self):
        """Build the dtrt_scene_desc. Returns (desc, keepalive); keep `keepalive`
        referenced while the description is in use."""
        keep = []

        def ptr(a, dtype=np.float32, shape=None):
            if a is None:
                return None
            arr = np.ascontiguousarray(np.asarray(a, dtype=dtype))
            if shape is not None:
                arr = arr.reshape(shape)
            keep.append(arr)
            ct = ctypes.c_float if dtype == np.float32 else ctypes.c_int
            return arr.ctypes.data_as(ctypes.POINTER(ct))

        n = self.nder
        d = _abi.SceneDesc()
        d.nder = n
        c = self.camera
        d.camera.width, d.camera.height = int(c.width), int(c.height)
        d.camera.cam_to_world = ptr(c.cam_to_world, shape=(16,))
        d.camera.cam_to_ndc = ptr(c.cam_to_ndc, shape=(9,))
        d.camera.clip_near = float(c.clip_near)
        d.camera.med_id = int(c.med_id)
        d.camera.velocities = ptr(c.velocities, shape=(2 * n * 3,)) if c.velocities is not None else None
        (d.camera.crop_offset_x, d.camera.crop_offset_y, d.camera.crop_width, d.camera.crop_height) = (
            int(x) for x in c.crop)

        shapes = (_abi.ShapeDesc * max(1, len(self.shapes)))()
        for i, s in enumerate(self.shapes):
            sd = shapes[i]
            sd.vertices = ptr(s.vertices)
            sd.indices = ptr(s.indices, dtype=np.int32)
            sd.uvs = ptr(s.uvs)
            sd.normals = ptr(s.normals)
            sd.num_vertices = int(np.asarray(s.vertices).shape[0])
            sd.num_triangles = int(np.asarray(s.indices).shape[0])
            sd.light_id, sd.bsdf_id = int(s.light_id), int(s.bsdf_id)
            sd.med_int_id, sd.med_ext_id = int(s.med_int_id), int(s.med_ext_id)
            sd.velocities = ptr(s.velocities)
        keep.append(shapes)
        d.num_shapes, d.shapes = len(self.shapes), shapes

        bsdfs = (_abi.BsdfDesc * max(1, len(self.bsdfs)))()
        for i, b in enumerate(self.bsdfs):
            bd = bsdfs[i]
            bd.type = b.type
            bd.diffuse[:] = [float(x) for x in np.broadcast_to(np.asarray(b.diffuse, np.float32), 3)]
            bd.specular[:] = [float(x) for x in np.broadcast_to(np.asarray(b.specular, np.float32), 3)]
            bd.exponent, bd.alpha = float(b.exponent), float(b.alpha)
            bd.int_ior, bd.ext_ior = float(b.int_ior), float(b.ext_ior)
            bd.d_diffuse, bd.d_specular = ptr(b.d_diffuse), ptr(b.d_specular)
            bd.d_exponent, bd.d_alpha, bd.d_eta = ptr(b.d_exponent), ptr(b.d_alpha), ptr(b.d_eta)
        keep.append(bsdfs)
        d.num_bsdfs, d.bsdfs = len(self.bsdfs), bsdfs

        ems = (_abi.EmitterDesc * max(1, len(self.emitters)))()
        for i, e in enumerate(self.emitters):
            ed = ems[i]
            ed.type, ed.shape_id = e.type, int(e.shape_id)
            ed.intensity[:] = [float(x) for x in np.broadcast_to(np.asarray(e.intensity, np.float32), 3)]
            ed.two_sided, ed.kappa = int(bool(e.two_sided)), float(e.kappa)
            ed.d_intensity, ed.d_kappa = ptr(e.d_intensity), ptr(e.d_kappa)
        keep.append(ems)
        d.num_emitters, d.emitters = len(self.emitters), ems

        phs = (_abi.PhaseDesc * max(1, len(self.phases)))()
        for i, p in enumerate(self.phases):
            phs[i].type, phs[i].g, phs[i].d_g = p.type, float(p.g), ptr(p.d_g)
        keep.append(phs)
        d.num_phases, d.phases = len(self.phases), phs

        meds = (_abi.MediumDesc * max(1, len(self.media)))()
        for i, m in enumerate(self.media):
            md = meds[i]
            md.type, md.phase_id = m.type, int(m.phase_id)
            md.sigma_t = float(m.sigma_t)
            md.albedo[:] = [float(x) for x in np.broadcast_to(np.asarray(m.albedo, np.float32), 3)]
            md.d_sigma_t, md.d_albedo = ptr(m.d_sigma_t), ptr(m.d_albedo)
            if m.density_file is not None:
                b = m.density_file.encode()
                keep.append(b)
                md.density_file = b
            if m.density is not None:
                md.density = ptr(m.density)
                rz, ry, rx = np.asarray(m.density).shape[:3]
                md.res[:] = [rx, ry, rz]
            md.vol_min[:] = [float(x) for x in m.vol_min]
            md.vol_max[:] = [float(x) for x in m.vol_max]
            if m.albedo_file is not None:
                b = m.albedo_file.encode()
                keep.append(b)
                md.albedo_file = b
            if m.albedo_grid is not None:
                md.albedo_grid = ptr(m.albedo_grid)
                rz, ry, rx = np.asarray(m.albedo_grid).shape[:3]
                md.albedo_res[:] = [rx, ry, rz]
            md.albedo_min[:] = [float(x) for x in m.albedo_min]
            md.albedo_max[:] = [float(x) for x in m.albedo_max]
            md.to_world[:] = [float(x) for x in np.asarray(m.to_world, np.float32).reshape(16)]
            md.density_scale = float(m.density_scale)
            md.d_density_scale = ptr(m.d_density_scale)
            md.trans_velocities, md.rot_velocities = ptr(m.trans_velocities), ptr(m.rot_velocities)
        keep.append(meds)
        d.num_media, d.media = len(self.media), meds
        d.edge_weights = ptr(self.edge_weights)
        return d, keep


# ----------------------------------------------------------------------------- configs
def _camera(width, height, fov_deg=45.0, pos=(0.0, 0.0, 4.0), target=(0.0, 0.0, 0.0), up=(0.0, 1.0, 0.0),
            nder=1, med_id=-1):
    f = 1.0 / math.tan(math.radians(0.5 * fov_deg))
    ndc = np.diag([f, f, 1.0]).astype(np.float32)
    return CameraSpec(width, height, look_at(pos, target, up), ndc, 1e-2, med_id, None)


def _stage(shapes, bsdfs, emitters, ground_albedo=0.5):
    """Ground quad (2 tris at y=-1, 4x4, diffuse) and a 1x1 light quad at y=2
    facing -y with radiance 10 (its BSDF is diffuse 0, a non-null BSDF)."""
    gv, gf = quad((0.0, -1.0, 0.0), 2.0, 2.0, +1.0)
    bsdfs.append(BsdfSpec(_abi.BSDF_DIFFUSE, diffuse=(ground_albedo,) * 3))
    shapes.append(ShapeSpec(gv, gf, bsdf_id=len(bsdfs) - 1))
    lv, lf = quad((0.0, 2.0, 0.0), 0.5, 0.5, -1.0)
    bsdfs.append(BsdfSpec(_abi.BSDF_DIFFUSE, diffuse=(0.0, 0.0, 0.0)))
    shapes.append(ShapeSpec(lv, lf, bsdf_id=len(bsdfs) - 1, light_id=len(emitters)))
    emitters.append(EmitterSpec(shape_id=len(shapes) - 1, intensity=(10.0, 10.0, 10.0)))


def config0(width=256, height=256, subdiv=3, nder=1):
    """C0: null-bounded homogeneous icosphere, derivative = sphere x-translation."""
    shapes, bsdfs, emitters = [], [], []
    sv, sf = icosphere(subdiv, 0.7)
    bsdfs.append(BsdfSpec(_abi.BSDF_NULL))
    vel = np.zeros((nder * sv.shape[0], 3), np.float32)
    vel[: sv.shape[0], 0] = 1.0  # SHAPE_TRANSLATE (1,0,0) on derivative slot 0
    shapes.append(ShapeSpec(sv, sf, bsdf_id=0, med_int_id=0, velocities=vel))
    _stage(shapes, bsdfs, emitters)
    media = [MediumSpec(_abi.MEDIUM_HOMOGENEOUS, phase_id=0, sigma_t=1.0, albedo=(0.8, 0.8, 0.8))]
    phases = [PhaseSpec(_abi.PHASE_ISOTROPIC)]
    return SceneSpec(nder, _camera(width, height, nder=nder), shapes, bsdfs, emitters, phases, media, name="C0")


def config1(width=512, height=512, res=64, seed=1, nder=3):
    """C1: smooth-dielectric cube (alpha at its 1e-4 floor, IOR 1.5) around a blob
    grid; derivatives = density scale, albedo, HG g."""
    shapes, bsdfs, emitters = [], [], []
    cv, cf = box((-0.5, -0.5, -0.5), (0.5, 0.5, 0.5))
    bsdfs.append(BsdfSpec(_abi.BSDF_ROUGHDIELECTRIC, alpha=1e-4, int_ior=1.5, ext_ior=1.0))
    shapes.append(ShapeSpec(cv, cf, bsdf_id=0, med_int_id=0))
    _stage(shapes, bsdfs, emitters)
    grid, _ = blob_grid(res, 8, seed)
    d_scale = np.zeros(nder, np.float32)
    d_alb = np.zeros((nder, 3), np.float32)
    d_g = np.zeros(nder, np.float32)
    if nder >= 3:
        d_scale[0], d_alb[1, :], d_g[2] = 1.0, 1.0, 1.0
    media = [MediumSpec(_abi.MEDIUM_HETEROGENEOUS, phase_id=0, albedo=(0.9, 0.9, 0.9), density=grid,
                        vol_min=(-0.5, -0.5, -0.5), vol_max=(0.5, 0.5, 0.5), density_scale=5.0,
                        d_density_scale=d_scale, d_albedo=d_alb,
                        trans_velocities=np.zeros((nder, 3), np.float32),
                        rot_velocities=np.zeros((nder, 3), np.float32))]
    phases = [PhaseSpec(_abi.PHASE_HG, g=0.3, d_g=d_g)]
    return SceneSpec(nder, _camera(width, height, nder=nder), shapes, bsdfs, emitters, phases, media, name="C1")


def config2(width=256, height=256, subdiv=5, nder=8, seed=2, displaced=False, sigma=0.01):
    """C2: diffuse icosphere (no vertex normals: faceted, every non-flat edge is a
    silhouette candidate); nder seeded unit directions in vertex space."""
    shapes, bsdfs, emitters = [], [], []
    sv, sf = icosphere(subdiv, 0.7)
    rng = np.random.default_rng(seed)
    if displaced:
        nrm = vertex_normals(sv, sf)
        sv = (sv + nrm * rng.normal(0.0, sigma, size=(sv.shape[0], 1))).astype(np.float32)
    dirs = rng.normal(size=(nder, sv.shape[0] * 3))
    dirs /= np.linalg.norm(dirs, axis=1, keepdims=True)
    bsdfs.append(BsdfSpec(_abi.BSDF_DIFFUSE, diffuse=(0.6, 0.6, 0.6)))
    shapes.append(ShapeSpec(sv, sf, bsdf_id=0, velocities=dirs.reshape(nder * sv.shape[0], 3).astype(np.float32)))
    _stage(shapes, bsdfs, emitters)
    return SceneSpec(nder, _camera(width, height, nder=nder), shapes, bsdfs, emitters, [], [], name="C2")


def config3(width=512, height=512, res=128, seed=3, nder=8, amp_jitter=None, param_slots=True, nblobs=32):
    """C3: 128^3 grid of 32 blobs inside a null-bounded unit cube (scale 8, albedo
    0.95, HG 0.5). Forward-mode slots: scale, albedo, g, volume translation x/y/z,
    volume rotation about y and about x. param_slots=False leaves every slot empty
    (for per-voxel density directions set on the scene afterwards)."""
    shapes, bsdfs, emitters = [], [], []
    cv, cf = box((-0.5, -0.5, -0.5), (0.5, 0.5, 0.5))
    bsdfs.append(BsdfSpec(_abi.BSDF_NULL))
    shapes.append(ShapeSpec(cv, cf, bsdf_id=0, med_int_id=0))
    _stage(shapes, bsdfs, emitters)
    grid, _ = blob_grid(res, nblobs, seed, amp_jitter=amp_jitter)
    d_scale = np.zeros(nder, np.float32)
    d_alb = np.zeros((nder, 3), np.float32)
    d_g = np.zeros(nder, np.float32)
    tv = np.zeros((nder, 3), np.float32)
    rv = np.zeros((nder, 3), np.float32)
    slots = [("scale", None), ("albedo", None), ("g", None), ("tx", 0), ("ty", 1), ("tz", 2), ("ry", 1), ("rx", 0)]
    for j in range(nder if param_slots else 0):
        kind, ax = slots[j % len(slots)]
        if kind == "scale":
            d_scale[j] = 1.0
        elif kind == "albedo":
            d_alb[j, :] = 1.0
        elif kind == "g":
            d_g[j] = 1.0
        elif kind.startswith("t"):
            tv[j, ax] = 1.0
        else:
            rv[j, ax] = 1.0
    media = [MediumSpec(_abi.MEDIUM_HETEROGENEOUS, phase_id=0, albedo=(0.95, 0.95, 0.95), density=grid,
                        vol_min=(-0.5, -0.5, -0.5), vol_max=(0.5, 0.5, 0.5), density_scale=8.0,
                        d_density_scale=d_scale, d_albedo=d_alb, trans_velocities=tv, rot_velocities=rv)]
    phases = [PhaseSpec(_abi.PHASE_HG, g=0.5, d_g=d_g)]
    return SceneSpec(nder, _camera(width, height, nder=nder), shapes, bsdfs, emitters, phases, media, name="C3")


def with_crop(spec, width, height, x=None, y=None):
    """Render only a width x height window of the camera's image (dtrt Camera.set_rect,
    src/dtrt.cpp:35-37); the window is centred when x / y are None."""
    W, H = spec.camera.width, spec.camera.height
    x = (W - width) // 2 if x is None else int(x)
    y = (H - height) // 2 if y is None else int(y)
    if not (0 <= x and 0 <= y and x + width <= W and y + height <= H):
        raise ValueError("crop window outside the image")
    spec.camera.crop = (x, y, int(width), int(height))
    return spec


def config4(index, seed=4, nder=1, side_scale=1.0, spp_scale=1.0):
    """One of the 64 uneven C4 scenes: an icosphere or a displaced plane of
    1k-50k triangles (log-uniform), 50% with a 32^3-128^3 blob grid. Image side
    128-512 and spp 16-256 (both scaled down by side_scale / spp_scale for small tests)."""
    rng = np.random.default_rng([seed, index])
    ntri = int(math.exp(rng.uniform(math.log(1000), math.log(50000))))
    side = max(8, int(int(rng.choice([128, 192, 256, 384, 512])) * side_scale))
    spp = max(1, int(int(2 ** rng.integers(4, 9)) * spp_scale))
    depth = int(rng.integers(4, 17))
    shapes, bsdfs, emitters, media, phases = [], [], [], [], []
    if rng.uniform() < 0.5:
        sub = max(2, min(6, int(round(math.log(ntri / 20.0, 4)))))
        v, f = icosphere(sub, 0.7)
    else:
        k = max(2, int(math.sqrt(ntri / 2)))
        xs = np.linspace(-0.8, 0.8, k + 1)
        xx, zz = np.meshgrid(xs, xs)
        yy = -0.3 + 0.1 * rng.normal(size=xx.shape)
        v = np.stack([xx, yy, zz], -1).reshape(-1, 3).astype(np.float32)
        f = []
        for i in range(k):
            for j in range(k):
                a = i * (k + 1) + j
                f += [(a, a + k + 1, a + 1), (a + 1, a + k + 1, a + k + 2)]
        f = np.array(f, np.int32)
    vel = np.zeros((nder * v.shape[0], 3), np.float32)
    vel[: v.shape[0], 0] = 1.0
    bsdfs.append(BsdfSpec(_abi.BSDF_DIFFUSE, diffuse=(0.6, 0.6, 0.6)))
    shapes.append(ShapeSpec(v, f, bsdf_id=0, velocities=vel))
    _stage(shapes, bsdfs, emitters)
    if rng.uniform() < 0.5:
        res = int(rng.choice([32, 64, 96, 128]))
        grid, _ = blob_grid(res, 8, int(rng.integers(1 << 30)))
        cv, cf = box((-0.9, -0.9, -0.9), (0.9, 0.9, 0.9))
        bsdfs.append(BsdfSpec(_abi.BSDF_NULL))
        shapes.append(ShapeSpec(cv, cf, bsdf_id=len(bsdfs) - 1, med_int_id=0))
        phases.append(PhaseSpec(_abi.PHASE_HG, g=0.3))
        media.append(MediumSpec(_abi.MEDIUM_HETEROGENEOUS, phase_id=0, albedo=(0.9,) * 3, density=grid,
                                vol_min=(-0.9, -0.9, -0.9), vol_max=(0.9, 0.9, 0.9), density_scale=2.0))
    sc = SceneSpec(nder, _camera(side, side, nder=nder), shapes, bsdfs, emitters, phases, media, name=f"C4[{index}]")
    return sc, dict(spp=spp, max_bounces=depth)
