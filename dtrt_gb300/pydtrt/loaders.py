"""load_obj / load_mitsuba and image I/O of the pydtrt API (reference pydtrt/load_obj.py,
load_mitsuba.py, image.py).

OpenEXR and scikit-image are not available here; imwrite/imread handle .npy, .pfm
(float) and .ppm (8-bit, gamma 2.2) instead and raise for other extensions.
"""
import os
import re
import xml.etree.ElementTree as etree

import numpy as np
import torch

from .. import dtrt
from . import transform
from .scene_objects import (AreaLight, AreaLightEx, BSDF_diffuse, BSDF_null, BSDF_Phong, BSDF_roughdielectric,
                            Camera, HG, Heterogeneous, Homogeneous, Isotropic, Scene, Shape)


class TriangleMesh:
    def __init__(self, vertices, indices, uvs, normals):
        self.vertices, self.indices, self.uvs, self.normals = vertices, indices, uvs, normals


def load_obj(filename):
    """Wavefront OBJ -> [TriangleMesh] with per-(position, uv, normal) vertex
    de-duplication and quads split in two (load_obj.py:13-103)."""
    vpool, tpool, npool = [], [], []
    verts, uvs, normals, indices = [], [], [], []
    vmap = {}

    def resolve(tok, k, pool_len):
        f = int(tok.split("/")[k])
        return f + pool_len if f < 0 else f - 1

    def vid(tok):
        parts = tok.split("/")
        pi = resolve(tok, 0, len(verts))
        ti = resolve(tok, 1, len(uvs)) if len(parts) > 1 and parts[1] != "" else None
        ni = resolve(tok, 2, 0) if len(parts) > 2 and parts[2] != "" else None
        key = (pi, ti, ni)
        if key not in vmap:
            vmap[key] = len(verts)
            verts.append(vpool[pi])
            if ti is not None:
                uvs.append(tpool[ti])
            if ni is not None:
                normals.append(npool[ni])
        return vmap[key]

    with open(filename) as fh:
        for line in fh:
            s = re.split(r"\s+", line.strip())
            if s[0] == "v":
                vpool.append([float(x) for x in s[1:4]])
            elif s[0] == "vt":
                tpool.append([float(x) for x in s[1:3]])
            elif s[0] == "vn":
                npool.append([float(x) for x in s[1:4]])
            elif s[0] == "f":
                assert len(s) <= 5
                a, b, c = vid(s[1]), vid(s[2]), vid(s[3])
                indices.append([a, b, c])
                if len(s) == 5:
                    indices.append([a, c, vid(s[4])])
    return [TriangleMesh(torch.tensor(verts, dtype=torch.float32), torch.tensor(indices, dtype=torch.int32),
                         torch.tensor(uvs, dtype=torch.float32) if uvs else None,
                         torch.tensor(normals, dtype=torch.float32) if normals else None)]


def _parse_transform(node):
    ret = torch.eye(4)
    for child in node:
        if child.tag == "matrix":
            m = torch.from_numpy(np.reshape(np.array(child.attrib["value"].split(), dtype=np.float32), (4, 4)))
            ret = m @ ret
            continue
        d = 1.0 if child.tag == "scale" else 0.0
        x, y, z = (float(child.attrib.get(k, d)) for k in ("x", "y", "z"))
        if child.tag == "translate":
            ret = transform.gen_translate_matrix(torch.tensor([x, y, z])) @ ret
        elif child.tag == "scale":
            ret = transform.gen_scale_matrix(torch.tensor([x, y, z])) @ ret
        elif child.tag == "rotate":
            ret = transform.gen_rotate_matrix([x, y, z], float(child.attrib["angle"])) @ ret
    return ret


def _parse_vector(s):
    v = np.array([float(x) for x in re.split(r"[,\s]+", s.strip()) if x], dtype=np.float32)
    return torch.from_numpy(v)


def _parse_camera(node, media):
    fov, pos, target, up = torch.tensor([45.0]), None, None, None
    res, crop, med_id = [256, 256], [0, 0, -1, -1], -1
    for ch in node:
        name = ch.attrib.get("name")
        if name == "fov":
            fov = torch.tensor([float(ch.attrib["value"])])
        elif name == "toWorld":
            la = [g for g in ch if g.tag.lower() == "lookat"]
            if not la:
                raise ValueError("Unsupported Mitsuba scene format: please use a look at transform")
            pos, target, up = (_parse_vector(la[0].attrib[k]) for k in ("origin", "target", "up"))
        if ch.tag == "film":
            for g in ch:
                n, v = g.attrib.get("name"), g.attrib.get("value")
                idx = {"width": (res, 0), "height": (res, 1), "cropOffsetX": (crop, 0), "cropOffsetY": (crop, 1),
                       "cropWidth": (crop, 2), "cropHeight": (crop, 3)}.get(n)
                if idx:
                    idx[0][idx[1]] = int(v)
        if ch.tag == "ref":
            med_id = media[ch.attrib["id"]]
    return Camera(position=pos, look_at=target, up=up, fov=fov, clip_near=1e-2, resolution=res, med_id=med_id,
                  crop_rect=crop)


def _parse_bsdf(node):
    t, nid = node.attrib["type"], node.attrib.get("id")
    vals = {c.attrib.get("name"): c.attrib.get("value") for c in node}
    if t == "diffuse":
        return nid, BSDF_diffuse(_parse_vector(vals["reflectance"]) if "reflectance" in vals else torch.tensor([0.5] * 3))
    if t == "null":
        return nid, BSDF_null()
    if t == "phong":
        kd = _parse_vector(vals["diffuseReflectance"]) if "diffuseReflectance" in vals else torch.tensor([0.5] * 3)
        ks = _parse_vector(vals["specularReflectance"]) if "specularReflectance" in vals else torch.tensor([0.2] * 3)
        e = _parse_vector(vals["exponent"]) if "exponent" in vals else 30.0
        return nid, BSDF_Phong(kd, ks, e)
    if t == "roughdielectric":
        return nid, BSDF_roughdielectric(_parse_vector(vals["alpha"]), _parse_vector(vals["intIOR"]),
                                         _parse_vector(vals["extIOR"]))
    raise ValueError(f"Unsupported bsdf type: {t}")


def _parse_phase(node):
    if node.attrib["type"] == "isotropic":
        return Isotropic()
    g = [c.attrib["value"] for c in node if c.attrib.get("name") == "g"][0]
    return HG(_parse_vector(g))


def _parse_medium(node):
    nid, phase = node.attrib.get("id"), None
    if node.attrib["type"] == "homogeneous":
        sig = alb = None
        for c in node:
            if c.tag == "phase":
                phase = _parse_phase(c)
            elif c.attrib.get("name") == "sigmaT":
                sig = _parse_vector(c.attrib["value"])
            elif c.attrib.get("name") == "albedo":
                alb = _parse_vector(c.attrib["value"])
        return nid, Homogeneous(sigma_t=sig, albedo=alb, phase_id=-1), phase or Isotropic()
    scalar, to_world, to_world0, fn, albedo = 1.0, torch.eye(4), torch.eye(4), None, None
    for c in node:
        if c.tag == "volume" and c.attrib.get("name") == "density":
            for g in c:
                if g.attrib.get("name") == "filename":
                    fn = g.attrib["value"]
                elif g.attrib.get("name") == "toWorld":
                    to_world = _parse_transform(g)
        elif c.tag == "volume" and c.attrib.get("name") == "albedo":
            for g in c:
                if g.attrib.get("name") == "value":
                    albedo = _parse_vector(g.attrib["value"])
                elif g.attrib.get("name") == "filename":
                    albedo = g.attrib["value"]
                elif g.attrib.get("name") == "toWorld":
                    to_world0 = _parse_transform(g)
        elif c.tag == "phase":
            phase = _parse_phase(c)
        elif c.attrib.get("name") == "scale":
            scalar = _parse_vector(c.attrib["value"])
    if isinstance(albedo, str):
        assert torch.all(torch.abs(to_world - to_world0) < 1e-6)
    return nid, Heterogeneous(fn_density=fn, albedo=albedo, scalar=scalar, to_world=to_world.contiguous(),
                              phase_id=-1), phase or Isotropic()


def _parse_shape(node, bsdfs, media, shape_id):
    t = node.attrib["type"]
    if t not in ("obj", "rectangle"):
        raise ValueError(f"Unsupported shape type: {t}")
    to_world, bsdf_id, med_ext, med_int, light_I, kappa, fn = torch.eye(4), -1, -1, -1, None, None, ""
    for c in node:
        name = c.attrib.get("name")
        if name == "filename":
            fn = c.attrib["value"]
        elif name == "toWorld":
            to_world = _parse_transform(c)
        if c.tag == "ref":
            if name == "interior":
                med_int = media[c.attrib["id"]]
            elif name == "exterior":
                med_ext = media[c.attrib["id"]]
            else:
                bsdf_id = bsdfs[c.attrib["id"]]
        elif c.tag == "emitter":
            for g in c:
                if g.attrib.get("name") == "radiance":
                    light_I = _parse_vector(g.attrib["value"])
                    if light_I.shape[0] == 1:
                        light_I = light_I.repeat(3)
                elif g.attrib.get("name") == "kappa" and c.attrib["type"] == "areaEx":
                    kappa = float(g.attrib["value"])
    if fn == "":
        idx = torch.tensor([[0, 2, 1], [1, 2, 3]], dtype=torch.int32)
        v = torch.tensor([[-1.0, -1.0, 0.0], [-1.0, 1.0, 0.0], [1.0, -1.0, 0.0], [1.0, 1.0, 0.0]])
        uvs = nrm = None
    else:
        m = load_obj(fn)[0]
        v, idx, uvs, nrm = m.vertices, m.indices, m.uvs, m.normals
    vh = torch.cat((v, torch.ones(v.shape[0], 1)), dim=1) @ to_world.T
    v = (vh[:, 0:3] / vh[:, 3:4]).contiguous()
    if nrm is not None:
        nrm = (nrm @ torch.inverse(to_world.T)[:3, :3]).contiguous()
    light = None
    if light_I is not None:
        light = AreaLight(shape_id, light_I) if kappa is None else AreaLightEx(shape_id, light_I, kappa)
    return Shape(v, idx, uvs, nrm, bsdf_id, med_ext, med_int), light


def _parse_scene(root):
    cam, bsdfs, bmap, shapes, lights, mmap, media, phases, integ = None, [], {}, [], [], {}, [], [], None
    names = {"direct": "DirectIntegrator", "path": "PathTracer", "volpath_simple": "VolPathTracerSimple",
             "volpath": "VolPathTracer", "directAD": "DirectAD", "pathAD": "PathTracerAD",
             "volpathAD": "VolPathTracerAD", "ptracer": "ParticleTracer"}
    for c in root:
        if c.tag == "sensor":
            cam = _parse_camera(c, mmap)
        elif c.tag == "bsdf":
            nid, b = _parse_bsdf(c)
            if nid is not None:
                bmap[nid] = len(bsdfs)
                bsdfs.append(b)
        elif c.tag == "medium":
            nid, m, ph = _parse_medium(c)
            if nid is not None:
                mmap[nid] = len(media)
                media.append(m)
                m.phase_id = len(phases)
                phases.append(ph)
        elif c.tag == "shape":
            s, l = _parse_shape(c, bmap, mmap, len(shapes))
            shapes.append(s)
            if l is not None:
                lights.append(l)
        elif c.tag == "integrator":
            t = c.attrib["type"]
            if t not in names:
                raise ValueError(f"Integrator type [ {t} ] not supported!")
            integ = getattr(dtrt, names[t])()
    return Scene(cam, shapes, bsdfs, media, phases, lights), integ


def load_mitsuba(filename):
    """Mitsuba 0.5 XML subset -> (pydtrt Scene, integrator) (load_mitsuba.py:322-350)."""
    root = etree.parse(filename).getroot()
    cwd = os.getcwd()
    os.chdir(os.path.dirname(os.path.abspath(filename)))
    try:
        return _parse_scene(root)
    finally:
        os.chdir(cwd)


# ----------------------------------------------------------------------------- image I/O
def imwrite(img, filename, normalize=False):
    d = os.path.dirname(filename)
    if d and not os.path.exists(d):
        os.makedirs(d)
    a = img.detach().cpu().numpy() if torch.is_tensor(img) else np.asarray(img)
    a = a.astype(np.float32)
    if normalize:
        rng = a.max() - a.min()
        if rng > 0:
            a = (a - a.min()) / rng
    if a.ndim == 2:
        a = np.repeat(a[:, :, None], 3, 2)
    ext = os.path.splitext(filename)[1].lower()
    if ext == ".npy":
        np.save(filename, a)
    elif ext == ".pfm":
        with open(filename, "wb") as fh:
            fh.write(b"PF\n%d %d\n-1\n" % (a.shape[1], a.shape[0]))
            fh.write(np.ascontiguousarray(a[::-1, :, :3], dtype="<f4").tobytes())
    elif ext == ".ppm":
        q = (np.power(np.clip(a[:, :, :3], 0, 1), 1 / 2.2) * 255 + 0.5).astype(np.uint8)
        with open(filename, "wb") as fh:
            fh.write(b"P6\n%d %d\n255\n" % (q.shape[1], q.shape[0]))
            fh.write(q.tobytes())
    else:
        raise ValueError(f"unsupported image format {ext!r}: use .npy, .pfm or .ppm (no OpenEXR here)")


def imread(filename):
    ext = os.path.splitext(filename)[1].lower()
    if ext == ".npy":
        return torch.from_numpy(np.load(filename).astype(np.float32))
    if ext == ".pfm":
        with open(filename, "rb") as fh:
            assert fh.readline().strip() == b"PF"
            w, h = (int(x) for x in fh.readline().split())
            scale = float(fh.readline())
            data = np.frombuffer(fh.read(w * h * 12), dtype="<f4" if scale < 0 else ">f4").reshape(h, w, 3)
        return torch.from_numpy(data[::-1].copy().astype(np.float32))
    if ext == ".ppm":
        with open(filename, "rb") as fh:
            assert fh.readline().strip() == b"P6"
            w, h = (int(x) for x in fh.readline().split())
            fh.readline()
            q = np.frombuffer(fh.read(w * h * 3), dtype=np.uint8).reshape(h, w, 3)
        return torch.from_numpy(np.power(q.astype(np.float32) / 255.0, 2.2))
    raise ValueError(f"unsupported image format {ext!r}: use .npy, .pfm or .ppm (no OpenEXR here)")
