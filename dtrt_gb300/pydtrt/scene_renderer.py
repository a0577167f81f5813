"""serialize_scene / render_scene of the pydtrt API (reference pydtrt/scene_renderer.py).

The flat argument list has exactly the reference's layout (documented in
scene_manager.py), so SceneManager offsets and user code carry over unchanged.
render_scene builds the native objects through dtrt_gb300.dtrt (CPU tensors, copied
at construction like the reference), allocates the (nder+1, H, W, 3) float32 CPU
tensor and renders it on the GPU.
"""
import time

import torch

from .. import _abi, dtrt

print_timing = False

# Keep the device scene between render_scene calls and rebuild it in place when the next
# scene has the same triangles (Scene.update: BVH refit, cached edge adjacency, device
# arrays rewritten), as in an optimisation loop that moves vertices or changes materials.
# Off by default: the reference builds a new scene for every call.
reuse_scene = False
_kept = None


def serialize_scene(scene):
    """pydtrt Scene -> flat argument list (scene_renderer.py:6-108)."""
    cam = scene.camera
    for light_id, light in enumerate(scene.area_lights):
        scene.shapes[light.shape_id].light_id = light_id
    args = [len(scene.shapes), len(scene.bsdfs), len(scene.area_lights), len(scene.mediums), len(scene.phases),
            cam.cam_to_world, cam.cam_to_ndc, cam.clip_near, cam.resolution, cam.med_id, None, cam.crop_rect]
    for shape in scene.shapes:
        args += [shape.vertices, shape.indices, shape.uvs, shape.normals, shape.bsdf_id, shape.light_id,
                 shape.med_ext_id, shape.med_int_id, None]
    for bsdf in scene.bsdfs:
        args.append(bsdf.type)
        if bsdf.type == "diffuse":
            args += [bsdf.diffuse_reflectance, None]
        elif bsdf.type == "null":
            pass
        elif bsdf.type == "phong":
            args += [bsdf.diffuse_reflectance, bsdf.specular_reflectance, bsdf.exponent, None, None, None]
        elif bsdf.type == "roughdielectric":
            args += [bsdf.alpha, bsdf.intIOR, bsdf.extIOR, None, None]
        else:
            raise ValueError(f"unknown bsdf type {bsdf.type!r}")
    for light in scene.area_lights:
        args.append(light.type)
        if light.type == "area_light":
            args += [light.shape_id, light.intensity, light.two_sided]
        elif light.type == "area_lightEx":
            args += [light.shape_id, light.intensity, light.kappa, None, None]
        else:
            raise ValueError(f"unknown emitter type {light.type!r}")
    for medium in scene.mediums:
        args.append(medium.type)
        if medium.type == "homogeneous":
            args += [medium.sigma_t, medium.albedo, medium.phase_id, None, None]
        elif medium.type == "heterogeneous":
            args += [medium.fn_density, medium.albedo, medium.to_world, medium.scalar, medium.phase_id,
                     None, None, None, None]
        else:
            raise ValueError(f"unknown medium type {medium.type!r}")
    for phase in scene.phases:
        args.append(phase.type)
        if phase.type == "isotropic":
            pass
        elif phase.type == "hg":
            args += [phase.g, None]
        else:
            raise ValueError(f"unknown phase type {phase.type!r}")
    args.append(None)
    return args


def _fp(t):
    return dtrt.float_ptr(t.data_ptr()) if t is not None else 0


def _f(x):
    return float(x.reshape(-1)[0]) if torch.is_tensor(x) else float(x)


def _native_objects(*args):
    """The dtrt objects of a flat argument list (scene_renderer.py:110-316): camera,
    shapes, bsdfs, lights, phases, media, the edge weights (or None), the output (H, W)
    and the tensors that must stay alive while the objects are in use."""
    num_shapes, num_bsdfs, num_lights, num_medium, num_phases = args[0:5]
    cam_to_world, cam_to_ndc, clip_near, resolution, cam_med_id, cam_vel, rect = args[5:12]
    assert cam_to_world.is_contiguous()
    keep = [cam_to_world, cam_to_ndc]
    camera = dtrt.Camera(resolution[0], resolution[1], _fp(cam_to_world), _fp(cam_to_ndc.contiguous()), clip_near,
                         cam_med_id, _fp(cam_vel.contiguous()) if cam_vel is not None else 0)
    camera.set_rect(rect[0], rect[1], rect[2], rect[3])
    i = 12
    shapes = []
    for _ in range(num_shapes):
        v, f, uv, n, bsdf_id, light_id, med_ext, med_int, vel = args[i:i + 9]
        assert v.is_contiguous() and f.is_contiguous()
        shapes.append(dtrt.Shape(_fp(v), dtrt.int_ptr(f.data_ptr()), _fp(uv), _fp(n), int(v.shape[0]), int(f.shape[0]),
                                 light_id, bsdf_id, med_int, med_ext, _fp(vel.contiguous()) if vel is not None else 0))
        i += 9
    bsdfs = []
    for _ in range(num_bsdfs):
        t = args[i]
        if t == "null":
            bsdfs.append(dtrt.BSDF_null())
            i += 1
        elif t == "diffuse":
            r = args[i + 1]
            spec = dtrt.Spectrum3f(_f(r[0]), _f(r[1]), _f(r[2]))
            d = args[i + 2]
            bsdfs.append(dtrt.BSDF_diffuse(spec) if d is None else dtrt.BSDF_diffuse(spec, _fp(d.contiguous())))
            i += 3
        elif t == "phong":
            kd, ks, e = args[i + 1:i + 4]
            skd = dtrt.Spectrum3f(_f(kd[0]), _f(kd[1]), _f(kd[2]))
            sks = dtrt.Spectrum3f(_f(ks[0]), _f(ks[1]), _f(ks[2]))
            if args[i + 4] is None:
                bsdfs.append(dtrt.BSDF_Phong(skd, sks, _f(e)))
            else:
                bsdfs.append(dtrt.BSDF_Phong(skd, sks, _f(e), _fp(args[i + 4].contiguous()), _fp(args[i + 5].contiguous()),
                                             _fp(args[i + 6].contiguous())))
            i += 7
        elif t == "roughdielectric":
            a, ii, ee = _f(args[i + 1]), _f(args[i + 2]), _f(args[i + 3])
            if args[i + 4] is None:
                bsdfs.append(dtrt.BSDF_roughdielectric(a, ii, ee))
            else:
                bsdfs.append(dtrt.BSDF_roughdielectric(a, ii, ee, _fp(args[i + 4].contiguous()), _fp(args[i + 5].contiguous())))
            i += 6
        else:
            raise ValueError(f"unknown bsdf type {t!r}")
    lights = []
    for _ in range(num_lights):
        if args[i] == "area_light":
            inten = torch.as_tensor(args[i + 2], dtype=torch.float32).contiguous()
            keep.append(inten)
            lights.append(dtrt.AreaLight(args[i + 1], _fp(inten), bool(args[i + 3])))
            i += 4
        else:
            I = args[i + 2]
            spec = dtrt.Spectrum3f(_f(I[0]), _f(I[1]), _f(I[2]))
            if args[i + 4] is None:
                lights.append(dtrt.AreaLightEx(args[i + 1], spec, _f(args[i + 3])))
            else:
                lights.append(dtrt.AreaLightEx(args[i + 1], spec, _f(args[i + 3]), _fp(args[i + 4].contiguous()),
                                               _fp(args[i + 5].contiguous())))
            i += 6
    media = []
    for _ in range(num_medium):
        if args[i] == "homogeneous":
            sig, alb, ph = _f(args[i + 1]), args[i + 2], args[i + 3]
            spec = dtrt.Spectrum3f(_f(alb[0]), _f(alb[1]), _f(alb[2]))
            if args[i + 4] is None:
                media.append(dtrt.Homogeneous(sig, spec, ph))
            else:
                media.append(dtrt.Homogeneous(sig, spec, ph, _fp(args[i + 4].contiguous()), _fp(args[i + 5].contiguous())))
            i += 6
        elif args[i] == "heterogeneous":
            fn, alb, tw, scal, ph = args[i + 1:i + 6]
            tw = tw.contiguous()
            keep.append(tw)
            a = alb if isinstance(alb, str) else dtrt.Spectrum3f(_f(alb[0]), _f(alb[1]), _f(alb[2]))
            if args[i + 6] is None:
                media.append(dtrt.Heterogeneous(fn, _fp(tw), _f(scal), a, ph))
            else:
                d_alb, d_sc, tr, rot = args[i + 6:i + 10]
                media.append(dtrt.Heterogeneous(fn, _fp(tw), _f(scal), a, ph, _fp(tr.contiguous()), _fp(rot.contiguous()),
                                                _fp(d_sc.contiguous()),
                                                None if isinstance(alb, str) else _fp(d_alb.contiguous())))
            i += 10
        else:
            raise ValueError(f"unknown medium type {args[i]!r}")
    phases = []
    for _ in range(num_phases):
        if args[i] == "isotropic":
            phases.append(dtrt.Isotropic())
            i += 1
        elif args[i] == "hg":
            g = _f(args[i + 1])
            phases.append(dtrt.HG(g) if args[i + 2] is None else dtrt.HG(g, _fp(args[i + 2].contiguous())))
            i += 3
        else:
            raise ValueError(f"unknown phase type {args[i]!r}")
    weights = args[i].contiguous().float() if args[i] is not None else None
    if rect[2] == -1 or rect[3] == -1:
        hw = (resolution[1], resolution[0])
    else:
        hw = (rect[3], rect[2])
    return (camera, shapes, bsdfs, lights, phases, media), weights, hw, keep


def scene_spec(*args):
    """The scene description (dtrt_gb300.scenes.SceneSpec) of a flat argument list, built
    by the same parsing as render_scene but without a device (e.g. for a CPU check)."""
    objs, weights, hw, keep = _native_objects(*args)
    spec = dtrt.scene_spec(*objs)
    if weights is not None:
        spec.edge_weights = weights.numpy().copy()
    return spec


def build_native_scene(*args, reuse=None):
    """Native objects and the device scene from a flat argument list
    (scene_renderer.py:110-316). Returns (scene, (H, W)). With `reuse` (a dtrt.Scene),
    that scene is updated in place when its triangles match, else a new one is built."""
    (camera, shapes, bsdfs, lights, phases, media), weights, hw, keep = _native_objects(*args)
    scene = None
    if reuse is not None and reuse._nder == camera._nder:
        try:
            reuse.update(camera, shapes, bsdfs, lights, phases, media)
            scene = reuse
        except _abi.DtrtError as e:
            if e.status != _abi.DTRT_ERR_INVALID:
                raise
    if scene is None:
        scene = dtrt.Scene(camera, shapes, bsdfs, lights, phases, media)
    if weights is not None:
        scene.initEdges(dtrt.float_ptr(weights.data_ptr()))
    return scene, hw


def render_scene(integrator, options, *args):
    """Render the flat-argument scene; returns a float32 CPU tensor (nder+1, H, W, 3)."""
    global _kept
    scene, (h, w) = build_native_scene(*args, reuse=_kept if reuse_scene else None)
    if _kept is not None and _kept is not scene:
        _kept.close()
        _kept = None
    img = torch.zeros(scene._nder + 1, h, w, 3)
    start = time.time()
    integrator.render(scene, options, dtrt.float_ptr(img.data_ptr()))
    if reuse_scene:
        _kept = scene
    else:
        scene.close()
    if print_timing:
        print("Total rendering time: %.2fs" % (time.time() - start))
    return img
