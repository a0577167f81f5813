"""The Python module `dtrt_gb300.dtrt` against the reference's native module `dtrt`
(src/dtrt.cpp:24-155): every class, base class, constructor overload (by argument
count), method and attribute of the pybind module exists here with the same name and
argument order. The table below is the reference's module surface; when the reference
sources are present it is also re-derived from src/dtrt.cpp and compared."""
import inspect
import os
import re

import pytest

from dtrt_gb300 import dtrt

# name: (base, constructor argument counts, methods {name: argument count}, attributes)
REFERENCE_MODULE = {
    "float_ptr": (None, [1], {}, []),
    "int_ptr": (None, [1], {}, []),
    "Spectrum3f": (None, [3], {}, []),
    "Camera": (None, [7], {"set_rect": 4}, []),
    "Shape": (None, [11], {"has_uvs": 0, "has_normals": 0}, ["num_vertices"]),
    "BSDF": (None, None, {}, []),
    "BSDF_diffuse": ("BSDF", [1, 2], {}, []),
    "BSDF_null": ("BSDF", [0], {}, []),
    "BSDF_Phong": ("BSDF", [3, 6], {}, []),
    "BSDF_roughdielectric": ("BSDF", [3, 4, 5], {}, []),
    "Phase": (None, None, {}, []),
    "HG": ("Phase", [1, 2], {}, []),
    "Isotropic": ("Phase", [0], {}, []),
    "Emitter": (None, None, {}, []),
    "AreaLight": ("Emitter", [3], {}, []),
    "AreaLightEx": ("Emitter", [3, 5], {}, []),
    "Medium": (None, None, {}, []),
    "Homogeneous": ("Medium", [3, 5], {}, []),
    "Heterogeneous": ("Medium", [5, 9, 5, 8], {}, []),
    "Scene": (None, [6], {"initEdges": 1}, []),
    "RenderOptions": (None, [6, 7, 8], {},
                      ["seed", "spp", "sppe", "sppse", "max_bounces", "quiet", "mode", "ddistCoeff"]),
    "Integrator": (None, None, {}, []),
    "DirectIntegrator": ("Integrator", [0], {"render": 3}, []),
    "PathTracer": ("Integrator", [0], {"render": 3}, []),
    "ParticleTracer": ("Integrator", [0], {"render": 3}, []),
    "VolPathTracer": ("Integrator", [0], {"render": 3}, []),
    "VolPathTracerSimple": ("Integrator", [0], {"render": 3}, []),
    "DirectAD": ("Integrator", [0], {"render": 3}, []),
    "PathTracerAD": ("Integrator", [0], {"render": 3}, []),
    "VolPathTracerAD": ("Integrator", [0], {"render": 3}, []),
}
MODULE_ATTRS = ["nder", "angleEps"]

# the argument order of the overloads the scene builder relies on (src/dtrt.cpp:35-115)
ARG_ORDER = {
    "Camera": ["width", "height", "cam_to_world", "cam_to_ndc", "clip_near", "med_id", "velocities"],
    "Shape": ["vertices", "indices", "uvs", "normals", "num_vertices", "num_triangles", "light_id", "bsdf_id",
              "med_int_id", "med_ext_id", "velocities"],
    "Homogeneous": ["sigma_t", "albedo", "phase_id", "d_sigma_t", "d_albedo"],
    "Heterogeneous": ["density_file", "to_world", "scale", "albedo", "phase_id", "trans_velocities",
                      "rot_velocities", "d_scale", "d_albedo"],
    "RenderOptions": ["seed", "spp", "max_bounces", "sppe", "sppse", "quiet", "mode", "ddistCoeff"],
    "AreaLight": ["shape_id", "intensity", "two_sided"],
    "AreaLightEx": ["shape_id", "intensity", "kappa", "d_intensity", "d_kappa"],
    "BSDF_Phong": ["diffuse", "specular", "exponent", "d_diffuse", "d_specular", "d_exponent"],
    "BSDF_roughdielectric": ["alpha", "int_ior", "ext_ior", "d_alpha", "d_eta"],
}


def _arity(fn):
    if fn is object.__init__:
        return 0, 0
    ps = [p for p in inspect.signature(fn).parameters.values() if p.name != "self"]
    lo = sum(1 for p in ps if p.default is inspect.Parameter.empty)
    return lo, len(ps)


@pytest.mark.parametrize("name", sorted(REFERENCE_MODULE))
def test_class_surface_matches_reference(name):
    base, ctors, methods, attrs = REFERENCE_MODULE[name]
    cls = getattr(dtrt, name)
    assert inspect.isclass(cls)
    if base:
        assert issubclass(cls, getattr(dtrt, base)), f"{name} must derive from {base}"
    if ctors:
        lo, hi = _arity(cls.__init__)
        for n in ctors:
            assert lo <= n <= hi, f"{name}: the {n}-argument overload is not accepted ({lo}..{hi})"
    for m, n in methods.items():
        lo, hi = _arity(getattr(cls, m))
        assert lo <= n <= hi, f"{name}.{m} takes {n} arguments in the reference"
    for a in attrs:
        assert a in inspect.signature(cls.__init__).parameters or a in ("num_vertices",), (name, a)


def test_argument_order():
    for name, order in ARG_ORDER.items():
        ps = [p for p in inspect.signature(getattr(dtrt, name).__init__).parameters if p != "self"]
        assert ps == order, (name, ps)


def test_module_attributes():
    for a in MODULE_ATTRS:
        assert hasattr(dtrt, a)
    assert dtrt.nder in (1, 3, 4, 8)
    assert dtrt.angleEps == pytest.approx(1e-4)


def test_render_options_properties():
    o = dtrt.RenderOptions(1, 2, 3, 4, 5, True, 7, 0.5)
    assert (o.seed, o.spp, o.max_bounces, o.sppe, o.sppse, o.quiet, o.mode, o.ddistCoeff) == (1, 2, 3, 4, 5, True, 7,
                                                                                              0.5)
    o.spp = 9
    assert o._c().spp == 9


REF_SRC = "/root/reference/src/dtrt.cpp"


def _parse_reference(text):
    """{class: (base, [ctor arg counts], {method names}, [attributes])} from the pybind code."""
    out = {}
    blocks = re.split(r"py::class_<", text)[1:]
    for b in blocks:
        head = re.match(r"(.*?)>\(m,\s*\"(\w+)\"\)", b, re.S)
        if not head:
            continue
        parts = [p.strip() for p in head.group(1).split(",")]
        name = head.group(2)
        ctors = []
        for args in re.findall(r"py::init<(.*?)>\(\)\)", b, re.S):
            args = re.sub(r"<[^<>]*>", "", args).strip()
            ctors.append(0 if not args else args.count(",") + 1)
        methods = set(re.findall(r"\.def\(\"(\w+)\"", b))
        attrs = re.findall(r"\.def_read(?:only|write)\(\"(\w+)\"", b)
        out[name] = (parts[1] if len(parts) > 1 else None, ctors, methods, attrs)
    return out


@pytest.mark.skipif(not os.path.exists(REF_SRC), reason="reference sources not present")
def test_table_matches_reference_source():
    parsed = _parse_reference(open(REF_SRC).read())
    base_names = {"BSDF": "BSDF", "PhaseFunction": "Phase", "Emitter": "Emitter", "Medium": "Medium",
                  "Integrator": "Integrator"}
    assert set(parsed) == set(REFERENCE_MODULE)
    for name, (base, ctors, methods, attrs) in parsed.items():
        want = REFERENCE_MODULE[name]
        assert (base_names.get(base) if base else None) == want[0], name
        assert ctors == (want[1] or []), (name, ctors)
        assert methods == set(want[2]), (name, methods)
        assert sorted(attrs) == sorted(want[3]), (name, attrs)
