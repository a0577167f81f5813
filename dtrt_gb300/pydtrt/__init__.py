"""Drop-in replacement for the reference's `pydtrt` package: scene description,
serialization, SceneManager/SceneTransform, ADLossFunc, loaders and image I/O, over
the GPU renderer in dtrt_gb300.dtrt.

Use `dtrt_gb300.install_reference_names()` to make `import dtrt` / `import pydtrt`
resolve to these modules for unmodified reference scripts.
"""
from .. import dtrt as _dtrt
from .auto_grad import ADLossFunc, DensityRenderFunc, VertexRenderFunc, downsample
from .loaders import imread, imwrite, load_mitsuba, load_obj
from .scene_manager import SceneManager, SceneTransform
from .scene_objects import (AreaLight, AreaLightEx, BSDF_diffuse, BSDF_null, BSDF_Phong, BSDF_roughdielectric,
                            Camera, HG, Heterogeneous, Homogeneous, Isotropic, Scene, Shape, compute_vertex_normal)
from .scene_renderer import build_native_scene, render_scene, serialize_scene
from .transform import gen_rotate_matrix

nder = _dtrt.nder


def _sync_nder(n):
    global nder
    nder = n
