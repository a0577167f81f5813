"""Generate tests/golden/glass_1_args.pt from the reference's example scene
examples/glass_1 (scene.xml and its OBJ meshes), read from the reference checkout.

The scene is loaded the way the example's optimize.py loads it: under the reference's
module names (dtrt_gb300.install_reference_names), through pydtrt.load_mitsuba and
pydtrt.serialize_scene, then SceneManager with the example's four transforms (apple
translation along x, y, z and the tank's roughness) set to the example's target values.
The fixture is that flat render_scene argument list; tests render it on the GPU and on
the oracle without needing the reference checkout.

    python tests/golden/make_examples.py [reference root]
"""
import os
import sys

import torch

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

TARGET = [-5.0, -3.0, -4.0, -2.5]  # examples/glass_1/optimize.py:34


def glass_1_args(ref_root):
    import dtrt_gb300
    dtrt, pydtrt = dtrt_gb300.install_reference_names()
    dtrt.set_nder(4)
    scene, integrator = pydtrt.load_mitsuba(os.path.join(ref_root, "examples", "glass_1", "scene.xml"))
    args = pydtrt.serialize_scene(scene)
    T = pydtrt.SceneTransform
    transforms = [[T("SHAPE_TRANSLATE", torch.tensor([1.0, 0.0, 0.0]), 0)],
                  [T("SHAPE_TRANSLATE", torch.tensor([0.0, 1.0, 0.0]), 0)],
                  [T("SHAPE_TRANSLATE", torch.tensor([0.0, 0.0, 1.0]), 0)],
                  [T("BSDF_VARY", "roughdielectric", 0, 0.1, 0.0)]]
    sm = pydtrt.SceneManager(args, transforms)
    sm.set_arguments(torch.tensor(TARGET))
    return list(sm.args), type(integrator).__name__


if __name__ == "__main__":
    root = sys.argv[1] if len(sys.argv) > 1 else "/root/reference"
    args, integ = glass_1_args(root)
    torch.save({"scene": "examples/glass_1/scene.xml", "nder": 4, "target": TARGET, "integrator": integ,
                "args": args}, os.path.join(HERE, "glass_1_args.pt"))
    print("wrote", os.path.join(HERE, "glass_1_args.pt"))
