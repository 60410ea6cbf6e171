"""GPU: scene descriptor edge cases through the C-ABI.

- A descriptor with no mesh objects gives every triangle material 0 on both
  BVH builders, whatever `object_material` points at.
- `er_scene_set_camera` rejects a non-finite camera and leaves the handle's
  camera as it was.
"""
import dataclasses

import numpy as np
import pytest

from eleven import _abi as A
from eleven import _lib, scenes

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("builder", [A.ER_BUILDER_HOST, A.ER_BUILDER_GPU])
def test_no_objects_means_material_zero(builder):
    base = scenes.config0(x_res=32, y_res=24, n_spheres=3, subdiv=1, seed=6)
    one = dataclasses.replace(base, tri_object=np.zeros(base.tri_count, np.int32),
                              object_material=np.zeros(1, np.int32))
    # a non-NULL pointer with a count of 0: ignored
    none = dataclasses.replace(base, tri_object=None, object_material=np.full(0, 7, np.int32))
    out = []
    for arrays in (one, none):
        with _lib.Scene(arrays, builder=builder) as s:
            out.append(s.render(spp=2, max_depth=3, seed=1)["beauty"])
    assert np.array_equal(out[0].view(np.uint32), out[1].view(np.uint32))


def test_set_camera_rejects_non_finite_and_keeps_the_old_camera():
    arrays = scenes.config0(x_res=16, y_res=12, n_spheres=2, subdiv=0)
    with _lib.Scene(arrays) as s:
        before = s.render(spp=1, max_depth=2, seed=3)["beauty"]
        cam = s.camera()
        bad = s.camera()
        bad.rotation[2] = float("nan")
        with pytest.raises(_lib.ElevenError) as e:
            s.set_camera(bad)
        assert e.value.status == A.ER_ERR_INVALID_ARG
        now = s.camera()
        assert bytes(now) == bytes(cam)
        after = s.render(spp=1, max_depth=2, seed=3)["beauty"]
        assert np.array_equal(before.view(np.uint32), after.view(np.uint32))
