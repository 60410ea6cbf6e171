"""GPU: progressive readback (er_snapshot) while er_render runs on another
thread, as the reference's window loop polls getBuffers during renderCuda
(main.cpp:53, kernel.cu:688-710)."""
import threading
import time

import numpy as np
import pytest

from eleven import _abi as A
from eleven import _lib, scenes

pytestmark = pytest.mark.gpu


def test_snapshots_during_render():
    arrays = scenes.config0(x_res=160, y_res=120)
    scene = _lib.Scene(arrays)
    with pytest.raises(_lib.ElevenError):
        scene.snapshot()  # nothing rendered with snapshots yet
    result = {}

    def render():
        result["out"] = scene.render(256, max_depth=4, seed=1, spp_per_wave=1, flags=A.ER_RENDER_SNAPSHOTS)

    t = threading.Thread(target=render)
    t.start()
    seen = []
    while t.is_alive():
        try:
            beauty, samples = scene.snapshot()
            seen.append(int(samples.max()))
        except _lib.ElevenError:
            pass
        time.sleep(0.002)
    t.join()
    out = result["out"]
    # progressive: the sample counts seen never go down, and intermediate
    # films were observed
    assert seen == sorted(seen)
    assert any(0 < v < 256 for v in seen)
    beauty, samples = scene.snapshot()
    assert np.array_equal(samples, out["samples"])
    assert np.array_equal(beauty.view(np.uint32), out["beauty"].view(np.uint32))
    scene.close()
