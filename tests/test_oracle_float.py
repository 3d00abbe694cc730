"""The oracle's float mode (the GPU's arithmetic) against its double mode
(the reference's arithmetic) on the same scenes and random streams.

Float differs from double where the reference's formulas lose precision in
float: the quadric roots (solved without cancellation in float) and light
samples leaving a surface at a shallow angle (started off the surface in
float).  With those, per-pixel radiance agrees within 1e-3 relative on all
but a few pixels (silhouettes and exact ties)."""
import os

import numpy as np
import pytest

from sray_gb300 import scenegen


def _agreement(oracle_lib, opts, path):
    imgs = {}
    for fp64 in (True, False):
        o = oracle_lib.Oracle(fp64=fp64, rng_mode=1, **opts)
        o.load(path)
        imgs[fp64] = np.asarray(o.render(0), np.float64)[..., :3]
    a, b = imgs[True], imgs[False]
    rel = np.abs(a - b) / np.maximum(np.abs(a), 1e-3)
    return (rel.max(-1) > 1e-3).mean(), float(np.sqrt(np.mean((a - b) ** 2)))


@pytest.mark.parametrize("name,over", [
    ("small", dict(width=128, height=128)),
    ("learned", dict(width=160, height=90, gi_photons=100000)),
    ("production", dict(width=96, height=54, caust_photons=20000, gi_photons=50000, max_samples=1)),
    ("textured", dict()),
])
def test_float_mode_tracks_double(oracle_lib, name, over, monkeypatch):
    opts = scenegen.scene_opts(name, **over)
    path = scenegen.write_scene(name)
    if name == "textured":      # its images sit beside the scene file
        monkeypatch.setenv("SRAY_DATA_PATH", os.path.dirname(path))
    frac, rmse = _agreement(oracle_lib, opts, path)
    print("%s: pixels over 1e-3 relative %.4f%%, rmse %.2e" % (name, 100 * frac, rmse))
    assert frac <= 2e-3
