"""A scene given as tables (sray_gpu_upload_scene) renders as the same scene
loaded from its XML document (sray_gpu_load_scene): the same primary hits
and photon maps bit for bit, and the same image up to the order of float
additions into a pixel -- on scenes with
meshes, spheres and a cylinder, sphere and box lights with motion blur and
global photons, keyframed transforms of every kind, and textures with
normal maps."""
import numpy as np
import pytest
import torch

from sray_gb300 import scene_desc, scenegen

pytestmark = pytest.mark.gpu

CASES = [("small", dict(width=96, height=96, caust_photons=20000), 0),
         ("feature", dict(width=96, height=72, min_samples=1, max_samples=4, max_var=0.01, caust_photons=20000,
                          gi_photons=30000, iter=6, shadow_samples=2, diffuse_samples=2, mblur=1, shutter=40,
                          gather_dist=0.02), 0),
         ("animated", dict(width=96, height=72, caust_photons=20000, iter=5), 1350),
         ("textured", dict(width=96, height=72, caust_photons=20000, gi_photons=30000, iter=6, shadow_samples=2,
                           diffuse_samples=2, gather_dist=0.02), 0)]


def _hits(g, n, msec):
    out = [torch.empty(n, dtype=torch.int32, device="cuda"), torch.empty(n, dtype=torch.int32, device="cuda"),
           torch.empty(n, dtype=torch.float32, device="cuda"), torch.empty(n, dtype=torch.uint8, device="cuda")]
    g.primary_hits(*out, msec=msec)
    torch.cuda.synchronize()
    return [x.cpu().numpy() for x in out]


@pytest.mark.parametrize("name,opts,msec", CASES)
def test_upload_renders_as_load(gpu_lib, name, opts, msec, monkeypatch, tmp_path):
    path = scenegen.write_scene(name)
    if name == "textured":
        scenegen.write_textures(str(tmp_path))
        monkeypatch.setenv("SRAY_DATA_PATH", str(tmp_path))
    xml = open(path, "rb").read()
    n = opts["width"] * opts["height"]
    a = gpu_lib.GpuRenderer(**opts)
    a.load_xml(xml)
    hits_a = _hits(a, n, msec)
    img_a = a.render(msec)
    ph_a = [a.photons(w) for w in (0, 1)]
    a.close()
    b = gpu_lib.GpuRenderer(**opts)
    b.upload_scene(scene_desc.from_xml(xml, shutter=opts.get("shutter", 0)))
    info = b.scene_info()
    hits_b = _hits(b, n, msec)
    img_b = b.render(msec)
    ph_b = [b.photons(w) for w in (0, 1)]
    b.close()
    print("%s: %s, image max difference %g, photons %d/%d" % (name, info, np.abs(img_a - img_b).max(), len(ph_b[0]), len(ph_b[1])))
    for x, y in zip(hits_a, hits_b):
        assert np.array_equal(x, y)
    for x, y in zip(ph_a, ph_b):
        assert np.array_equal(x, y)
    # the same frame twice: equal up to the order in which light-sample and
    # gather contributions are added into a pixel (float atomics)
    rel = np.abs(img_a[..., :3] - img_b[..., :3]) / np.maximum(np.abs(img_a[..., :3]), 1e-3)
    assert (rel.max(-1) > 1e-3).mean() <= 1e-3 and np.array_equal(img_a[..., 3], img_b[..., 3])


def test_upload_rejects_bad_tables(gpu_lib):
    from sray_gb300 import gpu
    d = scene_desc.SceneDesc()
    d.add_material("m")
    d.add_object("o", "sphere", material=5)
    g = gpu_lib.GpuRenderer(width=32, height=32)
    with pytest.raises(gpu.SrayError) as ei:
        g.upload_scene(d)
    assert ei.value.code == gpu.SRAY_EINVAL and "material index" in str(ei.value)
    g.close()
