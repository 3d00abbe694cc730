"""Failure detection without a GPU fault: conditions the library detects
and reports, made to happen on the host (malformed scenes, empty light
coverage, no photons, injected allocation failures, a capped ray queue)
or by a wait limit that runs out (the persistent shading pool's bounded
wait).  Each call returns its SRAY_E* code and message, and the context
renders correctly afterwards.  The reference has no failure handling
beyond printing and returning false from its loader (src/scene.cc:79-90)
and signal handlers that exit (src/sray.cc:85-89)."""
import numpy as np
import pytest
import torch

from sray_gb300 import gpu, scenegen

pytestmark = pytest.mark.gpu


def _opts(**over):
    o = scenegen.scene_opts("small", width=96, height=96, caust_photons=20000)
    o.update(over)
    return o


def _raises(code, fn, *a, **kw):
    with pytest.raises(gpu.SrayError) as ei:
        fn(*a, **kw)
    print("%s -> %s" % (getattr(fn, "__name__", fn), ei.value))
    assert ei.value.code == code
    return str(ei.value)


def test_malformed_scene_documents(gpu_lib, small_scene_path):
    g = gpu_lib.GpuRenderer(**_opts())
    good = open(small_scene_path, "rb").read()
    assert "xml:" in _raises(gpu.SRAY_ELOAD, g.load_xml, good[:len(good) // 2])      # cut inside a tag
    assert "end of document" in _raises(gpu.SRAY_ELOAD, g.load_xml, good[:good.rindex(b"</scene>")])
    assert "root element" in _raises(gpu.SRAY_ELOAD, g.load_xml, b"not a scene")
    assert "unknown type" in _raises(gpu.SRAY_ELOAD, g.load_xml, b'<scene><object name="o" type="torus"/></scene>')
    assert _raises(gpu.SRAY_ELOAD, g.load, "/nonexistent/scene.xml")
    # nothing loaded: rendering is refused, not attempted
    _raises(gpu.SRAY_ESTATE, g.render, 0)
    g.load(small_scene_path)
    assert np.isfinite(g.render(0)).all()
    g.close()


def test_no_photons_and_empty_light_coverage(gpu_lib, oracle_lib):
    # caustic photons with no reflective or refractive material: the
    # specular projection map is empty (coverage 0), so photons leave the
    # light in every direction and none is stored (src/light.cc:134-138
    # guards the rejection sampling that would otherwise loop forever)
    xml = scenegen.small_xml_without_specular()
    opts = _opts(caust_photons=20000, gi_photons=20000)
    g = gpu_lib.GpuRenderer(**opts)
    g.load_xml(xml)
    o = oracle_lib.Oracle(fp64=False, rng_mode=1, **opts)
    o.load_xml(xml)
    o.prepare(0)
    img = g.render(0)
    nc, ng = len(g.photons(0)), len(g.photons(1))
    onc, ong, _ = o.photon_info()
    print("caustic %d (oracle %d), global %d (oracle %d)" % (nc, onc, ng, ong))
    assert nc == onc == 0 and ng == ong > 0
    ref = o.render(0)
    rel = np.abs(img[..., :3] - ref[..., :3]) / np.maximum(np.abs(ref[..., :3]), 1e-3)
    assert (rel.max(-1) > 1e-3).mean() <= 1e-3
    # and no photons at all
    g.set_opts(caust_photons=0, gi_photons=0)
    img0 = g.render(0)
    assert len(g.photons(0)) == 0 and len(g.photons(1)) == 0 and np.isfinite(img0).all()
    g.close()


def test_allocation_failure(gpu_lib, small_scene_path):
    g = gpu_lib.GpuRenderer(**_opts())
    g.load(small_scene_path)
    ref = g.render(0)
    # a larger frame needs new buffers: the first allocation fails
    g.set_opts(width=160, height=160)
    g.set_faults(fail_alloc_after=0)
    try:
        msg = _raises(gpu.SRAY_ENOMEM, g.render, 0)
        assert "out of memory" in msg
    finally:
        g.set_faults()
    img = g.render(0)
    assert img.shape == (160, 160, 4) and np.isfinite(img).all()
    g.set_opts(width=96, height=96)
    assert np.abs(g.render(0) - ref).max() == 0.0
    g.close()


def test_queue_overflow(gpu_lib, small_scene_path):
    g = gpu_lib.GpuRenderer(**_opts())
    g.load(small_scene_path)
    ref = g.render(0)
    g.set_faults(queue_cap=64)
    try:
        assert "queue overflow" in _raises(gpu.SRAY_EDEVICE, g.render, 0)
    finally:
        g.set_faults()
    assert np.abs(g.render(0) - ref).max() == 0.0
    g.close()


def test_pool_wait_runs_out(gpu_lib, small_scene_path):
    # the persistent shading pool (every bounce after the first) with its
    # bounded wait cut to one poll: threads that claim a slot whose ray is
    # not written yet give up, the kernel returns, the host reads the error
    # word; no trap, no hang, and the next frame is right
    g = gpu_lib.GpuRenderer(**_opts())
    g.load(small_scene_path)
    g.set_tuning(render_tail=1 << 20)
    ref = g.render(0)
    g.set_faults(pool_spin_limit=1)
    try:
        assert "wait for work ran out" in _raises(gpu.SRAY_EDEVICE, g.render, 0)
    finally:
        g.set_faults()
    img = g.render(0)
    assert np.abs(img - ref).max() <= 1e-6
    g.close()
