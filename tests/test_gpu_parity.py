"""GPU path against the FP32 oracle on the small scene (512x512 config at
reduced resolution for speed where stated).

Bars: primary-hit object and primitive ids bit-exact except on rays flagged
as exact-t ties; photon maps identical as sets; per-pixel radiance within
1e-3 relative (on 99.9% of pixels; the rest are counted and reported)."""
import os

import numpy as np
import pytest
import torch

from sray_gb300 import scenegen

pytestmark = pytest.mark.gpu

RTOL = 1e-3


def _opts(**over):
    o = scenegen.scene_opts("small")
    o.update(over)
    return o


@pytest.fixture(scope="module")
def small_pair(gpu_lib, oracle_lib, small_scene_path):
    def make(**over):
        opts = _opts(**over)
        g = gpu_lib.GpuRenderer(**opts)
        g.load(small_scene_path)
        o = oracle_lib.Oracle(fp64=False, rng_mode=1, **opts)
        o.load(small_scene_path)
        return g, o
    return make


def test_primary_hits_bit_exact(small_pair):
    g, o = small_pair()
    W, H = g.opts.width, g.opts.height
    n = W * H
    obj = torch.empty(n, dtype=torch.int32, device="cuda")
    prim = torch.empty(n, dtype=torch.int32, device="cuda")
    t = torch.empty(n, dtype=torch.float32, device="cuda")
    tie = torch.empty(n, dtype=torch.uint8, device="cuda")
    g.primary_hits(obj, prim, t, tie)
    torch.cuda.synchronize()
    oobj, oprim, ot, otie = o.primary_hits()
    gobj, gprim, gt, gtie = obj.cpu().numpy(), prim.cpu().numpy(), t.cpu().numpy(), tie.cpu().numpy()
    flagged = (gtie > 0) | (otie > 0)
    mism = (gobj != oobj) | (gprim != oprim)
    print("rays %d hits %d ties %d mismatches %d (unflagged %d)" % (
        n, (oobj >= 0).sum(), flagged.sum(), mism.sum(), (mism & ~flagged).sum()))
    assert (mism & ~flagged).sum() == 0
    hit = (oobj >= 0) & ~mism
    assert np.array_equal(gt[hit], ot[hit].astype(np.float32))


def _same_photons(ph_o, ph_g):
    if len(ph_o) != len(ph_g):
        return False
    ko = np.lexsort(ph_o[:, :12].T[::-1])
    kg = np.lexsort(ph_g[:, :12].T[::-1])
    return np.array_equal(ph_o[ko, :12], ph_g[kg, :12])


def test_photon_maps_identical(small_pair):
    # caustic and global maps: the same photons (position, direction,
    # normal, power) as sets
    g, o = small_pair(gi_photons=60000)
    o.prepare(0)
    nc, ng = g.shoot_photons(0, 0)
    for which, n in ((0, nc), (1, ng)):
        ph_o = o.photons(which)
        ph_g = g.photons(which)
        same = _same_photons(ph_o, ph_g)
        print("%s photons: oracle %d gpu %d identical %s" % (("caustic", "global")[which], len(ph_o), len(ph_g), same))
        assert len(ph_g) == n > 0
        assert same


def _compare(img_g, img_o, label):
    a = img_g[..., :3].astype(np.float64)
    b = img_o[..., :3].astype(np.float64)
    rel = np.abs(a - b) / np.maximum(np.abs(b), 1e-3)
    bad = (rel > RTOL).any(axis=-1)
    frac = bad.mean()
    print("%s: max rel %.3g, pixels over %.0e: %d of %d (%.4f%%)" % (
        label, rel.max(), RTOL, bad.sum(), bad.size, 100 * frac))
    return frac


def test_image_small_scene(small_pair):
    g, o = small_pair(width=256, height=256)
    img_g = g.render(0)
    img_o = o.render(0)
    assert _compare(img_g, img_o, "small 256^2 knn") <= 1e-3


@pytest.mark.parametrize("tuning", [dict(shadow_order=1), dict(stream_priority=1), dict(stream_priority=2),
                                    dict(warp_rays=1 << 24, warp_segments=1 << 24), dict(warp_rays=0, warp_segments=0),
                                    dict(side_gather=1), dict(side_gather=2), dict(queue_depth=4096),
                                    dict(queue_depth=1024, warp_rays=1 << 24, warp_segments=1 << 24),
                                    dict(sort_rays=1), dict(sort_rays=1, queue_depth=4096, warp_rays=0),
                                    dict(side_shadow=1), dict(side_shadow=1, queue_depth=4096, warp_segments=0),
                                    dict(side_shadow=1, render_tail=1 << 20)])
def test_tuning_keeps_the_image(small_pair, tuning):
    # light samples' any-hit traversal in node order instead of nearest
    # first; the photon stream or the frame's own stream given priority;
    # every closest-hit pass traced one ray per warp
    g, o = small_pair(width=192, height=192)
    g.set_tuning(**tuning)
    n = 192 * 192
    gobj, gprim, gt, gtie = _hits(g, n, 0)
    oobj, oprim, ot, otie = o.primary_hits(0)
    mism = ((gobj != oobj) | (gprim != oprim)) & ~((gtie > 0) | (otie > 0))
    assert mism.sum() == 0
    hit = (oobj >= 0) & (gobj == oobj) & (gprim == oprim)
    assert np.array_equal(gt[hit], ot[hit].astype(np.float32))
    img_g = g.render(0)
    img_o = o.render(0)
    assert _compare(img_g, img_o, "small 192^2 %s" % tuning) <= 1e-3
    fb = torch.empty((192, 192, 4), dtype=torch.float32, device="cuda")
    stream = torch.cuda.Stream()
    g.render(0, fb=fb, stream=stream)      # device framebuffer on a caller's stream
    stream.synchronize()
    assert _compare(fb.cpu().numpy(), img_o, "small 192^2 %s, device framebuffer" % tuning) <= 1e-3


def test_image_reference_range_gather(small_pair):
    # the reference's own gather: fixed radius (gather_dist of the scene diagonal), no k
    g, o = small_pair(width=192, height=192, caust_k=0, gather_dist=0.004)
    img_g = g.render(0)
    img_o = o.render(0)
    assert _compare(img_g, img_o, "small 192^2 range") <= 1e-3


def test_image_adaptive_supersampling(small_pair):
    # jittered samples, variance stop rule evaluated sample by sample
    g, o = small_pair(width=128, height=128, max_samples=8, max_var=0.0005)
    img_g = g.render(0)
    img_o = o.render(0)
    assert _compare(img_g, img_o, "small 128^2 1-8 spp") <= 1e-3


@pytest.fixture(scope="module")
def production_pair(gpu_lib, oracle_lib):
    def make(**over):
        opts = scenegen.scene_opts("production")
        opts.update(over)
        path = scenegen.write_scene("production")
        g = gpu_lib.GpuRenderer(**opts)
        g.load(path)
        o = oracle_lib.Oracle(fp64=False, rng_mode=1, **opts)
        o.load(path)
        return g, o
    return make


def test_image_production_reduced(production_pair):
    # terrain + instanced icospheres, sphere lights, global and caustic k-nearest gathers
    g, o = production_pair(width=192, height=108, caust_photons=50000, gi_photons=200000, max_samples=4)
    img_g = g.render(0)
    img_o = o.render(0)
    assert _compare(img_g, img_o, "production 192x108 1-4 spp") <= 1e-3


def test_cast_rays_kats(gpu_lib, oracle_lib):
    import kat_scene
    g = gpu_lib.GpuRenderer(width=32, height=32)
    g.load_xml(kat_scene.XML)
    g.build(0, 0)
    orig, dirs = kat_scene.rays()
    n = len(orig)
    o_t = torch.tensor(orig, dtype=torch.float32, device="cuda")
    d_t = torch.tensor(dirs, dtype=torch.float32, device="cuda")
    tm = torch.zeros(n, dtype=torch.int32, device="cuda")
    obj = torch.empty(n, dtype=torch.int32, device="cuda")
    prim = torch.empty(n, dtype=torch.int32, device="cuda")
    t = torch.empty(n, dtype=torch.float32, device="cuda")
    tie = torch.empty(n, dtype=torch.uint8, device="cuda")
    g.cast_rays(o_t, d_t, tm, obj, prim, t, tie)
    torch.cuda.synchronize()
    bad = kat_scene.check(obj.cpu().numpy(), prim.cpu().numpy(), t.cpu().numpy(), tie.cpu().numpy(), 1e-6)
    assert not bad, bad
    # and bit-exact against the FP32 oracle on the same rays
    o = oracle_lib.Oracle(fp64=False, rng_mode=1, width=32, height=32)
    o.load_xml(kat_scene.XML)
    oo, op, ot, _ = o.cast_rays(orig.astype(np.float32).astype(np.float64), dirs.astype(np.float32).astype(np.float64))
    assert np.array_equal(oo, obj.cpu().numpy()) and np.array_equal(op, prim.cpu().numpy())
    assert np.array_equal(ot.astype(np.float32), t.cpu().numpy())


@pytest.fixture
def textured_pair(gpu_lib, oracle_lib, monkeypatch, tmp_path):
    """The textured scene, its images found through SRAY_DATA_PATH."""
    def make(data_dir=None, **over):
        opts = scenegen.scene_opts("textured", **over)
        path = scenegen.write_scene("textured")
        monkeypatch.setenv("SRAY_DATA_PATH", data_dir or os.path.dirname(path))
        g = gpu_lib.GpuRenderer(**opts)
        g.load(path)
        o = oracle_lib.Oracle(fp64=False, rng_mode=1, **opts)
        o.load(path)
        return g, o
    return make


def test_textured_scene(textured_pair, tmp_path):
    # diffuse, specular, shininess, reflect and ior textures; normal maps on a
    # sphere, on a glass sphere (caustic photons through the bumped surface)
    # and on a mesh with vertex tangents; an untextured "normal" attribute
    # and a texture that fails to load
    g, o = textured_pair()
    o.prepare(0)
    nc, ng = g.shoot_photons(0, 0)
    for which, n in ((0, nc), (1, ng)):
        ph_o, ph_g = o.photons(which), g.photons(which)
        same = _same_photons(ph_o, ph_g)
        print("%s photons: oracle %d gpu %d identical %s" % (("caustic", "global")[which], len(ph_o), len(ph_g), same))
        assert len(ph_g) == n
        assert same
    img_g = g.render(0)
    img_o = o.render(0)
    assert _compare(img_g, img_o, "textured 128x96") <= 1e-3
    # the same scene with no image found: the attributes fall back to their
    # colours, and the picture changes
    g2, _ = textured_pair(data_dir=str(tmp_path))
    img_u = g2.render(0)
    changed = (np.abs(img_u[..., :3] - img_g[..., :3]).max(-1) > 1e-3).mean()
    print("pixels changed by the textures: %.1f%%" % (100 * changed))
    assert changed > 0.2


def test_textured_primary_hits_match_reference(gpu_lib, monkeypatch, tmp_path):
    # primary hits of the textured scene against the reference's own (the
    # golden fixture the oracle is pinned to)
    import gzip
    import json
    here = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
    d = np.load(os.path.join(here, "textured.npz"))
    opts = json.loads(bytes(d["opts"]).decode())
    with gzip.open(os.path.join(here, "textured.xml.gz")) as f:
        xml = f.read()
    scenegen.write_textures(str(tmp_path))
    monkeypatch.setenv("SRAY_DATA_PATH", str(tmp_path))
    g = gpu_lib.GpuRenderer(**opts)
    g.load_xml(xml)
    n = opts["width"] * opts["height"]
    obj = torch.empty(n, dtype=torch.int32, device="cuda")
    prim = torch.empty(n, dtype=torch.int32, device="cuda")
    t = torch.empty(n, dtype=torch.float32, device="cuda")
    tie = torch.empty(n, dtype=torch.uint8, device="cuda")
    g.primary_hits(obj, prim, t, tie)
    torch.cuda.synchronize()
    gobj, gprim = obj.cpu().numpy(), prim.cpu().numpy()
    mism = (gobj != d["obj"]) | (gprim != d["prim"])
    print("textured primary hits: %d mismatches of %d (ties %d)" % (mism.sum(), n, int((tie.cpu().numpy() > 0).sum())))
    assert mism.mean() <= 1e-3


def _hits(g, n, msec):
    obj = torch.empty(n, dtype=torch.int32, device="cuda")
    prim = torch.empty(n, dtype=torch.int32, device="cuda")
    t = torch.empty(n, dtype=torch.float32, device="cuda")
    tie = torch.empty(n, dtype=torch.uint8, device="cuda")
    g.primary_hits(obj, prim, t, tie, msec=msec)
    torch.cuda.synchronize()
    return obj.cpu().numpy(), prim.cpu().numpy(), t.cpu().numpy(), tie.cpu().numpy()


@pytest.mark.parametrize("msec", [0, 350, 1350])
def test_animated_scene(gpu_lib, oracle_lib, msec):
    # transforms evaluated on the device from the keyframe tracks: linear
    # keys repeated past the last one, Catmull-Rom positions, step keys,
    # slerped and lerped rotations, scale about a pivot, a moving light
    opts = dict(width=96, height=72, caust_photons=20000, iter=5)
    path = scenegen.write_scene("animated")
    g = gpu_lib.GpuRenderer(**opts)
    g.load(path)
    o = oracle_lib.Oracle(fp64=False, rng_mode=1, **opts)
    o.load(path)
    n = opts["width"] * opts["height"]
    gobj, gprim, gt, gtie = _hits(g, n, msec)
    oobj, oprim, ot, otie = o.primary_hits(msec)
    mism = ((gobj != oobj) | (gprim != oprim)) & ~((gtie > 0) | (otie > 0))
    print("animated %d ms: %d hits, %d unflagged mismatches" % (msec, int((oobj >= 0).sum()), mism.sum()))
    assert mism.sum() == 0
    img_g = g.render(msec)
    img_o = o.render(msec)
    assert _compare(img_g, img_o, "animated 96x72 at %d ms" % msec) <= 1e-3


def test_animated_primary_hits_match_reference(gpu_lib):
    # primary hits at 1350 ms against the reference's own (golden fixture)
    import gzip
    import json
    here = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
    d = np.load(os.path.join(here, "animated.npz"))
    opts = json.loads(bytes(d["opts"]).decode())
    with gzip.open(os.path.join(here, "animated.xml.gz")) as f:
        xml = f.read()
    g = gpu_lib.GpuRenderer(**opts)
    g.load_xml(xml)
    n = opts["width"] * opts["height"]
    gobj, gprim, gt, gtie = _hits(g, n, int(d["msec"]))
    mism = (gobj != d["obj"]) | (gprim != d["prim"])
    print("animated primary hits vs reference: %d mismatches of %d" % (mism.sum(), n))
    assert mism.mean() <= 1e-3


def test_feature_scene_motion_blur_area_lights(gpu_lib, oracle_lib):
    # sphere + box lights with 2 shadow samples, global photons with 2 final-gather
    # rays, shade_undef material, motion blur over a 40 ms shutter, 1-4 spp
    opts = dict(width=96, height=72, min_samples=1, max_samples=4, max_var=0.01, caust_photons=20000,
                gi_photons=30000, iter=6, shadow_samples=2, diffuse_samples=2, mblur=1, shutter=40, gather_dist=0.02)
    path = scenegen.write_scene("feature")
    g = gpu_lib.GpuRenderer(**opts)
    g.load(path)
    o = oracle_lib.Oracle(fp64=False, rng_mode=1, **opts)
    o.load(path)
    img_g = g.render(0)
    img_o = o.render(0)
    assert _compare(img_g, img_o, "feature 96x72 mblur") <= 1e-3


@pytest.mark.parametrize("k", [0, 50])
def test_photon_gather_points(small_pair, k):
    # irradiance_est / radiance_est at given points: fixed-radius (k=0, the
    # reference) and k-nearest within the radius cap
    g, o = small_pair(width=32, height=32, caust_k=k, gi_k=k, gi_photons=40000, gather_dist=0.004)
    nc, ng = g.shoot_photons(0, 0)
    o.prepare(0)
    ph = o.photons(0)
    rng = np.random.default_rng(7)
    pts = ph[rng.choice(len(ph), 4000), :3].astype(np.float64) + rng.normal(0, 0.01, (4000, 3))
    nrm = np.tile([0.0, 1.0, 0.0], (4000, 1))
    pts32 = pts.astype(np.float32)
    for which in (0, 1):
        out = torch.empty((4000, 3), dtype=torch.float32, device="cuda")
        g.photon_gather(which, torch.tensor(pts32, device="cuda"), torch.tensor(nrm, dtype=torch.float32, device="cuda"), out)
        torch.cuda.synchronize()
        est_g = out.cpu().numpy().astype(np.float64)
        est_o = o.gather(which, pts32.astype(np.float64), nrm)[:, :3]
        rel = np.abs(est_g - est_o) / np.maximum(np.abs(est_o), 1e-6)
        nz = (est_o != 0).any(axis=1).sum()
        print("gather which=%d k=%d: %d nonzero, max rel %.3g" % (which, k, nz, rel.max()))
        assert nz > 100
        assert (rel.max(axis=1) > 1e-4).mean() <= 1e-3


def test_image_vs_fp64_reference(gpu_lib, oracle_lib, small_scene_path):
    # the reference's own arithmetic (double): within 1e-3 relative on all but
    # a few pixels, and the image's RMSE against it
    opts = _opts(width=256, height=256)
    g = gpu_lib.GpuRenderer(**opts)
    g.load(small_scene_path)
    img_g = g.render(0)
    o = oracle_lib.Oracle(fp64=True, rng_mode=1, **opts)
    o.load(small_scene_path)
    img_o = o.render(0)
    d = img_g[..., :3].astype(np.float64) - img_o[..., :3].astype(np.float64)
    print("small 256^2 vs FP64 oracle: rmse %.3g" % np.sqrt(np.mean(d * d)))
    assert _compare(img_g, img_o, "small 256^2 vs FP64") <= 1e-3


def test_autotuner_keeps_the_image(gpu_lib, small_scene_path):
    # the tunables only move work between launches: the image is the same
    opts = _opts(width=128, height=128, max_samples=4, max_var=0.0005)
    g = gpu_lib.GpuRenderer(**opts)
    g.load(small_scene_path)
    fb = torch.zeros((128, 128, 4), dtype=torch.float32, device="cuda")
    g.render(0, fb)
    ref = fb.cpu().numpy().copy()
    best, ms, trials = g.autotune(fb, frames=1)
    print("autotuner: %d trials, best %s at %.3f ms" % (len(trials), best, ms))
    assert len(trials) >= 8 and ms > 0.0
    assert g.tuning() == best
    g.set_tuning(render_tail=1 << 20, pool_blocks_per_sm=1, photon_tail=0)
    g.render(0, fb)
    assert np.abs(fb.cpu().numpy() - ref).max() <= 1e-5
    g.set_tuning(render_tail=0, pool_blocks_per_sm=16, photon_tail=1 << 20)
    g.render(0, fb)
    assert np.abs(fb.cpu().numpy() - ref).max() <= 1e-5


def test_sidecar_load_renders_the_same(gpu_lib, small_scene_path, tmp_path):
    opts = _opts(width=96, height=96)
    g = gpu_lib.GpuRenderer(**opts)
    g.load(small_scene_path)
    ref = g.render(0)
    car = str(tmp_path / "small.srmesh")
    assert not g.load(small_scene_path, sidecar=car)      # written
    assert g.load(small_scene_path, sidecar=car)          # used
    img = g.render(0)
    assert np.abs(img - ref).max() <= 1e-6


def test_photon_dump_restore(small_pair, tmp_path):
    # the reference's dump format round trip: every field comes back within
    # the format's rounding (%f: 5e-7 absolute, plus float rounding); the image moves only by that
    # rounding of the photon powers (~1e-3 of a power)
    g, _ = small_pair(width=128, height=128)
    g.build(0, 0)
    g.shoot_photons(0, 0)
    ref = g.render_pixels(0)
    ph = g.photons(0)
    path = str(tmp_path / "caustics.dump")
    g.dump_photons(0, path)
    lines = open(path).read().splitlines()
    assert lines[0].startswith("energy ") and len(lines) == 1 + len(ph)
    assert lines[1].startswith("<") and lines[1].count("<") == 4
    g.build(0, 0)
    assert g.restore_photons(0, path) == len(ph)
    back = g.photons(0)
    from scipy.spatial import cKDTree
    _, j = cKDTree(back[:, :3].astype(np.float64)).query(ph[:, :3].astype(np.float64))
    assert np.abs(ph[:, :12] - back[j, :12]).max() <= 1e-6
    img = g.render_pixels(0)
    _compare(img, ref, "restored caustic map")
    rel = np.abs(img[..., :3] - ref[..., :3]) / np.maximum(np.abs(ref[..., :3]), 1e-3)
    assert rel.max() <= 1e-2


def test_batch_jobs_match_single_frames(gpu_lib, small_scene_path):
    # jobs of different sizes in one wavefront; at 1 spp without global
    # photons the small scene's image draws nothing per pixel, so each job
    # equals its own single render (job 0 would match at any spp: its
    # pixels keep their streams)
    sizes = [(96, 96), (64, 48), (128, 72)]
    g = gpu_lib.GpuRenderer(**_opts(width=96, height=96))
    g.load(small_scene_path)
    fbs = [torch.zeros((h, w, 4), dtype=torch.float32, device="cuda") for w, h in sizes]
    g.render_batch([(0, fb) for fb in fbs])
    st = g.stats()
    for (w, h), fb in zip(sizes, fbs):
        g.set_opts(width=w, height=h)
        ref = torch.zeros((h, w, 4), dtype=torch.float32, device="cuda")
        g.render(0, ref)
        d = np.abs(fb.cpu().numpy() - ref.cpu().numpy()).max()
        print("batch job %dx%d: max abs difference to its own frame %.3g" % (w, h, d))
        assert d <= 1e-5
    assert st["primary_rays"] == sum(w * h for w, h in sizes)


def test_batch_jobs_match_oracle_mblur_gi_spp(gpu_lib, oracle_lib):
    # a batch of the feature scene (motion blur over a 40 ms shutter, sphere
    # and box lights with 2 samples, global photons with 2 final-gather rays,
    # 1-4 adaptive jittered samples): jobs at different frame times and
    # resolutions, each against the FP32 oracle's frame at its time with its
    # pixels keyed by their place in the batch and its own photon maps
    opts = dict(width=96, height=72, min_samples=1, max_samples=4, max_var=0.01, caust_photons=20000,
                gi_photons=30000, iter=6, shadow_samples=2, diffuse_samples=2, mblur=1, shutter=40, gather_dist=0.02)
    path = scenegen.write_scene("feature")
    jobs = [(0, 96, 72), (40, 64, 48), (100, 128, 96)]    # the loaded aspect (4:3)
    g = gpu_lib.GpuRenderer(**opts)
    g.load(path)
    fbs = [torch.zeros((h, w, 4), dtype=torch.float32, device="cuda") for _, w, h in jobs]
    g.render_batch([(ms, fb) for (ms, _, _), fb in zip(jobs, fbs)])
    st = g.stats()
    assert st["samples"] > sum(w * h for _, w, h in jobs)          # some pixels took more than one sample
    base = 0
    for (ms, w, h), fb in zip(jobs, fbs):
        o = oracle_lib.Oracle(fp64=False, rng_mode=1, **dict(opts, width=w, height=h))
        o.load(path)
        o.set_pixel_base(base)
        img_o = o.render(ms)
        assert _compare(fb.cpu().numpy(), img_o, "batch job %dx%d at %d ms (pixel base %d)" % (w, h, ms, base)) <= 1e-3
        base += w * h


def _read_dump(text):
    """Photons of a dump in the reference's format: energy, then
    <pos> <dir> <norm> <col> per line (src/pmap.cc:180-205)."""
    lines = text.splitlines()
    assert lines[0].startswith("energy ")
    rows = [[float(v) for v in ln.replace("<", " ").replace(">", " ").split()] for ln in lines[1:] if ln.strip()]
    return float(lines[0].split()[1]), np.array(rows, np.float64).reshape(-1, 12)


def test_gpu_restores_reference_dumps(gpu_lib, tmp_path):
    # photon maps the reference itself dumped (PhotonMap::dump, compiled
    # from its sources): the GPU restores every photon, within the format's
    # six decimals, and renders from them as from the reference's photons
    import gzip
    import json
    here = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
    d = np.load(os.path.join(here, "feature.npz"))
    opts = json.loads(bytes(d["opts"]).decode())
    with gzip.open(os.path.join(here, "feature.xml.gz")) as f:
        xml = f.read()
    g = gpu_lib.GpuRenderer(**opts)
    g.load_xml(xml)
    shutter = opts["shutter"]
    g.build(-(shutter // 2), shutter - shutter // 2)
    from scipy.spatial import cKDTree
    for which, name in ((0, "caust"), (1, "gi")):
        path = str(tmp_path / ("%s.dump" % name))
        with gzip.open(os.path.join(here, "feature.%s.dump.gz" % name), "rt") as f:
            text = f.read()
        with open(path, "w") as f:
            f.write(text)
        energy, rows = _read_dump(text)
        n = g.restore_photons(which, path)
        back = g.photons(which).astype(np.float64)
        ref = d[name].astype(np.float64)          # the reference's photons in full precision
        assert n == len(rows) == len(ref) == len(back)
        _, j = cKDTree(back[:, :3]).query(rows[:, :3])
        assert len(np.unique(j)) == len(rows)
        fmt = np.abs(back[j, :12] - rows[:, :12]).max()
        _, k = cKDTree(back[:, :3]).query(ref[:, :3])
        full = np.abs(back[k, :12] - ref[:, :12]).max()
        print("restored %s: %d photons (energy %g); against the dump's text %.2g, against the reference's values %.2g"
              % (name, n, energy, fmt, full))
        assert fmt <= 1e-6 and full <= 1.5e-6


@pytest.mark.parametrize("tuning", [dict(queue_depth=4096), dict(queue_depth=8192, render_tail=1 << 20)],
                         ids=["waves", "waves+pool"])
def test_scene_set_batch_matches_oracle(gpu_lib, oracle_lib, tuning):
    # a scene set (three documents: the small scene, the feature scene with
    # moving objects and area lights, a terrain with instances) and one
    # batch mixing their jobs at different times, resolutions and photon
    # counts, in waves of 4096 primary rays, or of 8192 with each wave's
    # shading tail in the persistent pool launch: each job is its scene's
    # own frame (FP32 oracle, pixels keyed by their place in the batch)
    opts = dict(width=96, height=72, min_samples=1, max_samples=3, max_var=0.01, caust_photons=10000, gi_photons=20000,
                iter=5, shadow_samples=2, diffuse_samples=1, mblur=1, shutter=40, gather_dist=0.02)
    paths = [scenegen.write_scene("small"), scenegen.write_scene("feature"),
             scenegen.write_scene("production", grid=(60, 30), n_inst=12)]
    jobs = [(0, 96, 72, 0, {}), (40, 64, 48, 1, dict(caust_photons=5000, gi_photons=30000)),
            (0, 64, 48, 2, dict(gi_photons=15000)), (100, 96, 72, 1, {}), (0, 48, 36, 0, dict(caust_photons=20000))]
    g = gpu_lib.GpuRenderer(**opts)
    g.load_scene_set(paths)
    g.set_tuning(**tuning)
    fbs = [torch.zeros((h, w, 4), dtype=torch.float32, device="cuda") for _, w, h, _, _ in jobs]
    g.set_profiling(time_kernels=True)
    g.kernel_times(reset=True)
    g.render_batch([(ms, fb, dict(extra, scene=k)) for (ms, _, _, k, extra), fb in zip(jobs, fbs)])
    pool_launches = g.kernel_times(reset=True).get("render_pool", (0.0, 0))[1]
    g.set_profiling(False)
    assert (pool_launches > 0) == ("render_tail" in tuning), pool_launches
    with pytest.raises(gpu_lib.SrayError):
        g.render(0)                                  # a scene set renders through batches only
    base = 0
    for (ms, w, h, k, extra), fb in zip(jobs, fbs):
        o = oracle_lib.Oracle(fp64=False, rng_mode=1, **dict(opts, width=w, height=h, **extra))
        o.load(paths[k])
        o.set_pixel_base(base)
        img_o = o.render(ms)
        assert _compare(fb.cpu().numpy(), img_o, "scene %d job %dx%d at %d ms (pixel base %d)" % (k, w, h, ms, base)) <= 1e-3
        base += w * h


def test_batch_photon_groups_keep_images(gpu_lib):
    # a batch's photon maps traced in groups of jobs (each group its own
    # wavefront, its maps copied out before the next) give the images of
    # the batch traced as one wavefront
    opts = dict(width=96, height=72, min_samples=1, max_samples=3, max_var=0.01, caust_photons=10000, gi_photons=20000,
                iter=5, shadow_samples=2, diffuse_samples=1, mblur=1, shutter=40, gather_dist=0.02)
    paths = [scenegen.write_scene("small"), scenegen.write_scene("feature")]
    jobs = [(0, 96, 72, 0, {}), (40, 64, 48, 1, dict(caust_photons=5000, gi_photons=30000)), (100, 96, 72, 1, {}),
            (0, 48, 36, 0, dict(caust_photons=20000))]
    imgs = []
    for group in (0, 40000):
        g = gpu_lib.GpuRenderer(**opts)
        g.load_scene_set(paths)
        g.set_faults(photon_group=group)
        fbs = [torch.zeros((h, w, 4), dtype=torch.float32, device="cuda") for _, w, h, _, _ in jobs]
        g.render_batch([(ms, fb, dict(extra, scene=k)) for (ms, _, _, k, extra), fb in zip(jobs, fbs)])
        g.set_faults()
        imgs.append([fb.cpu().numpy() for fb in fbs])
        g.close()
    for a, b in zip(*imgs):
        rel = np.abs(a - b) / np.maximum(np.abs(a), 1e-3)
        print("photon groups: max rel difference %.3g" % rel.max())
        assert rel.max() <= 1e-5
