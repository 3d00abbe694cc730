"""The radiance cache inside the renderer (opts.nrc), on the learned-gather
scene at reduced resolution.

1. Before any region is validated every region falls back, so the first
   frame with the cache on is the plain final gather's image.
2. What the trained network gains: after online training its image is much
   closer to the FP64 oracle's converged final gather (256 rays per vertex)
   than the plain gather with one ray per vertex, and an untrained network
   is not.
3. Validation catches a wrong network: outputs scaled up push every
   region's validation error over the threshold and the next frame falls
   back to the plain gather.
"""
import numpy as np
import pytest
import torch

from sray_gb300 import scenegen

pytestmark = pytest.mark.gpu

W, H = 320, 180
OPTS = dict(width=W, height=H, gi_photons=200000, nrc_fallback_samples=0)


@pytest.fixture(scope="module")
def learned(gpu_lib, oracle_lib):
    opts = scenegen.scene_opts("learned", **OPTS)
    path = scenegen.write_scene("learned")
    o = dict(opts)
    o["diffuse_samples"] = 256
    orc = oracle_lib.Oracle(fp64=True, rng_mode=1, **o)
    orc.load(path)
    orc.prepare(0)
    ref = np.asarray(orc.render(0), np.float64)
    g = gpu_lib.GpuRenderer(**opts)
    g.load(path)
    fb = torch.zeros((H, W, 4), dtype=torch.float32, device="cuda")
    yield g, fb, ref
    g.close()


def rmse(img, ref):
    d = np.asarray(img, np.float64)[..., :3] - ref[..., :3]
    return float(np.sqrt(np.mean(d * d)))


def frame(g, fb):
    g.render(0, fb)
    return fb.cpu().numpy().copy()


def test_unvalidated_cache_is_the_plain_gather(learned):
    g, fb, _ = learned
    g.set_opts(nrc=0, diffuse_samples=1)
    plain = frame(g, fb)
    g.nrc_reset()
    g.set_opts(nrc=1)
    first = frame(g, fb)
    st = g.nrc_stats()
    assert st["frames"] == 1 and st["cached"] == 0 and st["vertices"] > 0
    assert st["train_samples"] > 0 and st["val_samples"] > 0
    # same rays and gathers; only the order of the accumulators' float atomics differs
    assert np.abs(first - plain).max() <= 1e-5


def test_trained_cache_gains_over_plain_gather(learned):
    g, fb, ref = learned
    g.set_opts(nrc=0, diffuse_samples=1)
    e_plain1 = rmse(frame(g, fb), ref)
    g.set_opts(nrc=0, diffuse_samples=16)
    e_plain16 = rmse(frame(g, fb), ref)
    g.nrc_reset()
    g.set_opts(nrc=2, diffuse_samples=1)
    e_untrained = rmse(frame(g, fb), ref)
    for _ in range(400):
        g.render(0, fb)
    e_cache = rmse(frame(g, fb), ref)
    st = g.nrc_stats()
    print("rmse vs FP64 oracle: plain 1 ray %.5f, plain 16 rays %.5f, untrained cache %.5f, trained cache %.5f "
          "(%d frames, validation error %.3f)" % (e_plain1, e_plain16, e_untrained, e_cache, st["frames"], st["val_rel_err"]))
    assert e_untrained > e_plain1
    assert e_cache < 0.5 * e_plain1
    assert e_cache < e_plain16 * 1.5
    assert st["cached"] == st["vertices"]


def test_validation_catches_a_wrong_network(learned, gpu_lib):
    g, fb, _ = learned
    g.set_opts(nrc=1, diffuse_samples=1)
    for _ in range(50):
        g.render(0, fb)
    before = g.nrc_stats()
    assert before["regions_cached"] > 0 and before["cached"] > 0
    cache = gpu_lib.RadianceCache(seed=None)
    p = cache.params()
    n_w5 = 3 * 64
    # output layer x30: every prediction thirty times too bright.  Training
    # goes on and repairs the network within a few frames, so the first
    # frame's validation (before that frame's training steps) must catch it
    p[-(n_w5 + 3):] *= 30.0
    cache.set_params(p)
    for _ in range(2):
        g.render(0, fb)
    after = g.nrc_stats()
    print("regions served %d -> %d, vertices cached %.3f -> %.3f" % (
        before["regions_cached"], after["regions_cached"], before["cached"] / before["vertices"],
        after["cached"] / after["vertices"]))
    assert after["regions_cached"] == 0
    assert after["cached"] <= 0.02 * after["vertices"]


def test_cache_with_adaptive_sampling_and_two_batches(gpu_lib):
    # the production scene (reduced): two sample batches, area lights; the
    # cache queries both batches, records come from the first, and the
    # frame stays finite and close to the plain gather's (same estimator in
    # expectation; the untrained cache falls back everywhere at first)
    opts = scenegen.scene_opts("production", width=160, height=90, caust_photons=20000, gi_photons=80000, max_samples=4)
    g = gpu_lib.GpuRenderer(**opts)
    g.load(scenegen.write_scene("production"))
    plain = g.render(0)
    g.set_opts(nrc=1)
    g.nrc_reset(5)
    first = g.render(0)
    # nothing validated yet: the plain gather everywhere (up to the order of
    # float atomics, which can tip a pixel's variance test)
    assert (np.abs(first - plain).max(-1) > 1e-5).mean() <= 1e-3
    g.set_opts(nrc=2)
    for _ in range(30):
        img = g.render(0)
    st = g.nrc_stats()
    assert np.isfinite(img).all() and st["cached"] == st["vertices"] > 0 and st["train_samples"] > 0
    d = img[..., :3] - plain[..., :3]
    print("production 160x90, cache after 30 frames: rmse against the plain gather %.4f" % np.sqrt(np.mean(d * d)))
    g.close()


def test_cache_in_a_batch(gpu_lib):
    # the cache inside a batch of frames (one wavefront over the jobs): the
    # first batch, nothing validated, is the plain gather's batch; trained
    # online across batches, every job is served by the network and stays
    # close to its plain-gather frame
    opts = scenegen.scene_opts("production", width=160, height=90, caust_photons=20000, gi_photons=80000, max_samples=4)
    g = gpu_lib.GpuRenderer(**opts)
    g.load(scenegen.write_scene("production"))
    sizes = [(160, 90), (96, 54), (128, 72)]
    fbs = [torch.zeros((h, w, 4), dtype=torch.float32, device="cuda") for w, h in sizes]
    jobs = [(40 * i, fb) for i, fb in enumerate(fbs)]
    g.render_batch(jobs)
    plain = [fb.cpu().numpy().copy() for fb in fbs]
    g.set_opts(nrc=1)
    g.nrc_reset(5)
    g.render_batch(jobs)
    for fb, p in zip(fbs, plain):
        assert (np.abs(fb.cpu().numpy() - p).max(-1) > 1e-5).mean() <= 1e-3
    g.set_opts(nrc=2)
    for _ in range(30):
        g.render_batch(jobs)
    st = g.nrc_stats()
    assert st["frames"] == 31 and st["cached"] == st["vertices"] > 0
    for (w, h), fb, p in zip(sizes, fbs, plain):
        img = fb.cpu().numpy()
        d = img[..., :3] - p[..., :3]
        e = float(np.sqrt(np.mean(d * d)))
        print("batch job %dx%d, cache after 30 batches: rmse against the plain gather %.4f" % (w, h, e))
        assert np.isfinite(img).all() and e < 0.1
    g.close()
