"""The allocation-free photon gather against the allocating one.

sray_gpu_photon_gather_noalloc serves callers that cannot allocate device
memory while they run (an application whose device memory belongs to its own
pooling allocator, or a loop that cannot take the synchronisation of a
cudaMalloc).  It stages its requests in a fixed array inside the library
instead of a cudaMalloc'd buffer; its estimates must equal those of
sray_gpu_photon_gather, over two calls in a row on different points (the
second call reuses the array the first one filled), and it must refuse more
points than its fixed capacity.  This file is collected last on purpose.
"""
import numpy as np
import pytest
import torch

from sray_gb300 import scenegen

pytestmark = pytest.mark.gpu

RTOL = 1e-4   # the gather tolerance of test_gpu_parity.py


@pytest.fixture(scope="module")
def renderer(gpu_lib):
    opts = scenegen.scene_opts("small", width=32, height=32, caust_k=0, gi_k=0, gi_photons=40000, gather_dist=0.004)
    g = gpu_lib.GpuRenderer(**opts)
    g.load(scenegen.write_scene("small"))
    nc, ng = g.shoot_photons(0, 0)
    assert nc > 0 and ng > 0
    return g


def _points(g, seed, n):
    ph = g.photons(1)
    rng = np.random.default_rng(seed)
    pts = ph[rng.choice(len(ph), n), :3] + rng.normal(0, 0.01, (n, 3)).astype(np.float32)
    nrm = np.tile(np.array([0.0, 1.0, 0.0], np.float32), (n, 1))
    return torch.tensor(pts, device="cuda"), torch.tensor(nrm, device="cuda")


@pytest.mark.parametrize("which", [0, 1])
def test_noalloc_matches_allocating_gather(renderer, which):
    g = renderer
    for call, (seed, n) in enumerate([(11, 5000), (12, 3000)]):
        pos, nrm = _points(g, seed, n)
        ref = torch.empty((n, 3), dtype=torch.float32, device="cuda")
        out = torch.full((n, 3), -1.0, dtype=torch.float32, device="cuda")
        g.photon_gather(which, pos, nrm, ref)
        g.photon_gather_noalloc(which, pos, nrm, out)
        torch.cuda.synchronize()
        a, b = ref.cpu().numpy(), out.cpu().numpy()
        assert (a != 0).any(axis=1).sum() > 50, "too few non-zero estimates to compare"
        rel = np.abs(a - b) / np.maximum(np.abs(a), 1e-6)
        assert rel.max() <= RTOL, "call %d: max rel %.3g" % (call, rel.max())


def test_noalloc_rejects_oversized_calls(renderer, gpu_lib):
    n = 65536 + 1
    pos = torch.zeros((n, 3), dtype=torch.float32, device="cuda")
    out = torch.empty((n, 3), dtype=torch.float32, device="cuda")
    with pytest.raises(gpu_lib.SrayError, match="capacity"):
        renderer.photon_gather_noalloc(0, pos, pos, out)
