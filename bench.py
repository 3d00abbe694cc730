#!/usr/bin/env python
"""Frame benchmark of the GB300 renderer on the seeded production scene.

A step is one full frame through the renderer's own entry point
(sray_gpu_render: top-level octree build, projection maps, caustic and
global photon maps traced and sorted on the device, then the adaptive
<=16 spp wavefront render) with the scene resident in HBM.

Reported value: Mrays/s = every segment traced through cast_ray (primary,
secondary incl. final-gather rays, shadow rays) per second of frame time,
with ms/frame beside it.  The JSON line also carries:
  e2e          the same metric through the C-ABI with a HOST framebuffer
               (device->host copy and per-frame table uploads inside the timing)
  roofline     live CUDA-event time of the dominant kernel against its
               algorithmic bytes (counted in an untimed pass) and the
               measured HBM peak
  cpu_baseline the CPU restatement of the reference's path, FP64, all host
               threads, on a bounded sample of the same frame (see `sample`)
  clocks       nvidia-smi samples taken during the timed region

--impl reference times that CPU path alone, on the same metric.
"""
import argparse
import json
import os
import re
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Mrays/s & ms/frame at equal RMSE vs FP64 oracle: NRC vs plain gather, 1 GB300"
PEAKS_PATH = os.path.join(ROOT, "MEASURED_PEAKS.json")
FALLBACK_HBM = 6800.0


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", default="production",
                    choices=["production", "small", "learned", "stress", "batch", "stress-batch", "nrc-infer"])
    ap.add_argument("--nrc-samples", type=int, default=1 << 22,
                    help="samples per launch of the nrc-infer configuration (the default's 151 MB of inputs exceed the L2)")
    ap.add_argument("--batch-frames", type=int, default=16, help="frames per batch of the stress-batch configuration")
    ap.add_argument("--batch-jobs", type=int, default=64, help="jobs of the batch configuration")
    ap.add_argument("--batch-scenes", type=int, default=16, help="scenes of the batch configuration's scene set")
    ap.add_argument("--queue-depth", type=int, default=None,
                    help="primary rays per wave: of the batch configuration before (or without) autotuning "
                         "(default 2^20), of the stress-batch configuration (default 2^24)")
    ap.add_argument("--no-nrc", action="store_true", help="skip the radiance-cache comparison")
    ap.add_argument("--method", default="plain", choices=["plain", "cache", "cache-everywhere"],
                    help="final gather of the headline frames: the plain gather, the radiance cache with its "
                         "per-region fallback, or the cache in every region")
    ap.add_argument("--no-autotune", action="store_true", help="keep the default scheduler tuning")
    ap.add_argument("--tuning", default=None,
                    help="render_tail,pool_blocks_per_sm,photon_tail[,shadow_order[,stream_priority[,warp_rays"
                         "[,warp_segments[,side_gather[,sort_rays[,side_shadow]]]]]]]: set the scheduler tuning instead "
                         "of autotuning")
    ap.add_argument("--nrc-burn-in", type=int, default=600, help="frames of online training before the cache is timed")
    ap.add_argument("--nrc-ladder", default="1,2,4,8,16,32,64,128",
                    help="diffuse samples per vertex of the plain final gather, compared with the cache")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-rows", type=int, default=4, help="rows per band of the CPU baseline sample (16 bands)")
    ap.add_argument("--cpu-full-frame", action="store_true",
                    help="reference arm: also render one whole frame on the CPU and compare it with the projection")
    ap.add_argument("--no-parity", action="store_true", help="skip the untimed parity leg against the FP32 oracle")
    ap.add_argument("--res", default=None, help="WxH override (profiling runs on a reduced case)")
    ap.add_argument("--photon-scale", type=float, default=1.0, help="photon count multiplier (profiling)")
    return ap.parse_args()


def config_opts(args):
    from sray_gb300 import scenegen
    opts = scenegen.scene_opts(args.config)
    if args.res:
        w, h = args.res.lower().split("x")
        opts["width"], opts["height"] = int(w), int(h)
    if args.photon_scale != 1.0:
        opts["caust_photons"] = int(opts["caust_photons"] * args.photon_scale)
        opts["gi_photons"] = int(opts["gi_photons"] * args.photon_scale)
    method = getattr(args, "method", "plain")
    if method != "plain":
        opts["nrc"] = 1 if method == "cache" else 2
    return opts


def workload_desc(cfg):
    if cfg == "stress":
        return ("stress: 3840x2160, adaptive 1-16 spp (variance 0.05), depth 8, 4x4 displaced-grid terrain tiles "
                "(10M triangles) + 2000 instanced icospheres (10% moving over a 40 ms shutter, motion blur on), "
                "3 sphere lights, 20M global + 4M caustic photons, k=100 gathers within r<=0.5")
    if cfg == "learned":
        return ("learned gather: the small scene at 1920x1080, 1 spp, depth 5, 100k caustic photons (k=50), "
                "500k global photons (k=100 nearest within r<=0.5), final gather of indirect light by the radiance "
                "cache (12-band encoding, 4x64 ReLU, BF16 weights, FP32 accumulation, Adam 1e-3, 65,536 training "
                "vertices per frame, per-region fallback to the plain gather with 16 rays per vertex above 0.05 validation error) vs the plain photon gather")
    if cfg == "production":
        return ("production: 1920x1080, adaptive 1-16 spp (variance 0.05), depth 8, 1M-triangle displaced-grid "
                "terrain + 200 instanced icospheres (256k tris), 3 sphere lights, 2M global + 500k caustic photons, "
                "k=100 nearest-photon gathers within r<=0.5")
    return ("small: 512x512, 1 spp, depth 5, ground + 16 spheres + icosphere(4) + cylinder, point light, "
            "100k caustic photons, k=50 gather")


def reduce_over_ranks(ms_total, rays, e2e_s, e2e_rays, device="cpu"):
    """Replicas: the job's time is the slowest rank's, its work the sum of
    all ranks' (so value = all rays / max time)."""
    import torch
    import torch.distributed as dist
    t = torch.tensor([ms_total, rays, e2e_s, e2e_rays], dtype=torch.float64, device=device)
    tmax, tsum = t.clone(), t.clone()
    dist.all_reduce(tmax, op=dist.ReduceOp.MAX)
    dist.all_reduce(tsum, op=dist.ReduceOp.SUM)
    return float(tmax[0]), float(tsum[1]), float(tmax[2]), float(tsum[3])


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class ClockSampler:
    """nvidia-smi samples (200 ms) of SM clock, max clock and throttle reasons."""

    def __init__(self, index):
        self.index = index
        self.samples = []
        self.proc = None
        self.thread = None

    def start(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return

        def rd():
            for line in self.proc.stdout:
                self.samples.append([x.strip() for x in line.split(",")])
        self.thread = threading.Thread(target=rd, daemon=True)
        self.thread.start()

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for s in self.samples:
            try:
                sm.append(float(s[1]))
                mx.append(float(s[2]))
            except (ValueError, IndexError):
                continue
            for k, nm in enumerate(names):
                if len(s) > 5 + k and s[5 + k].lower().startswith("active"):
                    reasons.add(nm)
        sm.sort()
        return {"sm_mhz": sm[len(sm) // 2] if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def peaks():
    try:
        with open(PEAKS_PATH) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return FALLBACK_HBM, "fallback"


def bf16_peak():
    try:
        with open(PEAKS_PATH) as f:
            return float(json.load(f)["bf16_tflops"])
    except (OSError, KeyError, ValueError):
        return 1900.0


def algorithmic_bytes(st):
    """Algorithmic bytes of a frame per kernel kind, from the counted pass:
    (bytes, units, unit name, description)."""
    rays = st["primary_rays"] + st["secondary_rays"]
    return {
        "trace": (rays * (48 + 16) + st["node_visits"] * 128 + st["prim_tests"] * 48, rays, "rays",
                  "48 B ray + 16 B hit per ray, 128 B per 4-wide node read, 48 B per triangle tested"),
        "shadow": (st["shadow_rays"] * (48 + 16) + st["shadow_node_visits"] * 128 + st["shadow_prim_tests"] * 48,
                   st["shadow_rays"], "segments",
                   "48 B request + 16 B accumulator per light-sample segment, 128 B per node read, 48 B per triangle tested"),
        "gather": (st["gathers"] * (48 + 16 + 64) + st["gather_tested"] * 16 + st["gather_candidates"] * 32,
                   st["gathers"], "queries",
                   "48 B request + 16 B accumulator + 8 cells x 8 B per query, 16 B position per photon tested, "
                   "32 B more per photon within range"),
    }


PROFILE_TABLE = os.path.join(ROOT, "profiles", "roofline_kernels_960x540.md")


def committed_profile(kind):
    """Figures of the committed ncu capture for a kernel kind: machine-read
    lines `<kind>.<figure>: <value>` in the profile summary."""
    out = {"source": None}
    try:
        text = open(PROFILE_TABLE).read()
    except OSError:
        return out
    out["source"] = os.path.relpath(PROFILE_TABLE, ROOT)
    for key in ("dram_bytes_per_unit", "threads_per_instruction", "issue_active"):
        m = re.search(r"^%s\.%s:\s*([0-9.eE+-]+)" % (re.escape(kind), key), text, re.M)
        out[key] = float(m.group(1)) if m else None
    return out


def rays_of(st):
    return st["primary_rays"] + st["secondary_rays"] + st["shadow_rays"]


CPU_BANDS = 16


def band_rows(h, n=CPU_BANDS, rows=4):
    """n bands of `rows` image rows spread evenly over an image of h rows."""
    step = max(h // n, rows)
    return [(y, min(y + rows, h)) for y in range(step // 2 - rows // 2, h - rows + 1, step)][:n]


def cpu_sample(orc, h, bands, threads=0):
    """One bounded sample of the frame on the CPU restatement: prepare the
    frame (scene tree, projection maps, photon maps at the oracle's photon
    counts) and render the row bands.  Returns the phase times (s), the
    rays traced on the bands and their image."""
    import numpy as np
    t0 = time.perf_counter()
    orc.prepare(0)
    t_prep = time.perf_counter() - t0
    ph = orc.phase_ms()
    rows = [y for b0, b1 in bands for y in range(b0, b1)]
    t0 = time.perf_counter()
    img = orc.render_rows(rows, nthreads=threads)
    t_rows = time.perf_counter() - t0
    rays = orc.counters()["rays"]
    return {"prepare_s": t_prep, "build_s": ph["build"] / 1e3, "projmaps_s": ph["projmaps"] / 1e3,
            "photons_s": ph["photons"] / 1e3, "rows_s": t_rows, "rays": rays,
            "rows": sum(b1 - b0 for b0, b1 in bands), "image": img}


def cpu_baseline(opts, path, bands, threads=0):
    """The CPU restatement of the reference's path (FP64, all host threads)
    on a bounded sample of the frame: the frame's full preparation (scene
    tree, projection maps, both photon maps at full size: measured, not
    extrapolated) and the rows of `bands` spread over the image; the frame
    time is the preparation plus the rows' time scaled by the image's rows.
    Also returns the FP64 image of the bands (the RMSE reference)."""
    from oracle.oracle import Oracle
    o_opts = dict(opts)
    o_opts["threads"] = threads
    orc = Oracle(fp64=True, rng_mode=1, **o_opts)
    orc.load(path)
    h = opts["height"]
    smp = cpu_sample(orc, h, bands, threads)
    scale_rows = h / smp["rows"]
    t_frame = smp["prepare_s"] + smp["rows_s"] * scale_rows
    rays_frame = smp["rays"] * scale_rows
    cores = threads if threads > 0 else (os.cpu_count() or 1)
    return {
        "value": rays_frame / t_frame / 1e6, "unit": "Mrays/s", "cores": cores, "kind": "port",
        "ms_per_frame": t_frame * 1e3,
        "sample": "the frame's full preparation measured (%.1f s: scene tree %.1f, projection maps %.1f, %d+%d photons "
                  "traced and stored %.1f) and %d rows in %d bands spread over the %d-row image (%.1f s), the rows "
                  "scaled to the image; CPU restatement of the reference's path in FP64"
                  % (smp["prepare_s"], smp["build_s"], smp["projmaps_s"], opts["caust_photons"], opts["gi_photons"],
                     smp["photons_s"], smp["rows"], len(bands), h, smp["rows_s"]),
        "wall_s": smp["prepare_s"] + smp["rows_s"],
        "phases_s": {k: round(smp[k], 3) for k in ("build_s", "projmaps_s", "photons_s", "rows_s")},
    }, smp["image"]


def fp64_image_check(img, ref, bands):
    """The GPU frame's RMSE against the FP64 oracle (the reference's
    arithmetic, same seeds and photon counts) on the row bands, and the
    share of those pixels over 1e-3 relative."""
    import numpy as np
    rows = np.concatenate([np.arange(a, b) for a, b in bands])
    a = np.asarray(img, np.float64)[rows, :, :3]
    r = np.asarray(ref, np.float64)[rows, :, :3]
    rel = np.abs(a - r) / np.maximum(np.abs(r), 1e-3)
    return {"rmse": float(np.sqrt(np.mean((a - r) ** 2))), "pixels_over_1e-3": float((rel.max(-1) > 1e-3).mean()),
            "rows": len(rows), "bands": [list(b) for b in bands],
            "reference": "FP64 CPU oracle, same seeds and photon counts"}


def parity_leg(opts, path, g, img, bands):
    """Parity of the headline frame against the FP32 oracle (the GPU's
    arithmetic, same seeds and photon counts), untimed: primary-hit ids of
    every pixel (bit-exact except rays either side flags as an exact-t tie),
    both photon maps as sets, and the image within 1e-3 relative on the row
    bands."""
    import numpy as np
    import torch
    from oracle.oracle import Oracle
    H, W = opts["height"], opts["width"]
    t_start = time.perf_counter()
    o = Oracle(fp64=False, rng_mode=1, **opts)
    o.load(path)
    n = W * H
    obj = torch.empty(n, dtype=torch.int32, device="cuda")
    prim = torch.empty(n, dtype=torch.int32, device="cuda")
    t = torch.empty(n, dtype=torch.float32, device="cuda")
    tie = torch.empty(n, dtype=torch.uint8, device="cuda")
    g.primary_hits(obj, prim, t, tie)
    torch.cuda.synchronize()
    gobj, gprim, gt, gtie = obj.cpu().numpy(), prim.cpu().numpy(), t.cpu().numpy(), tie.cpu().numpy()
    oobj, oprim, ot, otie = o.primary_hits(0)
    flagged = (gtie > 0) | (otie > 0)
    mism = (gobj != oobj) | (gprim != oprim)
    same_t = (oobj >= 0) & ~mism & ~flagged
    maps = {}
    for which, name in ((0, "caustic"), (1, "global")):
        pg, po = g.photons(which), o.photons(which)
        same = len(pg) == len(po) and np.array_equal(po[np.lexsort(po[:, :12].T[::-1]), :12],
                                                      pg[np.lexsort(pg[:, :12].T[::-1]), :12])
        maps[name] = {"gpu": int(len(pg)), "oracle": int(len(po)), "identical": bool(same)}
    rows = np.concatenate([np.arange(a, b) for a, b in bands])
    ref = o.render_rows(rows)
    a = np.asarray(img, np.float64)[rows, :, :3]
    r = ref[rows, :, :3].astype(np.float64)
    rel = np.abs(a - r) / np.maximum(np.abs(r), 1e-3)
    over = rel.max(-1) > 1e-3
    return {"reference": "FP32 CPU oracle (the GPU's float arithmetic and path-keyed streams), same seeds and photon counts",
            "pixels": int(n), "primary_hits": int((oobj >= 0).sum()),
            "primary_mismatches": int(mism.sum()), "primary_unflagged_mismatches": int((mism & ~flagged).sum()),
            "ties": int(flagged.sum()), "primary_t_bit_exact": bool(np.array_equal(gt[same_t], ot[same_t].astype(np.float32))),
            "photon_maps": maps,
            "image_rows": int(len(rows)), "image_bands": len(bands),
            "image_pixels_over_1e-3": float(over.mean()), "image_max_rel": float(rel.max()),
            "pass": bool((mism & ~flagged).sum() == 0 and over.mean() <= 1e-3),
            "s": time.perf_counter() - t_start}


REF_DS = 256
REF_PHOTON_FRAC = 0.1
REF_BANDS = 16


def reference_bands(h, n=REF_BANDS, rows=8):
    """Row bands (y0, y1) spread evenly over an image of h rows."""
    step = max(h // n, rows)
    return [(y, min(y + rows, h)) for y in range(step // 2 - rows // 2, h - rows + 1, step)][:n]


def oracle_reference_rows(opts, path, ds=REF_DS, bands=None, threads=0):
    """The FP64 CPU oracle's image on row bands with `ds` final-gather rays
    per vertex: the converged reference of the final-gather estimators
    (same scene, photon maps, lights and camera).  Returns (image, rows, s)."""
    import numpy as np
    from oracle.oracle import Oracle
    o = dict(opts)
    o["diffuse_samples"] = ds
    o["threads"] = threads
    h, w = opts["height"], opts["width"]
    bands = bands or reference_bands(h)
    t0 = time.perf_counter()
    orc = Oracle(fp64=True, rng_mode=1, **o)
    orc.load(path)
    orc.prepare(0)
    rows = np.concatenate([np.arange(a, b) for a, b in bands])
    ref = np.asarray(orc.render_rows(rows, nthreads=threads), np.float64)
    return ref, rows, time.perf_counter() - t0


def image_rmse(img, ref, rows):
    import numpy as np
    d = np.asarray(img, np.float64)[rows, :, :3] - ref[rows, :, :3]
    return float(np.sqrt(np.mean(d * d)))


def equal_rmse_time(ladder, target):
    """Frame time of the plain method at the cache's RMSE: ladder = [(ds, ms,
    rmse)] with rmse falling as ds grows; interpolated linearly in log rmse
    against log ds, the time linearly in ds.  Returns (ms, ds, bracketed):
    bracketed False means the target lies outside the ladder, and the
    nearest end is returned (a bound, not an estimate)."""
    import math
    pts = sorted(ladder)
    if not pts:
        return None, None, False
    if target >= pts[0][2]:
        return pts[0][1], pts[0][0], target == pts[0][2]
    for (d0, m0, r0), (d1, m1, r1) in zip(pts, pts[1:]):
        if r0 >= target >= r1 and r0 > r1:
            f = (math.log(r0) - math.log(target)) / (math.log(r0) - math.log(r1))
            ds = math.exp(math.log(d0) + f * (math.log(d1) - math.log(d0)))
            ms = m0 + (ds - d0) / (d1 - d0) * (m1 - m0)
            return ms, ds, True
    return pts[-1][1], pts[-1][0], False


def nrc_vs_plain(args, reference):
    """Radiance cache vs the plain final gather on the learned-gather scene:
    the plain method's RMSE and frame time for each number of final-gather
    rays per vertex, the cache's after `--nrc-burn-in` frames of online
    training (timed frames keep training), and the plain frame time at the
    cache's RMSE.  reference = (image, rows) of the FP64 oracle, or None."""
    import numpy as np
    import torch
    from sray_gb300 import gpu, scenegen

    opts = scenegen.scene_opts("learned")
    path = scenegen.write_scene("learned")
    H, W = opts["height"], opts["width"]
    g = gpu.GpuRenderer(**opts)
    g.load(path)
    fb = torch.zeros((H, W, 4), dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream()
    steps = max(args.steps, 3)

    def timed(n):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        rays = 0
        for _ in range(n):
            g.render(0, fb, stream=stream)
            rays += rays_of(g.stats())
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / n
        return ms, rays / n / (ms / 1e3) / 1e6

    def err():
        if reference is None:
            return None
        return image_rmse(fb.cpu().numpy(), reference[0], reference[1])

    tuning = None
    if not args.no_autotune:
        g.set_opts(nrc=0, diffuse_samples=1)
        best, best_ms, _ = g.autotune(fb, frames=3, stream=stream)
        tuning = dict(best, ms_per_frame=best_ms)
    ladder = []
    for ds in [int(x) for x in args.nrc_ladder.split(",") if x]:
        g.set_opts(nrc=0, diffuse_samples=ds)
        for _ in range(2):
            g.render(0, fb, stream=stream)
        ms, mr = timed(steps)
        ladder.append({"diffuse_samples": ds, "ms_per_frame": ms, "mrays_per_s": mr, "rmse": err()})
    out = {"workload": workload_desc("learned"), "tuning": tuning, "plain": ladder,
           "reference": None if reference is None else
           "FP64 CPU oracle, %d final-gather rays per vertex, %d rows in %d bands" % (REF_DS, len(reference[1]), REF_BANDS)}
    g.set_opts(nrc=1, diffuse_samples=1)
    g.nrc_reset()
    t0 = time.perf_counter()
    for _ in range(args.nrc_burn_in):
        g.render(0, fb, stream=stream)
    torch.cuda.synchronize()
    burn_s = time.perf_counter() - t0
    for mode, name in ((1, "cache"), (2, "cache_no_fallback")):
        g.set_opts(nrc=mode)
        for _ in range(3):
            g.render(0, fb, stream=stream)
        ms, mr = timed(steps)      # as the plain ladder: without per-launch events
        g.set_profiling(time_kernels=True)
        g.kernel_times(reset=True)
        timed(steps)               # the same frames again for the kernels' durations
        kt = g.kernel_times(reset=True)
        g.set_profiling(False)
        st = g.nrc_stats()
        res = {"mode": mode, "ms_per_frame": ms, "mrays_per_s": mr, "rmse": err(),
               "cached_vertex_frac": st["cached"] / max(st["vertices"], 1), "frames_trained": st["frames"],
               "train_samples_per_frame": st["train_samples"], "val_samples_per_frame": st["val_samples"],
               "regions_validated": st["regions_validated"], "regions_cached": st["regions_cached"],
               "val_rel_err": st["val_rel_err"], "loss": st["loss"],
               "nrc_ms_per_frame": {k: round(v[0] / steps, 3) for k, v in kt.items() if k.startswith("nrc")},
               "gather_ms_per_frame": round(kt.get("gather", (0.0, 0))[0] / steps, 3)}
        # roofline of the query kernel: 2 x 26,304 FLOP per query against the measured bf16 peak
        q_ms = kt.get("nrc_query", (0.0, 0))[0] / steps
        if q_ms > 0 and st["cached"] > 0:
            tf = st["cached"] * 2 * 26304 / (q_ms / 1e3) / 1e12
            res["query_roofline"] = {"bound": "tensor", "achieved": tf, "peak": bf16_peak(), "unit": "TFLOP/s",
                                     "frac": tf / bf16_peak(), "queries_per_frame": st["cached"], "ms_per_frame": q_ms}
        # and of the frame's training steps: forward, backward and weight
        # gradients, about 3 x 2 x 26,304 FLOP per training sample
        t_ms = kt.get("nrc_train", (0.0, 0))[0] / steps
        if t_ms > 0 and st["train_samples"] > 0:
            tf = st["train_samples"] * 3 * 2 * 26304 / (t_ms / 1e3) / 1e12
            res["train_roofline"] = {"bound": "tensor", "achieved": tf, "peak": bf16_peak(), "unit": "TFLOP/s",
                                     "frac": tf / bf16_peak(), "samples_per_frame": st["train_samples"], "ms_per_frame": t_ms,
                                     "kernels": "warp-level mma.sync forward, backward and weight-gradient kernels and Adam, "
                                                "one CUDA graph per frame"}
        if res["rmse"] is not None:
            pts = [(p["diffuse_samples"], p["ms_per_frame"], p["rmse"]) for p in ladder]
            pms, pds, ok = equal_rmse_time(pts, res["rmse"])
            res["plain_at_equal_rmse"] = {"ms_per_frame": pms, "diffuse_samples": pds, "bracketed": ok,
                                          "time_ratio": ms / pms if pms else None}
        out[name] = res
    out["burn_in"] = {"frames": args.nrc_burn_in, "s": burn_s}
    g.close()
    return out


BATCH_SIZES = [(256, 256), (512, 512), (1280, 720), (1920, 1080)]


def batch_workload(n_jobs, n_scenes, seed=0x5EED0B):
    """The batched configuration: n_scenes seeded terrain-plus-moving-spheres
    scenes with triangle counts log-uniform in [10k, 2M]; n_jobs jobs, job j
    rendering scene j mod n_scenes at animation frame j div n_scenes (40 ms
    apart), its resolution drawn from 256^2, 512^2, 720p and 1080p, its
    photon count log-uniform in [100k, 2M] (a fifth caustic)."""
    import numpy as np
    rng = np.random.default_rng(seed)
    tris = np.exp(rng.uniform(np.log(1e4), np.log(2e6), n_scenes)).astype(int)
    sizes = [BATCH_SIZES[int(k)] for k in rng.integers(0, len(BATCH_SIZES), n_jobs)]
    photons = np.exp(rng.uniform(np.log(1e5), np.log(2e6), n_jobs)).astype(int)
    jobs = [dict(scene=j % n_scenes, msec=40 * (j // n_scenes), width=sizes[j][0], height=sizes[j][1],
                 caust_photons=int(photons[j] // 5), gi_photons=int(photons[j] - photons[j] // 5)) for j in range(n_jobs)]
    return [int(t) for t in tris], jobs


def run_batch(args):
    """Batched rendering: `--batch-jobs` jobs over a scene set of
    `--batch-scenes` scenes (batch_workload), motion blur over an 8 ms shutter
    (8 time samples), adaptive 1-16 spp, in one wavefront per batch
    (sray_gpu_render_batch) after the batch autotuner has picked the queue
    depth (65,536 / 262,144 / 1,048,576 primary rays per wave) and the
    traversal mode (thread per ray / warp per ray in the tails / warp per ray
    everywhere); against the same jobs rendered one frame at a time with
    sray_gpu_render, each scene loaded alone."""
    import torch
    from sray_gb300 import build as gbuild, gpu, scenegen
    torch.cuda.set_device(0)
    gbuild.build()
    tris, jobs = batch_workload(args.batch_jobs, args.batch_scenes)
    t0 = time.perf_counter()
    paths = [scenegen.write_scene("batch", seed=1000 + k, tris=t) for k, t in enumerate(tris)]
    gen_s = time.perf_counter() - t0
    opts = scenegen.scene_opts("production", mblur=1, shutter=8)
    g = gpu.GpuRenderer(**opts)
    t0 = time.perf_counter()
    g.load_scene_set(paths)
    load_s = time.perf_counter() - t0
    stream = torch.cuda.current_stream()
    fbs = [torch.zeros((J["height"], J["width"], 4), dtype=torch.float32, device="cuda") for J in jobs]
    spec = [(J["msec"], fb, dict(scene=J["scene"], caust_photons=J["caust_photons"], gi_photons=J["gi_photons"]))
            for J, fb in zip(jobs, fbs)]
    free0 = torch.cuda.mem_get_info()[0]

    def timed(fn, n):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        rays = 0
        for _ in range(n):
            rays += fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / n, rays / n

    def batch():
        g.render_batch(spec, stream=stream)
        return rays_of(g.stats())


    g.set_tuning(queue_depth=args.queue_depth or 1 << 20)      # bounded queues from the first batch on
    batch()
    tuning = None
    if not args.no_autotune:
        best, best_ms, trials = g.autotune_batch(spec, frames=1, stream=stream)
        tuning = {"chosen": best, "ms_per_batch": best_ms,
                  "trials": [dict(queue_depth=t["queue_depth"], warp_rays=t["warp_rays"], render_tail=t["render_tail"], ms=round(ms, 2)) for t, ms in trials]}
    for _ in range(args.warmup):
        batch()
    device_mb = (free0 - torch.cuda.mem_get_info()[0]) / 1e6
    clocks = ClockSampler(torch.cuda.current_device())
    clocks.start()
    ms_b, rays_b = timed(batch, args.steps)
    clk = clocks.stop()
    st = g.stats()
    # where a batch's time goes: kernel event times of one more batch
    g.set_profiling(time_kernels=True)
    g.kernel_times(reset=True)
    batch()
    kt_all = g.kernel_times(reset=True, host=True)
    kt = {k: v for k, v in kt_all.items() if not k.startswith("host.")}
    g.set_profiling(False)
    g.close()
    # the same jobs one frame at a time, as the reference renders them: each
    # scene loaded alone (untimed), its jobs rendered with sray_gpu_render
    ms_s, rays_s = 0.0, 0
    for k, p in enumerate(paths):
        mine = [J for J in jobs if J["scene"] == k]
        if not mine:
            continue
        g1 = gpu.GpuRenderer(**opts)
        g1.load(p)
        fb = torch.zeros((1080, 1920, 4), dtype=torch.float32, device="cuda")
        for J in mine:
            g1.set_opts(width=J["width"], height=J["height"], caust_photons=J["caust_photons"], gi_photons=J["gi_photons"])
            view = fb.view(-1)[:J["width"] * J["height"] * 4].view(J["height"], J["width"], 4)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            e0.record(stream)
            g1.render(J["msec"], view, stream=stream)
            e1.record(stream)
            torch.cuda.synchronize()
            ms_s += e0.elapsed_time(e1)
            rays_s += rays_of(g1.stats())
        g1.close()
    line = {
        "metric": METRIC, "value": rays_b / (ms_b / 1e3) / 1e6, "unit": "Mrays/s", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_b, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic (seeded scene generator, no dataset)",
        "config": {"workload": "batch: %d jobs over %d scenes (terrain + 24 moving spheres, %d to %d triangles, %.1fM in "
                               "all), each job a scene at its own animation frame, resolution from 256^2, 512^2, 1280x720, "
                               "1920x1080, 100k-2M photons, motion blur over an 8 ms shutter (8 time samples), adaptive "
                               "1-16 spp, depth 8, k=100 gathers within r<=0.5; one wavefront per batch"
                               % (len(jobs), len(tris), min(tris), max(tris), sum(tris) / 1e6),
                   "method": "plain gather", "tuning": tuning,
                   "pixels": sum(J["width"] * J["height"] for J in jobs),
                   "photons": sum(J["caust_photons"] + J["gi_photons"] for J in jobs)},
        "kernels_ms_per_batch": {k: round(v[0], 2) for k, v in kt.items()},
        "host_ms_per_batch": {k[5:]: [round(v[0], 2), v[1]] for k, v in kt_all.items() if k.startswith("host.")},
        "batch_vs_single": {"batch_ms": ms_b, "jobs_one_at_a_time_ms": ms_s, "speedup": ms_s / ms_b,
                            "batch_mrays_per_s": rays_b / (ms_b / 1e3) / 1e6,
                            "single_mrays_per_s": rays_s / (ms_s / 1e3) / 1e6},
        "frame": {"rays": rays_of(st), "primary": st["primary_rays"], "samples": st["samples"],
                  "device_mb": device_mb, "load_s": load_s, "scene_gen_s": gen_s},
        "gpu_launches": st["kernel_launches"], "clocks": clk,
        "e2e": None, "roofline": None, "cpu_baseline": None,
        "note": "a step renders every job once; e2e, roofline and the CPU baseline are reported for the production "
                "configuration; per-job parity of scene-set batches against the FP32 oracle is "
                "tests/test_gpu_parity.py::test_scene_set_batch_matches_oracle",
    }
    print(json.dumps(line))
    return 0


def run_stress_batch(args):
    """The combined stress configuration: the stress scene (10M triangles,
    2,000 instances, 24M photons, 3840x2160, adaptive 1-16 spp, motion blur)
    as batches of `--batch-frames` motion-blurred frames 2 ms apart, each
    batch one wavefront (waves of 16M primary rays), first with the plain
    gather, then with the radiance cache trained online across the batches:
    ms/frame, Mrays/s and device memory of both, and both images' RMSE
    against the FP64 oracle's converged final gather (64 rays per vertex) on
    row bands of frame 0, all at the full photon counts."""
    import numpy as np
    import torch
    from sray_gb300 import build as gbuild, gpu, scenegen
    torch.cuda.set_device(0)
    gbuild.build()
    opts = scenegen.scene_opts("stress")
    t0 = time.perf_counter()
    path = scenegen.write_scene("stress")
    gen_s = time.perf_counter() - t0
    H, W = opts["height"], opts["width"]
    free_start = torch.cuda.mem_get_info()[0]
    g = gpu.GpuRenderer(**opts)
    t0 = time.perf_counter()
    g.load(path)
    load_s = time.perf_counter() - t0
    stream = torch.cuda.current_stream()
    nf = args.batch_frames
    fbs = [torch.zeros((H, W, 4), dtype=torch.float32, device="cuda") for _ in range(nf)]
    jobs = [(2 * j, fb) for j, fb in enumerate(fbs)]
    g.set_tuning(queue_depth=args.queue_depth or 1 << 24)

    def timed(n):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        rays = 0
        for _ in range(n):
            g.render_batch(jobs, stream=stream)
            rays += rays_of(g.stats())
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / n
        return ms, rays / n

    free0 = torch.cuda.mem_get_info()[0]
    for _ in range(args.warmup):
        g.render_batch(jobs, stream=stream)
    torch.cuda.synchronize()
    mem_plain = (free_start - torch.cuda.mem_get_info()[0]) / 1e6
    clocks = ClockSampler(torch.cuda.current_device())
    clocks.start()
    ms_plain, rays_plain = timed(args.steps)
    clk = clocks.stop()
    launches = g.stats()["kernel_launches"]
    img_plain = fbs[0].cpu().numpy().copy()
    # the learned configuration's training rate per frame (65,536 records, 4
    # Adam steps), so a batch of nf frames trains on nf times as many
    g.set_opts(nrc=1, nrc_train_samples=min(65536 * nf, 1 << 20), nrc_train_steps=4 * nf)
    g.nrc_reset()
    t0 = time.perf_counter()
    for _ in range(args.nrc_burn_in):
        g.render_batch(jobs, stream=stream)
    torch.cuda.synchronize()
    burn_s = time.perf_counter() - t0
    mem_cache = (free_start - torch.cuda.mem_get_info()[0]) / 1e6
    ms_cache, rays_cache = timed(args.steps)
    st = g.nrc_stats()
    img_cache = fbs[0].cpu().numpy().copy()
    g.close()
    del fbs
    ref_info = None
    if not args.no_cpu_baseline:
        bands = band_rows(H, 8, 2)
        ref, rows, ref_s = oracle_reference_rows(opts, path, ds=64, bands=bands)
        ref_info = {"rmse_plain": image_rmse(img_plain, ref, rows), "rmse_cache": image_rmse(img_cache, ref, rows),
                    "rows": int(len(rows)), "bands": [list(b) for b in bands], "s": ref_s,
                    "reference": "FP64 CPU oracle of frame 0 (same seeds, full photon counts), 64 final-gather rays per "
                                 "vertex (the converged plain estimator)"}
    line = {
        "metric": METRIC, "value": rays_cache / (ms_cache / 1e3) / 1e6, "unit": "Mrays/s", "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_cache, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded scene generator, no dataset)",
        "config": {"workload": workload_desc("stress") + "; %d frames 2 ms apart per batch, one wavefront per batch "
                                                         "(waves of %d primary rays)" % (nf, args.queue_depth or 1 << 24),
                   "method": "radiance cache with per-region fallback, trained online across batches"},
        "stress_batch": {"frames_per_batch": nf,
                         "plain": {"ms_per_batch": ms_plain, "ms_per_frame": ms_plain / nf,
                                   "mrays_per_s": rays_plain / (ms_plain / 1e3) / 1e6, "device_mb": mem_plain},
                         "cache": {"ms_per_batch": ms_cache, "ms_per_frame": ms_cache / nf,
                                   "mrays_per_s": rays_cache / (ms_cache / 1e3) / 1e6, "device_mb": mem_cache,
                                   "burn_in_batches": args.nrc_burn_in, "burn_in_s": burn_s, "frames_trained": st["frames"],
                                   "train_samples_per_batch": st["train_samples"], "val_samples_per_batch": st["val_samples"],
                                   "cached_vertex_frac": st["cached"] / max(st["vertices"], 1),
                                   "regions_cached": st["regions_cached"], "val_rel_err": st["val_rel_err"]},
                         "cache_over_plain_time": ms_cache / ms_plain,
                         "image_vs_fp64_oracle": ref_info,
                         "scene_gen_s": gen_s, "load_s": load_s},
        "gpu_launches": launches, "clocks": clk, "e2e": None, "roofline": None, "cpu_baseline": None,
        "note": "a step is one batch of frames; e2e, roofline and the CPU baseline are reported for the production "
                "configuration",
    }
    print(json.dumps(line))
    return 0


def run_reference(args):
    """The reference arm: the CPU restatement of the reference's path (FP64,
    every host thread) on the same workload.  A step is one bounded sample
    of the frame: the frame's preparation (scene tree, projection maps and
    both photon maps at REF_PHOTON_FRAC of full size) and one row from each
    of 16 bands spread over the image.  The full frame's time is projected
    from each step: the tree and projection maps as measured, the photon
    phase from a line a + b * fraction fitted in the warm-up (photon maps at
    two fractions), the rows scaled to the image.  ms_per_step is the
    measured sample, projected_ms_per_frame the frame."""
    ws, rank, _ = dist_env()
    if rank != 0:
        return 0
    from sray_gb300 import scenegen
    from oracle import oracle as orc_mod
    from oracle.oracle import Oracle
    orc_mod.build()
    opts = config_opts(args)
    path = scenegen.write_scene(args.config)
    H = opts["height"]
    bands = band_rows(H, CPU_BANDS, 2)
    cores = os.cpu_count() or 1
    orc = Oracle(fp64=True, rng_mode=1, **dict(opts, threads=0))
    t0 = time.perf_counter()
    orc.load(path)
    load_s = time.perf_counter() - t0
    full = (opts["caust_photons"], opts["gi_photons"])
    sampled = args.config in ("production", "stress")
    f = REF_PHOTON_FRAC if sampled else 1.0

    def at(frac):
        orc.set_opts(caust_photons=int(round(full[0] * frac)), gi_photons=int(round(full[1] * frac)))

    fit = None
    if sampled:
        # the photon phase against the photon count: two fractions, warm-up
        pts = []
        for frac in (f, 3 * f):
            at(frac)
            orc.prepare(0)
            pts.append((frac, orc.phase_ms()["photons"] / 1e3))
        b = (pts[1][1] - pts[0][1]) / (pts[1][0] - pts[0][0])
        fit = {"photon_s_per_full_map": b, "photon_s_fixed": pts[0][1] - b * pts[0][0],
               "points": [[round(x, 4), round(y, 4)] for x, y in pts]}
    steps = []
    t_run = time.perf_counter()
    for i in range(args.warmup + args.steps):
        at(f)
        t0 = time.perf_counter()
        smp = cpu_sample(orc, H, bands)
        wall = time.perf_counter() - t0
        photons_full = smp["photons_s"] + (fit["photon_s_per_full_map"] * (1.0 - f) if fit else 0.0)
        frame_s = smp["build_s"] + smp["projmaps_s"] + photons_full + smp["rows_s"] * H / smp["rows"]
        rays = smp["rays"] * H / smp["rows"]
        if i >= args.warmup:
            steps.append({"wall_s": wall, "frame_s": frame_s, "rays": rays, "smp": smp})
    run_s = time.perf_counter() - t_run
    frame_ms = sum(x["frame_s"] for x in steps) / len(steps) * 1e3
    v = sum(x["rays"] for x in steps) / sum(x["frame_s"] for x in steps) / 1e6
    step_ms = sum(x["wall_s"] for x in steps) / len(steps) * 1e3
    last = steps[-1]["smp"]
    sample = ("each step: the frame's preparation with the photon maps at %g of full size (%d+%d photons) and %d rows "
              "from %d bands spread over the %d-row image; the frame's time projected from it (scene tree and "
              "projection maps as measured, the photon phase from a line fitted over photon maps at %g and %g of full "
              "size, the rows scaled to the image); CPU restatement of the reference's path in FP64 on %d threads"
              % (f, int(round(full[0] * f)), int(round(full[1] * f)), last["rows"], len(bands), H, f, 3 * f, cores)
              if sampled else
              "each step: the whole frame's preparation and %d rows from %d bands spread over the %d-row image, the rows "
              "scaled to the image; CPU restatement of the reference's path in FP64 on %d threads"
              % (last["rows"], len(bands), H, cores))
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": "Mrays/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": step_ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded scene)",
        "config": {"workload": workload_desc(args.config), "method": "plain gather"},
        "projected_ms_per_frame": frame_ms,
        "cpu_baseline": {"value": v, "unit": "Mrays/s", "cores": cores, "kind": "port", "sample": sample},
        "e2e": {"value": v, "unit": "Mrays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "photon_fit": fit, "load_s": load_s, "timed_steps_s": run_s,
        "phases_s_last_step": {k: round(last[k], 3) for k in ("build_s", "projmaps_s", "photons_s", "rows_s")},
        "note": "ms_per_step is the measured sample of each step; value and projected_ms_per_frame are the whole frame "
                "projected from it",
    }
    if args.cpu_full_frame:
        # the check of the projection: one whole frame (full photon maps, every row)
        at(1.0)
        t0 = time.perf_counter()
        orc.prepare(0)
        orc.render(0)
        full_s = time.perf_counter() - t0
        line["full_frame_check"] = {"measured_ms": full_s * 1e3, "projected_ms": frame_ms,
                                    "projected_over_measured": frame_ms / (full_s * 1e3)}
    print(json.dumps(line))
    return 0


def run_ours(args):
    import numpy as np
    import torch
    from sray_gb300 import build as gbuild, gpu, scenegen

    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    else:
        torch.cuda.set_device(0)
    dev = torch.cuda.current_device()
    if rank == 0:
        gbuild.build()
    if ws > 1:
        dist.barrier()
    opts = config_opts(args)
    path = scenegen.write_scene(args.config)
    free0 = torch.cuda.mem_get_info()[0]
    g = gpu.GpuRenderer(**opts)
    t0 = time.perf_counter()
    g.load(path)
    t_load = time.perf_counter() - t0
    info = g.scene_info()
    H, W = opts["height"], opts["width"]
    fb = torch.zeros((H, W, 4), dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream()

    for _ in range(args.warmup):
        g.render(0, fb, stream=stream)
    torch.cuda.synchronize()
    device_mb = (free0 - torch.cuda.mem_get_info()[0]) / 1e6

    # the library's autotuner picks the scheduler's queue depths (untimed setup)
    if args.tuning:
        vals = [int(v) for v in args.tuning.split(",")]
        g.set_tuning(**dict(zip(("render_tail", "pool_blocks_per_sm", "photon_tail", "shadow_order", "stream_priority",
                                 "warp_rays", "warp_segments", "side_gather", "sort_rays", "side_shadow"), vals)))
    tuning = {"chosen": g.tuning(), "autotuned": False}
    if not args.no_autotune and not args.tuning:
        best, best_ms, trials = g.autotune(fb, frames=3, stream=stream)
        tuning = {"chosen": best, "autotuned": True, "best_ms_per_frame": best_ms, "frames_per_trial": 3,
                  "trials": [dict(t, ms=round(ms, 3)) for t, ms in trials]}

    # untimed pass: traversal and gather work of the frame (algorithmic bytes)
    g.set_profiling(time_kernels=True, count_work=True)
    g.kernel_times(reset=True)
    g.render(0, fb, stream=stream)
    torch.cuda.synchronize()
    st_count = g.stats()
    g.kernel_times(reset=True)
    alg = algorithmic_bytes(st_count)

    # timed region: K frames, device timing on the launch stream
    g.set_profiling(False, False)
    clocks = ClockSampler(dev)
    if ws > 1:
        dist.barrier()
    torch.cuda.synchronize()
    clocks.start()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    rays = 0
    launches = 0
    for _ in range(args.steps):
        g.render(0, fb, stream=stream)
        st = g.stats()
        rays += rays_of(st)
        launches += st["kernel_launches"]
    e1.record(stream)
    torch.cuda.synchronize()
    ms_total = e0.elapsed_time(e1)
    clk = clocks.stop()
    st_last = st
    # the same K frames again with CUDA events around every launch, on the
    # launch's own stream: the kernels' durations (the events cost a few per
    # cent of the frame, so the frame time above is taken without them)
    g.set_profiling(time_kernels=True, count_work=False)
    g.kernel_times(reset=True)
    torch.cuda.synchronize()
    ek0 = torch.cuda.Event(enable_timing=True)
    ek1 = torch.cuda.Event(enable_timing=True)
    ek0.record(stream)
    for _ in range(args.steps):
        g.render(0, fb, stream=stream)
    ek1.record(stream)
    torch.cuda.synchronize()
    ms_profiled = ek0.elapsed_time(ek1) / args.steps
    kt = g.kernel_times(reset=True)
    ms_step = ms_total / args.steps
    g_nrc_stats = g.nrc_stats() if opts.get("nrc") else None

    # end to end through the C-ABI with a host framebuffer
    g.set_profiling(False, False)
    host_fb = np.zeros((H, W, 4), np.float32)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    e2e_rays = 0
    h2d = d2h = 0
    for _ in range(args.steps):
        g.render(0, host_fb)
        st = g.stats()
        e2e_rays += rays_of(st)
        h2d += st["h2d_bytes"]
        d2h += st["d2h_bytes"]
    e2e_s = time.perf_counter() - t0

    if ws > 1:
        import torch.distributed as dist
        ms_total, rays, e2e_s, e2e_rays = reduce_over_ranks(ms_total, rays, e2e_s, e2e_rays, device="cuda")
        ms_step = ms_total / args.steps
    value = rays / (ms_total / 1e3) / 1e6
    e2e_value = e2e_rays / e2e_s / 1e6

    # the roofline of the kernels that bound the frame's own stream (the
    # photon kernels run beside it on a stream of lower priority: their event
    # times include waiting for SM slots); `roofline` is the dominant one's
    dom = max(((k, v) for k, v in kt.items() if not k.startswith("photon")), key=lambda kv: kv[1][0])
    hbm, src = peaks()
    scaled = args.res is None and args.photon_scale == 1.0 and args.config == "production"
    kernels = {}
    for name, (bytes_frame, units, unit_name, desc) in alg.items():
        k_ms, k_n = kt.get(name, (0.0, 0))
        ms_frame = k_ms / args.steps
        achieved = bytes_frame / (ms_frame / 1e3) / 1e9 if ms_frame > 0 else 0.0
        launches_frame = k_n / args.steps
        prof = committed_profile(name)
        traffic = None
        if prof.get("dram_bytes_per_unit") is not None and launches_frame > 0:
            # DRAM bytes per unit of work from the committed small-case capture,
            # scaled to this frame's units per launch
            traffic = prof["dram_bytes_per_unit"] * units / launches_frame
        kernels[name] = {
            "bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
            "peak_source": src, "traffic": traffic,
            "algorithmic_bytes_per_launch": bytes_frame / launches_frame if launches_frame else None,
            "avg_launch_ms": ms_frame / launches_frame if launches_frame else None,
            "ms_per_frame": ms_frame, "launches_per_frame": launches_frame, unit_name + "_per_frame": units,
            "algorithmic_bytes": desc,
            "threads_per_instruction": prof.get("threads_per_instruction"), "issue_active": prof.get("issue_active"),
            "profile": prof.get("source")}
        if name == "trace":
            # the camera rays' passes run the warp-packet kernel
            pk = committed_profile("trace_packet")
            kernels[name]["first_bounce"] = {"kernel": "k_trace_packet",
                                             "threads_per_instruction": pk.get("threads_per_instruction"),
                                             "issue_active": pk.get("issue_active")}
    dom_name = dom[0] if dom[0] in kernels else max(kernels, key=lambda k: kernels[k]["ms_per_frame"])
    roof = dict(kernels[dom_name], kernel=dom_name, dominant_kernel=dom[0], kernels=kernels,
                note="achieved = algorithmic bytes of the frame's launches (counted in an untimed pass) over their "
                     "CUDA-event time in K frames timed right after the frame-time region (the same frames, events "
                     "around every launch on its own stream); traffic = DRAM bytes per unit from the committed ncu capture "
                     "of a smaller frame, times this frame's units per launch: the hierarchies and photon maps are "
                     "re-read from L1/L2, so DRAM traffic is a small fraction of the algorithmic bytes and the kernels "
                     "are bound by instruction issue at the SIMT efficiency beside each; with side_shadow the light "
                     "samples and gathers run beside the closest-hit launches, whose event time then includes the SMs "
                     "they share")
    roof["node_records_per_ray"] = st_count["node_visits"] / max(st_count["primary_rays"] + st_count["secondary_rays"], 1)
    roof["prim_tests_per_ray"] = st_count["prim_tests"] / max(st_count["primary_rays"] + st_count["secondary_rays"], 1)
    if not scaled:
        roof["note"] += " (reduced case: traffic from the capture is not scaled)"

    cpu = None
    check = None
    bands = band_rows(H, CPU_BANDS, args.cpu_rows)
    if rank == 0 and not args.no_cpu_baseline and args.config != "stress":
        try:
            cb, ref64 = cpu_baseline(opts, path, bands)
            cpu = {k: cb[k] for k in ("value", "unit", "cores", "kind", "sample", "ms_per_frame", "phases_s")}
            check = fp64_image_check(host_fb, ref64, bands)
        except Exception as exc:  # the CPU baseline is a report, not the measurement
            cpu = {"value": None, "unit": "Mrays/s", "cores": os.cpu_count(), "kind": "port",
                   "sample": "failed: %s" % exc}
    parity = None
    if rank == 0 and not args.no_parity and args.config in ("production", "small") and ws == 1:
        try:
            parity = parity_leg(opts, path, g, host_fb, band_rows(H, CPU_BANDS, 8))
        except Exception as exc:  # reported beside the measurement
            parity = {"error": str(exc)}

    # photons and gathers per second: of the frame, and of their own kernels
    ph_ms = sum(v[0] for k, v in kt.items() if k.startswith("photon")) / args.steps
    ga_ms = kt.get("gather", (0.0, 0))[0] / args.steps
    throughput = {"photons_per_frame": st_last["photons_emitted"], "gathers_per_frame": st_last["gathers"],
                  "photons_per_s": st_last["photons_emitted"] / (ms_step / 1e3),
                  "gathers_per_s": st_last["gathers"] / (ms_step / 1e3),
                  "photon_kernels_ms": ph_ms, "gather_kernels_ms": ga_ms,
                  "photons_per_s_of_photon_kernels": st_last["photons_emitted"] / (ph_ms / 1e3) if ph_ms else None,
                  "gathers_per_s_of_gather_kernels": st_last["gathers"] / (ga_ms / 1e3) if ga_ms else None,
                  "note": "photon kernels run on their own stream beside the first bounce; per-frame rates use the "
                          "frame time, kernel rates the CUDA-event time of the photon / gather launches"}

    stress_cache = None
    if args.config == "stress" and not args.no_nrc:
        # the same frames with the radiance cache (per-region fallback), trained online
        g.set_opts(nrc=1)
        free1 = torch.cuda.mem_get_info()[0]
        burn = args.nrc_burn_in
        for _ in range(burn):
            g.render(0, fb, stream=stream)
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        crays = 0
        for _ in range(args.steps):
            g.render(0, fb, stream=stream)
            crays += rays_of(g.stats())
        e1.record(stream)
        torch.cuda.synchronize()
        cms = e0.elapsed_time(e1) / args.steps
        st_c = g.nrc_stats()
        stress_cache = {"ms_per_frame": cms, "mrays_per_s": crays / args.steps / (cms / 1e3) / 1e6, "burn_in_frames": burn,
                        "plain_ms_per_frame": ms_step, "frames_trained": st_c["frames"],
                        "cached_vertex_frac": st_c["cached"] / max(st_c["vertices"], 1),
                        "regions_cached": st_c["regions_cached"], "val_rel_err": st_c["val_rel_err"],
                        "device_mb_plain": device_mb,
                        "device_mb_extra_for_cache": (free1 - torch.cuda.mem_get_info()[0]) / 1e6,
                        "note": "RMSE against the FP64 oracle is not computed for this scene (the CPU oracle would "
                                "trace 24M photons over 10M triangles in double)"}

    nrc = None
    if rank == 0 and not args.no_nrc and ws == 1 and args.res is None and args.config != "stress":
        g.close()
        ref = None
        if not args.no_cpu_baseline:
            from sray_gb300 import scenegen as sg
            lopts = sg.scene_opts("learned")
            img, rows, ref_s = oracle_reference_rows(lopts, sg.write_scene("learned"))
            ref = (img, rows)
        try:
            nrc = nrc_vs_plain(args, ref)
            if ref is not None:
                nrc["reference_s"] = ref_s
        except Exception as exc:  # reported, the headline stands on its own
            nrc = {"error": str(exc)}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "Mrays/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded scene generator, no dataset)",
            "config": {"workload": workload_desc(args.config) + ("" if not args.res and args.photon_scale == 1.0 else
                                                                  " [reduced: %s, photons x%g]" % (args.res, args.photon_scale)),
                       "method": {"plain": "plain gather", "cache": "radiance cache with per-region fallback",
                                  "cache-everywhere": "radiance cache in every region"}[args.method],
                       "parallelism": "replicas" if ws > 1 else "single",
                       "tuning": tuning,
                       "l2": "inputs larger than L2: %.0f MB of triangle records + photon maps rebuilt every frame"
                             % (info["triangles"] * 48 / 1e6),
                       "scene": info},
            "e2e": {"value": e2e_value, "unit": "Mrays/s", "h2d_bytes_per_step": h2d // args.steps,
                    "d2h_bytes_per_step": d2h // args.steps, "ms_per_step": e2e_s / args.steps * 1e3},
            "roofline": roof,
            "cpu_baseline": cpu,
            "gpu_launches": launches,
            "clocks": clk,
            "nrc_vs_plain": nrc,
            "stress_cache_vs_plain": stress_cache,
            "kernels_ms_per_step": {k: round(v[0] / args.steps, 3) for k, v in kt.items()},
            "kernel_timing": {"ms_per_step_with_events": ms_profiled,
                              "note": "kernel durations (roofline, kernels_ms_per_step) from CUDA events around every "
                                      "launch in a second run of the same K frames right after the timed one"},
            "frame": {"rays": rays_of(st_last), "primary": st_last["primary_rays"],
                      "secondary": st_last["secondary_rays"], "shadow": st_last["shadow_rays"],
                      "gathers": st_last["gathers"], "samples": st_last["samples"],
                      "photons_stored": st_last["photons_stored"], "load_s": t_load, "device_mb": device_mb,
                      "gather_slots_per_query": st_last["gather_tested"] / max(st_last["gathers"], 1),
                      "gather_candidates_per_query": st_last["gather_candidates"] / max(st_last["gathers"], 1),
                      "gather_select_frac": st_last["gather_selects"] / max(st_last["gathers"], 1),
                      "gather_spill_frac": st_last["gather_spills"] / max(st_last["gathers"], 1),
                      "bvh_fallbacks": st_last["bvh_fallbacks"],
                      "nrc": g_nrc_stats},
            "throughput": throughput,
            "primary_mrays_per_s": st_last["primary_rays"] / (ms_step / 1e3) / 1e6,
            "image_vs_fp64_oracle": check,
            "parity": parity,
        }
        print(json.dumps(line))
    if nrc is None:
        g.close()
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return 0


def run_nrc_infer(args):
    """The radiance cache's tensor-core inference alone: `--nrc-samples`
    uniform inputs, `--warmup` untimed calls, then `--steps` launches
    enqueued back to back (sray_nrc_infer_async: one k_nrc_forward_tc launch
    each, the error word read once after them by sray_nrc_check) timed with
    CUDA events -- the kernel's rate -- and `--steps` synchronous calls
    (sray_nrc_infer: the launch, a wait and a read of the error word each);
    TFLOP/s of the 2 x 26,304 FLOP per sample against the measured bf16
    peak."""
    import torch
    from sray_gb300 import build as gbuild, gpu
    torch.cuda.set_device(0)
    gbuild.build()
    n = args.nrc_samples
    cache = gpu.RadianceCache(seed=1)
    gen = torch.Generator(device="cuda").manual_seed(3)
    x = torch.rand((n, 9), device="cuda", generator=gen)
    y = torch.empty((n, 3), device="cuda")
    stream = torch.cuda.current_stream()
    for _ in range(args.warmup):
        cache.infer(x, y, stream=stream)
    torch.cuda.synchronize()

    def timed(sync):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.steps):
            cache.infer(x, y, stream=stream, sync=sync)
        e1.record(stream)
        cache.check(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / args.steps

    ms = timed(False)
    ms_sync = timed(True)
    tflops = 2 * 26304 * n / (ms / 1e3) / 1e12
    peak = bf16_peak()
    print(json.dumps({"metric": "radiance-cache inference (k_nrc_forward_tc)", "value": tflops, "unit": "TFLOP/s",
                      "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
                      "ms_per_synchronous_call": ms_sync,
                      "tflops_synchronous_calls": 2 * 26304 * n / (ms_sync / 1e3) / 1e12,
                      "higher_is_better": True, "dtype": "bf16", "data": "synthetic (uniform inputs)",
                      "config": {"workload": "nrc-infer: %d samples per launch" % n,
                                 "l2": "inputs of %.0f MB per launch%s" % (n * 36 / 1e6, " (larger than L2)" if n * 36 > 129e6 else "")},
                      "roofline": {"bound": "tensor", "achieved": tflops, "peak": peak, "unit": "TFLOP/s",
                                   "frac": tflops / peak if peak else None},
                      "finite": bool(torch.isfinite(y).all())}))
    return 0


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    if args.config == "nrc-infer":
        return run_nrc_infer(args)
    if args.config == "batch":
        return run_batch(args)
    if args.config == "stress-batch":
        return run_stress_batch(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
