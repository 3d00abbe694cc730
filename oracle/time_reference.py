"""TEST INFRASTRUCTURE: time the reference's own CPU frame against the CPU
restatement (the port that bench.py's reference arm runs where the
reference's sources are absent), on the same scene, options and threads.

The reference side is its unmodified frame entry point, rend_init +
render(msec) (src/render.cc:22-55: the scene octree, projection maps and a
serial photon loop, then 48x48 tiles on its pthread tpool,
src/tpool.cc:48-225), built by oracle/build_ref.py and timed by its own
get_msec.  The port side is the FP64 oracle's prepare + render of the whole
frame.  Both run the reference's fixed-radius gathers (no k-nearest).
Only runs where the compiled reference exists:
    python oracle/time_reference.py [--config small|production] [--threads N] [--reps R]
Prints one JSON line with both times and their ratio.
"""
import argparse
import json
import os
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def cli_of(o):
    """The reference's command-line options (src/opt.c:61-88) for sray_opts fields."""
    a = ["-s", "%dx%d" % (o["width"], o["height"]), "-r", "%d-%d" % (o.get("min_samples", 1), o.get("max_samples", 1)),
         "-i", str(o.get("iter", 7)), "-c", str(o.get("caust_photons", 0)), "-g", str(o.get("gi_photons", 0)),
         "-shadowrays", str(o.get("shadow_samples", 1)), "-diffuserays", str(o.get("diffuse_samples", 1))]
    if "max_var" in o:
        a += ["-d", repr(float(o["max_var"]))]
    if "gather_dist" in o:
        a += ["-gatherdisc", repr(float(o["gather_dist"]))]
    for k, f in (("scnoct_max_depth", "-soctdepth"), ("scnoct_max_items", "-soctitems"),
                 ("meshoct_max_depth", "-moctdepth"), ("meshoct_max_items", "-moctitems")):
        if k in o:
            a += [f, str(o[k])]
    return a


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--config", default="small")
    ap.add_argument("--threads", type=int, default=os.cpu_count() or 1)
    ap.add_argument("--reps", type=int, default=3)
    ap.add_argument("--res", default=None, help="WxH override")
    ap.add_argument("--photon-scale", type=float, default=1.0, help="photon count multiplier")
    args = ap.parse_args()
    from oracle import build_ref
    from oracle.oracle import Oracle
    from sray_gb300 import scenegen
    harness = build_ref.build()
    if not harness:
        print(json.dumps({"unavailable": "the reference's sources are not present"}))
        return 0
    opts = scenegen.scene_opts(args.config)
    if args.res:
        w, h = args.res.split("x")
        opts["width"], opts["height"] = int(w), int(h)
    opts["caust_k"] = opts["gi_k"] = 0          # the reference's fixed-radius gathers
    opts["caust_photons"] = int(round(opts.get("caust_photons", 0) * args.photon_scale))
    opts["gi_photons"] = int(round(opts.get("gi_photons", 0) * args.photon_scale))
    path = scenegen.write_scene(args.config)
    cmd = [harness, "--time", path, str(args.reps)] + cli_of(opts) + ["-t", str(args.threads)]
    out = subprocess.run(cmd, capture_output=True, text=True, check=True).stdout.strip().splitlines()[-1]
    ref = json.loads(out)
    orc = Oracle(fp64=True, rng_mode=0, **dict(opts, threads=args.threads))
    orc.load(path)
    port_ms = []
    for _ in range(args.reps):
        orc.set_opts()                         # forget the prepared frame
        t0 = time.perf_counter()
        orc.prepare(0)
        orc.render(0, nthreads=args.threads)
        port_ms.append((time.perf_counter() - t0) * 1e3)
    r_med = sorted(ref["render_ms"])[len(ref["render_ms"]) // 2]
    p_med = sorted(port_ms)[len(port_ms) // 2]
    print(json.dumps({"config": args.config, "width": opts["width"], "height": opts["height"], "threads": args.threads,
                      "photons": [opts["caust_photons"], opts["gi_photons"]],
                      "machine": os.uname().machine, "reference_render_ms": ref["render_ms"],
                      "port_frame_ms": [round(x, 1) for x in port_ms],
                      "reference_over_port": r_med / p_med}))
    return 0


if __name__ == "__main__":
    sys.exit(main())
