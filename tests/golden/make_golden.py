"""Generate the golden fixtures that pin the CPU oracle.

Runs the reference's own rendering code (compiled from its unmodified
sources by oracle/build_ref.py, with the project's libvmath/kdtree/imago
stand-ins and a Philox stream per photon and per pixel sample) on five
seeded scenes (the textured one reads the images of scenegen.textures()
through SRAY_DATA_PATH; the animated one is rendered at 1350 ms) and stores, per case: the scene XML, the options, the
primary-hit ids and t, the stored caustic and global photons, and the
rendered image with its per-pixel sample counts; for the feature scene
also both photon maps as the reference's PhotonMap::dump writes them.

Only runs where the reference sources are present:
    python tests/golden/make_golden.py [case ...]
"""
import gzip
import json
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

SEED = 0x5EED0001

# case: (scene generator, generator kwargs, reference command-line options, oracle options)
CASES = {
    "small_range": ("small", {}, ["-s", "64x64", "-c", "20000", "-i", "5", "-soctdepth", "8", "-soctitems", "8",
                                  "-moctdepth", "8", "-moctitems", "8"],
                    dict(width=64, height=64, caust_photons=20000, iter=5, scnoct_max_depth=8, scnoct_max_items=8,
                         meshoct_max_depth=8, meshoct_max_items=8)),
    "feature": ("feature", {}, ["-s", "64x48", "-r", "1-4", "-d", "0.01", "-c", "20000", "-g", "30000", "-i", "6",
                                "-shadowrays", "2", "-diffuserays", "2", "-m", "-u", "40", "-gatherdisc", "0.02"],
                dict(width=64, height=48, min_samples=1, max_samples=4, max_var=0.01, caust_photons=20000,
                     gi_photons=30000, iter=6, shadow_samples=2, diffuse_samples=2, mblur=1, shutter=40,
                     gather_dist=0.02)),
    "terrain": ("production", {"grid": (60, 30), "n_inst": 12},
                ["-s", "64x36", "-r", "1-2", "-d", "0.05", "-c", "5000", "-g", "20000", "-i", "4", "-gatherdisc", "0.01",
                 "-moctdepth", "8", "-moctitems", "8"],
                dict(width=64, height=36, min_samples=1, max_samples=2, max_var=0.05, caust_photons=5000,
                     gi_photons=20000, iter=4, gather_dist=0.01, meshoct_max_depth=8, meshoct_max_items=8)),
    "textured": ("textured", {}, ["-s", "64x48", "-r", "1-2", "-d", "0.02", "-c", "20000", "-g", "30000", "-i", "6",
                                  "-shadowrays", "2", "-diffuserays", "2", "-gatherdisc", "0.02"],
                 dict(width=64, height=48, min_samples=1, max_samples=2, max_var=0.02, caust_photons=20000,
                      gi_photons=30000, iter=6, shadow_samples=2, diffuse_samples=2, gather_dist=0.02)),
    # keyframes in every interpolation / extrapolation mode, rendered at 1350 ms
    "animated": ("animated", {}, ["-s", "64x48", "-c", "20000", "-i", "5"],
                 dict(width=64, height=48, caust_photons=20000, iter=5), 1350),
}


# cases whose photon maps are also stored as the reference's dump files
DUMP_CASES = {"feature"}


def run_case(harness, name, spec):
    from sray_gb300 import scenegen
    gen, kw, cli, oopts = spec[:4]
    msec = spec[4] if len(spec) > 4 else 0
    path = scenegen.write_scene(gen, **kw)
    xml = open(path, "rb").read()
    # textures are found through the first directory of SRAY_DATA_PATH; the
    # frame time is SRAY_REF_MSEC
    env = dict(os.environ, SRAY_DATA_PATH=os.path.dirname(path), SRAY_REF_MSEC=str(msec))
    with tempfile.TemporaryDirectory() as td:
        prefix = os.path.join(td, name)
        h = oopts["height"]
        subprocess.check_call([harness, path, prefix, hex(SEED), "0", str(h)] + cli, stdout=subprocess.DEVNULL,
                              env=env)
        hits = np.fromfile(prefix + ".hits", dtype=np.dtype([("o", "<i4"), ("p", "<i4"), ("t", "<f8")]))
        caust = np.fromfile(prefix + ".caust", dtype=np.float32).reshape(-1, 16)
        gi = np.fromfile(prefix + ".gi", dtype=np.float32).reshape(-1, 16)
        img = np.fromfile(prefix + ".img", dtype=np.float32).reshape(h, oopts["width"], 5)
        if name in DUMP_CASES:
            # the maps in the reference's own dump format (PhotonMap::dump)
            for which in ("caust", "gi"):
                with open(prefix + ".%s.dump" % which, "rb") as f, gzip.open(os.path.join(HERE, "%s.%s.dump.gz" % (name, which)), "wb") as g:
                    g.write(f.read())
    out = os.path.join(HERE, name + ".npz")
    np.savez_compressed(out, obj=hits["o"], prim=hits["p"], t=hits["t"], caust=caust[:, :13], gi=gi[:, :13],
                        img=img[..., :4], spp=img[..., 4].astype(np.int32), msec=np.int64(msec),
                        opts=np.frombuffer(json.dumps(oopts).encode(), dtype=np.uint8),
                        cli=np.frombuffer(json.dumps(cli).encode(), dtype=np.uint8))
    with gzip.open(os.path.join(HERE, name + ".xml.gz"), "wb") as f:
        f.write(xml)
    print("%s: %d hits, %d caustic, %d global photons, spp %s" % (
        name, int((hits["o"] >= 0).sum()), len(caust), len(gi), np.unique(img[..., 4]).tolist()))


def main():
    from oracle import build_ref
    harness = build_ref.build()
    if not harness:
        print("reference sources not present; nothing to do")
        return 0
    names = sys.argv[1:] or list(CASES)
    for name in names:
        run_case(harness, name, CASES[name])
    with open(os.path.join(HERE, "MACHINE"), "w") as f:
        f.write(os.uname().machine + "\n")
    return 0


if __name__ == "__main__":
    sys.exit(main())
