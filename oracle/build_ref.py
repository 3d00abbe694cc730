"""TEST INFRASTRUCTURE: compile the reference's own sources into the harness
that pins the CPU oracle.

The reference (S-ray) builds against three libraries it does not ship:
libvmath, kdtree and libimago.  oracle/refshim/ holds project-written
stand-ins with the semantics its call sites require; expat (XML) is taken
from the system.  Every .c/.cc of the reference's src/ except sray.cc (its
main) is compiled unmodified from where it lies, with rand() routed to the
harness's Philox streams, no fast-math and no FMA contraction.  Output goes
to oracle/_ref/ (git-ignored).  This only runs where the reference sources
are present.
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE = os.path.join(ROOT, "oracle")
SHIM = os.path.join(ORACLE, "refshim")
OUT = os.path.join(ORACLE, "_ref")
REF_SRC = os.environ.get("SRAY_REFERENCE_SRC", "/root/reference/src")
BIN = os.path.join(OUT, "ref_harness")

COMMON = ["-O2", "-ffp-contract=off", "-fno-fast-math", "-w", "-I" + SHIM, "-I" + ORACLE,
          "-I" + os.path.join(ROOT, "include"), "-I" + REF_SRC]
FORCE = ["-include", os.path.join(SHIM, "shim_rng.h")]


def sources():
    files = sorted(f for f in os.listdir(REF_SRC) if f.endswith((".c", ".cc")) and f != "sray.cc")
    return [os.path.join(REF_SRC, f) for f in files]


def compile_one(src):
    obj = os.path.join(OUT, os.path.basename(src) + ".o")
    if src.endswith(".c"):
        cmd = ["gcc", "-std=gnu99"] + COMMON + FORCE + ["-c", src, "-o", obj]
    elif src.startswith(REF_SRC):
        cmd = ["g++", "-std=gnu++11"] + COMMON + FORCE + ["-c", src, "-o", obj]
    else:
        cmd = ["g++", "-std=gnu++11"] + COMMON + ["-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("compile failed: %s\n%s" % (" ".join(cmd), r.stderr[-4000:]))
    return obj


def build(force=False):
    if not os.path.isdir(REF_SRC):
        return None
    srcs = sources() + [os.path.join(SHIM, "shim_libs.cc"), os.path.join(ORACLE, "ref_harness.cc")]
    deps = srcs + [os.path.join(SHIM, f) for f in ("shim_rng.h", "kdtree.h", "imago2.h")] + \
        [os.path.join(SHIM, "vmath", "vmath.h"), os.path.join(ORACLE, "vmath_core.h"), os.path.abspath(__file__)]
    if not force and os.path.exists(BIN) and all(os.path.getmtime(d) <= os.path.getmtime(BIN) for d in deps):
        return BIN
    os.makedirs(OUT, exist_ok=True)
    with ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
        objs = list(ex.map(compile_one, srcs))
    cmd = ["g++", "-o", BIN] + objs + ["-lexpat", "-lpthread", "-lrt", "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed: %s\n%s" % (" ".join(cmd), r.stderr[-4000:]))
    return BIN


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
