"""Build libsray_gpu.so in-tree for sm_103a (GB300).

Device code is compiled with -fmad=false and IEEE division/sqrt so every
float operation rounds like the CPU oracle's float path; host code with
-ffp-contract=off for the same reason (GCC contracts by default on Arm).
Translation units compile in parallel; the result goes to sray_gb300/_lib/.
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
OUT = os.path.join(PKG, "_lib")
LIB = os.path.join(OUT, "libsray_gpu.so")

NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
INC = ["-I" + os.path.join(ROOT, "include"), "-I" + CSRC]
CU_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-fmad=false", "-prec-div=true", "-prec-sqrt=true",
            "-Xcompiler", "-fPIC,-ffp-contract=off", "--expt-relaxed-constexpr", "-Xptxas", "-warn-spills"]
CC_FLAGS = ["-O3", "-std=c++17", "-fPIC", "-ffp-contract=off", "-fno-fast-math", "-I/usr/local/cuda/include"]

SOURCES = ["render.cu", "photon.cu", "nrc.cu", "scene_host.cc", "bvh_host.cc"]
HEADERS = ["dev_common.cuh", "renderer.h", "scene_host.h", "sray_device.h", "range_ff.h", "nrc.h", "anim_eval.h", "slot_order.h"]


def _deps():
    files = [os.path.join(CSRC, f) for f in SOURCES + HEADERS]
    files += [os.path.join(ROOT, "include", f) for f in ("sray_gpu.h", "sray_rng.h")]
    files.append(os.path.abspath(__file__))
    return files


def up_to_date():
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(f) <= t for f in _deps())


def _compile(src):
    obj = os.path.join(OUT, os.path.splitext(src)[0] + ".o")
    path = os.path.join(CSRC, src)
    if src.endswith(".cu"):
        cmd = [NVCC] + ARCH + CU_FLAGS + INC + ["-c", path, "-o", obj]
    else:
        cmd = ["g++"] + CC_FLAGS + INC + ["-c", path, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("compile failed: %s\n%s\n%s" % (" ".join(cmd), r.stdout, r.stderr))
    return obj, r.stderr


def build(force=False, verbose=False):
    if not force and up_to_date():
        return LIB
    os.makedirs(OUT, exist_ok=True)
    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        results = list(ex.map(_compile, SOURCES))
    if verbose:
        for _, err in results:
            if err.strip():
                print(err, file=sys.stderr)
    tmp = LIB + ".tmp%d" % os.getpid()
    cmd = [NVCC] + ARCH + ["-shared", "-o", tmp] + [o for o, _ in results] + ["-cudart", "static", "-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed: %s\n%s\n%s" % (" ".join(cmd), r.stdout, r.stderr))
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
