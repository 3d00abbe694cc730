"""TEST INFRASTRUCTURE: build recipe and ctypes binding of the CPU oracle.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use
this module; the GPU library never imports it.
"""
import ctypes
import os
import subprocess
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE_DIR = os.path.join(ROOT, "oracle")
BUILD_DIR = os.path.join(ORACLE_DIR, "_build")
LIB = os.path.join(BUILD_DIR, "liboracle.so")

sys.path.insert(0, ROOT)
from sray_gb300.options import SrayOpts, make_opts  # noqa: E402


def build(force=False):
    """Compile the oracle with the host compiler (no FMA contraction, so the
    float path rounds exactly like the device code built with -fmad=false)."""
    src = [os.path.join(ORACLE_DIR, "sray_oracle.cc")]
    deps = src + [os.path.join(ORACLE_DIR, "vmath_core.h"), os.path.join(ORACLE_DIR, "sray_oracle.h"),
                  os.path.join(ROOT, "include", "sray_rng.h"), os.path.join(ROOT, "include", "sray_gpu.h")]
    if not force and os.path.exists(LIB):
        t = os.path.getmtime(LIB)
        if all(os.path.getmtime(d) <= t for d in deps):
            return LIB
    os.makedirs(BUILD_DIR, exist_ok=True)
    tmp = LIB + ".tmp%d" % os.getpid()
    cmd = ["g++", "-O3", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math",
           "-I" + os.path.join(ROOT, "include"), "-I" + ORACLE_DIR, "-o", tmp] + src + ["-lpthread"]
    subprocess.check_call(cmd)
    os.replace(tmp, LIB)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB)
        vp, ip, dp, fp, cp = ctypes.c_void_p, ctypes.c_int, ctypes.c_double, ctypes.c_float, ctypes.c_char_p
        L.orc_create.restype = vp
        L.orc_create.argtypes = [ctypes.POINTER(SrayOpts), ip, ip]
        L.orc_destroy.argtypes = [vp]
        L.orc_load.argtypes = [vp, cp]
        L.orc_load_mem.argtypes = [vp, cp, ctypes.c_size_t]
        L.orc_error.restype = cp
        L.orc_error.argtypes = [vp]
        L.orc_scene_info.argtypes = [vp, vp, vp, vp, vp]
        L.orc_prepare_frame.argtypes = [vp, ctypes.c_long]
        L.orc_photon_info.argtypes = [vp, vp, vp, vp]
        L.orc_get_photons.argtypes = [vp, ip, vp, ip]
        L.orc_render_rows.argtypes = [vp, ctypes.c_long, ip, ip, vp, ip, ip, vp]
        L.orc_primary_hits.argtypes = [vp, ctypes.c_long, vp, vp, vp, vp]
        L.orc_cast_rays.argtypes = [vp, ip, vp, vp, vp, vp, vp, vp, vp]
        L.orc_gather.argtypes = [vp, ip, ip, vp, vp, vp]
        L.orc_counters.argtypes = [vp, vp, vp, vp, vp, vp]
        L.orc_set_pixel_base.argtypes = [vp, ip]
        L.orc_render_row_list.argtypes = [vp, ctypes.c_long, ip, vp, vp, ip, ip, vp]
        L.orc_set_opts.argtypes = [vp, ctypes.POINTER(SrayOpts)]
        L.orc_phase_ms.argtypes = [vp, vp]
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p) if a is not None else None


class Oracle:
    """CPU restatement of the reference's rendering path.

    fp64=True: the reference's double arithmetic; fp64=False: the float
    arithmetic of the CUDA kernels.  rng_mode 0 = depth-first draw order
    (as the compiled reference consumes its stream), 1 = path-keyed draws
    (as the GPU wavefront consumes them)."""

    def __init__(self, opts=None, fp64=True, rng_mode=1, **kw):
        self.L = lib()
        self.opts = opts if isinstance(opts, SrayOpts) else make_opts(**(opts or {}), **kw)
        self.h = self.L.orc_create(ctypes.byref(self.opts), int(fp64), int(rng_mode))

    def __del__(self):
        if getattr(self, "h", None):
            self.L.orc_destroy(self.h)
            self.h = None

    def _chk(self, r):
        if r < 0:
            raise RuntimeError("oracle: %s (%d)" % (self.L.orc_error(self.h).decode(), r))
        return r

    def load(self, path):
        self._chk(self.L.orc_load(self.h, path.encode()))

    def load_xml(self, xml):
        b = xml.encode() if isinstance(xml, str) else xml
        self._chk(self.L.orc_load_mem(self.h, b, len(b)))

    def scene_info(self):
        a, b, c = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        d = ctypes.c_int64()
        self.L.orc_scene_info(self.h, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c), ctypes.byref(d))
        return dict(objects=a.value, lights=b.value, materials=c.value, triangles=d.value)

    def prepare(self, msec=0):
        self._chk(self.L.orc_prepare_frame(self.h, msec))

    def photon_info(self):
        a, b = ctypes.c_int(), ctypes.c_int()
        g = ctypes.c_double()
        self._chk(self.L.orc_photon_info(self.h, ctypes.byref(a), ctypes.byref(b), ctypes.byref(g)))
        return a.value, b.value, g.value

    def photons(self, which):
        nc, ng, _ = self.photon_info()
        n = ng if which else nc
        out = np.zeros((max(n, 1), 16), dtype=np.float32)
        self._chk(self.L.orc_get_photons(self.h, which, _p(out), n))
        return out[:n]

    def render(self, msec=0, rows=None, nthreads=0, quirk_sum=False, want_spp=False):
        o = self.opts
        fb = np.zeros((o.height, o.width, 4), dtype=np.float32)
        spp = np.zeros((o.height, o.width), dtype=np.int32) if want_spp else None
        y0, y1 = rows if rows else (0, o.height)
        self._chk(self.L.orc_render_rows(self.h, msec, y0, y1, _p(fb), nthreads, int(quirk_sum), _p(spp)))
        return (fb, spp) if want_spp else fb

    def render_rows(self, rows, msec=0, nthreads=0, quirk_sum=False):
        """The listed image rows (the rest of the returned image is zero)."""
        o = self.opts
        fb = np.zeros((o.height, o.width, 4), dtype=np.float32)
        r = np.ascontiguousarray(rows, np.int32)
        self._chk(self.L.orc_render_row_list(self.h, msec, len(r), _p(r), _p(fb), nthreads, int(quirk_sum), None))
        return fb

    def primary_hits(self, msec=0):
        o = self.opts
        n = o.width * o.height
        obj = np.zeros(n, np.int32)
        prim = np.zeros(n, np.int32)
        t = np.zeros(n, np.float64)
        tie = np.zeros(n, np.uint8)
        self._chk(self.L.orc_primary_hits(self.h, msec, _p(obj), _p(prim), _p(t), _p(tie)))
        return obj, prim, t, tie

    def cast_rays(self, orig, dirs, times=None):
        orig = np.ascontiguousarray(orig, np.float64)
        dirs = np.ascontiguousarray(dirs, np.float64)
        n = len(orig)
        tm = None if times is None else np.ascontiguousarray(times, np.int32)
        obj = np.zeros(n, np.int32)
        prim = np.zeros(n, np.int32)
        t = np.zeros(n, np.float64)
        tie = np.zeros(n, np.uint8)
        self._chk(self.L.orc_cast_rays(self.h, n, _p(orig), _p(dirs), _p(tm), _p(obj), _p(prim), _p(t), _p(tie)))
        return obj, prim, t, tie

    def gather(self, which, pos, norm):
        pos = np.ascontiguousarray(pos, np.float64)
        norm = np.ascontiguousarray(norm, np.float64)
        out = np.zeros((len(pos), 4), np.float64)
        self._chk(self.L.orc_gather(self.h, which, len(pos), _p(pos), _p(norm), _p(out)))
        return out

    def set_opts(self, **kw):
        """Change options of the loaded scene (photon counts, samples...);
        the next call prepares the frame again."""
        for k, v in kw.items():
            setattr(self.opts, k, v)
        self._chk(self.L.orc_set_opts(self.h, ctypes.byref(self.opts)))

    def set_pixel_base(self, base):
        """Key pixel p's streams as pixel base + p (a job of a GPU batch)."""
        self._chk(self.L.orc_set_pixel_base(self.h, int(base)))

    def phase_ms(self):
        """(scene tree + frame tables, projection maps, photons) of the last
        prepare, wall ms."""
        ms = np.zeros(3, np.float64)
        self._chk(self.L.orc_phase_ms(self.h, _p(ms)))
        return dict(build=float(ms[0]), projmaps=float(ms[1]), photons=float(ms[2]))

    def counters(self):
        v = [ctypes.c_int64() for _ in range(5)]
        self._chk(self.L.orc_counters(self.h, *[ctypes.byref(x) for x in v]))
        return dict(zip(["rays", "node_visits", "prim_tests", "shadow_rays", "gathers"], [x.value for x in v]))
