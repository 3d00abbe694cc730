"""ctypes binding of libsray_gpu.so (include/sray_gpu.h).

There is no CPU fallback: if the native library is missing or no CUDA
device is present, every call raises.  Device buffers can be torch CUDA
tensors (passed by data_ptr) or raw device pointers.
"""
import ctypes
import os

import numpy as np

from .options import SrayOpts, make_opts

_LIB = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_lib", "libsray_gpu.so")
_lib = None

EXPORTS = ["sray_default_opts", "sray_gpu_init", "sray_gpu_set_opts", "sray_gpu_load_scene", "sray_gpu_load_scene_mem",
           "sray_gpu_load_scene_sidecar", "sray_gpu_add_data_path",
           "sray_gpu_scene_info", "sray_gpu_build", "sray_gpu_shoot_photons", "sray_gpu_render",
           "sray_gpu_render_pixels", "sray_gpu_cast_rays", "sray_gpu_primary_hits", "sray_gpu_photon_gather", "sray_gpu_photon_gather_noalloc",
           "sray_gpu_get_photons", "sray_gpu_dump_photons", "sray_gpu_restore_photons", "sray_gpu_render_batch",
           "sray_gpu_get_stats", "sray_gpu_nrc_stats", "sray_gpu_nrc_reset", "sray_gpu_get_tuning",
           "sray_gpu_set_tuning", "sray_gpu_autotune", "sray_gpu_set_profiling", "sray_gpu_kernel_times", "sray_gpu_last_error",
           "sray_gpu_shutdown", "sray_gpu_set_faults", "sray_gpu_upload_scene", "sray_gpu_load_scene_set",
           "sray_gpu_autotune_batch", "sray_nrc_reset", "sray_nrc_set_params", "sray_nrc_get_params", "sray_nrc_infer",
           "sray_nrc_infer_async", "sray_nrc_check", "sray_nrc_gradients", "sray_nrc_train", "sray_nrc_last_error"]

NRC_PARAMS = 26563


class SrayStats(ctypes.Structure):
    _fields_ = [("primary_rays", ctypes.c_int64), ("shadow_rays", ctypes.c_int64),
                ("secondary_rays", ctypes.c_int64), ("gather_rays", ctypes.c_int64),
                ("photons_emitted", ctypes.c_int64), ("photons_stored", ctypes.c_int64),
                ("gathers", ctypes.c_int64), ("samples", ctypes.c_int64),
                ("node_visits", ctypes.c_int64), ("prim_tests", ctypes.c_int64),
                ("kernel_launches", ctypes.c_int), ("pad", ctypes.c_int),
                ("h2d_bytes", ctypes.c_int64), ("d2h_bytes", ctypes.c_int64),
                ("gather_tested", ctypes.c_int64), ("gather_candidates", ctypes.c_int64),
                ("gather_selects", ctypes.c_int64), ("gather_spills", ctypes.c_int64),
                ("bvh_fallbacks", ctypes.c_int64),
                ("shadow_node_visits", ctypes.c_int64), ("shadow_prim_tests", ctypes.c_int64)]


class SrayNrcStats(ctypes.Structure):
    _fields_ = [("frames", ctypes.c_int64), ("vertices", ctypes.c_int64), ("cached", ctypes.c_int64),
                ("train_samples", ctypes.c_int64), ("val_samples", ctypes.c_int64),
                ("regions", ctypes.c_int), ("regions_validated", ctypes.c_int), ("regions_cached", ctypes.c_int),
                ("val_rel_err", ctypes.c_float), ("loss", ctypes.c_float), ("pad", ctypes.c_int),
                ("reserved", ctypes.c_int64 * 4)]


class SrayJob(ctypes.Structure):
    _fields_ = [("msec", ctypes.c_long), ("width", ctypes.c_int), ("height", ctypes.c_int), ("fb", ctypes.c_void_p),
                ("scene", ctypes.c_int), ("caust_photons", ctypes.c_int), ("gi_photons", ctypes.c_int),
                ("reserved", ctypes.c_int)]


class SrayFaults(ctypes.Structure):
    _fields_ = [("fail_alloc_after", ctypes.c_int), ("queue_cap", ctypes.c_int), ("pool_spin_limit", ctypes.c_int),
                ("photon_group", ctypes.c_int), ("reserved", ctypes.c_int * 4)]


class SrayTuning(ctypes.Structure):
    _fields_ = [("render_tail", ctypes.c_int), ("pool_blocks_per_sm", ctypes.c_int), ("photon_tail", ctypes.c_int),
                ("shadow_order", ctypes.c_int), ("stream_priority", ctypes.c_int), ("warp_rays", ctypes.c_int),
                ("warp_segments", ctypes.c_int), ("queue_depth", ctypes.c_int), ("side_gather", ctypes.c_int),
                ("sort_rays", ctypes.c_int), ("side_shadow", ctypes.c_int)]


class SrayTuneTrial(ctypes.Structure):
    _fields_ = [("tuning", SrayTuning), ("ms_per_frame", ctypes.c_float), ("pad", ctypes.c_int)]


def _tuning_dict(t):
    return {f[0]: getattr(t, f[0]) for f in SrayTuning._fields_ if f[0] != "reserved"}


class SrayError(RuntimeError):
    """A failed call: the library's message and its SRAY_E* code."""

    def __init__(self, msg, code=None):
        super().__init__(msg)
        self.code = code


# the library's status codes (include/sray_gpu.h)
SRAY_EINVAL, SRAY_ELOAD, SRAY_ECUDA, SRAY_ESTATE, SRAY_EDEVICE, SRAY_ENOMEM, SRAY_EIO = -1, -2, -3, -4, -5, -6, -7


def lib_path():
    return _LIB


def load_library():
    """Load the native library (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(_LIB):
        raise SrayError("libsray_gpu.so not built: run sray_gb300.build.build() (%s)" % _LIB)
    L = ctypes.CDLL(_LIB)
    vp, ip, lp = ctypes.c_void_p, ctypes.c_int, ctypes.c_long
    L.sray_default_opts.argtypes = [ctypes.POINTER(SrayOpts)]
    L.sray_gpu_init.argtypes = [ctypes.POINTER(SrayOpts)]
    L.sray_gpu_set_opts.argtypes = [ctypes.POINTER(SrayOpts)]
    L.sray_gpu_load_scene.argtypes = [ctypes.c_char_p]
    L.sray_gpu_load_scene_mem.argtypes = [ctypes.c_char_p, ctypes.c_size_t]
    L.sray_gpu_load_scene_sidecar.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.POINTER(ctypes.c_int)]
    L.sray_gpu_add_data_path.argtypes = [ctypes.c_char_p]
    L.sray_gpu_scene_info.argtypes = [vp, vp, vp, vp, vp]
    L.sray_gpu_build.argtypes = [lp, lp]
    L.sray_gpu_shoot_photons.argtypes = [lp, lp, vp, vp, vp]
    L.sray_gpu_render.argtypes = [lp, vp, ip, vp]
    L.sray_gpu_render_pixels.argtypes = [lp, vp, ip, vp]
    L.sray_gpu_cast_rays.argtypes = [ip, vp, vp, vp, vp, vp, vp, vp, vp]
    L.sray_gpu_primary_hits.argtypes = [lp, vp, vp, vp, vp, vp]
    L.sray_gpu_photon_gather.argtypes = [ip, ip, vp, vp, vp, vp]
    L.sray_gpu_photon_gather_noalloc.argtypes = [ip, ip, vp, vp, vp, vp]
    L.sray_gpu_get_photons.argtypes = [ip, vp, ip, vp]
    L.sray_gpu_dump_photons.argtypes = [ip, ctypes.c_char_p]
    L.sray_gpu_render_batch.argtypes = [ctypes.POINTER(SrayJob), ip, vp]
    L.sray_gpu_load_scene_set.argtypes = [ctypes.POINTER(ctypes.c_char_p), ip]
    L.sray_gpu_autotune_batch.argtypes = [ctypes.POINTER(SrayJob), ip, ip, vp, ctypes.POINTER(SrayTuning),
                                          ctypes.POINTER(ctypes.c_float), ctypes.POINTER(SrayTuneTrial), ip,
                                          ctypes.POINTER(ctypes.c_int)]
    L.sray_gpu_restore_photons.argtypes = [ip, ctypes.c_char_p, ctypes.POINTER(ctypes.c_int)]
    L.sray_gpu_get_stats.argtypes = [ctypes.POINTER(SrayStats)]
    L.sray_gpu_nrc_stats.argtypes = [ctypes.POINTER(SrayNrcStats)]
    L.sray_gpu_nrc_reset.argtypes = [ctypes.c_uint64]
    L.sray_gpu_get_tuning.argtypes = [ctypes.POINTER(SrayTuning)]
    L.sray_gpu_set_tuning.argtypes = [ctypes.POINTER(SrayTuning)]
    L.sray_gpu_autotune.argtypes = [lp, vp, ip, vp, ctypes.POINTER(SrayTuning), ctypes.POINTER(ctypes.c_float),
                                    ctypes.POINTER(SrayTuneTrial), ip, ctypes.POINTER(ctypes.c_int)]
    L.sray_gpu_set_profiling.argtypes = [ip]
    L.sray_gpu_kernel_times.argtypes = [ctypes.c_char_p, ctypes.c_size_t, vp, vp, ip, vp, ip]
    L.sray_gpu_last_error.argtypes = [ctypes.c_char_p, ctypes.c_size_t]
    L.sray_gpu_set_faults.argtypes = [ctypes.POINTER(SrayFaults)]
    from .scene_desc import SceneDescC
    L.sray_gpu_upload_scene.argtypes = [ctypes.POINTER(SceneDescC)]
    L.sray_gpu_shutdown.argtypes = []
    L.sray_gpu_shutdown.restype = None
    L.sray_nrc_reset.argtypes = [ctypes.c_uint64]
    L.sray_nrc_set_params.argtypes = [vp, ip]
    L.sray_nrc_get_params.argtypes = [vp, ip]
    L.sray_nrc_infer.argtypes = [ip, vp, vp, vp]
    L.sray_nrc_infer_async.argtypes = [ip, vp, vp, vp]
    L.sray_nrc_check.argtypes = [vp]
    L.sray_nrc_gradients.argtypes = [ip, vp, vp, vp, vp, vp]
    L.sray_nrc_train.argtypes = [ip, vp, vp, vp, vp]
    L.sray_nrc_last_error.argtypes = [ctypes.c_char_p, ctypes.c_size_t]
    _lib = L
    return L


class RadianceCache:
    """The radiance-cache MLP through its C-ABI (inputs and outputs are CUDA
    tensors: x [n, 9] float32, targets [n, 3])."""

    def __init__(self, seed=1):
        """seed: re-initialise the network from it; None: use the network as it
        is (the one the renderer trains)."""
        self.L = load_library()
        if seed is not None:
            self._chk(self.L.sray_nrc_reset(seed))

    def _chk(self, r):
        if r != 0:
            buf = ctypes.create_string_buffer(512)
            self.L.sray_nrc_last_error(buf, 512)
            raise SrayError("radiance cache error %d: %s" % (r, buf.value.decode(errors="replace")))

    def set_params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        self._chk(self.L.sray_nrc_set_params(_ptr(p), p.size))

    def params(self):
        p = np.zeros(NRC_PARAMS, np.float32)
        self._chk(self.L.sray_nrc_get_params(_ptr(p), p.size))
        return p

    def infer(self, x, y, stream=None, sync=True):
        """y = network(x); with sync=False the launch is only enqueued and
        check() reports a device-side failure."""
        f = self.L.sray_nrc_infer if sync else self.L.sray_nrc_infer_async
        self._chk(f(x.shape[0], _ptr(x), _ptr(y), _stream(stream)))

    def check(self, stream=None):
        self._chk(self.L.sray_nrc_check(_stream(stream)))

    def gradients(self, x, t, grad, loss, stream=None):
        self._chk(self.L.sray_nrc_gradients(x.shape[0], _ptr(x), _ptr(t), _ptr(grad), _ptr(loss), _stream(stream)))

    def train(self, x, t, loss=None, stream=None):
        self._chk(self.L.sray_nrc_train(x.shape[0], _ptr(x), _ptr(t), _ptr(loss), _stream(stream)))


def _ptr(x):
    if x is None:
        return None
    if isinstance(x, int):
        return ctypes.c_void_p(x)
    if hasattr(x, "data_ptr"):
        return ctypes.c_void_p(x.data_ptr())
    if isinstance(x, np.ndarray):
        return x.ctypes.data_as(ctypes.c_void_p)
    raise TypeError("unsupported buffer %r" % type(x))


def _stream(stream):
    if stream is None:
        return None
    if hasattr(stream, "cuda_stream"):
        return ctypes.c_void_p(stream.cuda_stream)
    return ctypes.c_void_p(int(stream))


class GpuRenderer:
    """The GPU renderer context (one per process)."""

    def __init__(self, opts=None, **kw):
        self.L = load_library()
        self.opts = opts if isinstance(opts, SrayOpts) else make_opts(**(opts or {}), **kw)
        self._chk(self.L.sray_gpu_init(ctypes.byref(self.opts)))

    def _chk(self, r):
        if r != 0:
            buf = ctypes.create_string_buffer(1024)
            self.L.sray_gpu_last_error(buf, 1024)
            raise SrayError("%s (code %d)" % (buf.value.decode(errors="replace"), r), r)
        return r

    def set_opts(self, **kw):
        for k, v in kw.items():
            setattr(self.opts, k, v)
        self._chk(self.L.sray_gpu_set_opts(ctypes.byref(self.opts)))

    def load(self, path, sidecar=None):
        """Load an XML scene; with `sidecar`, through the binary side-car of its
        meshes (written when missing or stale).  Returns True when the side-car
        was used."""
        if sidecar is None:
            self._chk(self.L.sray_gpu_load_scene(path.encode()))
            return False
        used = ctypes.c_int()
        self._chk(self.L.sray_gpu_load_scene_sidecar(path.encode(), sidecar.encode(), ctypes.byref(used)))
        return bool(used.value)

    def upload_scene(self, desc):
        """Load a scene given as tables (sray_gb300.scene_desc.SceneDesc)."""
        c = desc.c()
        self._chk(self.L.sray_gpu_upload_scene(ctypes.byref(c)))

    def load_xml(self, xml):
        b = xml.encode() if isinstance(xml, str) else xml
        self._chk(self.L.sray_gpu_load_scene_mem(b, len(b)))

    def add_data_path(self, directory):
        """Prepend a directory to the texture search path (SRAY_DATA_PATH);
        textures are looked up in its first directory only."""
        self._chk(self.L.sray_gpu_add_data_path(directory.encode()))

    def scene_info(self):
        a, b, c, e = ctypes.c_int(), ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        d = ctypes.c_int64()
        self._chk(self.L.sray_gpu_scene_info(ctypes.byref(a), ctypes.byref(b), ctypes.byref(c), ctypes.byref(d),
                                             ctypes.byref(e)))
        return dict(objects=a.value, lights=b.value, materials=c.value, triangles=d.value, unique_meshes=e.value)

    def build(self, t0=0, t1=0):
        self._chk(self.L.sray_gpu_build(t0, t1))

    def shoot_photons(self, t0=0, t1=0, stream=None):
        c, g = ctypes.c_int(), ctypes.c_int()
        self._chk(self.L.sray_gpu_shoot_photons(t0, t1, ctypes.byref(c), ctypes.byref(g), _stream(stream)))
        return c.value, g.value

    def render(self, msec=0, fb=None, stream=None):
        """Full frame (accel build + photons + pixels).  fb: None -> returns a
        host numpy [h, w, 4]; a CUDA tensor / device pointer -> written in place."""
        if fb is None:
            out = np.zeros((self.opts.height, self.opts.width, 4), np.float32)
            self._chk(self.L.sray_gpu_render(msec, _ptr(out), 0, _stream(stream)))
            return out
        if isinstance(fb, np.ndarray):
            self._chk(self.L.sray_gpu_render(msec, _ptr(fb), 0, _stream(stream)))
            return fb
        self._chk(self.L.sray_gpu_render(msec, _ptr(fb), 1, _stream(stream)))
        return fb

    @staticmethod
    def _jobs(jobs):
        arr = (SrayJob * len(jobs))()
        for i, job in enumerate(jobs):
            msec, fb = job[0], job[1]
            extra = job[2] if len(job) > 2 else {}
            arr[i].msec = msec
            arr[i].height, arr[i].width = int(fb.shape[0]), int(fb.shape[1])
            arr[i].fb = fb.data_ptr()
            arr[i].scene = int(extra.get("scene", 0))
            arr[i].caust_photons = int(extra.get("caust_photons", 0))
            arr[i].gi_photons = int(extra.get("gi_photons", 0))
        return arr

    def render_batch(self, jobs, stream=None):
        """Render several frames in one wavefront: jobs = [(msec, fb)] or
        [(msec, fb, {"scene": k, "caust_photons": c, "gi_photons": g})], fb a
        CUDA tensor [height, width, 4] float32 per job."""
        self._chk(self.L.sray_gpu_render_batch(self._jobs(jobs), len(jobs), _stream(stream)))

    def load_scene_set(self, paths):
        """Load several documents as one scene set (jobs pick theirs by index)."""
        arr = (ctypes.c_char_p * len(paths))(*[p.encode() for p in paths])
        self._chk(self.L.sray_gpu_load_scene_set(arr, len(paths)))

    def autotune_batch(self, jobs, frames=2, stream=None):
        """The batch autotuner: queue depth x traversal mode; returns (tuning,
        ms per batch, [(tuning, ms) per trial])."""
        best = SrayTuning()
        ms = ctypes.c_float()
        log = (SrayTuneTrial * 16)()
        n = ctypes.c_int()
        self._chk(self.L.sray_gpu_autotune_batch(self._jobs(jobs), len(jobs), frames, _stream(stream), ctypes.byref(best),
                                                 ctypes.byref(ms), log, 16, ctypes.byref(n)))
        trials = [(_tuning_dict(log[i].tuning), log[i].ms_per_frame) for i in range(min(n.value, 16))]
        return _tuning_dict(best), ms.value, trials

    def render_pixels(self, msec=0, fb=None, stream=None):
        if fb is None:
            out = np.zeros((self.opts.height, self.opts.width, 4), np.float32)
            self._chk(self.L.sray_gpu_render_pixels(msec, _ptr(out), 0, _stream(stream)))
            return out
        dev = 0 if isinstance(fb, np.ndarray) else 1
        self._chk(self.L.sray_gpu_render_pixels(msec, _ptr(fb), dev, _stream(stream)))
        return fb

    def primary_hits(self, obj, prim, t, tie, msec=0, stream=None):
        """Device buffers of width*height entries (int32, int32, float32, uint8)."""
        self._chk(self.L.sray_gpu_primary_hits(msec, _ptr(obj), _ptr(prim), _ptr(t), _ptr(tie), _stream(stream)))

    def cast_rays(self, orig, dirs, times, obj, prim, t, tie, stream=None):
        n = int(orig.shape[0])
        self._chk(self.L.sray_gpu_cast_rays(n, _ptr(orig), _ptr(dirs), _ptr(times), _ptr(obj), _ptr(prim), _ptr(t),
                                            _ptr(tie), _stream(stream)))

    def photon_gather(self, which, pos, norm, out, stream=None):
        """Estimates at caller points (device arrays n*3 float32)."""
        n = int(pos.shape[0])
        self._chk(self.L.sray_gpu_photon_gather(which, n, _ptr(pos), _ptr(norm), _ptr(out), _stream(stream)))
        return out

    def photon_gather_noalloc(self, which, pos, norm, out, stream=None):
        """Same estimates as photon_gather without any device allocation (at
        most SRAY_NOALLOC_MAX_POINTS = 65536 points per call)."""
        n = int(pos.shape[0])
        self._chk(self.L.sray_gpu_photon_gather_noalloc(which, n, _ptr(pos), _ptr(norm), _ptr(out), _stream(stream)))
        return out

    def photons(self, which):
        n = ctypes.c_int()
        self._chk(self.L.sray_gpu_get_photons(which, None, 0, ctypes.byref(n)))
        out = np.zeros((max(n.value, 1), 16), np.float32)
        self._chk(self.L.sray_gpu_get_photons(which, _ptr(out), n.value, ctypes.byref(n)))
        return out[:n.value]

    def dump_photons(self, which, path):
        """Write map `which` (0 caustic, 1 global) in the reference's dump format."""
        self._chk(self.L.sray_gpu_dump_photons(which, path.encode()))

    def restore_photons(self, which, path):
        """Rebuild map `which` from a dump (after build()); returns the photon count."""
        n = ctypes.c_int()
        self._chk(self.L.sray_gpu_restore_photons(which, path.encode(), ctypes.byref(n)))
        return n.value

    def stats(self):
        st = SrayStats()
        self._chk(self.L.sray_gpu_get_stats(ctypes.byref(st)))
        return {f[0]: getattr(st, f[0]) for f in SrayStats._fields_ if f[0] not in ("reserved", "pad")}

    def nrc_stats(self):
        """Radiance-cache state: frames trained, the last frame's final-gather
        vertices and how many the network served, training / validation
        records, regions validated and served, validation relative error, loss."""
        st = SrayNrcStats()
        self._chk(self.L.sray_gpu_nrc_stats(ctypes.byref(st)))
        return {f[0]: getattr(st, f[0]) for f in SrayNrcStats._fields_ if f[0] not in ("reserved", "pad")}

    def nrc_reset(self, seed=None):
        """Re-initialise the network and forget the regions' validation history."""
        self._chk(self.L.sray_gpu_nrc_reset(self.opts.seed if seed is None else seed))

    def set_faults(self, fail_alloc_after=-1, queue_cap=0, pool_spin_limit=0, photon_group=0):
        """Host-side fault injection for tests (sray_gpu_set_faults); the
        defaults turn it off."""
        f = SrayFaults(fail_alloc_after, queue_cap, pool_spin_limit, photon_group)
        self._chk(self.L.sray_gpu_set_faults(ctypes.byref(f)))

    def tuning(self):
        t = SrayTuning()
        self._chk(self.L.sray_gpu_get_tuning(ctypes.byref(t)))
        return _tuning_dict(t)

    def set_tuning(self, **kw):
        t = SrayTuning()
        self._chk(self.L.sray_gpu_get_tuning(ctypes.byref(t)))
        for k, v in kw.items():
            setattr(t, k, v)
        self._chk(self.L.sray_gpu_set_tuning(ctypes.byref(t)))

    def autotune(self, fb, msec=0, frames=3, stream=None):
        """Pick the fastest tuning for frame `msec` (device framebuffer `fb`);
        returns (tuning, ms per frame, [(tuning, ms) per trial])."""
        best = SrayTuning()
        ms = ctypes.c_float()
        log = (SrayTuneTrial * 64)()
        n = ctypes.c_int()
        self._chk(self.L.sray_gpu_autotune(msec, _ptr(fb), frames, _stream(stream), ctypes.byref(best), ctypes.byref(ms),
                                           log, 64, ctypes.byref(n)))
        trials = [(_tuning_dict(log[i].tuning), log[i].ms_per_frame) for i in range(min(n.value, 64))]
        return _tuning_dict(best), ms.value, trials

    def set_profiling(self, time_kernels=False, count_work=False):
        self._chk(self.L.sray_gpu_set_profiling((1 if time_kernels else 0) | (2 if count_work else 0)))

    def kernel_times(self, reset=True, host=False):
        """{kernel kind: (total ms, launches)} accumulated since the last reset;
        with host=True also the host phases ("host.<phase>": total ms, times
        entered) timed beside them."""
        names = ctypes.create_string_buffer(4096)
        ms = np.zeros(64, np.float64)
        ln = np.zeros(64, np.int64)
        n = ctypes.c_int()
        self._chk(self.L.sray_gpu_kernel_times(names, 4096, _ptr(ms), _ptr(ln), 64, ctypes.byref(n), int(reset)))
        keys = names.raw.split(b"\0")[:n.value]
        out = {k.decode(): (float(ms[i]), int(ln[i])) for i, k in enumerate(keys)}
        return out if host else {k: v for k, v in out.items() if not k.startswith("host.")}

    def close(self):
        self.L.sray_gpu_shutdown()
