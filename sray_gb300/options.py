"""ctypes mirror of `sray_opts` (include/sray_gpu.h) and its defaults.

Field meanings and defaults follow the reference's `struct options`
(src/opt.h:38-62, defaults src/opt.c:357-388); the trailing fields are
extensions of this library (k-nearest gathers, path-keyed random streams,
the Philox seed, the radiance cache).
"""
import ctypes

__all__ = ["SrayOpts", "make_opts", "DEFAULTS"]


class SrayOpts(ctypes.Structure):
    _fields_ = [
        ("width", ctypes.c_int), ("height", ctypes.c_int),
        ("min_samples", ctypes.c_int), ("max_samples", ctypes.c_int),
        ("max_var", ctypes.c_float), ("min_energy", ctypes.c_float),
        ("shadow_samples", ctypes.c_int), ("diffuse_samples", ctypes.c_int),
        ("threads", ctypes.c_int), ("blk_sz", ctypes.c_int), ("iter", ctypes.c_int),
        ("fps", ctypes.c_int), ("mblur", ctypes.c_int), ("shutter", ctypes.c_int),
        ("time_start", ctypes.c_int), ("time_end", ctypes.c_int),
        ("caust_photons", ctypes.c_int), ("gi_photons", ctypes.c_int),
        ("gather_dist", ctypes.c_float), ("photon_energy", ctypes.c_float),
        ("scnoct_max_depth", ctypes.c_int), ("scnoct_max_items", ctypes.c_int),
        ("meshoct_max_depth", ctypes.c_int), ("meshoct_max_items", ctypes.c_int),
        ("caust_k", ctypes.c_int), ("gi_k", ctypes.c_int), ("gather_rcap", ctypes.c_float),
        ("rng_paths", ctypes.c_int), ("seed", ctypes.c_uint64),
        ("nrc", ctypes.c_int), ("nrc_train_samples", ctypes.c_int), ("nrc_max_rel_err", ctypes.c_float),
        ("nrc_train_steps", ctypes.c_int), ("nrc_fallback_samples", ctypes.c_int),
        ("reserved", ctypes.c_int * 3),
    ]


DEFAULTS = dict(width=640, height=480, min_samples=1, max_samples=1, max_var=0.005, min_energy=0.0001,
                shadow_samples=1, diffuse_samples=1, threads=0, blk_sz=48, iter=7, fps=30, mblur=0,
                shutter=0, time_start=0, time_end=0, caust_photons=0, gi_photons=0, gather_dist=0.001,
                photon_energy=300.0, scnoct_max_depth=5, scnoct_max_items=5, meshoct_max_depth=7,
                meshoct_max_items=14, caust_k=0, gi_k=0, gather_rcap=0.5, rng_paths=1, seed=0x5EED0001,
                nrc=0, nrc_train_samples=65536, nrc_max_rel_err=0.05, nrc_train_steps=4,
                nrc_fallback_samples=0)


def make_opts(**kw):
    """sray_opts with the reference defaults, overridden by keyword."""
    d = dict(DEFAULTS)
    for k in kw:
        if k not in d:
            raise KeyError("unknown option %r" % k)
    d.update(kw)
    o = SrayOpts()
    for k, v in d.items():
        setattr(o, k, v)
    return o
