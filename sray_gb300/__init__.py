"""sray_gb300 -- S-ray's rendering hot path rebuilt for one NVIDIA GB300."""
from .options import SrayOpts, make_opts  # noqa: F401
