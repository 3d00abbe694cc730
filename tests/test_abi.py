"""The C-ABI library loads and exports every entry point its header declares
(no GPU needed: nothing is called)."""
import ctypes
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared(header):
    src = open(os.path.join(ROOT, "include", header)).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(sray_[a-z0-9_]+)\s*\(", src)))


def test_library_exports_header():
    from sray_gb300 import build, gpu
    build.build()
    lib = ctypes.CDLL(gpu.lib_path())
    names = declared("sray_gpu.h")
    assert len(names) >= 15
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    assert sorted(gpu.EXPORTS) == names
