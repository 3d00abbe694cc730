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


def test_struct_layouts_match_header(tmp_path):
    """The ctypes mirrors have the header's sizes and field offsets."""
    import subprocess
    from sray_gb300.options import SrayOpts
    from sray_gb300.gpu import SrayStats, SrayNrcStats, SrayTuning, SrayTuneTrial, SrayJob, SrayFaults
    mirrors = {"sray_opts": SrayOpts, "sray_stats": SrayStats, "sray_nrc_stats": SrayNrcStats, "sray_tuning": SrayTuning,
               "sray_tune_trial": SrayTuneTrial, "sray_job": SrayJob, "sray_faults": SrayFaults}
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "sray_gpu.h"', "int main(void) {"]
    for cname, py in mirrors.items():
        lines.append('printf("%s %%zu\\n", sizeof(%s));' % (cname, cname))
        for f in py._fields_:
            lines.append('printf("%s.%s %%zu\\n", offsetof(%s, %s));' % (cname, f[0], cname, f[0]))
    lines.append("return 0; }")
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.check_call(["gcc", "-I" + os.path.join(ROOT, "include"), str(src), "-o", str(exe)])
    got = dict(line.split() for line in subprocess.check_output([str(exe)], text=True).splitlines())
    for cname, py in mirrors.items():
        assert int(got[cname]) == ctypes.sizeof(py), cname
        for f in py._fields_:
            assert int(got["%s.%s" % (cname, f[0])]) == getattr(py, f[0]).offset, (cname, f[0])
