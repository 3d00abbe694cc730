"""Scenes given as tables (sray_gpu_upload_scene), on the host (no GPU):
the host scene the library builds from a sray_scene_desc equals the one its
XML loader builds from the same document -- materials, textures, objects,
meshes, lights, environment, and every object, light and camera transform
at every millisecond of a window (tests/desc_check.cc).  The tables come
from sray_gb300/scene_desc.py and, where the reference's sources are
present, from the reference-side adapter walking the reference's own
in-memory Scene (sray_gb300/adapter/render_gpu.cc)."""
import ctypes
import os
import subprocess

import pytest

from sray_gb300 import scene_desc, scenegen
from sray_gb300.options import make_opts

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "sray_gb300", "csrc")
# scene, its options, the window of milliseconds compared
CASES = [("small", {}, (0, 0)), ("feature", dict(mblur=1, shutter=40), (-45, 45)), ("animated", {}, (-5, 1400)),
         ("textured", {}, (0, 0)), ("production_small", {}, (0, 0))]


def _scene(name):
    if name == "production_small":
        return scenegen.write_scene("production", grid=(60, 30), n_inst=12)
    return scenegen.write_scene(name)


@pytest.fixture(scope="module")
def checker(tmp_path_factory):
    out = tmp_path_factory.mktemp("desc") / "libdesc_check.so"
    subprocess.check_call(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-I" + os.path.join(ROOT, "include"),
                           "-I" + CSRC, "-I/usr/local/cuda/include", os.path.join(ROOT, "tests", "desc_check.cc"),
                           os.path.join(CSRC, "scene_host.cc"), os.path.join(CSRC, "bvh_host.cc"), "-o", str(out), "-lpthread"])
    lib = ctypes.CDLL(str(out))
    lib.desc_matches_xml.argtypes = [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_size_t, ctypes.c_void_p, ctypes.c_int,
                                     ctypes.c_int, ctypes.c_int, ctypes.c_char_p, ctypes.c_size_t]
    return lib


@pytest.mark.parametrize("name,over,window", CASES)
def test_tables_build_the_xml_scene(checker, name, over, window, monkeypatch, tmp_path):
    path = _scene(name)
    if name == "textured":
        scenegen.write_textures(str(tmp_path))
        monkeypatch.setenv("SRAY_DATA_PATH", str(tmp_path))
    xml = open(path, "rb").read()
    opts = make_opts(**dict(scenegen.scene_opts("small"), width=96, height=72, **over))
    d = scene_desc.from_xml(xml, shutter=opts.shutter)
    c = d.c()
    msg = ctypes.create_string_buffer(512)
    ok = checker.desc_matches_xml(ctypes.byref(c), xml, len(xml), ctypes.byref(opts), window[0], window[1], 1, msg, 512)
    print("%s: %s" % (name, msg.value.decode()))
    assert ok == 1, msg.value.decode()


def _reference_objects():
    from oracle import build_ref
    harness = build_ref.build()
    if not harness:
        return None
    ref_dir = os.path.dirname(harness)
    objs = [os.path.join(ref_dir, f) for f in sorted(os.listdir(ref_dir))
            if f.endswith(".o") and f not in ("render.cc.o", "ref_harness.cc.o")]
    return build_ref, objs


def test_adapter_on_the_reference_scene(tmp_path):
    """The adapter flattens the reference's own Scene (loaded by its
    Scene::load) into tables that build the same host scene."""
    from sray_gb300 import build as gbuild
    ref = _reference_objects()
    if ref is None:
        pytest.skip("the reference's sources are not present")
    build_ref, objs = ref
    lib = gbuild.build()
    exe = tmp_path / "adapter_check"
    # the library's host scene (C++17) and the adapter against the reference's headers (its dialect)
    ours = []
    for src in (os.path.join(ROOT, "tests", "desc_check.cc"), os.path.join(CSRC, "scene_host.cc"), os.path.join(CSRC, "bvh_host.cc")):
        o = str(tmp_path / (os.path.basename(src) + ".o"))
        subprocess.check_call(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-I" + os.path.join(ROOT, "include"), "-I" + CSRC,
                               "-I/usr/local/cuda/include", "-c", src, "-o", o])
        ours.append(o)
    inc = ["-I" + build_ref.SHIM, "-I" + build_ref.ORACLE, "-I" + os.path.join(ROOT, "include"), "-I" + build_ref.REF_SRC,
           "-I" + os.path.join(ROOT, "sray_gb300", "adapter")]
    cmd = ["g++", "-std=gnu++11", "-O1", "-w", "-ffp-contract=off"] + inc + [
        os.path.join(ROOT, "tests", "adapter_check.cc"), os.path.join(ROOT, "sray_gb300", "adapter", "render_gpu.cc")] + ours + objs + [
        "-L" + os.path.dirname(lib), "-lsray_gpu", "-Wl,-rpath," + os.path.dirname(lib), "-lexpat", "-lpthread", "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    for name, over, window in CASES:
        if name == "textured":
            continue            # the reference keeps a texture's image private: the adapter sends colours only
        path = _scene(name)
        cli = ["-s", "96x72"]
        if over.get("mblur"):
            cli += ["-m", "-u", str(over["shutter"])]
        if name == "production_small":
            cli += ["-moctdepth", "8", "-moctitems", "8"]
        out = subprocess.run([str(exe), path, str(window[0]), str(window[1])] + cli, capture_output=True, text=True)
        print(out.stdout.strip())
        assert out.returncode == 0, out.stdout + out.stderr[-2000:]
