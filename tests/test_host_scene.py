"""Host-side scene loading (no GPU): texture files and their search path,
textured material attributes, and keyframe evaluation, checked by
tests/host_check.cc compiled with the scene loader."""
import os
import subprocess

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_textures_and_keyframes(tmp_path):
    from sray_gb300 import scenegen
    csrc = os.path.join(ROOT, "sray_gb300", "csrc")
    exe = tmp_path / "host_check"
    subprocess.check_call(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-I" + os.path.join(ROOT, "include"), "-I" + csrc,
                           "-I/usr/local/cuda/include", os.path.join(ROOT, "tests", "host_check.cc"),
                           os.path.join(csrc, "scene_host.cc"), os.path.join(csrc, "bvh_host.cc"), "-o", str(exe), "-lpthread"])
    out = subprocess.run([str(exe), str(tmp_path / "data"), scenegen.write_scene("animated")], capture_output=True, text=True)
    print(out.stdout)
    assert out.returncode == 0, out.stdout + out.stderr
