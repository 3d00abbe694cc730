"""The binary mesh side-car (host code, no GPU): compiled with the scene
loader and checked by tests/sidecar_check.cc on the small benchmark scene."""
import os
import subprocess

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_sidecar_round_trip(tmp_path):
    from sray_gb300 import scenegen
    csrc = os.path.join(ROOT, "sray_gb300", "csrc")
    exe = tmp_path / "sidecar_check"
    subprocess.check_call(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-I" + os.path.join(ROOT, "include"), "-I" + csrc,
                           "-I/usr/local/cuda/include", os.path.join(ROOT, "tests", "sidecar_check.cc"),
                           os.path.join(csrc, "scene_host.cc"), os.path.join(csrc, "bvh_host.cc"), "-o", str(exe), "-lpthread"])
    out = subprocess.run([str(exe), scenegen.write_scene("small"), str(tmp_path / "small.srmesh")], capture_output=True, text=True)
    print(out.stdout)
    assert out.returncode == 0, out.stdout + out.stderr
