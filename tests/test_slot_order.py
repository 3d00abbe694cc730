"""The first sample batch's slot -> pixel order (slot_pixel), checked on the
host: tests/slot_order_check.cc compiled against the product header."""
import os
import subprocess

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_slot_order(tmp_path):
    exe = tmp_path / "slot_order_check"
    subprocess.check_call(["g++", "-O2", "-std=c++17", "-I" + os.path.join(ROOT, "sray_gb300", "csrc"),
                           os.path.join(ROOT, "tests", "slot_order_check.cc"), "-o", str(exe)])
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
