"""Photon-map dumps between the GPU library and the reference, in the
reference's text format (PhotonMap::dump / restore, src/pmap.cc:180-251).

The GPU's maps of the golden feature scene, dumped by sray_gpu_dump_photons
on a GB300 (tests/golden/make_gpu_dump.py), are read by the reference's own
PhotonMap::restore (compiled from its sources into oracle/_ref, where they
are present): every photon comes back as the text says, and the photons
are the CPU oracle's float photon maps of that frame (which the GPU's equal
bit for bit) within the format's six decimals.  The other direction, the
GPU restoring the reference's own dumps, is
tests/test_gpu_parity.py::test_gpu_restores_reference_dumps."""
import gzip
import json
import os
import subprocess

import numpy as np
import pytest

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _read_dump(text):
    lines = text.splitlines()
    assert lines[0].startswith("energy ")
    rows = [[float(v) for v in ln.replace("<", " ").replace(">", " ").split()] for ln in lines[1:] if ln.strip()]
    return float(lines[0].split()[1]), np.array(rows, np.float64).reshape(-1, 12)


def test_gpu_dump_format():
    for name in ("caust", "gi"):
        with gzip.open(os.path.join(HERE, "feature.gpu.%s.dump.gz" % name), "rt") as f:
            text = f.read()
        energy, rows = _read_dump(text)
        assert energy == 300.0 and len(rows) > 1000
        first = text.splitlines()[1]
        assert first.count("<") == 4 and first.count(">") == 4


@pytest.mark.parametrize("name,which", [("caust", 0), ("gi", 1)])
def test_reference_restores_gpu_dump(oracle_lib, name, which, tmp_path):
    from oracle import build_ref
    harness = build_ref.build()
    if not harness:
        pytest.skip("the reference's sources are not present")
    with gzip.open(os.path.join(HERE, "feature.gpu.%s.dump.gz" % name), "rt") as f:
        text = f.read()
    dump = tmp_path / "map.dump"
    dump.write_text(text)
    out = tmp_path / "restored.bin"
    subprocess.check_call([harness, "--restore", str(dump), str(out)], stdout=subprocess.DEVNULL)
    got = np.fromfile(str(out), np.float32).reshape(-1, 16).astype(np.float64)
    energy, rows = _read_dump(text)
    assert len(got) == len(rows)
    # the reference read what the text says (its fscanf %f, times energy / energy = 1)
    assert np.allclose(got[:, :12], rows, rtol=2e-7, atol=0)
    # and that is the frame's photon map
    d = np.load(os.path.join(HERE, "feature.npz"))
    opts = json.loads(bytes(d["opts"]).decode())
    with gzip.open(os.path.join(HERE, "feature.xml.gz")) as f:
        xml = f.read()
    o = oracle_lib.Oracle(fp64=False, rng_mode=1, **opts)
    o.load_xml(xml)
    o.prepare(0)
    ph = o.photons(which).astype(np.float64)
    from scipy.spatial import cKDTree
    _, j = cKDTree(ph[:, :3]).query(got[:, :3])
    diff = np.abs(ph[j, :12] - got[:, :12]).max()
    print("%s: the reference restored %d GPU photons; against the oracle's map %.2g" % (name, len(got), diff))
    assert len(ph) == len(got) and len(np.unique(j)) == len(got) and diff <= 1.5e-6
