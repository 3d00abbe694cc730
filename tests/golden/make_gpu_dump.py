"""Write the GPU's photon maps of the golden feature scene as dump files in
the reference's format (sray_gpu_dump_photons), for the check that the
reference's own PhotonMap::restore reads them (tests/test_dump_interchange.py).

Needs a GPU:  python tests/golden/make_gpu_dump.py <output directory>
writes feature.gpu.caust.dump.gz and feature.gpu.gi.dump.gz there; the
committed copies sit beside this script.
"""
import gzip
import json
import os
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))


def main():
    import numpy as np
    from sray_gb300 import gpu
    out = sys.argv[1] if len(sys.argv) > 1 else HERE
    d = np.load(os.path.join(HERE, "feature.npz"))
    opts = json.loads(bytes(d["opts"]).decode())
    with gzip.open(os.path.join(HERE, "feature.xml.gz")) as f:
        xml = f.read()
    g = gpu.GpuRenderer(**opts)
    g.load_xml(xml)
    g.render(0)                      # the frame's photon maps
    with tempfile.TemporaryDirectory() as td:
        for which, name in ((0, "caust"), (1, "gi")):
            p = os.path.join(td, name)
            g.dump_photons(which, p)
            with open(p, "rb") as f, gzip.open(os.path.join(out, "feature.gpu.%s.dump.gz" % name), "wb") as z:
                z.write(f.read())
            print("%s: %d photons" % (name, len(g.photons(which))))
    g.close()
    return 0


if __name__ == "__main__":
    sys.exit(main())
