"""Known-answer intersections through the CPU oracle, FP64 and FP32."""
import pytest

import kat_scene


@pytest.mark.parametrize("fp64", [True, False])
def test_intersector_kats(oracle_lib, fp64):
    o = oracle_lib.Oracle(fp64=fp64, rng_mode=1, width=32, height=32)
    o.load_xml(kat_scene.XML)
    orig, dirs = kat_scene.rays()
    obj, prim, t, tie = o.cast_rays(orig, dirs)
    bad = kat_scene.check(obj, prim, t, tie, 1e-12 if fp64 else 1e-6)
    assert not bad, bad


def test_xml_numbers_are_floats(oracle_lib):
    # struct xml_attr keeps numbers as float (src/xmltree.h:31-33): a radius of
    # 0.1 is the float nearest to 0.1, visible in the hit parameter
    import numpy as np
    xml = kat_scene.XML.replace('<sphere rad="1.0"/>', '<sphere rad="0.1"/>')
    o = oracle_lib.Oracle(fp64=True, rng_mode=1, width=8, height=8)
    o.load_xml(xml)
    obj, _, t, _ = o.cast_rays(np.array([[0.0, 0.0, -1.0]]), np.array([[0.0, 0.0, 2.0]]))
    r = float(np.float32(0.1))
    assert obj[0] == 0 and t[0] == pytest.approx((1.0 - r) / 2.0, abs=1e-15)
