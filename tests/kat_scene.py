"""Known-answer rays for the intersectors (shared by the CPU and GPU tests).

Scene: unit sphere at the origin, cylinder r=0.5, y in [0, 2) at x=3,
triangle (6,0,0) (7,0,0) (6,1,0) and a second triangle coplanar with it
(same plane, covering it) to produce an exact tie.  Rays are segments:
the hit parameter t lies in [1e-6, 1] of origin + t * dir
(src/mesh.cc:117-165, src/sphere.cc:85-131, src/cylinder.cc:125-185)."""
import numpy as np

XML = """<?xml version="1.0"?>
<scene>
<material name="m" shader="phong"><mattr name="diffuse" value="0.5 0.5 0.5"/></material>
<object type="sphere" name="s"><matref name="m"/><sphere rad="1.0"/></object>
<object type="cylinder" name="c"><matref name="m"/><xform pos="3.0 0.0 0.0"/><cylinder rad="0.5" start="0.0" end="2.0"/></object>
<object type="mesh" name="t"><matref name="m"/><mesh>
<vertex id="0" val="6.0 0.0 0.0"/><vertex id="1" val="7.0 0.0 0.0"/><vertex id="2" val="6.0 1.0 0.0"/>
<vertex id="3" val="5.5 -0.5 0.0"/><vertex id="4" val="8.0 -0.5 0.0"/><vertex id="5" val="5.5 2.0 0.0"/>
<face><vref vertex="0"/><vref vertex="1"/><vref vertex="2"/></face>
</mesh></object>
<object type="mesh" name="t2"><matref name="m"/><xform pos="0.0 -3.0 0.0"/><mesh>
<vertex id="0" val="6.0 0.0 0.0"/><vertex id="1" val="7.0 0.0 0.0"/><vertex id="2" val="6.0 1.0 0.0"/>
<vertex id="3" val="5.5 -0.5 0.0"/><vertex id="4" val="8.0 -0.5 0.0"/><vertex id="5" val="5.5 2.0 0.0"/>
<face><vref vertex="0"/><vref vertex="1"/><vref vertex="2"/></face>
<face><vref vertex="3"/><vref vertex="4"/><vref vertex="5"/></face>
</mesh></object>
<camera type="free"><xform pos="0.0 0.0 -10.0"/></camera>
</scene>
"""

# (origin, dir, expected object, expected prim, expected t or None, tie expected)
CASES = [
    ((0, 0, -5), (0, 0, 10), 0, 0, 0.4, False),          # sphere front
    ((0, 0, 0), (0, 0, 10), 0, 0, 0.1, False),           # from inside: the positive root
    ((0, 2, -5), (0, 0, 10), -1, -1, None, False),        # miss above
    ((0, 0, -5), (0, 0, 3), -1, -1, None, False),         # segment ends before the sphere (t > 1)
    ((0, 0, -1), (0, 0, -10), -1, -1, None, False),       # starts on the surface going out: t < eps
    ((3, 1, -5), (0, 0, 10), 1, 0, 0.45, False),          # cylinder side
    ((3, 0, -5), (0, 0, 10), 1, 0, 0.45, False),          # y == start is inside [start, end)
    ((3, 2, -5), (0, 0, 10), -1, -1, None, False),        # y == end is outside
    ((6.25, 0.25, -1), (0, 0, 2), 2, 0, 0.5, False),      # triangle interior
    ((6.5, 0.0, -1), (0, 0, 2), 2, 0, 0.5, False),        # on an edge: check_clock >= 0 keeps it
    ((6.0, 0.0, -1), (0, 0, 2), -1, -1, None, False),     # on a vertex: origin on the box's x and y planes with
                                                          # dir.x = dir.y = 0 gives a NaN slab entry, the
                                                          # box test of src/aabb.cc:81-125 rejects it
    ((6.0, 0.5, -1), (0.0001, 0, 2), 2, 0, 0.5, False),   # on the x = 6 edge, entered through the slab
    ((7.0, 1.0, -1), (0, 0, 2), -1, -1, None, False),     # outside the triangle
    ((6.2, 0.2, 0.0), (2, 0, 0), -1, -1, None, False),    # parallel to the plane
    ((6.25, -2.75, -1), (0, 0, 2), 3, 0, 0.5, True),      # two coplanar faces: first kept, tie flagged
]


def rays():
    o = np.array([c[0] for c in CASES], np.float64)
    d = np.array([c[1] for c in CASES], np.float64)
    return o, d


def check(obj, prim, t, tie, tol):
    bad = []
    for i, (_, _, eo, ep, et, etie) in enumerate(CASES):
        ok = obj[i] == eo and (eo < 0 or prim[i] == ep)
        if ok and et is not None:
            ok = abs(float(t[i]) - et) <= tol * max(1.0, abs(et))
        if ok and etie:
            ok = bool(tie[i])
        if not ok:
            bad.append((i, CASES[i], int(obj[i]), int(prim[i]), float(t[i]), int(tie[i])))
    return bad
