"""Seeded synthetic S-ray scenes in the reference's XML format.

The reference ships no scenes and no benchmark data, so the benchmark scenes
are generated: the small scene (512x512, ground plane, 16 spheres, one
subdivision-4 icosphere, a cylinder, one point light, 100k caustic photons)
and the production scene (1920x1080, 1,000,000-triangle displaced-grid
terrain, 200 instanced subdivision-3 icospheres, 3 sphere lights, 2M global
and 500k caustic photons).  Everything is drawn from a numpy Generator
seeded from the scene seed, vertex data is float32 written with nine
significant digits (so parsing it back and rounding to float32 is exact).

The XML follows the reference's loader: <material> with <mattr>,
<env>, <object type="sphere|cylinder|mesh"> with <matref>/<xform>/<sphere>/
<cylinder>/<mesh>, <light type="point|sphere">, <camera type="target">
(src/scene.cc:93-183, src/meshload.cc:55-157, src/anim.cc:68-121).
Numbers always start with a digit or a sign, as the attribute typing of
src/xmltree.c:75-93 requires.
"""
import hashlib
import math
import os

import numpy as np

__all__ = ["icosphere", "value_noise_height", "small_scene", "production_scene", "feature_scene",
           "textured_scene", "animated_scene", "textures", "write_textures", "scene_opts", "write_scene", "CONFIGS"]


def _f(x):
    return "%.9g" % float(np.float32(x))


def _vec(v):
    return " ".join(_f(c) for c in v)


def icosphere(subdiv):
    """Unit icosphere: (vertices float32 [n,3], faces int32 [m,3])."""
    t = (1.0 + 5.0 ** 0.5) / 2.0
    v = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t),
         (0, -1, -t), (0, 1, -t), (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    f = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4),
         (11, 10, 2), (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8),
         (3, 8, 9), (4, 9, 5), (2, 4, 11), (6, 2, 10), (8, 6, 7), (9, 8, 1)]
    verts = [np.array(p, dtype=np.float64) / np.linalg.norm(p) for p in v]
    faces = list(f)
    for _ in range(subdiv):
        cache = {}

        def mid(a, b):
            key = (a, b) if a < b else (b, a)
            if key not in cache:
                m = verts[a] + verts[b]
                verts.append(m / np.linalg.norm(m))
                cache[key] = len(verts) - 1
            return cache[key]

        nf = []
        for a, b, c in faces:
            ab, bc, ca = mid(a, b), mid(b, c), mid(c, a)
            nf += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
        faces = nf
    return np.array(verts, dtype=np.float32), np.array(faces, dtype=np.int32)


def _lattice(rng, size):
    return rng.random((size, size), dtype=np.float64)


def value_noise_height(x, z, seed, octaves=6, amplitude=2.0, base_freq=0.05):
    """Seeded value noise, `octaves` octaves, smoothstep-interpolated lattice,
    normalised to [-amplitude/2, amplitude/2] * 2 (peak-to-peak ~amplitude*2)."""
    rng = np.random.default_rng(seed)
    h = np.zeros_like(x, dtype=np.float64)
    norm = 0.0
    size = 256
    for o in range(octaves):
        lat = _lattice(rng, size)
        freq = base_freq * (2.0 ** o)
        fx = x * freq + 1000.0
        fz = z * freq + 1000.0
        ix = np.floor(fx).astype(np.int64)
        iz = np.floor(fz).astype(np.int64)
        tx = fx - ix
        tz = fz - iz
        tx = tx * tx * (3 - 2 * tx)
        tz = tz * tz * (3 - 2 * tz)
        x0, x1 = ix % size, (ix + 1) % size
        z0, z1 = iz % size, (iz + 1) % size
        a = lat[x0, z0] * (1 - tx) + lat[x1, z0] * tx
        b = lat[x0, z1] * (1 - tx) + lat[x1, z1] * tx
        w = 0.5 ** o
        h += (a * (1 - tz) + b * tz - 0.5) * w
        norm += w
    return amplitude * 2.0 * h / norm


def _mesh_xml(out, name, mat, verts, faces, normals=None, xform=None, texcoords=None, tangents=None):
    out.append('<object type="mesh" name="%s">\n<matref name="%s"/>\n' % (name, mat))
    if xform:
        out.append(xform)
    out.append("<mesh>\n")
    vs = np.char.mod("%.9g", verts.astype(np.float32).astype(np.float64))
    ids = np.arange(len(verts))
    out.append("".join('<vertex id="%d" val="%s %s %s"/>\n' % (i, a, b, c)
                       for i, (a, b, c) in zip(ids, vs)))
    if texcoords is not None:
        # every vertex carries a normal, a texture coordinate and a tangent
        ns = np.char.mod("%.9g", normals.astype(np.float32).astype(np.float64))
        ts = np.char.mod("%.9g", texcoords.astype(np.float32).astype(np.float64))
        gs = np.char.mod("%.9g", tangents.astype(np.float32).astype(np.float64))
        for i in ids:
            out.append('<normal id="%d" val="%s %s %s"/>\n' % (i, *ns[i]))
            out.append('<texcoord id="%d" val="%s %s"/>\n' % (i, *ts[i]))
            out.append('<tangent id="%d" val="%s %s %s"/>\n' % (i, *gs[i]))
        out.append("".join(
            "<face>%s</face>\n" % "".join('<vref vertex="%d" normal="%d" texcoord="%d" tangent="%d"/>' % (v, v, v, v)
                                          for v in f)
            for f in faces.tolist()))
    elif normals is not None:
        ns = np.char.mod("%.9g", normals.astype(np.float32).astype(np.float64))
        out.append("".join('<normal id="%d" val="%s %s %s"/>\n' % (i, a, b, c)
                           for i, (a, b, c) in zip(ids, ns)))
        out.append("".join(
            '<face><vref vertex="%d" normal="%d"/><vref vertex="%d" normal="%d"/>'
            '<vref vertex="%d" normal="%d"/></face>\n' % (a, a, b, b, c, c)
            for a, b, c in faces.tolist()))
    else:
        out.append("".join(
            '<face><vref vertex="%d"/><vref vertex="%d"/><vref vertex="%d"/></face>\n' % (a, b, c)
            for a, b, c in faces.tolist()))
    out.append("</mesh>\n</object>\n")


def _material(out, name, kd, ks=0.3, shin=30.0, refl=None, refr=None, ior=None):
    out.append('<material name="%s" shader="phong">\n' % name)
    out.append('<mattr name="diffuse" value="%s"/>\n' % _vec(kd))
    if np.ndim(ks) == 0:
        ks = (ks, ks, ks)
    out.append('<mattr name="specular" value="%s"/>\n' % _vec(ks))
    out.append('<mattr name="shininess" value="%s"/>\n' % ("%.1f" % shin))
    if refl is not None:
        out.append('<mattr name="reflect" value="%.3f"/>\n' % refl)
    if refr is not None:
        out.append('<mattr name="refract" value="%.3f"/>\n' % refr)
    if ior is not None:
        out.append('<mattr name="ior" value="%.3f"/>\n' % ior)
    out.append("</material>\n")


def _xform(pos=None, scale=None, axisrot=None, time=None):
    s = "<xform"
    if time is not None:
        s += ' time="%d"' % time
    if pos is not None:
        s += ' pos="%s"' % _vec(pos)
    if scale is not None:
        s += ' scale="%s"' % _vec(scale)
    if axisrot is not None:
        s += ' axisrot="%s"' % _vec(axisrot)
    return s + "/>\n"


def small_scene(seed=0x5EED0001):
    """The 512x512 scene: ground quad, 16 spheres, icosphere(4), cylinder, point light."""
    rng = np.random.default_rng(seed)
    out = ["<?xml version=\"1.0\"?>\n<scene>\n"]
    out.append('<env ambient="0.05 0.05 0.05" bgcolor="0.1 0.12 0.18"/>\n')
    _material(out, "ground", (0.6, 0.6, 0.55), ks=0.1, shin=10.0)
    n_sph = 16
    centres = np.stack([rng.uniform(-5, 5, n_sph), rng.uniform(0.5, 3.0, n_sph),
                        rng.uniform(-5, 5, n_sph)], axis=1)
    radii = rng.uniform(0.3, 1.0, n_sph)
    kinds = np.array(["phong"] * n_sph, dtype=object)
    order = rng.permutation(n_sph)
    kinds[order[:2]] = "glass"
    kinds[order[2:6]] = "mirror"            # 4 of 16 = 25% mirrors
    for i in range(n_sph):
        kd = rng.uniform(0.1, 0.9, 3)
        if kinds[i] == "glass":
            _material(out, "m%d" % i, kd * 0.1, ks=1.0, shin=80.0, refr=1.0, ior=1.5)
        elif kinds[i] == "mirror":
            _material(out, "m%d" % i, kd, ks=1.0, shin=60.0, refl=0.8)
        else:
            _material(out, "m%d" % i, kd, ks=0.4, shin=30.0)
    _material(out, "ico", rng.uniform(0.1, 0.9, 3), ks=0.5, shin=40.0)
    _material(out, "cyl", rng.uniform(0.1, 0.9, 3), ks=0.3, shin=20.0)
    g = 20.0
    gv = np.array([[-g, 0, -g], [g, 0, -g], [g, 0, g], [-g, 0, g]], dtype=np.float32)
    gf = np.array([[0, 2, 1], [0, 3, 2]], dtype=np.int32)
    _mesh_xml(out, "ground", "ground", gv, gf)
    for i in range(n_sph):
        out.append('<object type="sphere" name="s%d">\n<matref name="m%d"/>\n%s<sphere rad="%s"/>\n</object>\n'
                   % (i, i, _xform(pos=centres[i]), "%.6f" % radii[i]))
    iv, ifc = icosphere(4)
    _mesh_xml(out, "ico", "ico", iv, ifc, normals=iv,
              xform=_xform(pos=(2.5, 1.3, 6.0), scale=(1.3, 1.3, 1.3)))
    out.append('<object type="cylinder" name="cyl">\n<matref name="cyl"/>\n%s'
               '<cylinder rad="0.5" start="0.0" end="2.0"/>\n</object>\n' % _xform(pos=(-6.5, 0.0, -2.0)))
    out.append('<light type="point" color="1.0">\n%s</light>\n' % _xform(pos=(0.0, 8.0, 0.0)))
    out.append('<camera type="target" fov="50.0">\n%s<target>\n%s</target>\n</camera>\n'
               % (_xform(pos=(0.5, 7.0, 16.0)), _xform(pos=(0.0, 0.8, 0.0))))
    out.append("</scene>\n")
    return "".join(out)


def small_xml_without_specular(seed=0x5EED0001):
    """The small scene with no reflective or refractive material: a light's
    projection map of specular objects is empty (coverage 0)."""
    return "".join(line for line in small_scene(seed).splitlines(True)
                   if 'name="reflect"' not in line and 'name="refract"' not in line)


def production_scene(seed=0x5EED0002, grid=(1000, 500), extent=(100.0, 50.0), n_inst=200):
    """The 1080p scene: displaced-grid terrain of 2*grid[0]*grid[1] triangles
    (6-octave value noise, amplitude 2), n_inst subdivision-3 icosphere
    instances with seeded transforms, 3 sphere lights."""
    rng = np.random.default_rng(seed)
    nx, nz = grid
    ex, ez = extent
    out = ["<?xml version=\"1.0\"?>\n<scene>\n"]
    out.append('<env ambient="0.04 0.04 0.05" bgcolor="0.35 0.45 0.6"/>\n')
    _material(out, "terrain", (0.45, 0.5, 0.32), ks=0.05, shin=8.0)
    n_mirror = n_inst // 4
    n_glass = n_inst // 10
    kinds = np.array(["phong"] * n_inst, dtype=object)
    order = rng.permutation(n_inst)
    kinds[order[:n_glass]] = "glass"
    kinds[order[n_glass:n_glass + n_mirror]] = "mirror"
    for i in range(n_inst):
        kd = rng.uniform(0.1, 0.9, 3)
        if kinds[i] == "glass":
            _material(out, "m%d" % i, kd * 0.1, ks=1.0, shin=80.0, refr=1.0, ior=1.5)
        elif kinds[i] == "mirror":
            _material(out, "m%d" % i, kd, ks=1.0, shin=60.0, refl=0.8)
        else:
            _material(out, "m%d" % i, kd, ks=0.4, shin=30.0)
    hseed = _terrain(out, rng, nx, nz, ex, ez)
    # instances
    iv, ifc = icosphere(3)
    px = rng.uniform(-0.4 * ex, 0.4 * ex, n_inst)
    pz = rng.uniform(-0.4 * ez, 0.4 * ez, n_inst)
    sc = rng.uniform(0.4, 1.5, n_inst)
    lift = rng.uniform(0.0, 2.0, n_inst)
    hy = value_noise_height(px, pz, hseed)
    axes = rng.normal(size=(n_inst, 3))
    axes /= np.linalg.norm(axes, axis=1, keepdims=True)
    angles = rng.uniform(0, 360, n_inst)
    for i in range(n_inst):
        xf = _xform(pos=(px[i], hy[i] + sc[i] + lift[i], pz[i]), scale=(sc[i],) * 3,
                    axisrot=(angles[i], axes[i][0], axes[i][1], axes[i][2]))
        _mesh_xml(out, "inst%d" % i, "m%d" % i, iv, ifc, normals=iv, xform=xf)
    for i, (lx, lz) in enumerate([(-20.0, 5.0), (15.0, -8.0), (5.0, 15.0)]):
        out.append('<light type="sphere" color="0.7">\n%s<sphere rad="0.8"/>\n</light>\n'
                   % _xform(pos=(lx, 18.0 + 2.0 * i, lz)))
    out.append('<camera type="target" fov="50.0">\n%s<target>\n%s</target>\n</camera>\n'
               % (_xform(pos=(0.7, 14.0, 42.0)), _xform(pos=(0.0, 0.0, -4.0))))
    out.append("</scene>\n")
    return "".join(out)


def batch_scene(seed=0x5EED0007, tris=100000, n_movers=24):
    """A job of the batched configuration: a displaced-grid terrain of about
    `tris` triangles (2:1 grid, 6-octave value noise) and `n_movers` spheres
    moving on linear keyframes (two keys 1 s apart: under an 8 ms shutter
    each sample of a pixel sees one of 8 integer times), 2 sphere lights; a
    quarter of the spheres are mirrors and two are glass."""
    rng = np.random.default_rng(seed)
    nz = max(2, int(round(math.sqrt(tris / 4.0))))
    nx = 2 * nz
    ex, ez = 80.0, 40.0
    out = ["<?xml version=\"1.0\"?>\n<scene>\n"]
    out.append('<env ambient="0.04 0.04 0.05" bgcolor="0.35 0.45 0.6"/>\n')
    _material(out, "terrain", (0.45, 0.5, 0.32), ks=0.05, shin=8.0)
    kinds = np.array(["phong"] * n_movers, dtype=object)
    order = rng.permutation(n_movers)
    kinds[order[:2]] = "glass"
    kinds[order[2:2 + n_movers // 4]] = "mirror"
    for i in range(n_movers):
        kd = rng.uniform(0.1, 0.9, 3)
        if kinds[i] == "glass":
            _material(out, "m%d" % i, kd * 0.1, ks=1.0, shin=80.0, refr=1.0, ior=1.5)
        elif kinds[i] == "mirror":
            _material(out, "m%d" % i, kd, ks=1.0, shin=60.0, refl=0.8)
        else:
            _material(out, "m%d" % i, kd, ks=0.4, shin=30.0)
    hseed = _terrain(out, rng, nx, nz, ex, ez)
    px = rng.uniform(-0.35 * ex, 0.35 * ex, n_movers)
    pz = rng.uniform(-0.35 * ez, 0.35 * ez, n_movers)
    rad = rng.uniform(0.5, 1.8, n_movers)
    hy = value_noise_height(px, pz, hseed)
    vel = rng.uniform(-4.0, 4.0, (n_movers, 2))      # scene units per second
    for i in range(n_movers):
        y = hy[i] + rad[i] + 0.3
        out.append('<object type="sphere" name="s%d">\n<matref name="m%d"/>\n' % (i, i))
        out.append(_xform(pos=(px[i], y, pz[i]), time=0).replace("<xform", '<xform interpolate="linear"'))
        out.append(_xform(pos=(px[i] + vel[i][0], y, pz[i] + vel[i][1]), time=1000))
        out.append('<sphere rad="%.4f"/>\n</object>\n' % rad[i])
    for i, (lx, lz) in enumerate([(-18.0, 4.0), (14.0, -6.0)]):
        out.append('<light type="sphere" color="0.8">\n%s<sphere rad="0.8"/>\n</light>\n'
                   % _xform(pos=(lx, 18.0 + 2.0 * i, lz)))
    out.append('<camera type="target" fov="50.0">\n%s<target>\n%s</target>\n</camera>\n'
               % (_xform(pos=(0.7, 14.0, 38.0)), _xform(pos=(0.0, 0.0, -4.0))))
    out.append("</scene>\n")
    return "".join(out)


def _terrain(out, rng, nx, nz, ex, ez):
    """A displaced-grid terrain mesh of 2 nx nz triangles over ex x ez;
    returns the height seed."""
    xs = np.linspace(-ex / 2, ex / 2, nx + 1)
    zs = np.linspace(-ez / 2, ez / 2, nz + 1)
    X, Z = np.meshgrid(xs, zs, indexing="ij")
    hseed = int(rng.integers(1 << 31))
    H = value_noise_height(X, Z, hseed)
    verts = np.stack([X, H, Z], axis=-1).reshape(-1, 3).astype(np.float32)
    dx = ex / nx
    dz = ez / nz
    Hp = np.pad(H, 1, mode="edge")
    gx = (Hp[2:, 1:-1] - Hp[:-2, 1:-1]) / (2 * dx)
    gz = (Hp[1:-1, 2:] - Hp[1:-1, :-2]) / (2 * dz)
    nrm = np.stack([-gx, np.ones_like(gx), -gz], axis=-1)
    nrm /= np.linalg.norm(nrm, axis=-1, keepdims=True)
    nrm = nrm.reshape(-1, 3).astype(np.float32)
    idx = np.arange((nx + 1) * (nz + 1)).reshape(nx + 1, nz + 1)
    a = idx[:-1, :-1].ravel()
    b = idx[1:, :-1].ravel()
    c = idx[1:, 1:].ravel()
    d = idx[:-1, 1:].ravel()
    faces = np.empty((a.size * 2, 3), dtype=np.int64)
    faces[0::2] = np.stack([a, d, c], axis=1)
    faces[1::2] = np.stack([a, c, b], axis=1)
    _mesh_xml(out, "terrain", "terrain", verts, faces, normals=nrm)
    return hseed


def stress_scene(seed=0x5EED0005, tiles=(4, 4), tile_grid=(625, 500), tile_extent=(100.0, 80.0), n_inst=2000,
                 moving=0.1, shutter_ms=40):
    """The stress scene, as chunks of XML: tiles[0] x tiles[1] displaced-grid
    terrain meshes of 2 * tile_grid[0] * tile_grid[1] triangles each (one
    continuous 6-octave value-noise height field, amplitude 2), n_inst
    subdivision-3 icosphere instances (a `moving` fraction with a two-key
    linear motion over the shutter), 3 sphere lights."""
    rng = np.random.default_rng(seed)
    tx, tz = tiles
    gx_, gz_ = tile_grid
    ex, ez = tile_extent
    EX, EZ = ex * tx, ez * tz
    out = ["<?xml version=\"1.0\"?>\n<scene>\n", '<env ambient="0.04 0.04 0.05" bgcolor="0.35 0.45 0.6"/>\n']
    _material(out, "terrain", (0.45, 0.5, 0.32), ks=0.05, shin=8.0)
    n_mirror, n_glass = n_inst // 4, n_inst // 10
    kinds = np.array(["phong"] * n_inst, dtype=object)
    order = rng.permutation(n_inst)
    kinds[order[:n_glass]] = "glass"
    kinds[order[n_glass:n_glass + n_mirror]] = "mirror"
    for i in range(n_inst):
        kd = rng.uniform(0.1, 0.9, 3)
        if kinds[i] == "glass":
            _material(out, "m%d" % i, kd * 0.1, ks=1.0, shin=80.0, refr=1.0, ior=1.5)
        elif kinds[i] == "mirror":
            _material(out, "m%d" % i, kd, ks=1.0, shin=60.0, refl=0.8)
        else:
            _material(out, "m%d" % i, kd, ks=0.4, shin=30.0)
    yield "".join(out)
    hseed = int(rng.integers(1 << 31))
    for ti in range(tx):
        for tj in range(tz):
            x0, z0 = -EX / 2 + ti * ex, -EZ / 2 + tj * ez
            xs = np.linspace(x0, x0 + ex, gx_ + 1)
            zs = np.linspace(z0, z0 + ez, gz_ + 1)
            X, Z = np.meshgrid(xs, zs, indexing="ij")
            H = value_noise_height(X, Z, hseed)
            verts = np.stack([X, H, Z], axis=-1).reshape(-1, 3).astype(np.float32)
            d = 1e-3
            gx = (value_noise_height(X + d, Z, hseed) - value_noise_height(X - d, Z, hseed)) / (2 * d)
            gz = (value_noise_height(X, Z + d, hseed) - value_noise_height(X, Z - d, hseed)) / (2 * d)
            nrm = np.stack([-gx, np.ones_like(gx), -gz], axis=-1)
            nrm /= np.linalg.norm(nrm, axis=-1, keepdims=True)
            nrm = nrm.reshape(-1, 3).astype(np.float32)
            idx = np.arange((gx_ + 1) * (gz_ + 1)).reshape(gx_ + 1, gz_ + 1)
            a, b = idx[:-1, :-1].ravel(), idx[1:, :-1].ravel()
            c, dd = idx[1:, 1:].ravel(), idx[:-1, 1:].ravel()
            faces = np.empty((a.size * 2, 3), dtype=np.int64)
            faces[0::2] = np.stack([a, dd, c], axis=1)
            faces[1::2] = np.stack([a, c, b], axis=1)
            chunk = []
            _mesh_xml(chunk, "terrain_%d_%d" % (ti, tj), "terrain", verts, faces, normals=nrm)
            yield "".join(chunk)
    iv, ifc = icosphere(3)
    px = rng.uniform(-0.45 * EX, 0.45 * EX, n_inst)
    pz = rng.uniform(-0.45 * EZ, 0.45 * EZ, n_inst)
    sc = rng.uniform(0.4, 1.5, n_inst)
    lift = rng.uniform(0.0, 2.0, n_inst)
    hy = value_noise_height(px, pz, hseed)
    axes = rng.normal(size=(n_inst, 3))
    axes /= np.linalg.norm(axes, axis=1, keepdims=True)
    angles = rng.uniform(0, 360, n_inst)
    move = rng.uniform(0, 1, n_inst) < moving
    vel = rng.normal(size=(n_inst, 3)) * 0.5
    chunk = []
    for i in range(n_inst):
        p0 = (px[i], hy[i] + sc[i] + lift[i], pz[i])
        if move[i]:
            p1 = tuple(np.asarray(p0) + vel[i])
            xf = (_xform(pos=p0, scale=(sc[i],) * 3, axisrot=(angles[i], axes[i][0], axes[i][1], axes[i][2]), time=0)
                  + _xform(pos=p1, scale=(sc[i],) * 3, axisrot=(angles[i], axes[i][0], axes[i][1], axes[i][2]),
                           time=shutter_ms))
        else:
            xf = _xform(pos=p0, scale=(sc[i],) * 3, axisrot=(angles[i], axes[i][0], axes[i][1], axes[i][2]))
        _mesh_xml(chunk, "inst%d" % i, "m%d" % i, iv, ifc, normals=iv, xform=xf)
        if len(chunk) > 400:
            yield "".join(chunk)
            chunk = []
    for i, (lx, lz) in enumerate([(-60.0, 20.0), (45.0, -30.0), (15.0, 50.0)]):
        chunk.append('<light type="sphere" color="0.9">\n%s<sphere rad="1.5"/>\n</light>\n'
                     % _xform(pos=(lx, 45.0 + 4.0 * i, lz)))
    chunk.append('<camera type="target" fov="55.0">\n%s<target>\n%s</target>\n</camera>\n'
                 % (_xform(pos=(2.0, 40.0, 150.0)), _xform(pos=(0.0, 0.0, -10.0))))
    chunk.append("</scene>\n")
    yield "".join(chunk)


def feature_scene(seed=0x5EED0003):
    """A small scene touching the reference's less common paths: sphere and
    box lights, a default (shade_undef) material, a cylinder, a mirror and a
    glass sphere, a two-key linear motion track, a target camera."""
    rng = np.random.default_rng(seed)
    out = ["<?xml version=\"1.0\"?>\n<scene>\n"]
    out.append('<env ambient="0.1" bgcolor="0.2 0.25 0.3" ior="1.0"/>\n')
    _material(out, "floor", (0.7, 0.65, 0.6), ks=0.2, shin=12.0)
    _material(out, "mirror", (0.2, 0.2, 0.2), ks=1.0, shin=90.0, refl=0.9)
    _material(out, "glass", (0.05, 0.05, 0.05), ks=1.0, shin=90.0, refr=1.0, ior=1.45)
    _material(out, "red", (0.8, 0.2, 0.15), ks=0.5, shin=25.0)
    out.append('<material name="plain"/>\n')
    g = 8.0
    gv = np.array([[-g, 0, -g], [g, 0, -g], [g, 0, g], [-g, 0, g]], dtype=np.float32)
    gf = np.array([[0, 2, 1], [0, 3, 2]], dtype=np.int32)
    _mesh_xml(out, "floor", "floor", gv, gf)
    out.append('<object type="sphere" name="m">\n<matref name="mirror"/>\n%s<sphere rad="1.0"/>\n</object>\n'
               % _xform(pos=(-1.5, 1.0, 0.0)))
    out.append('<object type="sphere" name="g">\n<matref name="glass"/>\n%s<sphere rad="0.8"/>\n</object>\n'
               % _xform(pos=(1.2, 0.8, 1.0)))
    out.append('<object type="sphere" name="mover">\n<matref name="red"/>\n%s%s<sphere rad="0.5"/>\n</object>\n'
               % (_xform(pos=(0.0, 0.5, -2.0), time=0), _xform(pos=(0.6, 0.5, -2.0), time=40)))
    out.append('<object type="cylinder" name="c">\n<matref name="plain"/>\n%s'
               '<cylinder rad="0.4" start="0.0" end="1.5"/>\n</object>\n' % _xform(pos=(2.5, 0.0, -1.5)))
    iv, ifc = icosphere(2)
    _mesh_xml(out, "ico", "red", iv, ifc, normals=iv,
              xform=_xform(pos=(-2.6, 0.7, 2.2), scale=(0.7, 0.7, 0.7), axisrot=(30.0, 0.0, 1.0, 0.0)))
    out.append('<light type="sphere" color="0.8 0.75 0.7">\n%s<sphere rad="0.6"/>\n</light>\n'
               % _xform(pos=(0.5, 6.0, 2.0)))
    out.append('<light type="box" color="0.3">\n%s<aabox min="-0.5 -0.1 -0.5" max="0.5 0.1 0.5"/>\n</light>\n'
               % _xform(pos=(-3.0, 5.0, -1.0)))
    out.append('<camera type="target" fov="45.0">\n%s<target>\n%s</target>\n</camera>\n'
               % (_xform(pos=(0.3, 4.5, 9.0)), _xform(pos=(0.0, 0.6, 0.0))))
    out.append("</scene>\n")
    del rng
    return "".join(out)


def _ppm(w, h, rgb):
    """Binary PPM (P6) bytes of an [h, w, 3] uint8 image."""
    return b"P6\n%d %d\n255\n" % (w, h) + np.ascontiguousarray(rgb, dtype=np.uint8).tobytes()


def textures():
    """The images of the textured scene, {file name: PPM bytes}.  Integer
    formulas only, so that every machine writes the same bytes."""
    y, x = np.mgrid[0:64, 0:64].astype(np.int64)
    blk = ((x >> 3) + (y >> 3)) & 3
    pal = np.array([[230, 210, 180], [60, 90, 160], [200, 60, 50], [90, 170, 80]], dtype=np.int64)
    tiles = np.clip(pal[blk] - ((x * 7 + y * 13) & 31)[..., None], 0, 255)
    y, x = np.mgrid[0:32, 0:32].astype(np.int64)
    dx, dy = (x & 15) - 8, (y & 15) - 8
    bumps = np.stack([128 + dx * 12, 128 + dy * 12, np.full_like(dx, 220)], axis=-1)
    y, x = np.mgrid[0:16, 0:16].astype(np.int64)
    stripes = 80 + ((x + y) & 3) * 55
    mask = np.stack([stripes, stripes, stripes], axis=-1)
    y, x = np.mgrid[0:8, 0:8].astype(np.int64)
    ramp = 200 + x * 7
    iorm = np.stack([ramp, ramp, ramp], axis=-1)
    return {"tiles.ppm": _ppm(64, 64, tiles), "bumps.ppm": _ppm(32, 32, bumps),
            "stripes.ppm": _ppm(16, 16, mask), "ior.ppm": _ppm(8, 8, iorm)}


def write_textures(directory):
    """Write the textured scene's images into `directory` (the directory a
    renderer searches through SRAY_DATA_PATH)."""
    os.makedirs(directory, exist_ok=True)
    for name, data in textures().items():
        path = os.path.join(directory, name)
        if not os.path.exists(path) or open(path, "rb").read() != data:
            tmp = path + ".tmp%d" % os.getpid()
            with open(tmp, "wb") as f:
                f.write(data)
            os.replace(tmp, path)


def _uv_sphere_frame(v):
    """Texture coordinates and tangents of a unit sphere's vertices, with the
    sphere primitive's own mapping (src/sphere.cc:118-124)."""
    th = np.arctan2(v[:, 2], v[:, 0]) + np.pi
    ph = np.arccos(np.clip(v[:, 1], -1.0, 1.0))
    tc = np.stack([th / (2 * np.pi), ph / np.pi], axis=1)
    tg = np.cross(np.array([0.0, 1.0, 0.0]), v)
    n = np.linalg.norm(tg, axis=1, keepdims=True)
    tg = np.where(n > 1e-6, tg / np.maximum(n, 1e-12), np.array([1.0, 0.0, 0.0]))
    return tc, tg


def textured_scene():
    """A small scene of textured materials (the files of textures()): a tiled
    floor mesh with texture coordinates and tangents, a normal-mapped sphere
    with striped specular and shininess, a normal-mapped glass sphere with a
    textured index of refraction (caustic photons through a bumped surface),
    a striped mirror, a tiled cylinder, a textured icosphere, one material
    with an untextured "normal" attribute and one whose texture fails to
    load; a point and a sphere light."""
    out = ["<?xml version=\"1.0\"?>\n<scene>\n"]
    out.append('<env ambient="0.08" bgcolor="0.15 0.18 0.25" ior="1.0"/>\n')
    out.append('<material name="floor" shader="phong">\n<mattr name="diffuse" value="0.9" map="tiles.ppm"/>\n'
               '<mattr name="specular" value="0.15"/>\n<mattr name="shininess" value="20.0"/>\n</material>\n')
    out.append('<material name="bumpy" shader="phong">\n<mattr name="diffuse" value="0.75 0.5 0.3"/>\n'
               '<mattr name="specular" value="0.7" map="stripes.ppm"/>\n'
               '<mattr name="shininess" value="60.0" map="stripes.ppm"/>\n'
               '<mattr name="normal" value="1.5" map="bumps.ppm"/>\n</material>\n')
    out.append('<material name="glass" shader="phong">\n<mattr name="diffuse" value="0.05"/>\n'
               '<mattr name="specular" value="1.0"/>\n<mattr name="shininess" value="80.0"/>\n'
               '<mattr name="refract" value="1.0"/>\n<mattr name="ior" value="1.6" map="ior.ppm"/>\n'
               '<mattr name="normal" value="0.6" map="bumps.ppm"/>\n</material>\n')
    out.append('<material name="mirror" shader="phong">\n<mattr name="diffuse" value="0.2"/>\n'
               '<mattr name="specular" value="1.0"/>\n<mattr name="shininess" value="90.0"/>\n'
               '<mattr name="reflect" value="0.9" map="stripes.ppm"/>\n</material>\n')
    out.append('<material name="pillar" shader="phong">\n<mattr name="diffuse" value="0.8 0.8 0.7" map="tiles.ppm"/>\n'
               '<mattr name="specular" value="0.3"/>\n<mattr name="shininess" value="25.0"/>\n'
               '<mattr name="normal" value="1.0"/>\n</material>\n')
    out.append('<material name="lost" shader="phong">\n<mattr name="diffuse" value="0.3 0.6 0.4" map="no_such.ppm"/>\n'
               '<mattr name="specular" value="0.4"/>\n<mattr name="shininess" value="30.0"/>\n</material>\n')
    g = 8.0
    gv = np.array([[-g, 0, -g], [g, 0, -g], [g, 0, g], [-g, 0, g]], dtype=np.float32)
    gf = np.array([[0, 2, 1], [0, 3, 2]], dtype=np.int32)
    gn = np.tile(np.array([[0.0, 1.0, 0.0]]), (4, 1))
    gt = np.array([[0.0, 0.0], [3.0, 0.0], [3.0, 3.0], [0.0, 3.0]])     # three repeats across the floor
    gg = np.tile(np.array([[1.0, 0.0, 0.0]]), (4, 1))
    _mesh_xml(out, "floor", "floor", gv, gf, normals=gn, texcoords=gt, tangents=gg)
    out.append('<object type="sphere" name="bumpy">\n<matref name="bumpy"/>\n%s<sphere rad="1.1"/>\n</object>\n'
               % _xform(pos=(-1.6, 1.1, 0.2)))
    out.append('<object type="sphere" name="glass">\n<matref name="glass"/>\n%s<sphere rad="0.8"/>\n</object>\n'
               % _xform(pos=(1.3, 1.3, 1.4)))
    out.append('<object type="sphere" name="mirror">\n<matref name="mirror"/>\n%s<sphere rad="0.9"/>\n</object>\n'
               % _xform(pos=(1.2, 0.9, -2.2)))
    out.append('<object type="cylinder" name="pillar">\n<matref name="pillar"/>\n%s'
               '<cylinder rad="0.45" start="0.0" end="2.4"/>\n</object>\n' % _xform(pos=(3.2, 0.0, -0.6)))
    iv, ifc = icosphere(2)
    tc, tg = _uv_sphere_frame(iv.astype(np.float64))
    _mesh_xml(out, "ico", "bumpy", iv, ifc, normals=iv, texcoords=tc, tangents=tg,
              xform=_xform(pos=(-2.8, 0.6, 2.6), scale=(0.6, 0.6, 0.6)))
    out.append('<object type="sphere" name="lost">\n<matref name="lost"/>\n%s<sphere rad="0.5"/>\n</object>\n'
               % _xform(pos=(0.2, 0.5, 2.8)))
    out.append('<light type="point" color="0.9">\n%s</light>\n' % _xform(pos=(2.0, 7.0, 3.0)))
    out.append('<light type="sphere" color="0.4 0.38 0.35">\n%s<sphere rad="0.5"/>\n</light>\n'
               % _xform(pos=(-3.0, 5.5, -1.0)))
    out.append('<camera type="target" fov="50.0">\n%s<target>\n%s</target>\n</camera>\n'
               % (_xform(pos=(0.5, 4.0, 9.0)), _xform(pos=(0.0, 0.8, 0.0))))
    out.append("</scene>\n")
    return "".join(out)


def animated_scene():
    """Keyframed objects in every interpolation and extrapolation mode of
    the reference's tracks (src/anim.cc:68-121, src/anim.inl:189-273):
    linear position keys repeated past the last key, cubic (Catmull-Rom)
    position keys, step keys, rotations by axis-angle and by quaternion with
    slerp (cubic) and component-wise lerp (linear), scale keys about a pivot,
    a moving point light; rendered at a time between or past the keys."""
    def xf(time, interp=None, extrap=None, **kw):
        s = '<xform time="%d"' % time
        if interp:
            s += ' interpolate="%s"' % interp
        if extrap:
            s += ' extrapolate="%s"' % extrap
        for k, v in kw.items():
            s += ' %s="%s"' % (k, _vec(v))
        return s + "/>\n"
    out = ["<?xml version=\"1.0\"?>\n<scene>\n"]
    out.append('<env ambient="0.1" bgcolor="0.2 0.2 0.25" ior="1.0"/>\n')
    _material(out, "floor", (0.6, 0.6, 0.55), ks=0.2, shin=15.0)
    _material(out, "a", (0.8, 0.3, 0.2), ks=0.5, shin=30.0)
    _material(out, "b", (0.2, 0.7, 0.3), ks=0.5, shin=30.0)
    _material(out, "c", (0.3, 0.4, 0.9), ks=0.4, shin=20.0)
    _material(out, "d", (0.8, 0.8, 0.2), ks=0.6, shin=50.0)
    _material(out, "glass", (0.05, 0.05, 0.05), ks=1.0, shin=80.0, refr=1.0, ior=1.5)
    g = 8.0
    gv = np.array([[-g, 0, -g], [g, 0, -g], [g, 0, g], [-g, 0, g]], dtype=np.float32)
    gf = np.array([[0, 2, 1], [0, 3, 2]], dtype=np.int32)
    _mesh_xml(out, "floor", "floor", gv, gf)
    # linear, repeated: keys at 0, 500, 1000
    out.append('<object type="sphere" name="rep">\n<matref name="a"/>\n%s%s%s<sphere rad="0.7"/>\n</object>\n'
               % (xf(0, "linear", "repeat", pos=(-3.0, 0.7, 0.0)), xf(500, pos=(-1.0, 1.5, -1.0)),
                  xf(1000, pos=(-3.0, 0.7, 0.0))))
    # cubic positions: keys at 0, 300, 600, 900
    out.append('<object type="sphere" name="cub">\n<matref name="glass"/>\n%s%s%s%s<sphere rad="0.6"/>\n</object>\n'
               % (xf(0, "cubic", pos=(0.0, 0.6, 2.0)), xf(300, pos=(0.8, 1.4, 1.5)), xf(600, pos=(1.6, 0.9, 2.2)),
                  xf(900, pos=(2.2, 0.6, 1.0))))
    # step keys
    out.append('<object type="cylinder" name="stp">\n<matref name="c"/>\n%s%s%s'
               '<cylinder rad="0.4" start="0.0" end="1.8"/>\n</object>\n'
               % (xf(0, "step", pos=(2.5, 0.0, -2.0)), xf(400, pos=(3.0, 0.0, -1.5)), xf(800, pos=(3.5, 0.0, -1.0))))
    # axis-angle rotation keys (cubic: slerp), scale keys, a pivot
    iv, ifc = icosphere(2)
    rot_xml = (xf(0, "cubic", pos=(-1.0, 1.0, -3.0), axisrot=(0.0, 0.0, 1.0, 0.0), scale=(0.8, 0.8, 0.8),
                  pivot=(0.3, 0.0, 0.0))
               + xf(700, axisrot=(120.0, 0.3, 1.0, 0.2), scale=(1.0, 0.6, 1.2))
               + xf(1400, axisrot=(250.0, 0.0, 1.0, 0.5), scale=(0.7, 0.9, 0.8)))
    _mesh_xml(out, "spin", "d", iv, ifc, normals=iv, xform=rot_xml)
    # quaternion keys, linear (component-wise lerp)
    box = np.array([[-1, -1, -1], [1, -1, -1], [1, 1, -1], [-1, 1, -1], [-1, -1, 1], [1, -1, 1], [1, 1, 1], [-1, 1, 1]],
                   dtype=np.float32) * 0.5
    bf = np.array([[0, 2, 1], [0, 3, 2], [4, 5, 6], [4, 6, 7], [0, 1, 5], [0, 5, 4], [2, 3, 7], [2, 7, 6],
                   [1, 2, 6], [1, 6, 5], [0, 4, 7], [0, 7, 3]], dtype=np.int32)
    quat_xml = (xf(0, "linear", pos=(1.0, 0.6, -0.5), rot=(1.0, 0.0, 0.0, 0.0))
                + xf(600, rot=(0.7, 0.2, 0.6, 0.3)) + xf(1200, rot=(0.3, 0.5, 0.1, 0.8)))
    _mesh_xml(out, "tumble", "b", box, bf, xform=quat_xml)
    out.append('<light type="point" color="1.0">\n%s%s</light>\n'
               % (xf(0, pos=(0.0, 7.0, 2.0)), xf(1000, pos=(3.0, 6.0, 4.0))))
    out.append('<camera type="target" fov="50.0">\n%s<target>\n%s</target>\n</camera>\n'
               % (_xform(pos=(0.5, 5.0, 9.5)), _xform(pos=(0.0, 0.8, 0.0))))
    out.append("</scene>\n")
    return "".join(out)


# option sets (sray_opts fields) of the benchmark configurations
CONFIGS = {
    "small": dict(width=512, height=512, min_samples=1, max_samples=1, iter=5,
                  caust_photons=100000, gi_photons=0, caust_k=50, gi_k=0, gather_rcap=0.5,
                  scnoct_max_depth=8, scnoct_max_items=8, meshoct_max_depth=8, meshoct_max_items=8),
    # the radiance-cache comparison: the small scene at 1080p with a global
    # map, one final-gather ray per vertex (the plain method) or the network
    "learned": dict(width=1920, height=1080, min_samples=1, max_samples=1, iter=5,
                    caust_photons=100000, gi_photons=500000, caust_k=50, gi_k=100, gather_rcap=0.5,
                    diffuse_samples=1, nrc_fallback_samples=16, scnoct_max_depth=8, scnoct_max_items=8,
                    meshoct_max_depth=8, meshoct_max_items=8),
    # the stress configuration: 10M triangles (4x4 terrain tiles) + 2000
    # instances at 3840x2160, 20M global + 4M caustic photons, motion blur
    "stress": dict(width=3840, height=2160, min_samples=1, max_samples=16, max_var=0.05, iter=8,
                   caust_photons=4000000, gi_photons=20000000, caust_k=100, gi_k=100, gather_rcap=0.5,
                   mblur=1, shutter=40, time_start=0, time_end=0,
                   scnoct_max_depth=8, scnoct_max_items=8, meshoct_max_depth=10, meshoct_max_items=8),
    # textured materials and normal maps (the reference's fixed-radius gathers)
    "textured": dict(width=128, height=96, min_samples=1, max_samples=2, max_var=0.02, iter=6,
                     caust_photons=20000, gi_photons=30000, shadow_samples=2, diffuse_samples=2, gather_dist=0.02),
    "production": dict(width=1920, height=1080, min_samples=1, max_samples=16, max_var=0.05, iter=8,
                       caust_photons=500000, gi_photons=2000000, caust_k=100, gi_k=100, gather_rcap=0.5,
                       scnoct_max_depth=8, scnoct_max_items=8, meshoct_max_depth=10, meshoct_max_items=8),
}


def scene_opts(name, **over):
    d = dict(CONFIGS[name])
    d.update(over)
    return d


def write_scene(name, cache_dir=None, **kw):
    """Generate (or reuse from cache_dir) the XML of scene `name`; returns the path."""
    gen = {"small": small_scene, "learned": small_scene, "production": production_scene, "feature": feature_scene,
           "stress": stress_scene, "textured": textured_scene, "animated": animated_scene, "batch": batch_scene}[name]
    key = hashlib.sha1(repr((name, sorted(kw.items()), 3)).encode()).hexdigest()[:12]
    cache_dir = cache_dir or os.environ.get("SRAY_SCENE_CACHE", "/tmp/sray_scenes")
    os.makedirs(cache_dir, exist_ok=True)
    path = os.path.join(cache_dir, "%s_%s.xml" % (name, key))
    if not os.path.exists(path):
        xml = gen(**kw)
        tmp = path + ".tmp%d" % os.getpid()
        with open(tmp, "w") as f:
            if isinstance(xml, str):
                f.write(xml)
            else:
                for chunk in xml:      # generators write their document in pieces
                    f.write(chunk)
        os.replace(tmp, path)
    if name == "textured":
        write_textures(cache_dir)
    return path
