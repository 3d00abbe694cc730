"""Scenes given as tables: ctypes mirrors of include/sray_gpu.h's
sray_scene_desc and a builder that keeps the arrays alive while the
library reads them (sray_gpu_upload_scene).

The tables are the reference's scene classes flattened (Scene, Object with
Sphere / Cylinder / Mesh, Material attributes, Light with SphLight /
BoxLight, Camera / TargetCamera and XFormNode keyframe tracks; see the
header).  `from_xml` builds them from an S-ray XML document with the
loader's rules, so that a scene can go either way and render the same.
"""
import ctypes
import math
import os

import numpy as np

ATTRS = ["diffuse", "specular", "shininess", "reflect", "refract", "ior", "normal"]
OBJ_TYPES = {"sphere": 0, "cylinder": 1, "mesh": 2}
LIGHT_TYPES = {"point": 0, "sphere": 1, "box": 2}
INTERP = {"step": 0, "linear": 1, "cubic": 2}
EXTRAP = {"clamp": 0, "repeat": 1, "pingpong": 2}


class TrackDesc(ctypes.Structure):
    _fields_ = [("nkeys", ctypes.c_int), ("interp", ctypes.c_int), ("extrap", ctypes.c_int),
                ("time", ctypes.POINTER(ctypes.c_int)), ("val", ctypes.POINTER(ctypes.c_double))]


class XformDesc(ctypes.Structure):
    _fields_ = [("pos", TrackDesc), ("rot", TrackDesc), ("scale", TrackDesc), ("pivot", ctypes.c_double * 3)]


class TextureDesc(ctypes.Structure):
    _fields_ = [("width", ctypes.c_int), ("height", ctypes.c_int), ("pixels", ctypes.POINTER(ctypes.c_float))]


class MatAttrDesc(ctypes.Structure):
    _fields_ = [("present", ctypes.c_int), ("col", ctypes.c_double * 4), ("texture", ctypes.c_int)]


class MaterialDesc(ctypes.Structure):
    _fields_ = [("name", ctypes.c_char_p), ("phong", ctypes.c_int), ("attr", MatAttrDesc * 7)]


class ObjectDesc(ctypes.Structure):
    _fields_ = [("name", ctypes.c_char_p), ("type", ctypes.c_int), ("material", ctypes.c_int), ("xform", XformDesc),
                ("rad", ctypes.c_double), ("start", ctypes.c_double), ("end", ctypes.c_double), ("nfaces", ctypes.c_int),
                ("pos", ctypes.POINTER(ctypes.c_double)), ("normal", ctypes.POINTER(ctypes.c_double)),
                ("tangent", ctypes.POINTER(ctypes.c_double)), ("texcoord", ctypes.POINTER(ctypes.c_double))]


class LightDesc(ctypes.Structure):
    _fields_ = [("type", ctypes.c_int), ("color", ctypes.c_double * 4), ("xform", XformDesc), ("radius", ctypes.c_double),
                ("dim", ctypes.c_double * 3)]


class CameraDesc(ctypes.Structure):
    _fields_ = [("target", ctypes.c_int), ("vfov", ctypes.c_double), ("shutter", ctypes.c_int), ("xform", XformDesc),
                ("target_xform", XformDesc)]


class SceneDescC(ctypes.Structure):
    _fields_ = [("n_materials", ctypes.c_int), ("n_objects", ctypes.c_int), ("n_lights", ctypes.c_int),
                ("n_textures", ctypes.c_int), ("materials", ctypes.POINTER(MaterialDesc)),
                ("objects", ctypes.POINTER(ObjectDesc)), ("lights", ctypes.POINTER(LightDesc)),
                ("textures", ctypes.POINTER(TextureDesc)), ("camera", ctypes.POINTER(CameraDesc)),
                ("env_ambient", ctypes.c_double * 4), ("env_color", ctypes.c_double * 4), ("env_ior", ctypes.c_double),
                ("reserved", ctypes.c_int * 4)]


class Xform:
    """An XFormNode's tracks: {time: value} per track, interpolation and
    extrapolation per track, and the pivot."""

    def __init__(self):
        self.keys = {"pos": {}, "rot": {}, "scale": {}}
        self.interp = {"pos": 1, "rot": 1, "scale": 1}
        self.extrap = {"pos": 0, "rot": 0, "scale": 0}
        self.pivot = (0.0, 0.0, 0.0)

    def key(self, track, time, value):
        self.keys[track][int(time)] = tuple(float(v) for v in value)
        return self


class SceneDesc:
    """A scene as tables; .c() gives the sray_scene_desc the library reads."""

    def __init__(self):
        self.textures, self.materials, self.objects, self.lights = [], [], [], []
        self.camera = None
        self.env_ambient = (0.0, 0.0, 0.0, 0.0)
        self.env_color = (0.0, 0.0, 0.0, 0.0)
        self.env_ior = 1.0
        self._keep = []

    def add_texture(self, rgba):
        rgba = np.ascontiguousarray(rgba, np.float32)
        self.textures.append(rgba)
        return len(self.textures) - 1

    def add_material(self, name, phong=True, attrs=None):
        """attrs: {attribute name: (rgba colour, texture index or -1)}."""
        self.materials.append((name, bool(phong), dict(attrs or {})))
        return len(self.materials) - 1

    def add_object(self, name, kind, material=-1, xform=None, rad=1.0, start=-1.0, end=1.0, pos=None, normal=None,
                   tangent=None, texcoord=None):
        self.objects.append(dict(name=name, type=OBJ_TYPES[kind], material=material, xform=xform or Xform(), rad=rad,
                                 start=start, end=end, pos=pos, normal=normal, tangent=tangent, texcoord=texcoord))
        return len(self.objects) - 1

    def add_light(self, kind, color, xform=None, radius=1.0, dim=(1.0, 1.0, 1.0)):
        self.lights.append(dict(type=LIGHT_TYPES[kind], color=color, xform=xform or Xform(), radius=radius, dim=dim))

    def set_camera(self, target, vfov, shutter, xform, target_xform=None):
        self.camera = dict(target=int(target), vfov=vfov, shutter=shutter, xform=xform, target_xform=target_xform or Xform())

    # ---- ctypes ----
    def _arr(self, a, ctype):
        if a is None:
            return None
        a = np.ascontiguousarray(a, np.float64 if ctype is ctypes.c_double else np.int32)
        self._keep.append(a)
        return a.ctypes.data_as(ctypes.POINTER(ctype))

    def _xform(self, xf):
        d = XformDesc()
        for tr, width in (("pos", 3), ("rot", 4), ("scale", 3)):
            ks = sorted(xf.keys[tr].items())
            t = getattr(d, tr)
            t.nkeys = len(ks)
            t.interp = xf.interp[tr]
            t.extrap = xf.extrap[tr]
            if ks:
                t.time = self._arr([k for k, _ in ks], ctypes.c_int)
                t.val = self._arr(np.array([v for _, v in ks], np.float64).reshape(-1, width), ctypes.c_double)
        d.pivot[:] = xf.pivot
        return d

    def c(self):
        self._keep = []
        d = SceneDescC()
        d.n_textures = len(self.textures)
        tex = (TextureDesc * max(1, len(self.textures)))()
        for i, t in enumerate(self.textures):
            tex[i].height, tex[i].width = t.shape[:2]
            tex[i].pixels = t.ctypes.data_as(ctypes.POINTER(ctypes.c_float))
        d.textures = tex
        mats = (MaterialDesc * max(1, len(self.materials)))()
        for i, (name, phong, attrs) in enumerate(self.materials):
            b = name.encode()
            self._keep.append(b)
            mats[i].name = b
            mats[i].phong = int(phong)
            for a, (col, texi) in attrs.items():
                k = ATTRS.index(a)
                mats[i].attr[k].present = 1
                mats[i].attr[k].col[:] = tuple(col)
                mats[i].attr[k].texture = texi
            for k in range(7):
                if ATTRS[k] not in attrs:
                    mats[i].attr[k].texture = -1
        d.n_materials = len(self.materials)
        d.materials = mats
        objs = (ObjectDesc * max(1, len(self.objects)))()
        for i, o in enumerate(self.objects):
            b = o["name"].encode()
            self._keep.append(b)
            objs[i].name = b
            objs[i].type = o["type"]
            objs[i].material = o["material"]
            objs[i].xform = self._xform(o["xform"])
            objs[i].rad, objs[i].start, objs[i].end = o["rad"], o["start"], o["end"]
            if o["pos"] is not None:
                objs[i].nfaces = len(o["pos"]) // 9
                objs[i].pos = self._arr(o["pos"], ctypes.c_double)
                objs[i].normal = self._arr(o["normal"], ctypes.c_double)
                objs[i].tangent = self._arr(o["tangent"], ctypes.c_double)
                objs[i].texcoord = self._arr(o["texcoord"], ctypes.c_double)
        d.n_objects = len(self.objects)
        d.objects = objs
        lts = (LightDesc * max(1, len(self.lights)))()
        for i, L in enumerate(self.lights):
            lts[i].type = L["type"]
            lts[i].color[:] = tuple(L["color"])
            lts[i].xform = self._xform(L["xform"])
            lts[i].radius = L["radius"]
            lts[i].dim[:] = tuple(L["dim"])
        d.n_lights = len(self.lights)
        d.lights = lts
        if self.camera:
            cam = CameraDesc()
            cam.target = self.camera["target"]
            cam.vfov = self.camera["vfov"]
            cam.shutter = self.camera["shutter"]
            cam.xform = self._xform(self.camera["xform"])
            cam.target_xform = self._xform(self.camera["target_xform"])
            self._keep.append(cam)
            d.camera = ctypes.pointer(cam)
        d.env_ambient[:] = self.env_ambient
        d.env_color[:] = self.env_color
        d.env_ior = self.env_ior
        self._keep += [tex, mats, objs, lts, d]
        return d


# ---- from an XML document, with the loader's rules ----
def _f32(x):
    return float(np.float32(x))


def _num_start(s):
    return len(s) > 0 and (s[0].isdigit() or (s[0] in "+-" and len(s) > 1 and s[1].isdigit()))


def _strtod(s):
    """strtod's leading number of s (0.0 if none)."""
    import re
    m = re.match(r"\s*[+-]?(\d+\.?\d*([eE][+-]?\d+)?|\.\d+([eE][+-]?\d+)?)", s)
    return float(m.group(0)) if m else 0.0


def _typed(v):
    """The typed value of an attribute (src/xmltree.c:75-93): a string
    starting with a number is an int (no '.') or a float; two or more
    numbers make a vector padded with 1.0; every number rounded to float."""
    if v is None:
        return None
    if not _num_start(v):
        return ("str", v)
    vv = [1.0, 1.0, 1.0, 1.0]
    parts = v.split()
    for i in range(min(4, len(parts))):
        vv[i] = _f32(_strtod(parts[i]))
    if len(parts) > 1:
        return ("vec", vv)
    return ("flt" if "." in v else "int", _f32(_strtod(v)), int(_strtod(v)) if "." not in v else None)


def _fval(v):
    """The attribute's first number as a float (0 when it is not a number)."""
    return _f32(_strtod(v)) if v is not None and _num_start(v) else 0.0


def _load_ppm(path):
    with open(path, "rb") as f:
        data = f.read()
    if data[:2] != b"P6":
        return None
    vals, pos = [], 2
    while len(vals) < 3:
        while data[pos:pos + 1].isspace() or data[pos:pos + 1] == b"#":
            if data[pos:pos + 1] == b"#":
                pos = data.index(b"\n", pos)
            pos += 1
        end = pos
        while data[end:end + 1].isdigit():
            end += 1
        vals.append(int(data[pos:end]))
        pos = end
    w, h, maxv = vals
    pos += 1
    rgb = np.frombuffer(data[pos:pos + w * h * 3], np.uint8).reshape(h, w, 3)
    out = np.ones((h, w, 4), np.float32)
    out[..., :3] = rgb.astype(np.float32) / np.float32(255.0)
    return out


def _texture_path(name):
    """find_file's search: the first directory of SRAY_DATA_PATH only."""
    if os.path.exists(name):
        return name
    dp = os.environ.get("SRAY_DATA_PATH", "")
    first = dp.split(":")[0] if dp else ""
    p = os.path.join(first, name) if first else None
    return p if p and os.path.exists(p) else None


def _xform_into(node, xf):
    interp = node.get("interpolate")
    if interp in INTERP:
        for k in xf.interp:
            xf.interp[k] = INTERP[interp]
    extrap = node.get("extrapolate")
    if extrap in EXTRAP:
        for k in xf.extrap:
            xf.extrap[k] = EXTRAP[extrap]
    t = _typed(node.get("time"))
    msec = t[2] if t and t[0] == "int" else 0
    p = _typed(node.get("pos"))
    if p and p[0] == "vec":
        xf.key("pos", msec, p[1][:3])
    r = _typed(node.get("rot"))
    if r and r[0] == "vec":
        q = r[1]
        ln = math.sqrt(q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3])
        xf.key("rot", msec, [c / ln for c in q] if ln > 0.0 else q)
    a = _typed(node.get("axisrot"))
    if a and a[0] == "vec":
        v = a[1]
        ang = (v[0] * math.pi) / 180.0
        half = ang * 0.5
        sn = math.sin(half)
        xf.key("rot", msec, (math.cos(half), v[1] * sn, v[2] * sn, v[3] * sn))
    s = _typed(node.get("scale"))
    if s and s[0] == "vec":
        xf.key("scale", msec, s[1][:3])
    pv = _typed(node.get("pivot"))
    if pv and pv[0] == "vec":
        xf.pivot = tuple(pv[1][:3])


def _read_val(v):
    if v is None or not _num_start(v):
        return None
    parts = v.split()
    if len(parts) < 2:
        return None
    return [_f32(_strtod(p)) for p in parts[:3]] + [1.0] * (3 - min(3, len(parts)))


def _mesh(node, name):
    names = ["vertex", "normal", "texcoord", "tangent"]
    el = {k: [] for k in names}
    faces = []
    for c in node:
        if c.tag in el:
            idv = c.get("id")
            i = int(idv) if idv is not None and _num_start(idv) and "." not in idv else len(el[c.tag])
            v = _read_val(c.get("val")) or [0.0, 0.0, 0.0]
            el[c.tag].append((i, v))
        elif c.tag == "face":
            f = []
            for vr in c:
                if vr.tag != "vref" or len(f) == 3:
                    continue
                f.append([int(vr.get(a)) if vr.get(a) is not None else 0 for a in ("vertex", "normal", "tangent", "texcoord")])
            while len(f) < 3:
                f.append([0, 0, 0, 0])
            faces.append(f)
    arr = {}
    for k in names:
        e = sorted(el[k], key=lambda x: x[0])
        if e and e[-1][0] != len(e) - 1:
            raise ValueError("error loading mesh %s: missing vertex elements" % name)
        arr[k] = [v for _, v in e]
    nf = len(faces)
    pos = np.zeros((nf, 3, 3))
    nrm = np.zeros((nf, 3, 3)) if arr["normal"] else None
    tng = np.zeros((nf, 3, 3)) if arr["tangent"] else None
    tc = np.zeros((nf, 3, 2)) if arr["texcoord"] else None
    for i, f in enumerate(faces):
        for j, (vi, ni, gi, ti) in enumerate(f):
            pos[i, j] = arr["vertex"][vi]
            if nrm is not None:
                nrm[i, j] = arr["normal"][ni]
            if tng is not None:
                tng[i, j] = arr["tangent"][gi]
            if tc is not None:
                tc[i, j] = arr["texcoord"][ti][:2]
    flat = [None if a is None else a.reshape(-1) for a in (pos, nrm, tng, tc)]
    return flat


def from_xml(xml, shutter=0):
    """A SceneDesc of an S-ray XML document (materials first, then env,
    objects, lights and the first camera, as Scene::load reads them);
    `shutter` is the option's, for a camera without a shutter attribute."""
    import xml.etree.ElementTree as ET
    root = ET.fromstring(xml if isinstance(xml, (bytes, str)) else bytes(xml))
    d = SceneDesc()
    mat_index = {}
    for m in root.findall("material"):
        attrs = {}
        for a in m.findall("mattr"):
            an, av = a.get("name"), _typed(a.get("value"))
            if an is None or av is None or av[0] == "str":
                continue
            col = av[1][:3] + [1.0] if av[0] == "vec" else [av[1]] * 3 + [1.0]
            tex = -1
            if a.get("map") is not None:
                p = _texture_path(a.get("map"))
                img = _load_ppm(p) if p else None
                if img is not None:
                    tex = d.add_texture(img)
            if an in ATTRS:
                attrs[an] = (col, tex)
        mat_index.setdefault(m.get("name"), len(d.materials))
        d.add_material(m.get("name"), m.get("shader") == "phong", attrs)
    for n in root:
        if n.tag == "env":
            a = _typed(n.get("ambient"))
            if a and a[0] == "vec":
                d.env_ambient = tuple(a[1][:3]) + (1.0,)
            elif a and a[0] in ("int", "flt"):
                d.env_ambient = (a[1],) * 3 + (1.0,)
            b = _typed(n.get("bgcolor"))
            if b and b[0] == "vec":
                d.env_color = tuple(b[1][:3]) + (1.0,)
            i = _typed(n.get("ior"))
            if i and i[0] == "flt":
                d.env_ior = i[1]
        elif n.tag == "object":
            kind = n.get("type")
            xf = Xform()
            mat, rad, start, end, mesh = -1, 1.0, -1.0, 1.0, [None] * 4
            for c in n:
                if c.tag == "matref":
                    mat = mat_index[c.get("name")]
                elif c.tag == "xform":
                    _xform_into(c, xf)
                elif c.tag == kind == "sphere":
                    if c.get("rad") is not None:
                        rad = _fval(c.get("rad"))
                elif c.tag == kind == "cylinder":
                    rad = _fval(c.get("rad")) if c.get("rad") is not None else rad
                    start = _fval(c.get("start")) if c.get("start") is not None else start
                    end = _fval(c.get("end")) if c.get("end") is not None else end
                elif c.tag == "mesh" and kind == "mesh":
                    mesh = _mesh(c, n.get("name"))
            d.add_object(n.get("name") or "", kind, mat, xf, rad, start, end, *mesh)
        elif n.tag == "light":
            kind = n.get("type")
            c = _typed(n.get("color"))
            col = (1.0, 1.0, 1.0, 1.0)
            if c and c[0] == "vec":
                col = tuple(c[1][:3]) + (1.0,)
            elif c and c[0] in ("int", "flt"):
                col = (c[1],) * 3 + (1.0,)
            xf, radius, dim = Xform(), 1.0, (1.0, 1.0, 1.0)
            for ch in n:
                if ch.tag == "xform":
                    _xform_into(ch, xf)
                elif ch.tag == "sphere" and kind == "sphere":
                    radius = _fval(ch.get("rad"))
                elif ch.tag == "aabox" and kind == "box":
                    a, b = _typed(ch.get("min"))[1], _typed(ch.get("max"))[1]
                    dim = (b[0] - a[0], b[1] - a[1], b[2] - a[2])
            d.add_light(kind, col, xf, radius, dim)
        elif n.tag == "camera" and d.camera is None:
            kind = n.get("type")
            xf, txf = Xform(), Xform()
            if kind == "target":
                xf.key("pos", 0, (0.0, 5.0, 10.0))
                txf.key("pos", 0, (0.0, 0.0, 0.0))
                txf.key("scale", 0, (0.0, 0.0, 0.0))
            sh = n.get("shutter")
            fov = _typed(n.get("fov"))
            target = None
            for ch in n:
                if ch.tag == "xform":
                    _xform_into(ch, xf)
                elif ch.tag == "target" and target is None:
                    target = ch
            if kind == "target" and target is not None:
                for cx in target:
                    if cx.tag == "xform":
                        _xform_into(cx, txf)
            d.set_camera(kind == "target", (fov[1] * math.pi) / 180.0 if fov and fov[0] in ("int", "flt") else math.pi / 4,
                         int(_fval(sh)) if sh is not None else int(shutter), xf, txf)
    return d
