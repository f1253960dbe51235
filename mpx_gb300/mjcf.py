"""MJCF (MuJoCo XML) reader for the whole-body terms.

Reads the subset of MJCF that defines the rigid-body dynamics of a
floating-base robot such as mpx/data/aliengo/aliengo.xml (the model that
mpx/config/config_srbd.py:6 names for the SRBD controller's whole-body
interface):

  * the body tree in document order (MuJoCo's body numbering), each body's
    `pos` and orientation (`quat`, `axisangle`, `euler` with the compiler's
    `angle` unit and `eulerseq`) in its parent's frame;
  * `<inertial>`: `mass`, `pos`, orientation, `diaginertia` or `fullinertia`;
  * one joint per body: `<freejoint/>` (no armature: MuJoCo's shortcut for a
    free joint with zero armature, damping and friction loss) or `<joint>`
    with `type` hinge / slide / free, `axis`, `pos`, `ref`, `armature`,
    resolved through the `<default>` classes (`class`, `childclass`);
  * `<option gravity>`;
  * the named geoms used as contact points (their `pos`, or the middle of
    `fromto`);
  * `<include file=...>` (the included file's top-level children take the
    element's place, paths relative to the including file), and repeated
    `<worldbody>` / `<default>` sections, read in order.

Everything else (meshes, visuals, actuators, sensors, limits, damping and
friction loss, which do not enter M or qfrc_bias) is ignored.  Bodies without
an `<inertial>` element would need MuJoCo's inertia-from-geom compilation and
are rejected unless they carry no geoms of their own.
"""
import os
import xml.etree.ElementTree as ET
from dataclasses import dataclass, field

import numpy as np

JNT_NONE, JNT_FREE, JNT_HINGE, JNT_SLIDE = 0, 1, 2, 3
_NDOF = {JNT_NONE: 0, JNT_FREE: 6, JNT_HINGE: 1, JNT_SLIDE: 1}
_NQ = {JNT_NONE: 0, JNT_FREE: 7, JNT_HINGE: 1, JNT_SLIDE: 1}


@dataclass
class RigidBodyModel:
    """A floating-base tree in MuJoCo's conventions (float64 numpy arrays).

    Bodies are listed parents first (index 0 is the first body under the
    world).  Inertias are about the body's centre of mass, in the body frame."""
    body_names: list
    parent: np.ndarray        # [nb] int, -1 = world
    body_pos: np.ndarray      # [nb,3]
    body_quat: np.ndarray     # [nb,4] (w, x, y, z)
    jnt_type: np.ndarray      # [nb] int
    jnt_pos: np.ndarray       # [nb,3]
    jnt_axis: np.ndarray      # [nb,3] unit
    jnt_names: list
    mass: np.ndarray          # [nb]
    com: np.ndarray           # [nb,3]
    inertia: np.ndarray       # [nb,3,3]
    armature: np.ndarray      # [nv]
    gravity: np.ndarray       # [3]
    contact_names: list = field(default_factory=list)
    contact_point_body: np.ndarray = None   # [C] int
    contact_jac_body: np.ndarray = None     # [C] int
    contact_point_pos: np.ndarray = None    # [C,3]
    geoms: dict = field(default_factory=dict)  # name -> (body index, pos)

    @property
    def nbody(self):
        return len(self.parent)

    @property
    def dof_adr(self):
        return np.concatenate([[0], np.cumsum([_NDOF[int(t)] for t in self.jnt_type])])[:-1].astype(np.int64)

    @property
    def qpos_adr(self):
        return np.concatenate([[0], np.cumsum([_NQ[int(t)] for t in self.jnt_type])])[:-1].astype(np.int64)

    @property
    def nv(self):
        return int(sum(_NDOF[int(t)] for t in self.jnt_type))

    @property
    def nq(self):
        return int(sum(_NQ[int(t)] for t in self.jnt_type))

    def body_id(self, name):
        return self.body_names.index(name)

    def with_contacts(self, geom_names, body_names):
        """Contact points = the named geoms, differentiated as attached to the
        named bodies (mjx.name2id of config.contact_frame / config.body_name,
        mpx/utils/mpc_wrapper_srbd.py:43-48)."""
        if len(geom_names) != len(body_names):
            raise ValueError("one body per contact geom")
        pb, jb, pp = [], [], []
        for g, b in zip(geom_names, body_names):
            if g not in self.geoms:
                raise KeyError("no geom named %r" % g)
            gb, gpos = self.geoms[g]
            pb.append(gb)
            pp.append(gpos)
            jb.append(self.body_id(b))
        self.contact_names = list(geom_names)
        self.contact_point_body = np.asarray(pb, dtype=np.int64)
        self.contact_jac_body = np.asarray(jb, dtype=np.int64)
        self.contact_point_pos = np.asarray(pp, dtype=np.float64).reshape(-1, 3)
        return self

    def to_struct(self):
        """The mpxg_wb_model of include/mpxg.h (float32)."""
        from . import _lib
        S = _lib.WbModel()
        nb, nv = self.nbody, self.nv
        nc = 0 if self.contact_point_body is None else len(self.contact_point_body)
        if nb > _lib.WB_MAX_BODY or nv > _lib.WB_MAX_DOF or nc > _lib.WB_MAX_CONTACT:
            raise ValueError("model too large for the kernel (%d bodies, %d dofs, %d contacts)" % (nb, nv, nc))
        S.nbody, S.nq, S.nv, S.n_contact = nb, self.nq, nv, nc
        dadr, qadr = self.dof_adr, self.qpos_adr
        for b in range(nb):
            S.parent[b] = int(self.parent[b])
            S.jnt_type[b] = int(self.jnt_type[b])
            S.qpos_adr[b] = int(qadr[b])
            S.dof_adr[b] = int(dadr[b])
            S.mass[b] = float(self.mass[b])
            for i in range(3):
                S.body_pos[b][i] = float(self.body_pos[b, i])
                S.jnt_pos[b][i] = float(self.jnt_pos[b, i])
                S.jnt_axis[b][i] = float(self.jnt_axis[b, i])
                S.com[b][i] = float(self.com[b, i])
            for i in range(4):
                S.body_quat[b][i] = float(self.body_quat[b, i])
            for i in range(9):
                S.inertia[b][i] = float(self.inertia[b].reshape(-1)[i])
        for j in range(nv):
            S.armature[j] = float(self.armature[j])
        for i in range(3):
            S.gravity[i] = float(self.gravity[i])
        for c in range(nc):
            S.contact_point_body[c] = int(self.contact_point_body[c])
            S.contact_jac_body[c] = int(self.contact_jac_body[c])
            for i in range(3):
                S.contact_point_pos[c][i] = float(self.contact_point_pos[c, i])
        return S


# ----------------------------------------------------------------- helpers
def _vec(s, n=None):
    v = np.array([float(t) for t in s.split()], dtype=np.float64)
    if n is not None and v.size != n:
        raise ValueError("expected %d numbers, got %r" % (n, s))
    return v


def _quat_mul(a, b):
    w1, x1, y1, z1 = a
    w2, x2, y2, z2 = b
    return np.array([w1 * w2 - x1 * x2 - y1 * y2 - z1 * z2, w1 * x2 + x1 * w2 + y1 * z2 - z1 * y2,
                     w1 * y2 - x1 * z2 + y1 * w2 + z1 * x2, w1 * z2 + x1 * y2 - y1 * x2 + z1 * w2])


def _axis_quat(axis, angle):
    axis = np.asarray(axis, dtype=np.float64)
    axis = axis / np.linalg.norm(axis)
    return np.concatenate([[np.cos(angle / 2)], np.sin(angle / 2) * axis])


def quat_to_mat(q):
    w, x, y, z = np.asarray(q, dtype=np.float64) / np.linalg.norm(q)
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y)],
                     [2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x)],
                     [2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)]])


def _expand_includes(el, base_dir, depth=0):
    """Replace every <include file=...> below el by the children of the
    included file's root element (recursively)."""
    if depth > 16:
        raise ValueError("MJCF includes nest deeper than 16 levels")
    i = 0
    while i < len(el):
        child = el[i]
        if child.tag == "include":
            if base_dir is None:
                raise ValueError("<include> needs the model to be read from a file")
            path = os.path.join(base_dir, child.get("file"))
            inc = ET.parse(path).getroot()
            _expand_includes(inc, os.path.dirname(path), depth + 1)
            el.remove(child)
            for k, c in enumerate(list(inc)):
                el.insert(i + k, c)
            i += len(inc)
        else:
            _expand_includes(child, base_dir, depth)
            i += 1


class _Defaults:
    """MJCF default classes: class name -> tag -> {attribute: value}, each
    class inheriting its parent class's values."""

    def __init__(self, root):
        self.cls = {"main": {}}
        for top in root.findall("default"):
            self._walk(top, "main", self.cls["main"])

    def _walk(self, el, name, inherited):
        own = {tag: dict(attrs) for tag, attrs in inherited.items()}
        for child in el:
            if child.tag == "default":
                continue
            own.setdefault(child.tag, {}).update(child.attrib)
        self.cls[name] = own
        for child in el:
            if child.tag == "default":
                self._walk(child, child.get("class", name), own)

    def get(self, el, tag, attr, cls):
        if attr in el.attrib:
            return el.get(attr)
        c = el.get("class", cls)
        if c not in self.cls:
            raise KeyError("unknown default class %r" % c)
        return self.cls[c].get(tag, {}).get(attr)


def _orientation(el, compiler):
    """quat / axisangle / euler of an element (identity if none)."""
    deg = compiler.get("angle", "degree") == "degree"
    unit = np.pi / 180.0 if deg else 1.0
    if "quat" in el.attrib:
        q = _vec(el.get("quat"), 4)
        return q / np.linalg.norm(q)
    if "axisangle" in el.attrib:
        v = _vec(el.get("axisangle"), 4)
        return _axis_quat(v[:3], v[3] * unit)
    if "euler" in el.attrib:
        seq = compiler.get("eulerseq", "xyz")
        ang = _vec(el.get("euler"), 3) * unit
        q = np.array([1.0, 0.0, 0.0, 0.0])
        for ch, a in zip(seq, ang):
            ax = {"x": [1, 0, 0], "y": [0, 1, 0], "z": [0, 0, 1]}[ch.lower()]
            r = _axis_quat(ax, a)
            # lower case: rotations about the moving axes; upper case: fixed axes
            q = _quat_mul(q, r) if ch.islower() else _quat_mul(r, q)
        return q
    for a in ("xyaxes", "zaxis"):
        if a in el.attrib:
            raise NotImplementedError("orientation attribute %r is not supported" % a)
    return np.array([1.0, 0.0, 0.0, 0.0])


def parse(source, contact_geoms=None, contact_bodies=None):
    """Read an MJCF file path (or XML text starting with '<') into a
    RigidBodyModel; contact_geoms / contact_bodies as in with_contacts()."""
    if source.lstrip().startswith("<"):
        root, base_dir = ET.fromstring(source), None
    else:
        root, base_dir = ET.parse(source).getroot(), os.path.dirname(os.path.abspath(source))
    _expand_includes(root, base_dir)
    compiler = {}
    for c in root.findall("compiler"):
        compiler.update(c.attrib)
    defaults = _Defaults(root)
    gravity = np.array([0, 0, -9.81])
    for opt in root.findall("option"):
        if "gravity" in opt.attrib:
            gravity = _vec(opt.get("gravity"), 3)
    names, parent, bpos, bquat = [], [], [], []
    jt, jpos, jaxis, jnames, armature = [], [], [], [], []
    mass, com, inertia = [], [], []
    geoms = {}

    def visit(el, par, cls):
        b = len(names)
        names.append(el.get("name", "body%d" % b))
        parent.append(par)
        bpos.append(_vec(el.get("pos", "0 0 0"), 3))
        bquat.append(_orientation(el, compiler))
        cls = el.get("childclass", cls)
        # inertia
        inert = el.find("inertial")
        own_geoms = el.findall("geom")
        if inert is None:
            # a body without <inertial> gets its inertia from its geoms in
            # MuJoCo (inertiafromgeom); only geom-less bodies are accepted
            if own_geoms:
                raise NotImplementedError("body %r: inertia from geoms is not supported; add <inertial>" % names[-1])
            mass.append(0.0)
            com.append(np.zeros(3))
            inertia.append(np.zeros((3, 3)))
        else:
            m = float(inert.get("mass"))
            ipos = _vec(inert.get("pos", "0 0 0"), 3)
            iq = _orientation(inert, compiler)
            if "diaginertia" in inert.attrib:
                d = _vec(inert.get("diaginertia"), 3)
                Ri = quat_to_mat(iq)
                I = Ri @ np.diag(d) @ Ri.T
            elif "fullinertia" in inert.attrib:
                f = _vec(inert.get("fullinertia"), 6)  # ixx iyy izz ixy ixz iyz
                I = np.array([[f[0], f[3], f[4]], [f[3], f[1], f[5]], [f[4], f[5], f[2]]])
            else:
                raise ValueError("body %r: <inertial> needs diaginertia or fullinertia" % names[-1])
            mass.append(m)
            com.append(ipos)
            inertia.append(0.5 * (I + I.T))
        # joint
        joints = [c for c in el if c.tag in ("joint", "freejoint")]
        if len(joints) > 1:
            raise NotImplementedError("body %r has %d joints; one joint per body is supported" % (names[-1], len(joints)))
        if not joints:
            jt.append(JNT_NONE)
            jpos.append(np.zeros(3))
            jaxis.append(np.array([0.0, 0.0, 1.0]))
            jnames.append(None)
        else:
            j = joints[0]
            jnames.append(j.get("name"))
            if j.tag == "freejoint":
                t, arm = JNT_FREE, 0.0
            else:
                t = {"hinge": JNT_HINGE, "slide": JNT_SLIDE, "free": JNT_FREE}.get(
                    defaults.get(j, "joint", "type", cls) or "hinge")
                if t is None:
                    raise NotImplementedError("joint type %r is not supported" % defaults.get(j, "joint", "type", cls))
                arm = float(defaults.get(j, "joint", "armature", cls) or 0.0)
            if t == JNT_FREE and par != -1:
                raise NotImplementedError("a free joint must attach a body to the world")
            jt.append(t)
            jpos.append(_vec(defaults.get(j, "joint", "pos", cls) or "0 0 0", 3) if t != JNT_FREE else np.zeros(3))
            ax = _vec(defaults.get(j, "joint", "axis", cls) or "0 0 1", 3)
            ax = ax / np.linalg.norm(ax)
            jaxis.append(ax)
            armature.extend([arm] * _NDOF[t])
            # MuJoCo measures a hinge / slide coordinate from the joint's
            # `ref`.  Rotations about one axis commute, so the offset folds
            # into the body's rest pose: the body turns by -ref about the axis
            # through the anchor (or moves by -ref along it), and q then
            # enters the kinematics as it is.
            ref = float(defaults.get(j, "joint", "ref", cls) or 0.0)
            if ref != 0.0 and t == JNT_HINGE:
                deg = compiler.get("angle", "degree") == "degree"
                th = -ref * (np.pi / 180.0 if deg else 1.0)
                Rb = quat_to_mat(bquat[-1])
                anchor = bpos[-1] + Rb @ jpos[-1]
                bquat[-1] = _quat_mul(bquat[-1], _axis_quat(ax, th))
                bpos[-1] = anchor - quat_to_mat(bquat[-1]) @ jpos[-1]
            elif ref != 0.0 and t == JNT_SLIDE:
                bpos[-1] = bpos[-1] - quat_to_mat(bquat[-1]) @ ax * ref
        for g in own_geoms:
            gname = g.get("name")
            if gname is None:
                continue
            if "fromto" in g.attrib:
                ft = _vec(g.get("fromto"), 6)
                gp = 0.5 * (ft[:3] + ft[3:])
            else:
                gp = _vec(defaults.get(g, "geom", "pos", cls) or "0 0 0", 3)
            geoms[gname] = (b, gp)
        for child in el.findall("body"):
            visit(child, b, cls)

    worlds = root.findall("worldbody")
    if not worlds:
        raise ValueError("no <worldbody>")
    for world in worlds:
        for child in world.findall("body"):
            visit(child, -1, "main")
    model = RigidBodyModel(
        body_names=names, parent=np.asarray(parent, dtype=np.int64), body_pos=np.asarray(bpos),
        body_quat=np.asarray(bquat), jnt_type=np.asarray(jt, dtype=np.int64), jnt_pos=np.asarray(jpos),
        jnt_axis=np.asarray(jaxis), jnt_names=jnames, mass=np.asarray(mass), com=np.asarray(com),
        inertia=np.asarray(inertia), armature=np.asarray(armature, dtype=np.float64), gravity=gravity, geoms=geoms)
    if model.nbody and model.jnt_type[0] != JNT_FREE and (model.jnt_type == JNT_FREE).any():
        raise NotImplementedError("a free joint is supported on the first body only")
    if contact_geoms is not None:
        model.with_contacts(contact_geoms, contact_bodies)
    return model


_NPZ_ARRAYS = ("parent", "body_pos", "body_quat", "jnt_type", "jnt_pos", "jnt_axis", "mass", "com", "inertia",
               "armature", "gravity", "contact_point_body", "contact_jac_body", "contact_point_pos")


def save_npz(model, path, **extra):
    """Write a parsed model (plus any extra arrays) to an .npz file."""
    arrays = {k: getattr(model, k) for k in _NPZ_ARRAYS if getattr(model, k) is not None}
    arrays["body_names"] = np.asarray(model.body_names)
    arrays["contact_names"] = np.asarray(model.contact_names)
    np.savez(path, **arrays, **extra)


def load_npz(path):
    """Read a model written by save_npz."""
    z = np.load(path, allow_pickle=False)
    kw = {k: z[k] for k in _NPZ_ARRAYS if k in z.files}
    m = RigidBodyModel(body_names=[str(s) for s in z["body_names"]], jnt_names=[None] * len(z["parent"]),
                       contact_names=[str(s) for s in z["contact_names"]], **kw)
    return m
