"""Mechanism descriptions: the reference's types, and their flattened tables.

The classes mirror gorilla-physics' mechanism API so that a caller of the
reference can describe a mechanism the same way:

* ``Transform3D(from_frame, to_frame, rotation, translation)``
  (src/spatial/transform.rs:54-58; rotation is a unit quaternion (x, y, z, w))
* ``RevoluteJoint / PrismaticJoint / FloatingJoint / FixedJoint``
  (src/joint/*.rs; the transform maps the child frame to the parent frame)
* ``SpatialInertia(frame, moment, cross_part, mass)`` (src/inertia.rs:31-37)
* ``RigidBody(inertia)`` (src/rigid_body.rs:62-80) with
  ``add_cuboid_collider(Cuboid.new_at_center(w, d, h))`` (src/rigid_body.rs:197-199),
  ``ContactPoint``
  (src/contact.rs:16-38), ``HalfSpace`` (src/collision/halfspace.rs:6-36)
* ``MechanismState(treejoints, bodies)`` (src/mechanism.rs:62-148): joint i's
  child must be body i and the parent is found by frame name, with the same
  assertion messages.

``Model`` holds the structure-of-arrays tables (``gpb_model``) of many
mechanisms — the form the GPU library consumes.
"""

from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field
from typing import Sequence

import numpy as np

from . import _abi

WORLD_FRAME = "world"  # src/lib.rs:44


@dataclass
class Transform3D:
    from_frame: str
    to_frame: str
    rotation: tuple = (0.0, 0.0, 0.0, 1.0)  # unit quaternion x, y, z, w
    translation: tuple = (0.0, 0.0, 0.0)

    @staticmethod
    def identity(from_frame: str, to_frame: str) -> "Transform3D":
        return Transform3D(from_frame, to_frame)

    @staticmethod
    def move_xyz(from_frame: str, to_frame: str, x: float, y: float, z: float) -> "Transform3D":
        return Transform3D(from_frame, to_frame, translation=(x, y, z))


@dataclass
class SpatialInertia:
    frame: str
    moment: np.ndarray
    cross_part: np.ndarray
    mass: float


@dataclass
class ContactPoint:
    frame: str
    location: tuple
    k: float = 50e3          # src/contact.rs:24-30
    radius: float = 0.0      # > 0: sphere of this radius centred at `location`
    damping: float = 0.0     # LINEAR_SPRING_DAMPER only


@dataclass
class HalfSpace:
    point: tuple
    normal: tuple
    alpha: float = 0.9       # src/collision/halfspace.rs:15-22
    mu: float = 0.5

    @staticmethod
    def new(normal, distance: float, alpha: float = 0.9, mu: float = 0.5) -> "HalfSpace":
        n = np.asarray(normal, float)
        return HalfSpace(tuple(n * distance), tuple(n), alpha, mu)


@dataclass
class Cuboid:
    """Cuboid collider centred on its body's frame (src/collision/cuboid.rs:7-15)."""
    w: float
    d: float
    h: float

    @staticmethod
    def new_at_center(w: float, d: float, h: float) -> "Cuboid":
        return Cuboid(float(w), float(d), float(h))

    @staticmethod
    def new_cube_at_center(l: float) -> "Cuboid":
        return Cuboid(float(l), float(l), float(l))


@dataclass
class RigidBody:
    inertia: SpatialInertia
    contact_points: list = field(default_factory=list)
    collider: Cuboid | None = None

    def add_cuboid_collider(self, cuboid: Cuboid) -> None:
        """RigidBody::add_cuboid_collider (src/rigid_body.rs:197-199).  The
        collider's pose follows the body (src/mechanism.rs:257-275)."""
        self.collider = cuboid

    def add_contact_point(self, cp: ContactPoint) -> None:
        if self.inertia.frame != cp.frame:
            raise ValueError(
                f"Contact point frame {cp.frame} does not match body frame {self.inertia.frame}")
        self.contact_points.append(cp)


@dataclass
class _Joint:
    transform: Transform3D
    axis: tuple = (0.0, 0.0, 1.0)
    spring: tuple | None = None  # (k, rest length), prismatic only
    kind: int = _abi.FIXED
    armature: float = 0.0        # reflected rotor inertia, revolute only

    def with_armature(self, armature: float) -> "_Joint":
        """Joint::with_armature (src/joint/mod.rs:105-109)."""
        if self.kind != _abi.REVOLUTE:
            raise AssertionError("armature is only supported on revolute joints")
        self.armature = float(armature)
        return self


def RevoluteJoint(transform: Transform3D, axis) -> _Joint:
    return _Joint(transform, tuple(float(a) for a in axis), None, _abi.REVOLUTE)


def PrismaticJoint(transform: Transform3D, axis, spring: tuple | None = None) -> _Joint:
    return _Joint(transform, tuple(float(a) for a in axis), spring, _abi.PRISMATIC)


def FloatingJoint(transform: Transform3D) -> _Joint:
    return _Joint(transform, (0.0, 0.0, 0.0), None, _abi.FLOATING)


def FixedJoint(transform: Transform3D) -> _Joint:
    return _Joint(transform, (0.0, 0.0, 0.0), None, _abi.FIXED)


def _nq(kind: int) -> int:
    return {_abi.FIXED: 0, _abi.REVOLUTE: 1, _abi.PRISMATIC: 1, _abi.FLOATING: 7}[kind]


def _nv(kind: int) -> int:
    return {_abi.FIXED: 0, _abi.REVOLUTE: 1, _abi.PRISMATIC: 1, _abi.FLOATING: 6}[kind]


class MechanismState:
    """One mechanism (MechanismState::new, src/mechanism.rs:62-148)."""

    def __init__(self, treejoints: Sequence[_Joint], bodies: Sequence[RigidBody]):
        self.treejoints = list(treejoints)
        self.bodies = list(bodies)
        self.parents: list[int] = []
        self.halfspaces: list[HalfSpace] = []
        self.contact_model = _abi.HUNT_CROSSLEY
        for index, j in enumerate(self.treejoints):
            assert j.transform.from_frame == self.bodies[index].inertia.frame, (
                f"joint {index + 1}'s child body is not body {index + 1}\n")
            if j.transform.to_frame == WORLD_FRAME:
                self.parents.append(0)
            else:
                for bi, b in enumerate(self.bodies):
                    if j.transform.to_frame == b.inertia.frame:
                        self.parents.append(bi + 1)
                        break
                else:
                    raise AssertionError(
                        f"joint {index + 1} has no parent body of frame {j.transform.to_frame}\n")
            if self.parents[-1] > index:
                raise AssertionError(
                    f"joint {index + 1}'s parent body {self.parents[-1]} comes after it")
        # zero state: joint zero / identity pose (src/mechanism.rs:68-88)
        self.q = np.concatenate([np.array([0, 0, 0, 1, 0, 0, 0], float) if j.kind == _abi.FLOATING
                                 else np.zeros(_nq(j.kind)) for j in self.treejoints] or [np.zeros(0)])
        self.v = np.zeros(sum(_nv(j.kind) for j in self.treejoints))

    @property
    def nq(self) -> int:
        return int(self.q.size)

    @property
    def nv(self) -> int:
        return int(self.v.size)

    def add_halfspace(self, h: HalfSpace) -> None:
        self.halfspaces.append(h)

    def add_contact_point(self, cp: ContactPoint) -> None:
        """Adds cp to the body with its frame (src/mechanism.rs:383-391)."""
        for b in self.bodies:
            if b.inertia.frame == cp.frame:
                b.add_contact_point(cp)
                return

    def update(self, q, v) -> None:
        """MechanismState::update with flattened q / v (src/joint/mod.rs:208-303 order)."""
        q = np.asarray(q, float).ravel()
        v = np.asarray(v, float).ravel()
        if q.size != self.nq or v.size != self.nv:
            raise ValueError(f"expected {self.nq} q and {self.nv} v values, got {q.size} and {v.size}")
        self.q = q.copy()
        self.v = v.copy()


class Model:
    """Structure-of-arrays tables of many mechanisms (``gpb_model``)."""

    FIELDS = ("joint_offset", "joint_type", "joint_parent", "joint_iso", "joint_axis",
              "joint_spring", "body_inertia", "contact_offset", "contact_body", "contact_params",
              "halfspace_offset", "halfspace_params", "contact_model", "joint_armature",
              "body_cuboid")

    def __init__(self, **arrays):
        i32 = ("joint_offset", "joint_type", "joint_parent", "contact_offset", "contact_body",
               "halfspace_offset", "contact_model")
        nj = len(np.asarray(arrays["joint_type"]).ravel())
        if arrays.get("joint_armature") is None:  # optional: no armature
            arrays["joint_armature"] = np.zeros(nj)
        if arrays.get("body_cuboid") is None:     # optional: no cuboid colliders
            arrays["body_cuboid"] = np.zeros(3 * nj)
        for name in self.FIELDS:
            a = arrays[name]
            dt = np.int32 if name in i32 else np.float64
            setattr(self, name, np.ascontiguousarray(np.asarray(a, dtype=dt).ravel()))
        self.n = int(self.joint_offset.size - 1)
        self._struct = None

    # -- construction -----------------------------------------------------
    @classmethod
    def from_mechanisms(cls, mechs: Sequence[MechanismState]) -> "Model":
        jo, jt, jp, iso, ax, sp, inert, arm, cub = [0], [], [], [], [], [], [], [], []
        co, cb, cp, ho, hp, cm = [0], [], [], [0], [], []
        for m in mechs:
            for j, b, p in zip(m.treejoints, m.bodies, m.parents):
                jt.append(j.kind)
                jp.append(p)
                iso.extend(list(j.transform.rotation) + list(j.transform.translation))
                ax.extend(j.axis)
                sp.extend(j.spring if j.spring is not None else (0.0, 0.0))
                arm.append(j.armature)
                cub.extend((b.collider.w, b.collider.d, b.collider.h) if b.collider else (0.0, 0.0, 0.0))
                I = b.inertia
                M = np.asarray(I.moment, float)
                inert.extend([I.mass, *np.asarray(I.cross_part, float),
                              M[0, 0], M[1, 1], M[2, 2], M[0, 1], M[0, 2], M[1, 2]])
            jo.append(len(jt))
            for bi, b in enumerate(m.bodies):
                for c in b.contact_points:
                    cb.append(bi + 1)
                    cp.extend([*c.location, c.k, c.radius, c.damping])
            co.append(len(cb))
            for h in m.halfspaces:
                hp.extend([*h.point, *h.normal, h.alpha, h.mu])
            ho.append(len(hp) // 8)
            cm.append(m.contact_model)
        return cls(joint_offset=jo, joint_type=jt, joint_parent=jp, joint_iso=iso, joint_axis=ax,
                   joint_spring=sp, body_inertia=inert, contact_offset=co, contact_body=cb,
                   contact_params=cp, halfspace_offset=ho, halfspace_params=hp, contact_model=cm,
                   joint_armature=arm, body_cuboid=cub)

    @classmethod
    def from_config(cls, config: int, n: int, seed: int = 0,
                    contact_model: int = _abi.LINEAR_SPRING_DAMPER):
        """Seeded benchmark mechanisms (gpb_config_build).  Returns (model, q0, v0, aux)."""
        L = _abi.lib()
        nj, nc, nh, nq, nv = (C.c_int64() for _ in range(5))
        _abi.check(L.gpb_config_sizes(config, n, seed, C.byref(nj), C.byref(nc), C.byref(nh),
                                      C.byref(nq), C.byref(nv)), "gpb_config_sizes")
        nj, nc, nh, nq, nv = nj.value, nc.value, nh.value, nq.value, nv.value
        a = dict(joint_offset=np.zeros(n + 1, np.int32), joint_type=np.zeros(nj, np.int32),
                 joint_parent=np.zeros(nj, np.int32), joint_iso=np.zeros(7 * nj),
                 joint_axis=np.zeros(3 * nj), joint_spring=np.zeros(2 * nj),
                 body_inertia=np.zeros(10 * nj), contact_offset=np.zeros(n + 1, np.int32),
                 contact_body=np.zeros(max(nc, 1), np.int32), contact_params=np.zeros(max(6 * nc, 1)),
                 halfspace_offset=np.zeros(n + 1, np.int32), halfspace_params=np.zeros(max(8 * nh, 1)),
                 contact_model=np.zeros(n, np.int32))
        q0, v0, aux = np.zeros(max(nq, 1)), np.zeros(max(nv, 1)), np.zeros(max(nv, 1))
        ptr = lambda x, t: x.ctypes.data_as(t)
        _abi.check(L.gpb_config_build(
            config, n, seed, contact_model,
            ptr(a["joint_offset"], _abi.P_i32), ptr(a["joint_type"], _abi.P_i32),
            ptr(a["joint_parent"], _abi.P_i32), ptr(a["joint_iso"], _abi.P_f64),
            ptr(a["joint_axis"], _abi.P_f64), ptr(a["joint_spring"], _abi.P_f64),
            ptr(a["body_inertia"], _abi.P_f64), ptr(a["contact_offset"], _abi.P_i32),
            ptr(a["contact_body"], _abi.P_i32), ptr(a["contact_params"], _abi.P_f64),
            ptr(a["halfspace_offset"], _abi.P_i32), ptr(a["halfspace_params"], _abi.P_f64),
            ptr(a["contact_model"], _abi.P_i32), ptr(q0, _abi.P_f64), ptr(v0, _abi.P_f64),
            ptr(aux, _abi.P_f64)), "gpb_config_build")
        a["contact_body"] = a["contact_body"][:nc]
        a["contact_params"] = a["contact_params"][:6 * nc]
        a["halfspace_params"] = a["halfspace_params"][:8 * nh]
        return cls(**a), q0[:nq], v0[:nv], aux[:nv]

    # -- queries ------------------------------------------------------------
    def dims(self, i: int) -> tuple[int, int, int]:
        """(nq, nv, ncontacts) of instance i."""
        t = self.joint_type[self.joint_offset[i]:self.joint_offset[i + 1]]
        nq = int(sum(_nq(int(k)) for k in t))
        nv = int(sum(_nv(int(k)) for k in t))
        return nq, nv, int(self.contact_offset[i + 1] - self.contact_offset[i])

    def offsets(self):
        """Per-instance flattened q / v / contact offsets ([n+1] each)."""
        if getattr(self, "_offsets", None) is None:
            self._offsets = self._compute_offsets()
        return self._offsets

    def _compute_offsets(self):
        t = self.joint_type
        nqj = np.choose(t, [0, 1, 1, 7])
        nvj = np.choose(t, [0, 1, 1, 6])
        cq = np.concatenate([[0], np.cumsum(nqj)])
        cv = np.concatenate([[0], np.cumsum(nvj)])
        return (cq[self.joint_offset].astype(np.int64), cv[self.joint_offset].astype(np.int64),
                self.contact_offset.astype(np.int64))

    def subset(self, idx) -> "Model":
        """The model of instances `idx` (in that order)."""
        idx = np.asarray(idx, int)
        parts = {k: [] for k in self.FIELDS}
        jo, co, ho = [0], [0], [0]
        for i in idx:
            j0, j1 = self.joint_offset[i], self.joint_offset[i + 1]
            c0, c1 = self.contact_offset[i], self.contact_offset[i + 1]
            h0, h1 = self.halfspace_offset[i], self.halfspace_offset[i + 1]
            parts["joint_type"].append(self.joint_type[j0:j1])
            parts["joint_parent"].append(self.joint_parent[j0:j1])
            parts["joint_iso"].append(self.joint_iso[7 * j0:7 * j1])
            parts["joint_axis"].append(self.joint_axis[3 * j0:3 * j1])
            parts["joint_spring"].append(self.joint_spring[2 * j0:2 * j1])
            parts["joint_armature"].append(self.joint_armature[j0:j1])
            parts["body_cuboid"].append(self.body_cuboid[3 * j0:3 * j1])
            parts["body_inertia"].append(self.body_inertia[10 * j0:10 * j1])
            parts["contact_body"].append(self.contact_body[c0:c1])
            parts["contact_params"].append(self.contact_params[6 * c0:6 * c1])
            parts["halfspace_params"].append(self.halfspace_params[8 * h0:8 * h1])
            parts["contact_model"].append(self.contact_model[i:i + 1])
            jo.append(jo[-1] + j1 - j0)
            co.append(co[-1] + c1 - c0)
            ho.append(ho[-1] + h1 - h0)
        out = {k: (np.concatenate(v) if v else np.zeros(0)) for k, v in parts.items() if k not in
               ("joint_offset", "contact_offset", "halfspace_offset")}
        return Model(joint_offset=jo, contact_offset=co, halfspace_offset=ho, **out)

    @classmethod
    def concat(cls, models: Sequence["Model"]) -> "Model":
        """The instances of `models`, one after the other."""
        out = {}
        for name in ("joint_type", "joint_parent", "joint_iso", "joint_axis", "joint_spring",
                     "body_inertia", "contact_body", "contact_params", "halfspace_params",
                     "contact_model", "joint_armature", "body_cuboid"):
            out[name] = np.concatenate([getattr(m, name)[:cls._used(m, name)] for m in models])
        for name in ("joint_offset", "contact_offset", "halfspace_offset"):
            parts, base = [np.zeros(1, np.int64)], 0
            for m in models:
                o = getattr(m, name).astype(np.int64)
                parts.append(o[1:] - o[0] + base)
                base = int(parts[-1][-1]) if parts[-1].size else base
            out[name] = np.concatenate(parts)
        return cls(**out)

    @staticmethod
    def _used(m: "Model", name: str) -> int:
        """Length of the used part of a table (struct() may pad empty tables to one entry)."""
        nj, nc, nh = int(m.joint_offset[-1]), int(m.contact_offset[-1]), int(m.halfspace_offset[-1])
        per = {"joint_type": nj, "joint_parent": nj, "joint_iso": 7 * nj, "joint_axis": 3 * nj,
               "joint_spring": 2 * nj, "joint_armature": nj, "body_cuboid": 3 * nj,
               "body_inertia": 10 * nj, "contact_body": nc,
               "contact_params": 6 * nc, "halfspace_params": 8 * nh, "contact_model": m.n}
        return per[name]

    def struct(self) -> _abi.GpbModel:
        """The ctypes gpb_model pointing at this object's arrays."""
        if self._struct is None:
            s = _abi.GpbModel()
            s.n_instances = self.n
            for name in self.FIELDS:
                arr = getattr(self, name)
                if arr.size == 0:  # keep a valid pointer
                    arr = np.zeros(1, arr.dtype)
                    setattr(self, name, arr)
                t = _abi.P_i32 if arr.dtype == np.int32 else _abi.P_f64
                setattr(s, name, arr.ctypes.data_as(t))
            self._struct = s
        return self._struct
