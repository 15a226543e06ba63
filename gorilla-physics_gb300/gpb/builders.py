"""Mechanism builders of gorilla-physics (src/helpers.rs) that carry cuboid
colliders: build_pusher, build_gripper, and a stack of free boxes."""

from __future__ import annotations

import numpy as np

from .model import (WORLD_FRAME, ContactPoint, Cuboid, FloatingJoint, HalfSpace, MechanismState,
                    PrismaticJoint, RevoluteJoint, RigidBody, SpatialInertia, Transform3D)


def cuboid_body(frame: str, m: float, w: float, d: float, h: float, collider: bool = True) -> RigidBody:
    """RigidBody::new_cuboid (src/rigid_body.rs:160-173), with
    add_cuboid_collider(Cuboid::new_at_center(w, d, h)) if `collider`."""
    mom = np.diag([m * (d * d + h * h) / 12.0, m * (w * w + h * h) / 12.0, m * (w * w + d * d) / 12.0])
    b = RigidBody(SpatialInertia(frame, mom, np.zeros(3), float(m)))
    if collider:
        b.add_cuboid_collider(Cuboid.new_at_center(w, d, h))
    return b


def cube_body(frame: str, m: float, l: float, collider: bool = True) -> RigidBody:
    """RigidBody::new_cube (src/rigid_body.rs:147-158), with a cube collider."""
    mom = m * l * l / 6.0
    b = RigidBody(SpatialInertia(frame, np.diag([mom] * 3), np.zeros(3), float(m)))
    if collider:
        b.add_cuboid_collider(Cuboid.new_cube_at_center(l))
    return b


def add_cube_contacts(state: MechanismState, frame: str, l: float) -> None:
    """add_cube_contacts (src/helpers.rs:388-421): the 8 corners, bottom face first."""
    h = l / 2.0
    for c in [(h, h, -h), (h, -h, -h), (-h, h, -h), (-h, -h, -h),
              (h, h, h), (h, -h, h), (-h, h, h), (-h, -h, h)]:
        state.add_contact_point(ContactPoint(frame, c))


def build_pusher(ground: bool = True) -> MechanismState:
    """build_pusher (src/helpers.rs:559-607): revolute base (about z, 2 m up),
    prismatic pusher along x (cuboid collider 0.2 × 0.2 × 1.75), free 0.5 m cube
    (collider, 8 corner contacts); `ground` adds the half-space z ≥ 0."""
    wb, hb = 0.5, 0.5
    base = cuboid_body("base", 1.0, wb, 0.5, hb, collider=False)
    wp, dp, hp = 0.2, 0.2, 1.75
    push = cuboid_body("pusher", 1.0, wp, dp, hp)
    lc = 0.5
    cube = cube_body("cube", 0.1, lc)
    joints = [RevoluteJoint(Transform3D.move_xyz("base", WORLD_FRAME, 0.0, 0.0, 2.0), (0, 0, 1)),
              PrismaticJoint(Transform3D.move_xyz("pusher", "base", wb / 2 + wp / 2, 0.0, -hb / 2 - hp / 2),
                             (1, 0, 0)),
              FloatingJoint(Transform3D.move_xyz("cube", WORLD_FRAME, wb + wp + 0.5, 0.0, lc / 2))]
    s = MechanismState(joints, [base, push, cube])
    add_cube_contacts(s, "cube", lc)
    if ground:
        s.add_halfspace(HalfSpace.new((0, 0, 1), 0.0))
    return s


def build_gripper(ground: bool = True) -> MechanismState:
    """build_gripper (src/helpers.rs:609-666): prismatic lift (along −z, 2 m
    up), two prismatic jaws along ∓x (cuboid colliders 0.1 × 0.4 × 0.4), free
    0.5 m cube (collider, 8 corner contacts); `ground` adds z ≥ 0."""
    wl, dl, hl = 0.2, 0.2, 1.0
    lift = cuboid_body("lift", 1.0, wl, dl, hl, collider=False)
    wg, dg, hg = 0.1, 0.4, 0.4
    left = cuboid_body("gripper_left", 0.5, wg, dg, hg)
    right = cuboid_body("gripper_right", 0.5, wg, dg, hg)
    lc = 0.5
    cube = cube_body("cube", 0.1, lc)
    joints = [PrismaticJoint(Transform3D.move_xyz("lift", WORLD_FRAME, 0.0, 0.0, 2.0), (0, 0, -1)),
              PrismaticJoint(Transform3D.move_xyz("gripper_left", "lift", -wl / 2 - wg / 2 - 0.3, 0.0,
                                                  -hl / 2 - hg / 2), (-1, 0, 0)),
              PrismaticJoint(Transform3D.move_xyz("gripper_right", "lift", wl / 2 + wg / 2 + 0.3, 0.0,
                                                  -hl / 2 - hg / 2), (1, 0, 0)),
              FloatingJoint(Transform3D.move_xyz("cube", WORLD_FRAME, 0.0, 0.0, lc / 2))]
    s = MechanismState(joints, [lift, left, right, cube])
    add_cube_contacts(s, "cube", lc)
    if ground:
        s.add_halfspace(HalfSpace.new((0, 0, 1), 0.0))
    return s


def build_box_stack(n_boxes: int = 3, l: float = 0.5, m: float = 1.0, ground: bool = True) -> MechanismState:
    """Free cubes (each a FloatingJoint to the world with a collider and its 8
    corner contacts): every pair of boxes is tested each evaluation."""
    joints, bodies = [], []
    for k in range(n_boxes):
        f = f"box{k}"
        joints.append(FloatingJoint(Transform3D(f, WORLD_FRAME)))
        bodies.append(cube_body(f, m, l))
    s = MechanismState(joints, bodies)
    for k in range(n_boxes):
        add_cube_contacts(s, f"box{k}", l)
    if ground:
        s.add_halfspace(HalfSpace.new((0, 0, 1), 0.0))
    return s


def _euler_quats(rng, n, scale):
    """UnitQuaternion::from_euler_angles of angles drawn in ±scale → (x, y, z, w)."""
    r = rng.uniform(-scale, scale, (n, 3))
    sr, cr = np.sin(r[:, 0] * .5), np.cos(r[:, 0] * .5)
    sp, cp = np.sin(r[:, 1] * .5), np.cos(r[:, 1] * .5)
    sy, cy = np.sin(r[:, 2] * .5), np.cos(r[:, 2] * .5)
    return np.stack([sr * cp * cy - cr * sp * sy, cr * sp * cy + sr * cp * sy, cr * cp * sy - sr * sp * cy,
                     cr * cp * cy + sr * sp * sy], 1)


def gripper_states(rng, n: int, closed: bool = True):
    """Seeded states of build_gripper: q = (lift, left jaw, right jaw, cube pose).
    closed: both jaws 0.02-0.07 m into the cube's sides (else 0.1 m clear of
    them); the cube near its rest pose on the ground (±0.01 m, ±0.05 rad);
    v ~ N(0, 0.1²)."""
    q = np.zeros((n, 10))
    q[:, 0] = rng.uniform(0.95, 1.05, n)
    lo, hi = (-0.22, -0.17) if closed else (0.05, 0.1)
    q[:, 1] = rng.uniform(lo, hi, n)
    q[:, 2] = rng.uniform(lo, hi, n)
    q[:, 3:7] = _euler_quats(rng, n, 0.05)
    q[:, 7:9] = rng.uniform(-0.01, 0.01, (n, 2))
    q[:, 9] = rng.uniform(-0.01, 0.01, n)
    v = rng.normal(0, 0.1, (n, 9))
    return q, v


def pusher_states(rng, n: int):
    """Seeded states of build_pusher: q = (base angle, pusher slide, cube pose),
    the pusher's lower end 0.01-0.05 m into the cube's face; v ~ N(0, 0.1²)."""
    q = np.zeros((n, 9))
    q[:, 0] = rng.uniform(-0.05, 0.05, n)
    # pusher x at slide s: 0.35 + s, its face at 0.45 + s; the cube's face at 0.95
    q[:, 1] = rng.uniform(0.51, 0.55, n)
    q[:, 2:6] = _euler_quats(rng, n, 0.05)
    q[:, 6:8] = rng.uniform(-0.01, 0.01, (n, 2))
    q[:, 8] = rng.uniform(-0.01, 0.01, n)
    v = rng.normal(0, 0.1, (n, 8))
    return q, v


def box_stack_states(rng, n: int, k: int = 3):
    """Seeded states of build_box_stack: k cubes stacked along z with 0.005-0.03 m
    overlaps, jittered by ±0.1 m in x, y and ±0.1 rad; v ~ N(0, 0.2²)."""
    q = np.zeros((n, 7 * k))
    z = np.full(n, 0.25 - 0.002)
    for b in range(k):
        q[:, 7 * b:7 * b + 4] = _euler_quats(rng, n, 0.1)
        q[:, 7 * b + 4:7 * b + 6] = rng.uniform(-0.1, 0.1, (n, 2))
        q[:, 7 * b + 6] = z
        z = z + 0.5 - rng.uniform(0.005, 0.03, n)
    v = rng.normal(0, 0.2, (n, 6 * k))
    return q, v


def cuboid_pairs(rng, n: int, kind: str = "shallow"):
    """Seeded independent cuboid pairs for collision-query workloads: poses
    (n, 7) = (qx, qy, qz, qw, tx, ty, tz) and sizes (n, 3) of A and B.
    "shallow": cubes of 0.5-2 m side with touching faces along x or y,
    0-1e-3 m deep, ±1e-2 rad (every pair collides; EPA does the work);
    "deep": cuboids of 0.2-2 m sides in uniformly random orientations with
    centres within one half-extent sum (about 45 % collide)."""
    if kind == "shallow":
        c = rng.uniform(-1.0, 1.0, (n, 3))
        la, lb = rng.uniform(0.5, 2.0, n), rng.uniform(0.5, 2.0, n)
        ax = rng.integers(0, 2, n)
        bc = c + rng.uniform(-1e-2, 1e-2, (n, 3))
        k = np.arange(n)
        bc[k, ax] = c[k, ax] + la / 2 + lb / 2 - rng.uniform(0.0, 1e-3, n)
        qa, qb = _euler_quats(rng, n, 1e-2), _euler_quats(rng, n, 1e-2)
        return (np.concatenate([qa, c], 1), np.stack([la] * 3, 1), np.concatenate([qb, bc], 1),
                np.stack([lb] * 3, 1))
    if kind == "deep":
        c = rng.uniform(-1, 1, (n, 3))
        da, db = rng.uniform(0.2, 2.0, (n, 3)), rng.uniform(0.2, 2.0, (n, 3))
        bc = c + rng.uniform(-1, 1, (n, 3)) * (da.max(1) / 2 + db.max(1) / 2)[:, None]
        qa = rng.normal(size=(n, 4))
        qa /= np.linalg.norm(qa, axis=1)[:, None]
        qb = rng.normal(size=(n, 4))
        qb /= np.linalg.norm(qb, axis=1)[:, None]
        return np.concatenate([qa, c], 1), da, np.concatenate([qb, bc], 1), db
    raise ValueError(f"unknown pair distribution {kind!r}")


def resting_cube_states(rng, model, scale_of, tilt: float = 0.2, depth: float = 2e-3):
    """States of one-cube mechanisms (a FloatingJoint with its 8 corner contacts
    on the ground z ≥ 0) resting near the ground: tilted by up to `tilt` rad,
    the lowest corner 0-`depth` m below the plane, v ~ N(0, 0.5²).  `scale_of(i)`
    is instance i's side length.  Returns flat (q, v)."""
    n = model.n
    q = np.zeros((n, 7))
    q[:, :4] = _euler_quats(rng, n, tilt)
    corners = np.array([[sx, sy, sz] for sx in (-.5, .5) for sy in (-.5, .5) for sz in (-.5, .5)])
    for i in range(n):
        x, y, z, w = q[i, :4]
        R = np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y)],
                      [2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x)],
                      [2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)]])
        zc = (corners * scale_of(i)) @ R[2]
        q[i, 4:6] = rng.uniform(-1.0, 1.0, 2)
        q[i, 6] = -zc.min() - rng.uniform(0.0, depth)
    v = rng.normal(0.0, 0.5, (n, 6))
    return q.ravel(), v.ravel()
