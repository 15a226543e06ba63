"""Cuboid–cuboid collision cases restated from gorilla-physics' own tests, the
reference's cuboid-collider mechanisms, and seeded generators with the
distributions of its randomised collision tests.

* ``SAMPLES``: gjk_sample..gjk_sample4 (src/collision/gjk.rs:137-199) and
  epa_sample, epa_sample3..epa_sample9 (src/collision/epa.rs:437-668) with the
  test's expected outcome or analytic values and tolerance.  epa_sample2 is
  #[ignore]d in the reference ("this exact test case does not pass").
* ``shallow_face_pairs`` / ``separated_pairs`` / ``small_separation_pairs`` /
  ``epa_face_pairs``: the distributions of gjk_face_shallow_penetration,
  gjk_no_penetration, gjk_small_separation (gjk.rs:201-343) and
  epa_face_face_shallow_penetration (epa.rs:365-435), drawn from a seeded numpy
  generator instead of rand::rng().
* ``pusher`` / ``gripper`` / ``box_stack``: the builders of gpb.builders
  (build_pusher / build_gripper, src/helpers.rs:559-666).
"""

from __future__ import annotations

import math

import numpy as np

from tests.golden.kats import quat_axis_angle, quat_euler

PI = math.pi
I = (0.0, 0.0, 0.0, 1.0)
S2 = math.sqrt(2.0)


def pose(q, t):
    return [*q, *t]


# (name, A pose, A sizes, B pose, B sizes, translate, checks) — translate False:
# the test calls gjk / epa on the shapes where they are; True: CollisionDetector.
# checks: ("hit", bool) | ("depth", value, tol) | ("cp", "a"|"b", axis, value, tol)
# | ("same", axis, tol) | ("depth_gt", value) | ("separates", scale)
def _samples():
    s = []
    s.append(("gjk_sample", pose(I, (0, 0, 0)), (3, 1, 2), pose(quat_euler(0, PI / 4, 0), (1.5, 0, 1)), (1, 1, 1),
              False, [("hit", True)]))
    s.append(("gjk_sample2", pose(I, (0, 0, 0)), (1, 1, 1), pose(I, (1.5, 0, 1)), (1, 1, 1), False, [("hit", False)]))
    s.append(("gjk_sample3", pose(I, (0, 0, 0)), (2, 2, 2), pose(I, (-S2, 0, S2)), (2, 2, 2), False,
              [("hit", True)]))
    q45 = quat_axis_angle((0, 1, 0), PI / 4)
    s.append(("gjk_sample4", pose(q45, (0, 0, 0)), (2, 2, 2), pose(q45, (-S2 - 1e-3, 0, S2)), (2, 2, 2), False,
              [("hit", False)]))
    s.append(("epa_sample", pose(quat_euler(-1e-2, 1e-2, -1e-2), (0, 0, 0)), (1.1, 1.1, 1.1),
              pose(I, (1.1 / 2 + 0.5 - 1e-3, 1e-2, 1e-2)), (1, 1, 1), False, [("hit", True), ("separates", 1e-3)]))
    s.append(("epa_sample3", pose(I, (0, 0, 0)), (2, 2, 2), pose(I, (1, 1, 0)), (2, 2, 2), False,
              [("hit", True), ("depth", 1.0, 1e-5), ("separates", 1e-3)]))
    s.append(("epa_sample4", pose(I, (0, 0, 0)), (2, 2, 2), pose(I, (1, 0, 0)), (2, 2, 2), False,
              [("hit", True), ("depth", 1.0, 1e-5), ("same", 1, 1e-5), ("same", 2, 1e-5), ("separates", 1e-3)]))
    s.append(("epa_sample5", pose(I, (1, 0, 0)), (2, 1, 1), pose(q45, (2, 0, 0)), (S2 / 2,) * 3, False,
              [("hit", True), ("depth", 0.5, 1e-5), ("cp", "a", 0, 2.0, 1e-5), ("cp", "a", 2, 0.0, 1e-5),
               ("cp", "b", 0, 1.5, 1e-5), ("cp", "b", 2, 0.0, 1e-5), ("same", 1, 1e-5)]))
    md = 0.15
    depth6 = S2 / 2 * (S2 / 2 - md)
    s.append(("epa_sample6", pose(quat_axis_angle((1, 0, 0), PI / 4), (0, 0, 0)), (1, 1, 1),
              pose(I, (0, 1 + md, 1.5)), (1, 2, 3), False,
              [("hit", True), ("depth", depth6, 1e-5), ("cp", "a", 1, S2 / 2 * depth6 + md, 1e-5),
               ("cp", "a", 2, S2 / 2 * depth6, 1e-5), ("cp", "b", 1, md, 1e-5), ("cp", "b", 2, 0.0, 1e-5),
               ("same", 0, 1e-5)]))
    s.append(("epa_sample7", pose(I, (2.5, 0, 1.0)), (0.5, 0.5, 2.0), pose(I, (3.0, 0, 0.25)), (0.5,) * 3, False,
              [("depth_if_hit", 0.0, 1e-6)]))
    s.append(("epa_sample8", pose(I, (2.5083275, 0, 0.9903475)), (0.5, 0.5, 2.0),
              pose(I, (3.0000002, 0, 0.2499184)), (0.5,) * 3, False, [("hit", True), ("depth_gt", 0.0)]))
    q9 = np.array([2.7207802e-6, -0.002590372, -3.0188437e-5, 0.99999666])
    q9 = tuple(q9 / np.linalg.norm(q9))  # UnitQuaternion::from_quaternion
    s.append(("epa_sample9", pose(I, (2.600148, 0, 0.9818603)), (0.5, 0.5, 2.0),
              pose(q9, (3.0916612, -6.926495e-6, 0.25050417)), (0.5,) * 3, False,
              [("hit", True), ("depth_gt", 0.0)]))
    return s


SAMPLES = _samples()


def _eul(r):
    """UnitQuaternion::from_euler_angles for rows (roll, pitch, yaw) → (x, y, z, w)."""
    sr, cr = np.sin(r[:, 0] * .5), np.cos(r[:, 0] * .5)
    sp, cp = np.sin(r[:, 1] * .5), np.cos(r[:, 1] * .5)
    sy, cy = np.sin(r[:, 2] * .5), np.cos(r[:, 2] * .5)
    return np.stack([sr * cp * cy - cr * sp * sy, cr * sp * cy + sr * cp * sy, cr * cp * sy - sr * sp * cy,
                     cr * cp * cy + sr * sp * sy], 1)


def _cubes(rng, n, center_range, offset_range, place, rot_range, signed=False):
    """A at a random centre; B offset by U(±offset_range), then moved along x or
    y (rng.random_range(0..2)) to place(la, lb) from A's centre (times a random
    sign if `signed`)."""
    c = rng.uniform(-center_range, center_range, (n, 3))
    la, lb = rng.uniform(0.5, 2.0, n), rng.uniform(0.5, 2.0, n)
    ax = rng.integers(0, 2, n)
    sgn = np.where(rng.random(n) < 0.5, 1.0, -1.0) if signed else np.ones(n)
    bc = c + rng.uniform(-offset_range, offset_range, (n, 3))
    k = np.arange(n)
    bc[k, ax] = c[k, ax] + sgn * place(la, lb)
    qa = _eul(rng.uniform(-rot_range, rot_range, (n, 3)))
    qb = _eul(rng.uniform(-rot_range, rot_range, (n, 3)))
    return (np.concatenate([qa, c], 1), np.stack([la] * 3, 1), np.concatenate([qb, bc], 1), np.stack([lb] * 3, 1))


def shallow_face_pairs(rng, n):
    """gjk_face_shallow_penetration: touching faces, penetration in [0, 1e-3)."""
    return _cubes(rng, n, 1.0, 1e-2, lambda la, lb: la / 2 + lb / 2 - rng.uniform(0.0, 1e-3, n), 1e-2)


def separated_pairs(rng, n):
    """gjk_no_penetration: centres l_a + l_b (± 1e-2) apart, any orientation."""
    return _cubes(rng, n, 1.0, 0.1, lambda la, lb: la + lb + rng.uniform(-1e-2, 1e-2, n), PI)


def small_separation_pairs(rng, n):
    """gjk_small_separation: faces 0.1-0.2 apart, near-aligned."""
    return _cubes(rng, n, 1.0, 0.1, lambda la, lb: la / 2 + lb / 2 + rng.uniform(0.1, 0.2, n), 1e-2)


def epa_face_pairs(rng, n):
    """epa_face_face_shallow_penetration: far from the origin (|c| ≤ 100), either
    side along x or y, penetration in [0, 1e-3)."""
    return _cubes(rng, n, 100.0, 1e-2, lambda la, lb: la / 2 + lb / 2 - rng.uniform(0.0, 1e-3, n), 1e-2,
                  signed=True)


def deep_pairs(rng, n):
    """Deep overlaps of arbitrary cuboids in arbitrary orientations (not a
    reference test: the stress case for the storage bounds)."""
    c = rng.uniform(-1, 1, (n, 3))
    da, db = rng.uniform(0.2, 2.0, (n, 3)), rng.uniform(0.2, 2.0, (n, 3))
    bc = c + rng.uniform(-1, 1, (n, 3)) * (da.max(1) / 2 + db.max(1) / 2)[:, None]
    qa = rng.normal(size=(n, 4))
    qa /= np.linalg.norm(qa, axis=1)[:, None]
    qb = rng.normal(size=(n, 4))
    qb /= np.linalg.norm(qb, axis=1)[:, None]
    return np.concatenate([qa, c], 1), da, np.concatenate([qb, bc], 1), db


# ---------------------------------------------------------------------------
# mechanisms with cuboid colliders: the package's builders (src/helpers.rs)

from gpb.builders import build_box_stack as box_stack  # noqa: E402
from gpb.builders import build_gripper as gripper  # noqa: E402
from gpb.builders import build_pusher as pusher  # noqa: E402


def unit_quats(rng, n, scale):
    """Small random rotations (Euler angles in ±scale)."""
    return _eul(rng.uniform(-scale, scale, (n, 3)))
