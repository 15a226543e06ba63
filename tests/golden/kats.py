"""Known-answer cases of the hot path, restated from gorilla-physics' own tests.

The reference ships no data files: its pins are inline values in #[test]
functions — analytic results, the closed-form double pendulum
(src/double_pendulum.rs:14-50) and two RigidBodyDynamics.jl vectors.  Each case
below rebuilds the test's mechanism with the gpb model classes and carries the
expected values and tolerance of the reference test it cites.
"""

from __future__ import annotations

import math

import numpy as np

from gpb import (WORLD_FRAME, ContactPoint, FloatingJoint, HalfSpace, MechanismState,
                 PrismaticJoint, RevoluteJoint, RigidBody, SpatialInertia, Transform3D)

G = 9.81
PI = math.pi


def quat_axis_angle(axis, angle):
    a = np.asarray(axis, float)
    a = a / np.linalg.norm(a)
    s, c = math.sin(angle / 2), math.cos(angle / 2)
    return (a[0] * s, a[1] * s, a[2] * s, c)


def quat_euler(roll, pitch, yaw):
    """UnitQuaternion::from_euler_angles (x, y, z, w)."""
    sr, cr = math.sin(roll * 0.5), math.cos(roll * 0.5)
    sp, cp = math.sin(pitch * 0.5), math.cos(pitch * 0.5)
    sy, cy = math.sin(yaw * 0.5), math.cos(yaw * 0.5)
    w = cr * cp * cy + sr * sp * sy
    x = sr * cp * cy - cr * sp * sy
    y = cr * sp * cy + sr * cp * sy
    z = cr * cp * sy - sr * sp * cy
    return (x, y, z, w)


def body(frame, m, moment_diag, cross):
    return RigidBody(SpatialInertia(frame, np.diag(moment_diag).astype(float),
                                    np.asarray(cross, float), float(m)))


def pendulum(m, moment, cross, rot=(0, 0, 0, 1), trans=(0, 0, 0), axis=(0, 1, 0)):
    """build_pendulum (src/helpers.rs:24-46)."""
    j = RevoluteJoint(Transform3D("rod", WORLD_FRAME, rot, trans), axis)
    return MechanismState([j], [body("rod", m, moment, cross)])


def double_pendulum(m, moment, cross, rod2_trans, axis=(0, 1, 0)):
    """build_double_pendulum (src/helpers.rs:49-83) with identity rod1_to_world."""
    j1 = RevoluteJoint(Transform3D("rod1", WORLD_FRAME), axis)
    j2 = RevoluteJoint(Transform3D("rod2", "rod1", translation=rod2_trans), axis)
    return MechanismState([j1, j2], [body("rod1", m, moment, cross), body("rod2", m, moment, cross)])


def double_pendulum2(m1, l1, m2, l2):
    """Point masses on massless rods hanging along −z (the closed form's model)."""
    j1 = RevoluteJoint(Transform3D("rod1", WORLD_FRAME), (0, 1, 0))
    j2 = RevoluteJoint(Transform3D("rod2", "rod1", translation=(0, 0, -l1)), (0, 1, 0))
    b1 = body("rod1", m1, (m1 * l1 * l1, m1 * l1 * l1, 0), (0, 0, -m1 * l1))
    b2 = body("rod2", m2, (m2 * l2 * l2, m2 * l2 * l2, 0), (0, 0, -m2 * l2))
    return MechanismState([j1, j2], [b1, b2])


def simple_double_pendulum(m1, m2, l1, l2, q1, q2, q1dot, q2dot):
    """SimpleDoublePendulum::dynamics (src/double_pendulum.rs:12-53)."""
    s1, s2, s12, c2 = math.sin(q1), math.sin(q2), math.sin(q1 + q2), math.cos(q2)
    I2 = m2 * l2 * l2
    m12 = I2 + m2 * l1 * l2 * c2
    M = np.array([[(m1 + m2) * l1 * l1 + I2 + 2 * m2 * l1 * l2 * c2, m12], [m12, I2]])
    Cm = np.array([[0.0, -m2 * l1 * l2 * (2 * q1dot + q2dot) * s2],
                   [0.5 * m2 * l1 * l2 * (2 * q1dot + q2dot) * s2, -0.5 * m2 * l1 * l2 * q1dot * s2]])
    tau_g = -G * np.array([(m1 + m2) * l1 * s1 + m2 * l2 * s12, m2 * l2 * s12])
    bias = Cm @ np.array([q1dot, q2dot]) - tau_g
    return np.linalg.solve(M, -bias)


def ball(m=5.0, r=1.0):
    mom = 2.0 / 5.0 * m * r * r
    return MechanismState([FloatingJoint(Transform3D("ball", WORLD_FRAME))],
                          [body("ball", m, (mom, mom, mom), (0, 0, 0))])


def cube(m, l):
    """build_cube + add_cube_contacts (src/helpers.rs:151-166,388-421)."""
    mom = m * l * l / 6.0
    s = MechanismState([FloatingJoint(Transform3D("cube", WORLD_FRAME))],
                       [body("cube", m, (mom, mom, mom), (0, 0, 0))])
    h = l / 2.0
    for c in [(h, h, -h), (h, -h, -h), (-h, h, -h), (-h, -h, -h),
              (h, h, h), (h, -h, h), (-h, h, h), (-h, -h, h)]:
        s.add_contact_point(ContactPoint("cube", c))
    return s


def motor_turning_mass():
    """src/dynamics.rs:1194-1251."""
    base = body("base", 1.0, (0.4, 0.4, 0.4), (0, 0, 0))
    mass = body("mass", 1.0, (1.0, 0.0, 1.0), (0, -1.0, 0))
    j = [FloatingJoint(Transform3D("base", WORLD_FRAME)),
         RevoluteJoint(Transform3D("mass", "base"), (0, 0, 1))]
    return MechanismState(j, [base, mass])


def mass_matrix_mech():
    """src/mechanism.rs:711-786 (floating body + two revolute legs)."""
    mb, wb, hb = 2.0, 1.0, 0.1
    body_ = body("body", mb, ((wb * wb + hb * hb) * mb / 12, (wb * wb + hb * hb) * mb / 12,
                              (wb * wb + wb * wb) * mb / 12), (0, 0, 0))
    ml, wl, hl = 1.0, 0.1, 1.0
    mx = ml * ((wl * wl + hl * hl) / 12 + (hl / 2 * hl / 2))
    mz = (wl * wl + wl * wl) * ml / 12
    leg = body("leg", ml, (mx, mx, mz), (0, 0, -hl / 2 * ml))
    leg2 = body("leg2", ml, (mx, mx, mz), (0, 0, -hl / 2 * ml))
    j = [FloatingJoint(Transform3D("body", WORLD_FRAME)),
         RevoluteJoint(Transform3D("leg", "body"), (0, 1, 0)),
         RevoluteJoint(Transform3D("leg2", "leg", translation=(0, 0, -hl)), (0, 1, 0))]
    return MechanismState(j, [body_, leg, leg2])


def supports_tree():
    """test_supports (src/mechanism.rs:793-832): 3 - 2 - 1 - 4 - 5 (1 floating)."""
    j = [FloatingJoint(Transform3D("1", WORLD_FRAME)),
         RevoluteJoint(Transform3D("2", "1", translation=(-1, 0, 0)), (0, 1, 0)),
         RevoluteJoint(Transform3D("3", "2", translation=(0, 0, 1)), (0, 1, 0)),
         RevoluteJoint(Transform3D("4", "1", translation=(1, 0, 0)), (0, 1, 0)),
         RevoluteJoint(Transform3D("5", "4", translation=(0, 0, 1)), (0, 1, 0))]
    b = [body(f, 1.0, (0.4, 0.4, 0.4), (0, 0, 0)) for f in "12345"]
    return MechanismState(j, b)


def cart(m=3.0, l=5.0):
    """build_cart (src/helpers.rs:86-108) as used by simulate.rs:177-214."""
    return MechanismState([PrismaticJoint(Transform3D("cart", WORLD_FRAME), (1, 0, 0))],
                          [body("cart", m, (0, m * l * l / 12, m * l * l / 12), (0, 0, 0))])


def cart_pole(mc=3.0, lc=1.0, mp=5.0, lp=7.0, axis_pole=(0, 1, 0)):
    """build_cart_pole (src/helpers.rs:111-149) as used by simulate.rs:218-272."""
    j = [PrismaticJoint(Transform3D("cart", WORLD_FRAME), (1, 0, 0)),
         RevoluteJoint(Transform3D("pole", "cart"), axis_pole)]
    b = [body("cart", mc, (0, mc * lc * lc / 12, mc * lc * lc / 12), (0, 0, 0)),
         body("pole", mp, (mp * lp * lp, mp * lp * lp, 0), (0, 0, -lp * mp))]
    return MechanismState(j, b)


def spring_pair(m=1.0, r=0.1, k=50.0, l_rest=2.0 / 3.0):
    """spring_on_frictionless_ground (src/dynamics.rs:1133-1188): two spheres,
    A on a floating joint, B on a prismatic joint along A's x axis with a
    spring (k, l_rest); their sphere colliders take no part in the continuous
    dynamics, so the ground half-space exerts nothing."""
    mom = 2.0 / 5.0 * m * r * r
    s = MechanismState([FloatingJoint(Transform3D("A", WORLD_FRAME)),
                        PrismaticJoint(Transform3D("B", "A"), (1.0, 0.0, 0.0), spring=(k, l_rest))],
                       [body("A", m, (mom, mom, mom), (0, 0, 0)), body("B", m, (mom, mom, mom), (0, 0, 0))])
    s.add_halfspace(HalfSpace.new((0, 0, 1), 0.0, 1.0, 0.0))
    return s


def sphere_point(m=1.0, r=0.1):
    """mass_hit_ground (src/contact.rs:607-675): floating sphere + centre contact."""
    mom = 2.0 / 5.0 * m * r * r
    s = MechanismState([FloatingJoint(Transform3D("ball", WORLD_FRAME))],
                       [body("ball", m, (mom, mom, mom), (0, 0, 0))])
    s.add_contact_point(ContactPoint("ball", (0.0, 0.0, 0.0)))
    return s


# ---------------------------------------------------------------------------
# single-evaluation known answers: (name, mechanism, q, v, tau, expected q̈, tol, exact, source)

def dynamics_cases():
    m, l = 5.0, 7.0
    rod_mom = (0.0, m * l * l / 3, m * l * l / 3)
    rod_cross = (m * l / 2, 0, 0)
    cases = []
    p = pendulum(m, rod_mom, rod_cross)
    cases.append(("rod_pendulum_horizontal", p, [0.0], [0.0], [0.0], [3 * G / (2 * l)], 1e-12,
                  "src/dynamics.rs:883-908"))
    qx = quat_axis_angle((1, 0, 0), PI / 2)
    p = pendulum(m, rod_mom, rod_cross, rot=qx, axis=(0, 0, 1))
    cases.append(("rod_pendulum_rotated_frame", p, [0.0], [0.0], [0.0], [-3 * G / (2 * l)], 1e-12,
                  "src/dynamics.rs:916-941"))
    p = pendulum(m, rod_mom, rod_cross, rot=qx, trans=(11.0, 0, 0), axis=(0, 0, 1))
    cases.append(("rod_pendulum_moved_frame", p, [0.0], [0.0], [0.0], [-3 * G / (2 * l)], 1e-6,
                  "src/dynamics.rs:948-975"))
    p = pendulum(m, rod_mom, rod_cross)
    cases.append(("hold_horizontal_rod", p, [0.0], [0.0], [-m * G * l / 2], [0.0], 1e-6,
                  "src/dynamics.rs:979-1007"))
    p = pendulum(m, (0, m * l * l, m * l * l), (m * l, 0, 0))
    cases.append(("simple_pendulum_horizontal", p, [0.0], [0.0], [0.0], [G / l], 1e-12,
                  "src/dynamics.rs:1011-1033"))
    p = double_pendulum(m, (0, m * l * l, m * l * l), (m * l, 0, 0), (l, 0, 0))
    cases.append(("double_pendulum_horizontal", p, [0.0, 0.0], [0.0, 0.0], [0.0, 0.0],
                  [G / l, -G / l], 1e-6, "src/dynamics.rs:1038-1088"))
    m3, l5 = 3.0, 5.0
    p = double_pendulum(m3, (m3 * l5 * l5, m3 * l5 * l5, 0), (0, 0, -m3 * l5), (0, 0, -l5))
    cases.append(("double_pendulum_closed_form", p, [3.0, 5.0], [3.0, 5.0], [0.0, 0.0],
                  list(simple_double_pendulum(m3, m3, l5, l5, 3.0, 5.0, 3.0, 5.0)), 1e-5,
                  "src/dynamics.rs:1091-1130"))
    p = double_pendulum2(1.0, 2.0, 3.0, 4.0)
    cases.append(("double_pendulum_rbdjl", p, [1.0, 2.0], [3.0, 4.0], [0.0, 0.0],
                  [68.8824, -58.9877], 1e-4, "src/double_pendulum.rs:64-83 (RigidBodyDynamics.jl)"))
    b = ball()
    q = list(quat_euler(0.1, 0.2, 0.3)) + [1.0, 2.0, 3.0]
    cases.append(("ball_dynamics", b, q, [1, 2, 3, 4, 5, 6], [0.0] * 6,
                  [0.0, 0.0, 0.0, 4.948946, -6.959844, -6.566419], 1e-5,
                  "src/joint/floating.rs:82-128 (RigidBodyDynamics.jl)"))
    mt = motor_turning_mass()
    base_ang = -1.0 / 0.4
    base_lin_x = -1.0 / 1.0 / 1.0
    exp = [0, 0, base_ang, base_lin_x, 0, -G, -base_ang + 1.0 / 1.0 + -base_lin_x * 1.0]
    cases.append(("motor_turning_mass", mt, [0, 0, 0, 1, 0, 0, 0, 0.0], [0.0] * 7, [0.0] * 6 + [1.0],
                  exp, 1e-5, "src/dynamics.rs:1194-1251"))
    return cases
