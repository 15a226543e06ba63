"""Velocity stepping (src/integrators.rs:42-51; src/dynamics.rs:367-430,652-742).

The reference solves the friction-cone program of every step with Clarabel
0.11.1, a third-party interior-point solver that is not in the repository.
Its solution in velocity space is unique — the objective ½λᵀGλ + gᵀλ with
G = J M⁻¹ Jᵀ, g = J v_free depends on λ only through Jᵀλ — so any solver that
reaches the optimum gives the reference's v'.

CPU: the oracle (oracle/socp.cpp, oracle/gpb_oracle.cpp: velocity_step) is
pinned by the reference's own velocity-stepping tests (shoot a box onto a
tilted plane, drop a sphere, roll a sphere under torque) with their
tolerances, by the optimality certificate of every program it solves
(λ in the friction cones, the contact velocities J v' in the dual cones,
complementarity), and against scipy's SLSQP on small programs.

GPU (-m gpu): one step of cubes, spheres, quadrupeds, grippers and pushers
against the oracle (v' and q' within 1e-6 relative — both solvers stop at
1e-10 relative residual and gap), the reference scenarios run on the GPU, and
the argument checks.
"""

import math

import numpy as np
import pytest

import gpb
import oracle
from gpb import (WORLD_FRAME, Batch, ContactPoint, FloatingJoint, HalfSpace, MechanismState, Model,
                 Transform3D, builders)
from tests.golden import kats

VS = gpb.VELOCITY_STEPPING
MU = 0.95


def sphere(m, r, ground=True):
    """build_sphere (src/helpers.rs:812-821): the sphere collider is a contact
    point at the body origin with radius r."""
    mom = 2.0 / 5.0 * m * r * r
    s = MechanismState([FloatingJoint(Transform3D("sphere", WORLD_FRAME))],
                       [kats.body("sphere", m, (mom, mom, mom), (0, 0, 0))])
    s.add_contact_point(ContactPoint("sphere", (0, 0, 0), radius=r))
    if ground:
        s.add_halfspace(HalfSpace.new((0, 0, 1), 0.0))
    return s


def ground_cube(m, l):
    """build_cube (src/helpers.rs:151-166) on the ground z ≥ 0."""
    s = kats.cube(m, l)
    s.add_halfspace(HalfSpace.new((0, 0, 1), 0.0))
    return s


def shoot_box():
    """velocity_stepping_shoot_box (src/integrators.rs:340-382)."""
    s = kats.cube(1.0, 1.0)
    ang = math.radians(-10.0)
    n = (math.sin(ang), 0.0, math.cos(ang))
    s.add_halfspace(HalfSpace.new(n, 0.0))
    rot = kats.quat_axis_angle((0, 1, 0), math.pi / 2)
    # linear velocity rot⁻¹ (1, 0, 0) in the body frame: a quarter turn about y maps x to −z
    q0 = np.array([*rot, 0.0, 0.0, 1.0])
    v0 = np.array([0.0, 0.0, 0.0, 0.0, 0.0, 1.0])
    return s, q0, v0, np.array(n)


def run_oracle(M, q, v, dt, K, tau=None):
    for _ in range(K):
        q, v, st = oracle.step(M, 0, q, v, dt, tau, VS)
        assert st == 0
    return q, v


def euler_xyz(qx, qy, qz, qw):
    """UnitQuaternion::euler_angles (roll, pitch, yaw)."""
    roll = math.atan2(2 * (qw * qx + qy * qz), 1 - 2 * (qx * qx + qy * qy))
    pitch = math.asin(max(-1.0, min(1.0, 2 * (qw * qy - qz * qx))))
    yaw = math.atan2(2 * (qw * qz + qx * qy), 1 - 2 * (qy * qy + qz * qz))
    return roll, pitch, yaw


# ---------------------------------------------------------------------------
# CPU: the oracle against the reference's tests


def test_oracle_shoot_box(built):
    s, q0, v0, n = shoot_box()
    M = Model.from_mechanisms([s])
    dt = 1.0 / 600.0
    q, v = run_oracle(M, q0, v0, dt, int(2.0 / dt))
    assert abs(np.dot(q[4:7], n) - 0.5) <= 1e-2
    assert abs(q[5]) <= 1e-5
    assert np.all(np.abs(v) <= 1e-5)


def test_oracle_sphere_hit_ground(built):
    """sphere_hit_ground (src/collision/sphere.rs:55-86)."""
    M = Model.from_mechanisms([sphere(1.0, 1.0)])
    q, _ = run_oracle(M, np.array([0, 0, 0, 1, 0, 0, 1.5]), np.zeros(6), 1e-3, 2000)
    np.testing.assert_allclose(q[4:7], [0, 0, 1], atol=1e-3)


def test_oracle_sphere_roll_forward(built):
    """sphere_roll_forward (src/collision/sphere.rs:88-131): exact zeros out of
    the rolling plane, rolling without slip (r·θ = x)."""
    r = 0.5
    M = Model.from_mechanisms([sphere(1.0, r)])
    q, _ = run_oracle(M, np.array([0, 0, 0, 1, 0, 0, r]), np.zeros(6), 1e-3, 2000,
                      tau=np.array([0, 0.1, 0, 0, 0, 0]))
    roll, pitch, yaw = euler_xyz(*q[:4])
    assert roll == 0.0 and yaw == 0.0 and q[5] == 0.0
    assert abs(q[6] - r) <= 1e-5
    assert abs(r * pitch - q[4]) <= 1e-4


def test_oracle_box_pusher(built):
    """velocity_stepping_box_pusher (src/integrators.rs:416-440), PusherController
    (src/control/pusher_control.rs:13-30).  The box stays on the ground (z within
    1e-2) and within the test's ±0.2 m band in y, but it does not reach x > 3:
    the single EPA contact point of the face-face pusher/box contact moves
    between the corners of the contact patch (y = ±0.1, near the box's bottom
    or top edge), tipping and yawing the box until it slides off the pusher at
    x ≈ 2.5.  The reference test marks the case as sensitive to friction
    ("needs friction mu to be < 1.0")."""
    M = Model.from_mechanisms([builders.build_pusher()])
    q = np.array([0, 0, 0, 0, 0, 1, 0, 0, 0], float)
    v = np.zeros(8)
    dt = 1.0 / 120.0
    for _ in range(int(5.0 / dt)):
        qd = 3.0 - q[1]
        vt = math.copysign(10.0 * min(abs(qd), 0.1), qd)
        tau = np.array([0, 20.0 * (vt - v[1]), 0, 0, 0, 0, 0, 0])
        q, v, st = oracle.step(M, 0, q, v, dt, tau, VS)
        assert st == 0
    box = q[6:9] + np.array([1.2, 0.0, 0.25])  # world centre (init translation + q)
    assert abs(box[1]) <= 0.2 and abs(box[2] - 0.25) <= 1e-2
    assert box[0] > 2.0


def test_oracle_box_pusher_cause(built):
    """Why the restated box pusher stops short of x > 3 (the cause, shown).

    The pusher's face (0.2 m wide, 1.75 m tall) covers the whole height of the
    box's back face, so their contact is a 0.2 × 0.5 m patch, but
    CollisionDetector returns one contact point (EPA's closest point of the
    Minkowski difference, src/collision/epa.rs), which for a face-face contact
    lands on a corner of the patch.  Along the oracle's trajectory the point sits
    on the box's top or bottom edge in most contact steps, never near the face's
    centre, and flips between the two edges: the single off-centre push tips
    and yaws the box (about 1 rad by the time it slides off the pusher at
    x ≈ 2.45), so it never reaches x = 3.  The reference runs the same
    single-point contact, and its own test notes that it depends on friction
    ("needs friction mu to be < 1.0")."""
    from scipy.spatial.transform import Rotation

    M = Model.from_mechanisms([builders.build_pusher()])
    q = np.array([0, 0, 0, 0, 0, 1, 0, 0, 0], float)
    v = np.zeros(8)
    dt = 1.0 / 120.0
    zrel, yaw_hit, box_x = [], [], []
    for _ in range(int(5.0 / dt)):
        Rz = Rotation.from_euler("z", q[0])
        pc = np.array([0, 0, 2.0]) + Rz.apply([0.35 + q[1], 0, -1.125])  # pusher centre
        bc = q[6:9] + np.array([1.2, 0, 0.25])                            # box centre
        r, _, cb = oracle.collide_cuboids(np.r_[Rz.as_quat(), pc][None], [[0.2, 0.2, 1.75]],
                                          np.r_[q[2:6], bc][None], [[0.5, 0.5, 0.5]])
        if r[0] == oracle.COL_HIT:
            zrel.append(cb[0][2] - bc[2])
            yaw_hit.append(Rotation.from_quat(q[2:6]).as_euler("xyz")[2])
            box_x.append(bc[0])
        qd = 3.0 - q[1]
        vt = math.copysign(10.0 * min(abs(qd), 0.1), qd)
        tau = np.array([0, 20.0 * (vt - v[1]), 0, 0, 0, 0, 0, 0])
        q, v, st = oracle.step(M, 0, q, v, dt, tau, VS)
        assert st == 0
    z = np.array(zrel)
    assert z.size > 50
    assert np.mean(np.abs(z) >= 0.24) > 0.75       # on the top or bottom edge (half height 0.25)
    assert np.all(np.abs(z) > 0.1)                 # never near the middle of the face
    assert np.sum(np.diff(np.sign(z)) != 0) >= 10  # flips between the two edges
    assert abs(yaw_hit[-1]) > 0.5 and box_x[-1] < 3.0


def cube_states(rng, n):
    """Cubes of side 0.4-1.0 m tilted by up to 0.2 rad, the lowest corners
    0-2 mm below the ground, random velocities (1-4 corner contacts)."""
    from scipy.spatial.transform import Rotation

    ls = rng.uniform(0.4, 1.0, n)
    quats = Rotation.from_euler("xyz", rng.uniform(-0.2, 0.2, (n, 3))).as_quat()
    q, v = [], []
    corners = np.array([[sx, sy, sz] for sx in (-.5, .5) for sy in (-.5, .5) for sz in (-.5, .5)])
    for l, qu in zip(ls, quats):
        zc = (Rotation.from_quat(qu).apply(corners * l))[:, 2]
        z = -zc.min() - rng.uniform(0.0, 2e-3)
        q.append(np.array([*qu, rng.uniform(-1, 1), rng.uniform(-1, 1), z]))
        v.append(rng.normal(0, 0.5, 6))
    return ls, q, v


def vs_models(rng, n=24):
    """A mixed set of velocity-stepping cases: (model, q, v) per kind."""
    cases = {}
    ls, q, v = cube_states(rng, n)
    cases["cube"] = (Model.from_mechanisms([ground_cube(1.0, l) for l in ls]), np.concatenate(q),
                     np.concatenate(v))
    rs = rng.uniform(0.2, 1.0, n)
    qs = np.concatenate([[0, 0, 0, 1, 0, 0, r - rng.uniform(0, 2e-3)] for r in rs])
    cases["sphere"] = (Model.from_mechanisms([sphere(1.0, r) for r in rs]), qs, rng.normal(0, 0.5, 6 * n))
    Mq, q0, v0, _ = Model.from_config(3, n, seed=5)
    qo, vo, _ = Mq.offsets()
    for i in range(n):  # lower each torso until a foot touches the ground
        qi = q0[qo[i]:qo[i + 1]]
        while oracle.vs_step(Mq, i, qi, v0[vo[i]:vo[i + 1]], 1e-3)["nc"] == 0:
            qi[6] -= 0.005
        qi[6] -= 0.002
    cases["quadruped"] = (Mq, q0, v0)
    Mg = Model.from_mechanisms([builders.build_gripper()] * n)
    qg, vg = builders.gripper_states(rng, n)
    cases["gripper"] = (Mg, qg.ravel(), vg.ravel())
    Mp = Model.from_mechanisms([builders.build_pusher()] * n)
    qp, vp = builders.pusher_states(rng, n)
    cases["pusher"] = (Mp, qp.ravel(), vp.ravel())
    return cases


def test_oracle_program_certificates(built):
    """Every program of one step: λ in K = {‖λ_t‖ ≤ μ λ_n}, the contact-frame
    velocities u = J v' in the dual cone {u_n ≥ μ ‖u_t‖}, λ_i·u_i ≈ 0, and
    v' = v_free + M⁻¹Jᵀλ."""
    rng = np.random.default_rng(2)
    seen = 0
    for kind, (M, q, v) in vs_models(rng).items():
        qo, vo, _ = M.offsets()
        for i in range(M.n):
            d = oracle.vs_step(M, i, q[qo[i]:qo[i + 1]], v[vo[i]:vo[i + 1]], 1e-3)
            assert d["status"] == 0, (kind, i)
            if d["nc"] == 0:
                continue
            seen += 1
            lam = d["lam"].reshape(-1, 3)
            u = (d["J"] @ d["vnext"]).reshape(-1, 3)
            ls = max(np.abs(lam).max(), 1.0)
            us = max(np.abs(d["J"] @ d["vfree"]).max(), 1.0)
            assert np.all(np.linalg.norm(lam[:, 1:], axis=1) <= MU * lam[:, 0] + 1e-9 * ls), (kind, i)
            assert np.all(MU * np.linalg.norm(u[:, 1:], axis=1) <= u[:, 0] + 1e-7 * us), (kind, i)
            assert np.all(np.abs(np.sum(lam * u, axis=1)) <= 1e-7 * ls * us), (kind, i)
            back = d["vfree"] + np.linalg.solve(d["M"], d["J"].T @ d["lam"])
            np.testing.assert_allclose(back, d["vnext"], rtol=0, atol=1e-9 * max(1, np.abs(d["vnext"]).max()))
    assert seen > 60


def test_oracle_program_against_slsqp(built):
    """A different method cannot do better: scipy's SLSQP, started from a
    feasible point and from the interior-point solution, never finds a lower
    objective than the oracle's (the program is convex, so a solution no
    feasible descent improves is the optimum)."""
    from scipy.optimize import minimize

    rng = np.random.default_rng(4)
    ls, q, v = cube_states(rng, 16)
    M = Model.from_mechanisms([ground_cube(1.0, l) for l in ls])
    checked = 0
    for i in range(M.n):
        d = oracle.vs_step(M, i, q[i], v[i], 1e-3)
        k = d["nc"]
        if k == 0:
            continue
        J, Mm, vf = d["J"], d["M"], d["vfree"]
        G = J @ np.linalg.solve(Mm, J.T)
        g = J @ vf
        f = lambda x: 0.5 * x @ G @ x + g @ x
        cons = []
        for c in range(k):
            cons.append({"type": "ineq", "fun": lambda x, c=c: MU * x[3 * c] - np.hypot(x[3 * c + 1], x[3 * c + 2])})
        obj = f(d["lam"])
        for x0 in (np.tile([1e-3, 0.0, 0.0], k), d["lam"]):
            res = minimize(f, x0, jac=lambda x: G @ x + g, constraints=cons, method="SLSQP",
                           options={"ftol": 1e-15, "maxiter": 1000})
            feas = min(con["fun"](res.x) for con in cons)
            if feas >= -1e-9:
                assert obj <= res.fun + 1e-10 * max(1.0, abs(obj)), (i, obj, res.fun)
        checked += 1
    assert checked >= 8


# ---------------------------------------------------------------------------
# GPU


@pytest.mark.gpu
@pytest.mark.parametrize("kind", ["cube", "sphere", "quadruped", "gripper", "pusher"])
def test_gpu_one_step(ctx, kind):
    rng = np.random.default_rng(7)
    M, q, v = vs_models(rng)[kind]
    qo, vo, _ = M.offsets()
    B = Batch(M, ctx)
    B.update(q, v)
    B.step(1e-3, None, VS)
    qg, vg = B.state()
    assert np.all(B.status() == 0)
    contacts = 0
    for i in range(M.n):
        d = oracle.vs_step(M, i, q[qo[i]:qo[i + 1]], v[vo[i]:vo[i + 1]], 1e-3)
        assert d["status"] == 0
        contacts += d["nc"]
        sc = max(1.0, np.abs(d["v"]).max())
        assert np.max(np.abs(vg[vo[i]:vo[i + 1]] - d["v"])) <= 1e-6 * sc, (kind, i)
        assert np.max(np.abs(qg[qo[i]:qo[i + 1]] - d["q"])) <= 1e-8 * max(1.0, np.abs(d["q"]).max()), (kind, i)
    assert contacts > 0


@pytest.mark.gpu
def test_gpu_reference_scenarios(ctx):
    """The reference's shoot-box and sphere-roll tests run on the GPU."""
    s, q0, v0, n = shoot_box()
    B = Batch(Model.from_mechanisms([s]), ctx)
    B.update(q0, v0)
    dt = 1.0 / 600.0
    B.simulate_steps(int(2.0 / dt), dt, VS)
    q, v = B.state()
    assert B.status()[0] == 0
    assert abs(np.dot(q[4:7], n) - 0.5) <= 1e-2 and abs(q[5]) <= 1e-5 and np.all(np.abs(v) <= 1e-5)
    r = 0.5
    B = Batch(Model.from_mechanisms([sphere(1.0, r)]), ctx)
    B.update(np.array([0, 0, 0, 1, 0, 0, r]), np.zeros(6))
    B.simulate_steps(2000, 1e-3, VS, tau=np.array([0, 0.1, 0, 0, 0, 0]))
    q, _ = B.state()
    roll, pitch, yaw = euler_xyz(*q[:4])
    assert abs(roll) <= 1e-12 and abs(yaw) <= 1e-12 and abs(q[5]) <= 1e-12
    assert abs(q[6] - r) <= 1e-5 and abs(r * pitch - q[4]) <= 1e-4


@pytest.mark.gpu
def test_gpu_trajectories(ctx):
    """200 steps of falling / sliding cubes and quadrupeds against the oracle."""
    rng = np.random.default_rng(9)
    for kind in ("cube", "quadruped"):
        M, q, v = vs_models(rng, 16)[kind]
        qo, vo, _ = M.offsets()
        B = Batch(M, ctx)
        B.update(q, v)
        B.simulate_steps(200, 1e-3, VS)
        qg, vg = B.state()
        assert np.all(B.status() == 0)
        for i in range(M.n):
            qr, vr = q[qo[i]:qo[i + 1]].copy(), v[vo[i]:vo[i + 1]].copy()
            for _ in range(200):
                qr, vr, st = oracle.step(M, i, qr, vr, 1e-3, None, VS)
                assert st == 0
            assert np.max(np.abs(vg[vo[i]:vo[i + 1]] - vr)) <= 1e-5 * max(1.0, np.abs(vr).max()), (kind, i)
            assert np.max(np.abs(qg[qo[i]:qo[i + 1]] - qr)) <= 1e-6 * max(1.0, np.abs(qr).max()), (kind, i)


@pytest.mark.gpu
def test_gpu_velocity_stepping_arguments(ctx):
    B = Batch(Model.from_mechanisms([kats.cube(1.0, 0.5)]), ctx)
    with pytest.raises(gpb.GpbError):
        B.step(1e-3, None, VS, gpb.MIXED)
    # a cube with 8 corners against 3 half-spaces: 24 potential contacts > 16
    s = kats.cube(1.0, 0.5)
    for nrm in ((0, 0, 1), (1, 0, 0), (0, 1, 0)):
        s.add_halfspace(HalfSpace.new(nrm, -5.0))
    B = Batch(Model.from_mechanisms([s]), ctx)
    with pytest.raises(gpb.GpbError):
        B.step(1e-3, None, VS)
