"""The oracle against gorilla-physics' own known answers (CPU).

Pins the CPU restatement before it is trusted as the checker: every
single-evaluation known answer of the reference's tests, the mass-matrix
structure tests and the trajectory-level physical outcomes (which run the
reference's integrators, including RK4's q0 + dt·v0 position update).
"""

import math

import numpy as np
import pytest

import gpb
import oracle
from gpb import HalfSpace, Model
from tests.golden import kats

G = 9.81


@pytest.mark.parametrize("case", kats.dynamics_cases(), ids=lambda c: c[0])
@pytest.mark.parametrize("solver", [oracle.LU, oracle.CHOLESKY], ids=["lu", "cholesky"])
def test_dynamics_known_answers(built, case, solver):
    name, mech, q, v, tau, expected, tol, source = case
    M = Model.from_mechanisms([mech])
    qdd, st = oracle.dynamics(M, 0, q, v, tau, solver=solver)
    assert st == 0
    np.testing.assert_allclose(qdd, expected, rtol=0, atol=tol, err_msg=source)


def test_exact_pendulum_answers_are_exact(built):
    # dynamics.rs:904-907, 937-940, 1029-1032 use assert_eq!
    m, l = 5.0, 7.0
    p = kats.pendulum(m, (0.0, m * l * l / 3, m * l * l / 3), (m * l / 2, 0, 0))
    qdd, _ = oracle.dynamics(Model.from_mechanisms([p]), 0, [0.0], [0.0], [0.0])
    assert qdd[0] == 3.0 * G / (2.0 * l)


def test_mass_matrix_structure(built):
    # mechanism.rs:711-786: 8x8 with non-zero coupling rows for both legs
    M = Model.from_mechanisms([kats.mass_matrix_mech()])
    H = oracle.mass_matrix(M, 0, [0, 0, 0, 1, 0, 0, 0, 0, 0])
    assert H.shape == (8, 8)
    assert np.any(H[6, :6] != 0) and H[6, 6] != 0
    assert np.any(H[7, :6] != 0) and H[7, 6] != 0 and H[7, 7] != 0
    np.testing.assert_array_equal(H, H.T)
    assert np.all(np.linalg.eigvalsh(H) > 0)


def test_supports_sparsity(built):
    # mechanism.rs:793-832: supports = {1..5}, {2,3}, {3}, {4,5}, {5}; the
    # mass matrix couples two joints only if one supports the other.
    M = Model.from_mechanisms([kats.supports_tree()])
    H = oracle.mass_matrix(M, 0, [0, 0, 0, 1, 0, 0, 0, 0.3, -0.2, 0.5, 0.1])
    # revolute dofs 6..9 = joints 2..5; 2-4, 2-5, 3-4, 3-5 are unrelated
    for a, b in [(6, 8), (6, 9), (7, 8), (7, 9)]:
        assert H[a, b] == 0 and H[b, a] == 0
    for a, b in [(6, 7), (8, 9)]:
        assert H[a, b] != 0


def test_simulate_horizontal_rod_sie(built):
    # simulate.rs:129-174: SIE, 10 s at 1 ms — top of swing π, energy ≈ 0
    m, l = 5.0, 7.0
    M = Model.from_mechanisms([kats.pendulum(m, (0, m * l * l / 3, m * l * l / 3), (m * l / 2, 0, 0))])
    K = gpb.simulate_steps(10.0, 0.001)
    q, v, st, h = oracle.simulate(M, 0, [0.0], [0.0], 0.001, K, integrator=0, record_every=1)
    assert abs(h[:, 0].max() - math.pi) < 1e-2
    E = m * G * l / 2 * (-math.sin(q[0])) + 0.5 * (m * l * l / 3) * v[0] ** 2
    assert abs(E) < 1e-1


def test_cart_rk4(built):
    # simulate.rs:177-214
    M = Model.from_mechanisms([kats.cart()])
    K = gpb.simulate_steps(10.0, 0.02)
    q, v, st, _ = oracle.simulate(M, 0, [2.0], [-1.0], 0.02, K, integrator=2)
    assert abs(q[0] - (2.0 - 10.0)) < 2e-2
    assert abs(v[0] + 1.0) < 1e-6


def test_cart_pole_rk4(built):
    # simulate.rs:218-272: steady pole angle under constant cart force
    M = Model.from_mechanisms([kats.cart_pole()])
    F, acc = 1.0, 1.0 / 8.0
    theta = math.atan2(acc, G)
    K = gpb.simulate_steps(20.0, 1e-2)
    q, v, st, _ = oracle.simulate(M, 0, [0.0, theta], [0.0, 0.0], 1e-2, K, integrator=2,
                                  ctl=[F, 0.0])
    assert abs(abs(v[0] - acc * 20.0)) < 1e-4
    assert abs(q[1] - theta) < 1e-5


def test_double_pendulum_energy_sie(built):
    # energy.rs:82-128: energy drift of SIE over 2 s stays below 0.1
    m, l = 1.0, 1.0
    M = Model.from_mechanisms([kats.double_pendulum(m, (m * l * l, m * l * l, 0), (0, 0, -m * l), (0, 0, -l))])

    def energy(q, v):  # state.kinetic_energy() + double_pendulum_potential_energy (energy.rs:9-17)
        ke, _ = oracle.energy(M, 0, q, v)
        return ke + m * G * (-l * math.cos(q[0]) - l * math.cos(q[0]) - l * math.cos(q[0] + q[1]))

    e0 = energy([1.0, 1.0], [0.1, 0.1])
    q, v, st, _ = oracle.simulate(M, 0, [1.0, 1.0], [0.1, 0.1], 1e-3, gpb.simulate_steps(2.0, 1e-3))
    assert abs(energy(q, v) - e0) < 1e-1


def test_pendulum_hit_ground(built):
    # contact.rs:371-405: rests at 30° on the z = −5 half-space
    m, l = 1.5, 10.0
    p = kats.pendulum(m, (0, m * l * l, m * l * l), (m * l, 0, 0))
    p.add_contact_point(gpb.ContactPoint("rod", (l, 0.0, 0.0)))
    p.add_halfspace(HalfSpace.new((0, 0, 1), -5.0))
    M = Model.from_mechanisms([p])
    q, v, st, _ = oracle.simulate(M, 0, [0.0], [0.0], 1e-2, gpb.simulate_steps(5.0, 1e-2), integrator=2)
    assert abs(q[0] - math.radians(30.0)) < 1e-3


def test_cube_fall_and_slide(built):
    # contact.rs:408-441 and 444-489
    c = kats.cube(3.0, 1.0)
    c.add_halfspace(HalfSpace.new((0, 0, 1), -10.0))
    q, v, st, _ = oracle.simulate(Model.from_mechanisms([c]), 0, [0, 0, 0, 1, 0, 0, 0], [1] * 6, 1e-3,
                                  gpb.simulate_steps(5.0, 1e-3), integrator=2)
    assert abs(q[6] - (-10.0 + 0.5)) < 1e-2
    c = kats.cube(3.0, 1.0)
    c.add_halfspace(HalfSpace.new((0, 0, 1), -0.5, 1.0, 0.5))
    q, v, st, _ = oracle.simulate(Model.from_mechanisms([c]), 0, [0, 0, 0, 1, 0, 0, 0],
                                  [0, 0, 0, 1, 0, 0], 1e-3, gpb.simulate_steps(2.0, 1e-3), integrator=2)
    acc = -G * 0.5
    ts = 1.0 / -acc
    assert abs(q[6]) < 1e-2
    assert np.linalg.norm(v[3:]) < 5e-3 and np.linalg.norm(v[:3]) < 1e-2
    assert abs(q[4] - (ts + acc * ts * ts / 2)) < 1e-2


def test_mass_hit_ground(built):
    # contact.rs:607-675: analytic landing point + Coulomb sliding distance
    s = kats.sphere_point()
    s.add_halfspace(HalfSpace.new((0, 0, 1), -0.3, 1.0, 0.5))
    q, v, st, _ = oracle.simulate(Model.from_mechanisms([s]), 0, [0, 0, 0, 1, 0, 0, 0],
                                  [0, 0, 0, 2.0, 0, 0], 1e-3, gpb.simulate_steps(2.0, 1e-3), integrator=2)
    th = math.sqrt(0.3 * 2 / G)
    vx = 2.0 - G * th * 0.5
    ts = vx / (G * 0.5)
    x = th * 2.0 + vx * ts - G * 0.5 * ts * ts / 2
    assert abs(q[6] + 0.3) < 1e-2
    assert np.linalg.norm(v[3:]) < 1e-2 and np.linalg.norm(v[:3]) < 1e-3
    assert abs(q[4] - x) < 1e-2


def test_ball_fall(built):
    # joint/floating.rs:133-168: ballistic flight with spin about x
    M = Model.from_mechanisms([kats.ball()])
    q0 = list(kats.quat_axis_angle((1, 0, 0), math.pi / 2)) + [0, 0, 1.0]
    q, v, st, _ = oracle.simulate(M, 0, q0, [1.0, 0, 0, 0, 1.0, 0], 0.01, gpb.simulate_steps(5.0, 0.01),
                                  integrator=2, ctl=[0.0] * 6)
    z_expect = 1.0 + 1.0 * 5.0 - 0.5 * G * 25.0
    assert abs(q[4]) < 1e-4 and abs(q[5]) < 1e-2 and abs(q[6] - z_expect) < 1.0
    angle = 2 * math.acos(min(1.0, abs(q[3])))
    exp = (math.pi / 2 + 5.0) % (2 * math.pi)
    exp = min(exp, 2 * math.pi - exp)
    assert abs(angle - exp) < 1e-2


def spring_midpoint(q):
    """x of A, x of B and their midpoint for the spring pair's q = (floating A, prismatic B)."""
    x, y, z, w = q[0:4]
    r00 = 1.0 - 2.0 * (y * y + z * z)  # x component of A's x axis in the world
    xa = q[4]
    xb = xa + r00 * q[7]
    return xa, xb, 0.5 * (xa + xb)


def test_spring_on_frictionless_ground(built):
    """src/dynamics.rs:1133-1188: a prismatic spring between two free spheres,
    RK4 for 1.1 s — the midpoint stays at l_init/2 (1e-5), A at x > 0, B at x < l_init."""
    l_init = 2.0
    M = Model.from_mechanisms([kats.spring_pair(l_rest=l_init / 3.0)])
    K = gpb.simulate_steps(1.1, 1e-3)
    q0 = np.array([0, 0, 0, 1, 0, 0, 0, l_init], float)
    q, v, st, _ = oracle.simulate(M, 0, q0, np.zeros(7), 1e-3, K, gpb.RUNGE_KUTTA_4)
    assert st == 0
    xa, xb, mid = spring_midpoint(q)
    assert abs(mid - l_init / 2.0) < 1e-5
    assert xa > 0.0 and xb < l_init
    assert abs(q[7] - l_init) > 0.1  # the spring did move the spheres
