"""Mechanisms with cuboid colliders (src/contact.rs:191-242): every pair of
cuboid bodies goes through GJK/EPA and the collider contact law on top of the
point contacts against the ground.

CPU: model tables and the oracle's physics of the pair forces.
GPU (-m gpu): q̈ and trajectories of build_gripper / build_pusher and free-box
stacks against the oracle, through the C ABI, for both routes to q̈.

Tolerances (FP64 forms) as in test_gpu_parity: one evaluation within
max(1e-10, 5e-15·cond(M)) of the oracle (relative to max(|q̈|, 1)); one step
within 1e-11; 100-step trajectories within a bound scaled by the oracle's own
round-off sensitivity (test_gpu_trajectories).  MIXED: 1e-4 relative.
"""

import numpy as np
import pytest

import gpb
import oracle
from gpb import Batch, Model, builders
from tests.golden import cuboids as cb


def build(kind, n, rng, **kw):
    mech = {"gripper": cb.gripper, "pusher": cb.pusher, "stack": cb.box_stack}[kind]()
    states = {"gripper": builders.gripper_states, "pusher": builders.pusher_states,
              "stack": builders.box_stack_states}[kind]
    M = Model.from_mechanisms([mech] * n)
    q, v = states(rng, n, **kw)
    return M, q, v


def rel(a, b):
    return np.max(np.abs(np.asarray(a) - np.asarray(b))) / max(np.max(np.abs(b)), 1.0)


# ---------------------------------------------------------------------------
# CPU

def test_model_tables_carry_colliders(built):
    M = Model.from_mechanisms([cb.gripper(), cb.pusher()])
    assert M.body_cuboid.reshape(-1, 3).tolist() == [
        [0, 0, 0], [0.1, 0.4, 0.4], [0.1, 0.4, 0.4], [0.5, 0.5, 0.5],
        [0, 0, 0], [0.2, 0.2, 1.75], [0.5, 0.5, 0.5]]
    S = M.subset([1, 0])
    assert S.body_cuboid.reshape(-1, 3)[1].tolist() == [0.2, 0.2, 1.75]
    C = Model.concat([M, S])
    assert C.body_cuboid.size == 3 * 14


def test_oracle_pair_forces_push_apart(built):
    """Only the left jaw overlaps the cube: the cube is pushed along +x and the
    jaw back along its own axis (−x, so q̈_left > 0); the right jaw is free."""
    M = Model.from_mechanisms([cb.gripper(ground=False)])
    q = np.zeros(10)
    q[0], q[1], q[2] = 1.0, -0.2, 0.1
    q[3:7] = (0, 0, 0, 1)
    qdd, st = oracle.dynamics(M, 0, q, np.zeros(9))
    assert st == 0
    q_free = q.copy()
    q_free[1] = 0.1
    qdd0, _ = oracle.dynamics(M, 0, q_free, np.zeros(9))
    assert qdd[1] > 10.0 and abs(qdd0[1]) < 1e-9
    assert qdd[3 + 3] > 10.0                  # cube linear x (body frame = world, no rotation)
    np.testing.assert_allclose(qdd[2], qdd0[2], atol=1e-12)


def test_oracle_colliders_inert_when_apart(built):
    """Without overlap the colliders change nothing (same q̈ as the mechanism
    without colliders)."""
    rng = np.random.default_rng(5)
    M, q, v = build("gripper", 4, rng, closed=False)
    bare = cb.gripper()
    for b in bare.bodies:
        b.collider = None
    M0 = Model.from_mechanisms([bare] * 4)
    for i in range(4):
        a, sa = oracle.dynamics(M, i, q[i], v[i])
        b, sb = oracle.dynamics(M0, i, q[i], v[i])
        assert sa == sb == 0
        np.testing.assert_array_equal(a, b)


# ---------------------------------------------------------------------------
# GPU

@pytest.fixture(params=["crba", "aba"])
def algo(request):
    return {"crba": gpb.ALGO_CRBA, "aba": gpb.ALGO_ABA}[request.param]


@pytest.mark.gpu
@pytest.mark.parametrize("kind", ["gripper", "pusher", "stack"])
def test_gpu_dynamics_fp64(ctx, algo, kind):
    rng = np.random.default_rng({"gripper": 1, "pusher": 2, "stack": 3}[kind])
    n = 96
    M, q, v = build(kind, n, rng)
    B = Batch(M, ctx)
    B.set_algorithm(algo)
    B.update(q.ravel(), v.ravel())
    qdd = B.dynamics_continuous(None).reshape(n, -1)
    assert np.all(B.status() == 0)
    worst = 0.0
    for i in range(n):
        ref, st = oracle.dynamics(M, i, q[i], v[i], solver=oracle.LU)
        assert st == 0
        cond = np.linalg.cond(oracle.mass_matrix(M, i, q[i]))
        e = rel(qdd[i], ref)
        worst = max(worst, e)
        assert e <= max(1e-10, 5e-15 * cond), (kind, i, e, cond)
    # the pair forces are active in these states (not a vacuous comparison)
    M0 = Model.from_mechanisms([cb.box_stack() if kind == "stack" else
                                (cb.gripper() if kind == "gripper" else cb.pusher())])
    M0.body_cuboid[:] = 0.0
    d0, _ = oracle.dynamics(M0, 0, q[0], v[0])
    assert rel(d0, oracle.dynamics(M, 0, q[0], v[0])[0]) > 1e-3


@pytest.mark.gpu
@pytest.mark.parametrize("kind", ["gripper", "stack"])
def test_gpu_dynamics_mixed(ctx, algo, kind):
    rng = np.random.default_rng(11)
    n = 64
    M, q, v = build(kind, n, rng)
    B = Batch(M, ctx)
    B.set_algorithm(algo)
    B.update(q.ravel(), v.ravel())
    qdd = B.dynamics_continuous(None, precision=gpb.MIXED).reshape(n, -1)
    assert np.all(B.status() == 0)
    for i in range(n):
        ref, _ = oracle.dynamics(M, i, q[i], v[i], solver=oracle.CHOLESKY)
        assert rel(qdd[i], ref) <= 1e-4, (kind, i)


@pytest.mark.gpu
@pytest.mark.parametrize("integrator", [gpb.SEMI_IMPLICIT_EULER, gpb.RUNGE_KUTTA_4])
@pytest.mark.parametrize("kind", ["gripper", "pusher", "stack"])
def test_gpu_one_step(ctx, algo, kind, integrator):
    """One step from 96 contact states: q, v within 1e-11·max(|x|, 1)."""
    rng = np.random.default_rng(31)
    n = 96
    dt = {"gripper": 1e-5, "pusher": 1e-4, "stack": 2e-4}[kind]
    M, q, v = build(kind, n, rng)
    B = Batch(M, ctx)
    B.set_algorithm(algo)
    B.update(q.ravel(), v.ravel())
    B.step(dt, None, integrator)
    qg, vg = B.state()
    qo, vo, _ = M.offsets()
    assert np.all(B.status() == 0)
    for i in range(n):
        qr, vr, st = oracle.step(M, i, q[i], v[i], dt, None, integrator, oracle.CHOLESKY)
        assert st == 0
        assert rel(qg[qo[i]:qo[i + 1]], qr) <= 1e-11, (kind, i)
        assert rel(vg[vo[i]:vo[i + 1]], vr) <= 1e-11, (kind, i)


@pytest.mark.gpu
@pytest.mark.parametrize("integrator", [gpb.SEMI_IMPLICIT_EULER, gpb.RUNGE_KUTTA_4])
@pytest.mark.parametrize("kind", ["gripper", "pusher", "stack"])
def test_gpu_trajectories(ctx, algo, kind, integrator):
    """100 steps.  Contact trajectories amplify round-off: the squeezed 0.1 kg
    cube of the gripper makes the regularised friction very stiff (μπ/v_s with
    v_s = 1e-3; it runs at dt = 1e-5), and in box stacks a near-tie between two
    EPA faces can flip.  The oracle's own sensitivity d_i — how far its LU and
    Cholesky trajectories, which differ only in round-off, end apart — sets
    each instance's bound max(1e-7, 100·d_i); at least 3/4 of the instances must
    be smooth (d_i ≤ 1e-8).  Instances whose oracle trajectory stops (the
    reference's EPA panics on some face-face stacks) are left out."""
    rng = np.random.default_rng(21)
    n, K = 32, 100
    dt = {"gripper": 1e-5, "pusher": 1e-4, "stack": 2e-4}[kind]
    M, q, v = build(kind, n, rng)
    B = Batch(M, ctx)
    B.set_algorithm(algo)
    B.update(q.ravel(), v.ravel())
    B.simulate_steps(K, dt, integrator=integrator)
    qg, vg = B.state()
    stg = B.status()
    qo, vo, _ = M.offsets()
    smooth = 0
    for i in range(n):
        qr, vr, st, _ = oracle.simulate(M, i, q[i], v[i], dt, K, integrator, oracle.CHOLESKY)
        ql, vl, st2, _ = oracle.simulate(M, i, q[i], v[i], dt, K, integrator, oracle.LU)
        if st or st2:
            continue
        d = max(rel(ql, qr), rel(vl, vr))
        smooth += d <= 1e-8
        tol = max(1e-7, 100 * d)
        assert stg[i] == 0, (kind, i, stg[i])
        assert rel(qg[qo[i]:qo[i + 1]], qr) <= tol, (kind, i, d)
        assert rel(vg[vo[i]:vo[i + 1]], vr) <= tol, (kind, i, d)
    assert smooth >= 3 * n // 4


@pytest.mark.gpu
def test_gpu_mixed_batch_with_and_without_colliders(ctx, algo):
    """Lanes with and without cuboids share packs; each matches the oracle."""
    rng = np.random.default_rng(4)
    Mg, qg, vg = build("gripper", 40, rng)
    Mb = Model.from_config(1, 40, seed=9)
    M = Model.concat([Mg, Mb[0]])
    q = np.concatenate([qg.ravel(), Mb[1]])
    v = np.concatenate([vg.ravel(), Mb[2]])
    B = Batch(M, ctx)
    B.set_algorithm(algo)
    B.update(q, v)
    qdd = B.dynamics_continuous(None)
    qo, vo, _ = M.offsets()
    for i in range(M.n):
        ref, st = oracle.dynamics(M, i, q[qo[i]:qo[i + 1]], v[vo[i]:vo[i + 1]], solver=oracle.CHOLESKY)
        cond = np.linalg.cond(oracle.mass_matrix(M, i, q[qo[i]:qo[i + 1]])) if vo[i + 1] > vo[i] else 1.0
        assert rel(qdd[vo[i]:vo[i + 1]], ref) <= max(1e-10, 5e-15 * cond), i
