"""Body-parallel mapping of serial chains (gpb_batch_set_mapping): 2–32 lanes of
a warp step one instance, the sweeps as warp-shuffle scans, the mass matrix and
its Cholesky factor in shared memory; FP64 (also for GPB_MIXED requests).

Bounds, against the oracle (the reference's algorithm with a Cholesky solve):
  * one step: q, v within 1e-10 · max(|x|, 1), as the one-lane mapping;
  * 200-step trajectories: within 1e-8 · max(|x|, 1);
  * recorded history rows: the same 1e-8.
The scans sum in another order than the one-lane sweeps, so the two mappings
agree to rounding (checked at 1e-10 after one step), not bit for bit.
"""

import math

import numpy as np
import pytest

import gpb
import oracle
from gpb import Batch, HalfSpace, Model

pytestmark = pytest.mark.gpu


def rel_err(a, b):
    a, b = np.asarray(a), np.asarray(b)
    if b.size == 0:
        return 0.0
    return np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1.0)


def random_chains(rng, n, nb_lo, nb_hi, contacts=False):
    """n serial chains of nb_lo..nb_hi bodies: revolute joints about general
    axes with rotated, offset joint frames, revolute joints about ±x/±y/±z,
    prismatic joints (half of them sprung), fixed joints, armature on some
    revolute joints (which the step ignores: only Articulated::free_velocity
    puts it on the mass matrix, src/hybrid/articulated/mod.rs:244-247),
    inertias with off-diagonal moments and offset centres of mass; with
    `contacts`, point and sphere contacts on some bodies against one
    or two half-spaces, under either contact law."""
    from gpb.model import (WORLD_FRAME, ContactPoint, FixedJoint, MechanismState, PrismaticJoint,
                           RevoluteJoint, RigidBody, SpatialInertia, Transform3D)
    mechs = []
    for _ in range(n):
        joints, bodies = [], []
        for k in range(int(rng.integers(nb_lo, nb_hi + 1))):
            frame, parent = f"b{k}", WORLD_FRAME if k == 0 else f"b{k - 1}"
            kind = rng.choice(["general", "principal", "prismatic", "fixed"], p=[0.35, 0.35, 0.15, 0.15])
            if k == 0 and kind == "fixed":
                kind = "principal"
            if kind == "principal":
                axis = np.zeros(3)
                axis[rng.integers(0, 3)] = rng.choice([-1.0, 1.0])
                t = np.zeros(3)
                t[rng.integers(0, 3)] = rng.uniform(-0.6, 0.6)
                tr = Transform3D(frame, parent, translation=tuple(t))
            else:
                quat = rng.normal(size=4)
                quat /= np.linalg.norm(quat)
                axis = rng.normal(size=3)
                axis /= np.linalg.norm(axis)
                tr = Transform3D(frame, parent, rotation=tuple(quat), translation=tuple(rng.uniform(-0.6, 0.6, 3)))
            if kind == "fixed":
                j = FixedJoint(tr)
            elif kind == "prismatic":
                spring = (rng.uniform(5.0, 200.0), rng.uniform(-0.5, 0.5)) if rng.uniform() < 0.5 else None
                j = PrismaticJoint(tr, axis, spring=spring)
            else:
                j = RevoluteJoint(tr, axis)
                if rng.uniform() < 0.3:
                    j = j.with_armature(rng.uniform(0.01, 0.2))
            joints.append(j)
            m = rng.uniform(0.3, 2.0)
            r = rng.uniform(-0.3, 0.3, 3)
            a = rng.normal(size=(3, 3))
            jc = 0.05 * a @ a.T + 0.01 * np.eye(3)
            b = RigidBody(SpatialInertia(frame, jc + m * (r @ r * np.eye(3) - np.outer(r, r)), m * r, m))
            if contacts and rng.uniform() < 0.4:
                b.add_contact_point(ContactPoint(frame, tuple(rng.uniform(-0.3, 0.3, 3)), k=rng.uniform(1e3, 5e4),
                                                 radius=rng.choice([0.0, 0.05]), damping=rng.uniform(0.0, 50.0)))
            bodies.append(b)
        mech = MechanismState(joints, bodies)
        if contacts:
            mech.add_halfspace(HalfSpace.new((0, 0, 1), -0.4, 0.9, 0.5))
            if rng.uniform() < 0.5:
                nrm = rng.normal(size=3)
                mech.add_halfspace(HalfSpace.new(tuple(nrm / np.linalg.norm(nrm)), -0.8, 0.5, 0.8))
            mech.contact_model = int(rng.integers(0, 2))
        mechs.append(mech)
    return Model.from_mechanisms(mechs)


def lane_counts(nb_max):
    """The lane counts the mapping accepts: one or two bodies per lane of a
    warp, or a 4-warp block per instance (128)."""
    return [g for g in (2, 4, 8, 16, 32) if 2 * g >= nb_max] + [128]


def state(rng, M, qscale=math.pi):
    qo, vo, _ = M.offsets()
    return rng.uniform(-qscale, qscale, qo[-1]), rng.normal(size=vo[-1])


@pytest.mark.parametrize("nb_lo,nb_hi", [(1, 4), (5, 16), (17, 32), (33, 64)])
@pytest.mark.parametrize("integrator", [gpb.SEMI_IMPLICIT_EULER, gpb.RUNGE_KUTTA_2, gpb.RUNGE_KUTTA_4])
def test_one_step_against_oracle(ctx, nb_lo, nb_hi, integrator):
    """One step of random chains at every accepted lane count (1e-10), and the
    one-lane mapping of the same batch against it (1e-10)."""
    rng = np.random.default_rng(100 * nb_lo + integrator)
    n = 80  # three packs, the last one partial
    M = random_chains(rng, n, nb_lo, nb_hi, contacts=integrator == gpb.SEMI_IMPLICIT_EULER)
    qo, vo, _ = M.offsets()
    q0, v0 = state(rng, M)
    tau = rng.normal(size=vo[-1])
    dt = 1e-3
    ref = [oracle.step(M, i, q0[qo[i]:qo[i + 1]], v0[vo[i]:vo[i + 1]], dt, tau[vo[i]:vo[i + 1]], integrator,
                       solver=oracle.CHOLESKY) for i in range(n)]
    assert all(r[2] == 0 for r in ref)
    one = Batch(M, ctx)
    one.update(q0, v0)
    one.step(dt, tau, integrator)
    q1, v1 = one.state()
    one.close()
    for i in range(n):  # the one-lane mapping too (armature on revolute joints acts in free_velocity only)
        assert rel_err(q1[qo[i]:qo[i + 1]], ref[i][0]) < 1e-10, i
        assert rel_err(v1[vo[i]:vo[i + 1]], ref[i][1]) < 1e-10, i
    nb_max = int(np.max(np.diff(M.joint_offset)))
    for g in lane_counts(nb_max):
        B = Batch(M, ctx)
        B.set_mapping(g)
        B.update(q0, v0)
        B.step(dt, tau, integrator)
        q, v = B.state()
        assert np.all(B.status() == 0), g
        B.close()
        for i in range(n):
            assert rel_err(q[qo[i]:qo[i + 1]], ref[i][0]) < 1e-10, (g, i)
            assert rel_err(v[vo[i]:vo[i + 1]], ref[i][1]) < 1e-10, (g, i)
        assert rel_err(q, q1) < 1e-10 and rel_err(v, v1) < 1e-10, g


@pytest.mark.parametrize("control,lanes", [("host", 32), ("open_loop", 32), ("pd", 32), ("open_loop", 128)])
def test_trajectory_200_steps(ctx, control, lanes):
    """200 steps of C1 chains (2–48 DOF) with each control law, one warp per
    instance (two bodies per lane where needed) or a block per instance: final
    state and the recorded history against the oracle (1e-8)."""
    n = 64
    M, q0, v0, aux = Model.from_config(1, n, seed=31)
    qo, vo, _ = M.offsets()
    dt = 5e-4
    kw = dict(seed=77, resample_every=10, sigma=1.0, kp=50.0, kd=2.0)
    ctl = aux if control == "pd" else None
    B = Batch(M, ctx)
    B.set_mapping(lanes)
    B.update(q0, v0)
    hist = B.simulate_steps(200, dt, gpb.SEMI_IMPLICIT_EULER, gpb.FP64, control, tau=ctl, record_every=50, **kw)
    q, v = B.state()
    assert np.all(B.status() == 0)
    assert np.all(B.steps_done() == 200)
    for i in range(n):
        c = None if ctl is None else ctl[vo[i]:vo[i + 1]]
        qr, vr, st, hr = oracle.simulate(M, i, q0[qo[i]:qo[i + 1]], v0[vo[i]:vo[i + 1]], dt, 200, 0,
                                         oracle.CHOLESKY, control, c, record_every=50, **kw)
        assert st == 0
        assert rel_err(q[qo[i]:qo[i + 1]], qr) < 1e-8, i
        assert rel_err(v[vo[i]:vo[i + 1]], vr) < 1e-8, i
        nq = qo[i + 1] - qo[i]
        for r in range(4):
            assert rel_err(hist[r, qo[i]:qo[i + 1]], hr[r, :nq]) < 1e-8, (i, r)
            assert rel_err(hist[r, B.nq + vo[i]:B.nq + vo[i + 1]], hr[r, nq:]) < 1e-8, (i, r)
    B.close()


def test_acrobots_sixteen_per_warp(ctx):
    """C0 acrobots with two lanes per instance (sixteen instances per warp):
    1,000 steps against the oracle (1e-8), and the split horizon 2 × 500
    equal to one call of 1,000 (the open-loop draws are keyed by the step)."""
    n = 96
    M, q0, v0, _ = Model.from_config(0, n, seed=5)
    qo, vo, _ = M.offsets()
    kw = dict(seed=9, resample_every=10, sigma=0.5)
    A = Batch(M, ctx)
    A.set_mapping(2)
    A.update(q0, v0)
    A.simulate_steps(1000, 1e-3, gpb.SEMI_IMPLICIT_EULER, gpb.FP64, "open_loop", **kw)
    qa, va = A.state()
    for i in range(0, n, 5):
        qr, vr, st, _ = oracle.simulate(M, i, q0[qo[i]:qo[i + 1]], v0[vo[i]:vo[i + 1]], 1e-3, 1000, 0,
                                        oracle.CHOLESKY, "open_loop", None, **kw)
        assert st == 0 and rel_err(qa[qo[i]:qo[i + 1]], qr) < 1e-8 and rel_err(va[vo[i]:vo[i + 1]], vr) < 1e-8, i
    B = Batch(M, ctx)
    B.set_mapping(2)
    B.update(q0, v0)
    B.simulate_steps(500, 1e-3, gpb.SEMI_IMPLICIT_EULER, gpb.FP64, "open_loop", **kw)
    B.simulate_steps(500, 1e-3, gpb.SEMI_IMPLICIT_EULER, gpb.FP64, "open_loop", step0=500, **kw)
    np.testing.assert_array_equal(B.q, A.q)
    np.testing.assert_array_equal(B.v, A.v)
    A.close()
    B.close()


def test_failures_are_flagged_and_frozen(ctx):
    """A non-finite state sets GPB_ST_NONFINITE, negative inertias
    GPB_ST_CHOL_FAIL; those instances stop where they were and the others of
    their warp run on — in both mappings."""
    M, q0, v0, _ = Model.from_config(1, 48, seed=2)
    qo, _, _ = M.offsets()
    q0 = q0.copy()
    q0[qo[5]] = np.nan
    jo = M.joint_offset
    M.body_inertia[10 * jo[9]:10 * jo[10]] *= -1.0  # instance 9: every inertia negative
    for g in (1, 16, 32, 128):
        if g > 1 and 2 * g < int(np.max(np.diff(jo))):
            continue
        B = Batch(M, ctx)
        B.set_mapping(g)
        B.update(q0, v0)
        before = B.q.copy()
        B.simulate_steps(20, 5e-4)
        st = B.status()
        assert st[5] & 1 and st[9] & 2, (g, st[5], st[9])
        assert np.sum(st != 0) == 2
        done = B.steps_done()
        assert done[5] == 0 and done[9] == 0 and np.all(np.delete(done, [5, 9]) == 20)
        np.testing.assert_array_equal(B.q[qo[9]:qo[10]], before[qo[9]:qo[10]])
        B.close()


def test_mapping_rules(ctx):
    """Lane counts: 1 or a power of two in [2, 32] with at most two bodies per
    lane; only chain batches.  GPB_MIXED_REFINED keeps one lane per instance
    (bit-identical to a batch that never set the mapping); under the
    articulated-body setting the mapping still factors H, in agreement with the
    one-lane articulated-body route to rounding."""
    M, q0, v0, _ = Model.from_config(1, 40, seed=6)  # up to 48 bodies: only 32 lanes give ≤ 2 per lane
    nb_max = int(np.max(np.diff(M.joint_offset)))
    B = Batch(M, ctx)
    for bad in (0, 3, 64, 256):
        with pytest.raises(gpb.GpbError):
            B.set_mapping(bad)
    if nb_max > 32:
        with pytest.raises(gpb.GpbError):
            B.set_mapping(16)
    B.set_mapping(32)
    B.update(q0, v0)
    B.simulate_steps(20, 5e-4, gpb.SEMI_IMPLICIT_EULER, gpb.MIXED_REFINED)
    R = Batch(M, ctx)
    R.update(q0, v0)
    R.simulate_steps(20, 5e-4, gpb.SEMI_IMPLICIT_EULER, gpb.MIXED_REFINED)
    np.testing.assert_array_equal(B.q, R.q)
    B.set_algorithm(gpb.ALGO_ABA)
    R.set_algorithm(gpb.ALGO_ABA)
    B.update(q0, v0)
    R.update(q0, v0)
    B.simulate_steps(20, 5e-4)
    R.simulate_steps(20, 5e-4)
    assert rel_err(B.q, R.q) < 1e-10 and rel_err(B.v, R.v) < 1e-10
    B.close()
    R.close()
    Q, _, _, _ = Model.from_config(3, 4, seed=1)  # quadrupeds: trees with a floating base
    C = Batch(Q, ctx)
    with pytest.raises(gpb.GpbError):
        C.set_mapping(16)
    C.set_mapping(1)
    C.close()


def test_mixed_requests_run_fp64(ctx):
    """A GPB_MIXED step on the body-parallel mapping is its FP64 computation
    (bit-identical to a GPB_FP64 step on it), under either algorithm setting."""
    M, q0, v0, _ = Model.from_config(1, 96, seed=13)
    for algo in (gpb.ALGO_CRBA, gpb.ALGO_ABA):
        out = []
        for prec in (gpb.FP64, gpb.MIXED):
            B = Batch(M, ctx)
            B.set_algorithm(algo)
            B.set_mapping(32)
            B.update(q0, v0)
            B.simulate_steps(50, 5e-4, gpb.SEMI_IMPLICIT_EULER, prec, "open_loop", seed=2)
            out.append(B.state())
            B.close()
        assert np.array_equal(out[0][0], out[1][0]) and np.array_equal(out[0][1], out[1][1]), algo


def test_autotune_chooses_among_mappings(ctx):
    """A small batch of long chains: the autotuner times the one-lane and the
    body-parallel shapes, keeps one, restores the state; the run after it
    matches the oracle (1e-8)."""
    n = 64
    M, q0, v0, _ = Model.from_config(1, n, seed=12)
    qo, vo, _ = M.offsets()
    B = Batch(M, ctx)
    B.update(q0, v0)
    w, c, lanes = B.autotune(5e-4, gpb.SEMI_IMPLICIT_EULER, gpb.FP64, trial_steps=5)
    assert lanes in (1, 32, 128) and (lanes > 1 or w in (4, 8, 12, 16))
    q1, v1 = B.state()
    assert np.array_equal(q1, q0) and np.array_equal(v1, v0)
    B.simulate_steps(100, 5e-4)
    q, v = B.state()
    for i in range(0, n, 7):
        qr, vr, st, _ = oracle.simulate(M, i, q0[qo[i]:qo[i + 1]], v0[vo[i]:vo[i + 1]], 5e-4, 100, 0,
                                        oracle.CHOLESKY)
        assert st == 0 and rel_err(q[qo[i]:qo[i + 1]], qr) < 1e-8 and rel_err(v[vo[i]:vo[i + 1]], vr) < 1e-8
    B.close()
