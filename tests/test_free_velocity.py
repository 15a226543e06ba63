"""Articulated::free_velocity (src/hybrid/articulated/mod.rs:124-199): v + dt·M⁻¹(τ − c)
with the revolute armature on M's diagonal and gravity switchable.

CPU: the oracle's restatement against closed forms.  GPU: gpb_free_velocity
(both algorithms, FP64 and the refined form) against the oracle."""

import numpy as np
import pytest

import gpb
import oracle
from gpb import Batch, Model, RevoluteJoint, PrismaticJoint, Transform3D


def with_armature(M, seed=0):
    rng = np.random.default_rng(seed)
    arm = np.where(M.joint_type == gpb.REVOLUTE, rng.uniform(0.0, 0.5, M.joint_type.size), 0.0)
    parts = {k: getattr(M, k) for k in Model.FIELDS}
    parts["joint_armature"] = arm
    return Model(**parts)


def test_oracle_armature_scales_single_joint(built):
    M, q0, v0, _ = Model.from_config(0, 4, seed=1)          # acrobots: 2 revolute joints
    one = M.subset([0])
    parts = {k: getattr(one, k) for k in Model.FIELDS}
    # a single pendulum: keep the first joint of the acrobot
    pend = Model(joint_offset=[0, 1], joint_type=parts["joint_type"][:1], joint_parent=[0],
                 joint_iso=parts["joint_iso"][:7], joint_axis=parts["joint_axis"][:3],
                 joint_spring=[0, 0], body_inertia=parts["body_inertia"][:10], contact_offset=[0, 0],
                 contact_body=[], contact_params=[], halfspace_offset=[0, 0], halfspace_params=[],
                 contact_model=[1])
    q, v, dt = np.array([0.7]), np.array([0.3]), 1e-3
    H0 = oracle.mass_matrix(pend, 0, q)[0, 0]
    base, st = oracle.free_velocity(pend, 0, q, v, None, dt, True)
    assert st == 0
    # no armature: exactly dynamics_continuous (Cholesky) for a contact-free mechanism
    qdd, _ = oracle.dynamics(pend, 0, q, v, None, solver=oracle.CHOLESKY)
    np.testing.assert_allclose(base, v + dt * qdd, rtol=1e-15, atol=0)
    parts = {k: getattr(pend, k) for k in Model.FIELDS}
    parts["joint_armature"] = [0.25]
    armed = Model(**parts)
    out, _ = oracle.free_velocity(armed, 0, q, v, None, dt, True)
    np.testing.assert_allclose((out - v) / dt, (base - v) / dt * H0 / (H0 + 0.25), rtol=1e-13)
    # gravity off, at rest: q̈ = τ / (H + armature)
    out, _ = oracle.free_velocity(armed, 0, q, np.zeros(1), np.array([2.0]), dt, False)
    np.testing.assert_allclose(out / dt, 2.0 / (H0 + 0.25), rtol=1e-13)


def test_armature_only_on_revolute_joints():
    j = PrismaticJoint(Transform3D("a", "world"), (1, 0, 0))
    with pytest.raises(AssertionError, match="revolute"):
        j.with_armature(0.1)
    r = RevoluteJoint(Transform3D("a", "world"), (0, 1, 0)).with_armature(0.1)
    assert r.armature == 0.1


@pytest.mark.gpu
@pytest.mark.parametrize("algorithm", [gpb.ALGO_CRBA, gpb.ALGO_ABA])
@pytest.mark.parametrize("gravity", [True, False])
def test_free_velocity_matches_oracle(ctx, algorithm, gravity):
    A, qa, va, _ = Model.from_config(1, 192, seed=21)   # chains n ~ U{2..48}
    C, qc, vc, _ = Model.from_config(0, 64, seed=22)    # acrobots
    M = with_armature(Model.concat([A, C]), seed=3)
    q0, v0 = np.concatenate([qa, qc]), np.concatenate([va, vc])
    rng = np.random.default_rng(5)
    tau = rng.normal(size=v0.size)
    dt = 1e-3
    B = Batch(M, ctx)
    B.set_algorithm(algorithm)
    B.set_gravity(9.81 if gravity else 0.0)
    B.update(q0, v0)
    vf = B.free_velocity(dt, tau)
    qo, vo, _ = M.offsets()
    worst = 0.0
    for i in range(M.n):
        s = slice(vo[i], vo[i + 1])
        ref, st = oracle.free_velocity(M, i, q0[qo[i]:qo[i + 1]], v0[s], tau[s], dt, gravity)
        assert st == 0
        a = (vf[s] - v0[s]) / dt
        b = (ref - v0[s]) / dt
        H = oracle.mass_matrix(M, i, q0[qo[i]:qo[i + 1]]) + np.diag(
            [M.joint_armature[M.joint_offset[i] + k] for k in range(vo[i + 1] - vo[i])])
        bound = max(1e-10, 5e-15 * np.linalg.cond(H))
        e = np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1.0)
        worst = max(worst, e / bound)
    assert worst <= 1.0, worst
    assert not B.status().any()
    B.close()


@pytest.mark.gpu
def test_armature_in_refined_and_mixed_forms(ctx):
    A, q0, v0, _ = Model.from_config(1, 256, seed=31)
    M = with_armature(A, seed=4)
    B = Batch(M, ctx)
    B.update(q0, v0)
    a = B.dynamics_continuous(None, precision=gpb.FP64)
    r = B.dynamics_continuous(None, precision=gpb.MIXED_REFINED)
    B.set_algorithm(gpb.ALGO_ABA)
    x = B.dynamics_continuous(None, precision=gpb.MIXED)
    f = B.dynamics_continuous(None, precision=gpb.FP64)
    vo = B.v_offset
    rel = lambda u, w: max(np.max(np.abs(u - w)) / max(np.max(np.abs(w)), 1.0) for _ in [0])
    er = [rel(r[vo[i]:vo[i + 1]], a[vo[i]:vo[i + 1]]) for i in range(M.n)]
    ex = np.array([rel(x[vo[i]:vo[i + 1]], a[vo[i]:vo[i + 1]]) for i in range(M.n)])
    ef = [rel(f[vo[i]:vo[i + 1]], a[vo[i]:vo[i + 1]]) for i in range(M.n)]
    assert max(er) < 1e-7 and max(ef) < 1e-8
    assert ex.max() <= 1e-5, ex.max()
    B.close()
