"""GPU parity: the CUDA kernels (through the C ABI) against the oracle.

Tolerances
  * FP64 form, one dynamics evaluation: with e = ‖q̈_gpu − q̈_ref‖∞ / max(‖q̈_ref‖∞, 1),
    e ≤ max(1e-10, 5e-15·cond(M)) against both the oracle's Cholesky solve and the
    reference's LU solve.  Two FP64 evaluations that round differently differ by
    about cond(M)·ε, so 1e-10 holds for cond(M) ≤ 2e4 and the bound grows with
    cond(M) beyond that (long chains reach cond ≈ 1e6).
  * Contact forces: 1e-10 relative to max(|f|, 1).
  * One integrator step: q, v within 1e-12 · max(|x|, 1).
  * 200-step trajectories: within 1e-8 · max(|x|, 1) (chaotic chains amplify
    round-off; the bound holds over this horizon at these step sizes).
"""

import math
import sys

import numpy as np
import pytest

import gpb
import oracle
from gpb import Batch, HalfSpace, Model
from tests.golden import kats

pytestmark = pytest.mark.gpu
G = 9.81


@pytest.fixture(autouse=True, params=["crba", "aba"])
def algorithm(request, monkeypatch):
    """Every parity test runs with both routes to q̈: the reference's CRBA +
    solve and the articulated-body algorithm (same bounds)."""
    if request.param == "aba" and "refined" in request.node.name:
        pytest.skip("MIXED_REFINED always uses CRBA")
    algo = {"crba": gpb.ALGO_CRBA, "aba": gpb.ALGO_ABA}[request.param]

    class AlgoBatch(gpb.Batch):
        def __init__(self, *a, **k):
            super().__init__(*a, **k)
            self.set_algorithm(algo)

    monkeypatch.setattr(sys.modules[__name__], "Batch", AlgoBatch)
    return request.param


def rel_err(a, b):
    a, b = np.asarray(a), np.asarray(b)
    if b.size == 0:
        return 0.0
    return np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1.0)


def slices(M):
    qo, vo, co = M.offsets()
    return qo, vo, co


# ---------------------------------------------------------------------------
# single evaluations

def test_known_answers_fp64(ctx):
    cases = kats.dynamics_cases()
    mechs = [c[1] for c in cases]
    B = Batch(mechs, ctx)
    q = np.concatenate([np.asarray(c[2], float) for c in cases])
    v = np.concatenate([np.asarray(c[3], float) for c in cases])
    tau = np.concatenate([np.asarray(c[4], float) for c in cases])
    B.update(q, v)
    qdd = B.dynamics_continuous(tau)
    o = 0
    for name, mech, _, _, _, expected, tol, src in cases:
        n = len(expected)
        np.testing.assert_allclose(qdd[o:o + n], expected, rtol=0, atol=tol, err_msg=f"{name} {src}")
        o += n
    assert np.all(B.status() == 0)


@pytest.mark.parametrize("config,n,model", [(0, 256, 1), (1, 512, 1), (2, 256, 1), (2, 256, 0),
                                            (3, 96, 1), (3, 96, 0)])
def test_config_dynamics_fp64(ctx, config, n, model):
    M, q0, v0, aux = Model.from_config(config, n, seed=5, contact_model=model)
    qo, vo, co = slices(M)
    rng = np.random.default_rng(config)
    if config in (2, 3):
        # push some instances into the ground so contacts are active
        q0 = q0.copy()
        for i in range(n):
            q0[qo[i] + 6] = rng.uniform(-0.01, 0.5) if config == 2 else rng.uniform(0.38, 0.45)
    tau = rng.normal(size=v0.size)
    B = Batch(M, ctx)
    B.update(q0, v0)
    qdd, cf = B.dynamics_continuous(tau, contact_forces=True)
    worst = worst_cf = 0.0
    active = within = 0
    for i in range(n):
        qi, vi, ti = q0[qo[i]:qo[i + 1]], v0[vo[i]:vo[i + 1]], tau[vo[i]:vo[i + 1]]
        ref_c, st, cf_ref = oracle.dynamics(M, i, qi, vi, ti, solver=oracle.CHOLESKY, contact_forces=True)
        ref_l, _ = oracle.dynamics(M, i, qi, vi, ti, solver=oracle.LU)
        g = qdd[vo[i]:vo[i + 1]]
        cond = np.linalg.cond(oracle.mass_matrix(M, i, qi))
        bound = max(1e-10, 5e-15 * cond)
        e = max(rel_err(g, ref_c), rel_err(g, ref_l))
        worst = max(worst, e / bound)
        within += int(e <= 1e-10)
        gcf = cf[3 * co[i]:3 * co[i + 1]]
        worst_cf = max(worst_cf, rel_err(gcf, cf_ref))
        active += int(np.any(cf_ref != 0))
    assert worst <= 1.0, worst
    assert worst_cf <= 1e-10, worst_cf
    if config != 1:
        assert within == n  # short mechanisms: cond(M) small, 1e-10 everywhere
    if config in (2, 3):
        assert active > n // 4
    assert np.all(B.status() == 0)


@pytest.mark.parametrize("config,n,model", [(0, 1024, 1), (1, 16384, 1), (2, 4096, 1), (2, 4096, 0),
                                            (3, 2048, 1), (3, 2048, 0)])
def test_mixed_aba_error_bound(ctx, algorithm, config, n, model):
    """MIXED with the articulated-body algorithm (double-float articulated
    inertias and bias forces, FP32 kinematics): every instance's q̈ within 1e-5
    of FP64 (relative to max(|q̈|, 1))."""
    if algorithm != "aba":
        pytest.skip("the bound is a property of the ABA form of MIXED")
    M, q0, v0, _ = Model.from_config(config, n, seed=13, contact_model=model)
    qo, vo, _ = M.offsets()
    rng = np.random.default_rng(config + 3)
    if config in (2, 3):
        q0 = q0.copy()
        for i in range(n):
            q0[qo[i] + 6] = rng.uniform(0.0, 0.4) if config == 2 else rng.uniform(0.38, 0.45)
    tau = rng.normal(size=v0.size)
    B = Batch(M, ctx)
    B.update(q0, v0)
    a = B.dynamics_continuous(tau, precision=gpb.FP64)
    b = B.dynamics_continuous(tau, precision=gpb.MIXED)
    errs = np.array([rel_err(b[vo[i]:vo[i + 1]], a[vo[i]:vo[i + 1]]) for i in range(M.n)])
    assert errs.max() <= 1e-5, (errs.max(), int(np.argmax(errs)))


def _pack_kinds(M):
    """Contact / no-contact kinds of the lanes of every pack of 32, in the
    library's pack order (instances sorted by DOF, bodies and contacts, largest
    first; ties keep their order within a topology)."""
    qo, vo, co = M.offsets()
    nb = np.diff(M.joint_offset)
    nv, nc = np.diff(vo), np.diff(co)
    order = sorted(range(M.n), key=lambda i: (-nv[i], -nb[i], -nc[i]))
    return [{bool(nc[i] > 0) for i in order[k:k + 32]} for k in range(0, M.n, 32)]


@pytest.mark.parametrize("precision", [gpb.FP64, gpb.MIXED, gpb.MIXED_REFINED])
def test_mixed_contact_batches(ctx, algorithm, precision):
    """Quadrupeds (contacts) batched with serial chains (none), so that packs
    hold both kinds.  A lane reads and writes nothing of its neighbours: the
    quadrupeds' q̈ is bit-identical to the one they get in a batch of their own,
    and so is the chains' under CRBA.  Under ABA a pack of planar chains alone
    runs the articulated-body passes specialised for planar chains, a pack that
    also holds a quadruped the general ones: the chains then agree to round-off
    (FP64: 1e-9 relative to max(|q̈|, 1)) or to the mixed form's bound (2e-5:
    both within 1e-5 of FP64).  MIXED with the articulated-body algorithm stays
    within 1e-5 of FP64, MIXED_REFINED within 1e-6, and no status bit is set.
    A mixed pack once let the FP32 bias forces of its chain lanes overwrite the
    FP64 bias forces of its contact lanes."""
    if algorithm == "aba" and precision == gpb.MIXED_REFINED:
        pytest.skip("MIXED_REFINED always uses CRBA")
    M3, q3, v3, _ = Model.from_config(3, 75, seed=31)
    M1, q1, v1, _ = Model.from_config(1, 600, seed=32)
    qo3, _, _ = M3.offsets()
    rng = np.random.default_rng(31)
    q3 = q3.copy()
    for i in range(M3.n):  # feet in the ground
        q3[qo3[i] + 6] = rng.uniform(0.38, 0.45)
    M = Model.concat([M3, M1])
    q0, v0 = np.concatenate([q3, q1]), np.concatenate([v3, v1])
    tau = rng.normal(size=v0.size)
    assert sum(len(k) == 2 for k in _pack_kinds(M)) >= 2  # packs that straddle the kinds
    B = Batch(M, ctx)
    B.update(q0, v0)
    mix = B.dynamics_continuous(tau, precision=precision)
    st = B.status()
    ref = B.dynamics_continuous(tau, precision=gpb.FP64)
    n3 = int(v3.size)
    chain_tol = 0.0 if algorithm == "crba" else (2e-5 if precision == gpb.MIXED else 1e-9)
    for Mk, qk, vk, sl, tol in ((M3, q3, v3, slice(0, n3), 0.0), (M1, q1, v1, slice(n3, None), chain_tol)):
        A = Batch(Mk, ctx)
        A.update(qk, vk)
        alone = A.dynamics_continuous(tau[sl], precision=precision)
        if tol == 0.0:
            np.testing.assert_array_equal(mix[sl], alone)
        else:
            _, vk_off, _ = Mk.offsets()
            d = max(rel_err(mix[sl][vk_off[i]:vk_off[i + 1]], alone[vk_off[i]:vk_off[i + 1]]) for i in range(Mk.n))
            assert d <= tol, d
        A.close()
    # MIXED with CRBA is the FP32 mass-matrix form, limited by cond(H)·ε32: no bound
    bound = {gpb.FP64: 0.0, gpb.MIXED: 1e-5 if algorithm == "aba" else None, gpb.MIXED_REFINED: 1e-6}[precision]
    if bound is not None:
        _, vo, _ = M.offsets()
        errs = np.array([rel_err(mix[vo[i]:vo[i + 1]], ref[vo[i]:vo[i + 1]]) for i in range(M.n)])
        assert errs.max() <= bound, (errs.max(), int(np.argmax(errs)))
    assert np.all(st == 0)


def random_trees(rng, n):
    """n random trees of 3–9 bodies: revolute joints about general axes with
    rotated, offset joint frames, revolute joints about ±x/±y/±z with an offset
    along one axis, prismatic and fixed joints, random parents (branches),
    inertias with off-diagonal moments and offset centres of mass."""
    from gpb.model import (WORLD_FRAME, FixedJoint, MechanismState, PrismaticJoint, RevoluteJoint,
                           RigidBody, SpatialInertia, Transform3D)
    mechs = []
    for _ in range(n):
        joints, bodies = [], []
        for k in range(int(rng.integers(3, 10))):
            frame, parent = f"b{k}", WORLD_FRAME if k == 0 else f"b{int(rng.integers(0, k))}"
            kind = "general" if k == 0 else rng.choice(["general", "principal", "prismatic", "fixed"],
                                                        p=[0.4, 0.3, 0.2, 0.1])
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
            joints.append({"general": RevoluteJoint, "principal": RevoluteJoint,
                           "prismatic": PrismaticJoint}[kind](tr, axis) if kind != "fixed" else FixedJoint(tr))
            m = rng.uniform(0.3, 2.0)
            r = rng.uniform(-0.3, 0.3, 3)
            a = rng.normal(size=(3, 3))
            jc = 0.05 * a @ a.T + 0.01 * np.eye(3)
            bodies.append(RigidBody(SpatialInertia(frame, jc + m * (r @ r * np.eye(3) - np.outer(r, r)), m * r, m)))
        mechs.append(MechanismState(joints, bodies))
    return Model.from_mechanisms(mechs)


def test_general_trees(ctx, algorithm):
    """Random trees with every joint kind and transform the chain
    configurations do not have (general axes and joint rotations, offsets
    along several axes, prismatic and fixed joints, branches): FP64 against
    the oracle, and MIXED ABA (its general-rotation, general-shift, prismatic
    and fixed-joint double-float paths) against FP64."""
    rng = np.random.default_rng(44)
    M = random_trees(rng, 512)
    qo, vo, _ = M.offsets()
    q0 = rng.uniform(-math.pi, math.pi, qo[-1])
    v0 = rng.normal(size=vo[-1])
    tau = rng.normal(size=vo[-1])
    B = Batch(M, ctx)
    B.update(q0, v0)
    a = B.dynamics_continuous(tau, precision=gpb.FP64)
    for i in range(0, M.n, 8):
        ref, st = oracle.dynamics(M, i, q0[qo[i]:qo[i + 1]], v0[vo[i]:vo[i + 1]], tau[vo[i]:vo[i + 1]])
        assert st == 0
        assert rel_err(a[vo[i]:vo[i + 1]], ref) <= 1e-9, i
    if algorithm != "aba":
        return
    b = B.dynamics_continuous(tau, precision=gpb.MIXED)
    errs = np.array([rel_err(b[vo[i]:vo[i + 1]], a[vo[i]:vo[i + 1]]) for i in range(M.n)])
    assert errs.max() <= 1e-5, (errs.max(), int(np.argmax(errs)))
    assert np.all(B.status() == 0)


def test_spring_on_frictionless_ground_gpu(ctx):
    """src/dynamics.rs:1133-1188 through the GPU (RK4, 1.1 s): a prismatic spring
    between two free spheres keeps their midpoint at l_init/2 (1e-5); 64 copies
    with different initial extensions, each on the oracle's trajectory (1e-9)."""
    from tests.test_oracle_kats import spring_midpoint

    n = 64
    rng = np.random.default_rng(8)
    l0 = np.concatenate([[2.0], rng.uniform(0.5, 3.0, n - 1)])
    M = Model.from_mechanisms([kats.spring_pair(l_rest=2.0 / 3.0) for _ in range(n)])
    q0 = np.concatenate([[0, 0, 0, 1, 0, 0, 0, x] for x in l0])
    B = Batch(M, ctx)
    B.update(q0, np.zeros(7 * n))
    K = gpb.simulate_steps(1.1, 1e-3)
    B.simulate_steps(K, 1e-3, gpb.RUNGE_KUTTA_4)
    q, _ = B.state()
    assert np.all(B.status() == 0)
    xa, xb, mid = spring_midpoint(q[0:8])
    assert abs(mid - 1.0) < 1e-5 and xa > 0.0 and xb < 2.0
    for i in range(0, n, 9):
        qr, _, st, _ = oracle.simulate(M, i, q0[8 * i:8 * i + 8], np.zeros(7), 1e-3, K, gpb.RUNGE_KUTTA_4,
                                       oracle.CHOLESKY)
        assert st == 0 and rel_err(q[8 * i:8 * i + 8], qr) < 1e-9, i
        assert abs(spring_midpoint(q[8 * i:8 * i + 8])[2] - l0[i] / 2.0) < 1e-5


def test_sprung_prismatic_trees(ctx, algorithm):
    """Trees whose prismatic joints carry springs (src/dynamics.rs:298-315):
    FP64 q̈ against the oracle (1e-9), MIXED (ABA) against FP64 (1e-5)."""
    from gpb.model import (WORLD_FRAME, MechanismState, PrismaticJoint, RevoluteJoint, RigidBody,
                           SpatialInertia, Transform3D)

    rng = np.random.default_rng(12)
    mechs = []
    for _ in range(256):
        joints, bodies = [], []
        for k in range(int(rng.integers(2, 7))):
            frame, parent = f"b{k}", WORLD_FRAME if k == 0 else f"b{int(rng.integers(0, k))}"
            axis = rng.normal(size=3)
            axis /= np.linalg.norm(axis)
            tr = Transform3D(frame, parent, translation=tuple(rng.uniform(-0.5, 0.5, 3)))
            if k == 0 or rng.uniform() < 0.6:
                joints.append(PrismaticJoint(tr, axis, spring=(rng.uniform(5.0, 200.0), rng.uniform(-0.5, 0.5))))
            else:
                joints.append(RevoluteJoint(tr, axis))
            m = rng.uniform(0.3, 2.0)
            bodies.append(RigidBody(SpatialInertia(frame, np.diag(rng.uniform(0.01, 0.1, 3)), (0.0, 0.0, 0.0), m)))
        mechs.append(MechanismState(joints, bodies))
    M = Model.from_mechanisms(mechs)
    assert np.count_nonzero(M.joint_spring[0::2]) >= 256
    qo, vo, _ = M.offsets()
    q0 = rng.uniform(-1.0, 1.0, qo[-1])
    v0 = rng.normal(size=vo[-1])
    B = Batch(M, ctx)
    B.update(q0, v0)
    a = B.dynamics_continuous(None, precision=gpb.FP64)
    for i in range(M.n):
        ref, st = oracle.dynamics(M, i, q0[qo[i]:qo[i + 1]], v0[vo[i]:vo[i + 1]])
        assert st == 0 and rel_err(a[vo[i]:vo[i + 1]], ref) <= 1e-9, i
    # the spring term is present: without it the oracle's q̈ differs
    Mn = Model.from_mechanisms(mechs)
    Mn.joint_spring[:] = 0.0
    ref0, _ = oracle.dynamics(Mn, 0, q0[qo[0]:qo[1]], v0[vo[0]:vo[1]])
    assert rel_err(a[vo[0]:vo[1]], ref0) > 1e-3
    if algorithm == "aba":
        b = B.dynamics_continuous(None, precision=gpb.MIXED)
        errs = np.array([rel_err(b[vo[i]:vo[i + 1]], a[vo[i]:vo[i + 1]]) for i in range(M.n)])
        assert errs.max() <= 1e-5, errs.max()
    assert np.all(B.status() == 0)


def test_mixed_precision_error(ctx):
    """MIXED on C1 chains: finite, and the FP32 build error is what it is
    (reported by the benchmark; not the ≤1e-5 mode)."""
    M, q0, v0, _ = Model.from_config(1, 512, seed=9)
    B = Batch(M, ctx)
    B.update(q0, v0)
    a = B.dynamics_continuous(None, precision=gpb.FP64)
    b = B.dynamics_continuous(None, precision=gpb.MIXED)
    qo, vo, _ = M.offsets()
    errs = [rel_err(b[vo[i]:vo[i + 1]], a[vo[i]:vo[i + 1]]) for i in range(M.n)]
    assert np.all(np.isfinite(b))
    assert np.median(errs) < 1e-2, np.median(errs)


@pytest.mark.parametrize("config,n,model", [(0, 256, 1), (1, 512, 1), (2, 256, 1), (2, 128, 0),
                                            (3, 96, 1), (3, 96, 0)])
def test_refined_precision_error(ctx, config, n, model):
    """MIXED_REFINED: FP32 link-coordinate solve plus FP64-residual refinement
    brings every instance's q̈ within 1e-7 (relative to max(|q̈|, 1)) of the
    FP64 form."""
    M, q0, v0, _ = Model.from_config(config, n, seed=9, contact_model=model)
    qo, vo, co = M.offsets()
    rng = np.random.default_rng(config + 10)
    if config in (2, 3):
        q0 = q0.copy()
        for i in range(n):
            q0[qo[i] + 6] = rng.uniform(0.0, 0.4) if config == 2 else rng.uniform(0.38, 0.45)
    tau = rng.normal(size=v0.size)
    B = Batch(M, ctx)
    B.update(q0, v0)
    a, ca = B.dynamics_continuous(tau, precision=gpb.FP64, contact_forces=True)
    b, cb = B.dynamics_continuous(tau, precision=gpb.MIXED_REFINED, contact_forces=True)
    errs = [rel_err(b[vo[i]:vo[i + 1]], a[vo[i]:vo[i + 1]]) for i in range(M.n)]
    assert max(errs) < 1e-7, (max(errs), int(np.argmax(errs)))
    if M.contact_offset[-1]:
        assert rel_err(cb, ca) < 1e-9
    assert np.all(B.status() == 0)


def test_refined_trajectory(ctx):
    """200 open-loop steps of chains: MIXED_REFINED stays on the FP64 trajectory."""
    M, q0, v0, _ = Model.from_config(1, 128, seed=33)
    A = Batch(M, ctx)
    A.update(q0, v0)
    A.simulate_steps(200, 5e-4, 0, gpb.FP64, "open_loop", seed=5)
    B = Batch(M, ctx)
    B.update(q0, v0)
    B.simulate_steps(200, 5e-4, 0, gpb.MIXED_REFINED, "open_loop", seed=5)
    qo, vo, _ = M.offsets()
    qa, va = A.state()
    qb, vb = B.state()
    for i in range(M.n):
        assert rel_err(qb[qo[i]:qo[i + 1]], qa[qo[i]:qo[i + 1]]) < 1e-7
        assert rel_err(vb[vo[i]:vo[i + 1]], va[vo[i]:vo[i + 1]]) < 1e-6


# ---------------------------------------------------------------------------
# integrators

@pytest.mark.parametrize("integrator", [gpb.SEMI_IMPLICIT_EULER, gpb.RUNGE_KUTTA_2, gpb.RUNGE_KUTTA_4])
@pytest.mark.parametrize("config", [0, 1, 2, 3])
def test_one_step(ctx, integrator, config):
    n = 64
    M, q0, v0, _ = Model.from_config(config, n, seed=3)
    qo, vo, _ = slices(M)
    dt = {0: 1e-3, 1: 5e-4, 2: 1e-4, 3: 2e-4}[config]
    tau = np.random.default_rng(1).normal(size=v0.size)
    B = Batch(M, ctx)
    B.update(q0, v0)
    B.step(dt, tau, integrator)
    q, v = B.state()
    for i in range(n):
        qr, vr, st = oracle.step(M, i, q0[qo[i]:qo[i + 1]], v0[vo[i]:vo[i + 1]], dt,
                                 tau[vo[i]:vo[i + 1]], integrator, solver=oracle.CHOLESKY)
        assert rel_err(q[qo[i]:qo[i + 1]], qr) < 1e-10
        assert rel_err(v[vo[i]:vo[i + 1]], vr) < 1e-10


@pytest.mark.parametrize("config,control", [(0, "host"), (1, "open_loop"), (2, "host")])
def test_trajectory_200_steps(ctx, config, control):
    n = 64
    M, q0, v0, aux = Model.from_config(config, n, seed=21)
    qo, vo, _ = slices(M)
    dt = {0: 1e-3, 1: 5e-4, 2: 1e-4, 3: 2e-4}[config]
    kw = dict(seed=77, resample_every=10, sigma=1.0, kp=50.0, kd=2.0)
    B = Batch(M, ctx)
    B.update(q0, v0)
    ctl = aux if control == "pd" else None
    hist = B.simulate_steps(200, dt, gpb.SEMI_IMPLICIT_EULER, gpb.FP64, control, tau=ctl,
                            record_every=50, **kw)
    q, v = B.state()
    for i in range(n):
        c = None if ctl is None else ctl[vo[i]:vo[i + 1]]
        qr, vr, st, hr = oracle.simulate(M, i, q0[qo[i]:qo[i + 1]], v0[vo[i]:vo[i + 1]], dt, 200,
                                         0, oracle.CHOLESKY, control, c, record_every=50, **kw)
        assert rel_err(q[qo[i]:qo[i + 1]], qr) < 1e-8, i
        assert rel_err(v[vo[i]:vo[i + 1]], vr) < 1e-8, i
        nq = qo[i + 1] - qo[i]
        for r in range(4):
            assert rel_err(hist[r, qo[i]:qo[i + 1]], hr[r, :nq]) < 1e-8
    assert np.all(B.status() == 0)


@pytest.mark.parametrize("config,control,integ", [(3, "pd", 0), (1, "open_loop", 0), (2, "host", 2)])
def test_trajectory_segments(ctx, config, control, integ):
    """200 steps in 8 segments of 25: the oracle restarts from the GPU's state at
    every segment boundary and must land on the GPU's next recorded state.
    (The quadruped amplifies round-off ~10× per 25 steps — the reference's own
    LU and Cholesky variants drift apart by 1e-3 over 200 steps — so its
    trajectory is compared segment by segment.)"""
    n = 64
    M, q0, v0, aux = Model.from_config(config, n, seed=21)
    qo, vo, _ = slices(M)
    dt = {0: 1e-3, 1: 5e-4, 2: 1e-4, 3: 2e-4}[config]
    kw = dict(seed=77, resample_every=10, sigma=1.0, kp=50.0, kd=2.0)
    B = Batch(M, ctx)
    B.update(q0, v0)
    ctl = aux if control == "pd" else None
    hist = B.simulate_steps(200, dt, integ, gpb.FP64, control, tau=ctl, record_every=25, **kw)
    nqt = B.nq
    for i in range(n):
        c = None if ctl is None else ctl[vo[i]:vo[i + 1]]
        qs, vs = q0[qo[i]:qo[i + 1]], v0[vo[i]:vo[i + 1]]
        for r in range(8):
            qr, vr, st, _ = oracle.simulate(M, i, qs, vs, dt, 25, integ, oracle.CHOLESKY, control, c,
                                            step0=25 * r, **kw)
            qg = hist[r, qo[i]:qo[i + 1]]
            vg = hist[r, nqt + vo[i]:nqt + vo[i + 1]]
            assert rel_err(qg, qr) < 1e-9, (i, r)
            assert rel_err(vg, vr) < 1e-9, (i, r)
            qs, vs = qg, vg
    assert np.all(B.status() == 0)


def test_split_horizon_equals_one_call(ctx):
    """Open-loop draws are keyed by the global step: 2 × 100 steps == 200 steps."""
    M, q0, v0, _ = Model.from_config(1, 64, seed=4)
    A = Batch(M, ctx)
    A.update(q0, v0)
    A.simulate_steps(200, 5e-4, control="open_loop", seed=5)
    B = Batch(M, ctx)
    B.update(q0, v0)
    B.simulate_steps(100, 5e-4, control="open_loop", seed=5)
    B.simulate_steps(100, 5e-4, control="open_loop", seed=5, step0=100)
    np.testing.assert_array_equal(A.q, B.q)
    np.testing.assert_array_equal(A.v, B.v)


# ---------------------------------------------------------------------------
# reference trajectory tests through the GPU (physical outcomes)

def test_reference_trajectories_on_gpu(ctx):
    m, l = 5.0, 7.0
    rod = kats.pendulum(m, (0, m * l * l / 3, m * l * l / 3), (m * l / 2, 0, 0))
    B = Batch([rod], ctx)
    qs, vs = gpb.simulate(B, 10.0, 0.001, tau=[0.0])
    assert abs(qs[:, 0].max() - math.pi) < 1e-2  # simulate.rs:129-174
    E = m * G * l / 2 * (-math.sin(qs[-1, 0])) + 0.5 * (m * l * l / 3) * vs[-1, 0] ** 2
    assert abs(E) < 1e-1

    c = kats.cube(3.0, 1.0)
    c.add_halfspace(HalfSpace.new((0, 0, 1), -10.0))
    B = Batch([c], ctx)
    B.update([0, 0, 0, 1, 0, 0, 0], [1] * 6)
    B.simulate_steps(gpb.simulate_steps(5.0, 1e-3), 1e-3, gpb.RUNGE_KUTTA_4)
    assert abs(B.q[6] + 9.5) < 1e-2  # contact.rs:408-441

    s = kats.sphere_point()
    s.add_halfspace(HalfSpace.new((0, 0, 1), -0.3, 1.0, 0.5))
    B = Batch([s], ctx)
    B.update([0, 0, 0, 1, 0, 0, 0], [0, 0, 0, 2.0, 0, 0])
    B.simulate_steps(gpb.simulate_steps(2.0, 1e-3), 1e-3, gpb.RUNGE_KUTTA_4)
    th = math.sqrt(0.3 * 2 / G)
    vx = 2.0 - G * th * 0.5
    ts = vx / (G * 0.5)
    assert abs(B.q[4] - (th * 2.0 + vx * ts - G * 0.5 * ts * ts / 2)) < 1e-2  # contact.rs:607-675


# ---------------------------------------------------------------------------
# failure handling: per-instance status, never a fault

def test_nonfinite_state_is_flagged_and_frozen(ctx):
    M, q0, v0, _ = Model.from_config(0, 64, seed=1)
    B = Batch(M, ctx)
    q0 = q0.copy()
    q0[2 * 5] = np.nan
    B.update(q0, v0)
    B.simulate_steps(10, 1e-3)
    st = B.status()
    assert st[5] & 1 and np.all(np.delete(st, 5) == 0)
    q, _ = B.state()
    assert np.isnan(q[10])


def test_non_spd_mass_matrix_is_flagged(ctx):
    M, q0, v0, _ = Model.from_config(0, 32, seed=1)
    M.body_inertia[10 * 2 * 3:10 * 2 * 3 + 10] *= -1.0  # instance 3: negative inertia
    B = Batch(M, ctx)
    B.update(q0, v0)
    q_before = B.q.copy()
    B.simulate_steps(5, 1e-3)
    st = B.status()
    assert st[3] & 2
    np.testing.assert_array_equal(B.q[6:8], q_before[6:8])  # frozen
    assert np.sum(st != 0) == 1
