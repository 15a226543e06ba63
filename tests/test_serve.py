"""Serving engine (gpb_server_*): continuous batching of independent requests.

CPU tests cover the pool sizing (gpb_server_plan) and argument checks; the
GPU tests check that a request's final state is bit-identical whether it runs
alone or in a mix, equals the batch API's result, that admission respects the
pool capacity in FIFO order, and that a failing request is retired without
disturbing the others.
"""

import numpy as np
import pytest

import gpb
from gpb import Batch, Model
from gpb.serve import Server, SlotClass, plan

CONTROL = {0: "host", 1: "open_loop", 2: "host", 3: "pd"}
DT = {0: 1e-3, 1: 5e-4, 2: 1e-4, 3: 2e-4}


def test_plan_fixed_and_weighted_classes(built):
    fixed = SlotClass(2, 2, 2, packs=3)
    packs, nbytes = plan([fixed])
    assert packs.tolist() == [3] and nbytes[0] > 0
    w = [fixed, SlotClass(48, 48, 48, weight=3.0), SlotClass(13, 19, 18, 4, 1, weight=1.0)]
    budget = 1 << 30
    packs, nbytes = plan(w, hbm_budget_bytes=budget)
    assert packs[0] == 3
    rest = budget - 3 * nbytes[0]
    # each weighted class gets its share of what the fixed class left, in whole packs
    assert packs[1] == int(rest * 0.75 // nbytes[1]) and packs[2] == int(rest * 0.25 // nbytes[2])
    assert int(np.dot(packs, nbytes)) <= budget


def test_plan_rejects_bad_classes(built):
    with pytest.raises(gpb.GpbError, match="capacity"):
        plan([SlotClass(65, 1, 1, packs=1)])
    with pytest.raises(gpb.GpbError, match="exceed"):
        plan([SlotClass(48, 48, 48, packs=100)], hbm_budget_bytes=1 << 20)
    with pytest.raises(gpb.GpbError, match="budget"):
        plan([SlotClass(2, 2, 2, weight=1.0)])


def mix_model(seed=3, n=(40, 40, 5, 4)):
    parts = [Model.from_config(c, k, seed=seed + c) for c, k in zip(range(4), n)]
    M = Model.concat([p[0] for p in parts])
    q0 = np.concatenate([p[1] for p in parts])
    v0 = np.concatenate([p[2] for p in parts])
    aux = np.concatenate([p[3] if c == 3 else np.zeros_like(p[2]) for c, p in enumerate(parts)])
    cfg = np.concatenate([[c] * k for c, k in zip(range(4), n)])
    return M, q0, v0, aux, cfg


CLASSES = [SlotClass(2, 2, 2, packs=1), SlotClass(48, 48, 48, packs=1), SlotClass(1, 7, 6, 8, 1, packs=1),
           SlotClass(13, 19, 18, 4, 1, packs=1)]
# the same pool with the acrobot and chain classes for planar chains only
PLANAR_CLASSES = [SlotClass(2, 2, 2, packs=1, planar_only=True), SlotClass(48, 48, 48, packs=1, planar_only=True),
                  SlotClass(1, 7, 6, 8, 1, packs=1), SlotClass(13, 19, 18, 4, 1, packs=1)]


def submit_all(S, M, q0, v0, aux, cfg, horizons, idx):
    ids = {}
    for i in idx:
        c = int(cfg[i])
        rid = S.submit(M, int(i), 1, q0, v0, dt=DT[c], steps=int(horizons[i]), control=CONTROL[c],
                       tau=aux if c == 3 else None, seed=11 + i, kp=50.0, kd=2.0, keys=0)
        ids[int(i)] = int(rid[0])
    return ids


def run_server(ctx, M, q0, v0, aux, cfg, horizons, idx, precision, chunk=37, classes=CLASSES,
               algorithm=gpb.ALGO_CRBA):
    S = Server(ctx, classes, precision=precision, chunk_steps=chunk, algorithm=algorithm)
    ids = submit_all(S, M, q0, v0, aux, cfg, horizons, idx)
    S.drain(100000)
    out = {i: S.result(r) for i, r in ids.items()}
    S.close()
    return out


@pytest.mark.gpu
@pytest.mark.parametrize("precision,algorithm,classes", [
    (gpb.FP64, gpb.ALGO_CRBA, CLASSES), (gpb.MIXED, gpb.ALGO_CRBA, CLASSES),
    (gpb.MIXED_REFINED, gpb.ALGO_CRBA, CLASSES), (gpb.FP64, gpb.ALGO_ABA, CLASSES),
    (gpb.MIXED, gpb.ALGO_ABA, CLASSES), (gpb.FP64, gpb.ALGO_ABA, PLANAR_CLASSES),
    (gpb.MIXED, gpb.ALGO_ABA, PLANAR_CLASSES)], ids=lambda x: "planar" if x is PLANAR_CLASSES else
    ("general" if x is CLASSES else None))
def test_alone_equals_mix_bit_for_bit(ctx, precision, algorithm, classes):
    M, q0, v0, aux, cfg = mix_model()
    rng = np.random.default_rng(5)
    horizons = rng.integers(40, 300, size=M.n)
    mix = run_server(ctx, M, q0, v0, aux, cfg, horizons, range(M.n), precision, algorithm=algorithm,
                     classes=classes)
    # one pack (32 slots) per class: the 40 acrobots and 40 chains queue, and
    # later requests run in slots freed by others (of other sizes for the chains)
    for i in (0, 35, 42, 77, 82, 86, 88):
        alone = run_server(ctx, M, q0, v0, aux, cfg, horizons, [i], precision, chunk=53, algorithm=algorithm,
                           classes=classes)[i]
        qa, va, sa, da, _ = alone
        qm, vm, sm, dm, _ = mix[i]
        assert sa == sm and da == dm == horizons[i]
        assert np.array_equal(qa, qm) and np.array_equal(va, vm), i


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [gpb.FP64, gpb.MIXED])
def test_planar_classes_match_batch_api(ctx, precision):
    """Under the articulated-body algorithm a planar chain in a planar-only slot
    class runs the same specialised passes as a batch of planar chains: its
    result equals the batch of one bit for bit (acrobots and chains); the other
    mechanisms run the general passes in both."""
    M, q0, v0, aux, cfg = mix_model()
    qo, vo, _ = M.offsets()
    horizons = np.full(M.n, 120)
    res = run_server(ctx, M, q0, v0, aux, cfg, horizons, range(M.n), precision, classes=PLANAR_CLASSES,
                     algorithm=gpb.ALGO_ABA)
    for i in (1, 38, 45, 78, 81, 87):
        c = int(cfg[i])
        B = Batch(M.subset([i]), ctx)
        B.set_algorithm(gpb.ALGO_ABA)
        B.update(q0[qo[i]:qo[i + 1]], v0[vo[i]:vo[i + 1]])
        B.simulate_steps(120, DT[c], 0, precision, control=CONTROL[c],
                         tau=aux[vo[i]:vo[i + 1]] if c == 3 else None, seed=11 + i, resample_every=10,
                         sigma=1.0, kp=50.0, kd=2.0)
        qb, vb = B.state()
        B.close()
        qs, vs, st, done, _ = res[i]
        assert st == 0 and done == 120
        assert np.array_equal(qb, qs) and np.array_equal(vb, vs), i


@pytest.mark.gpu
def test_server_matches_batch_api(ctx):
    """A request through the server equals the same instance as a batch of one."""
    M, q0, v0, aux, cfg = mix_model()
    qo, vo, _ = M.offsets()
    horizons = np.full(M.n, 120)
    res = run_server(ctx, M, q0, v0, aux, cfg, horizons, range(M.n), gpb.FP64)
    for i in (1, 38, 45, 78, 81, 87):
        c = int(cfg[i])
        sub = M.subset([i])
        B = Batch(sub, ctx)
        B.update(q0[qo[i]:qo[i + 1]], v0[vo[i]:vo[i + 1]])
        B.simulate_steps(120, DT[c], 0, gpb.FP64, control=CONTROL[c],
                         tau=aux[vo[i]:vo[i + 1]] if c == 3 else None, seed=11 + i, resample_every=10,
                         sigma=1.0, kp=50.0, kd=2.0)
        qb, vb = B.state()
        B.close()
        qs, vs, st, done, _ = res[i]
        assert st == 0 and done == 120
        assert np.array_equal(qb, qs) and np.array_equal(vb, vs), i


@pytest.mark.gpu
def test_requests_keep_their_own_settings(ctx):
    """Requests in one pool with different step sizes, integrators and control
    laws each run with their own (the job's, not the launch's): every one
    equals the same instance as a batch of one with its settings."""
    M, q0, v0, _ = Model.from_config(0, 6, seed=7)
    qo, vo, _ = M.offsets()
    cases = [(1e-3, gpb.SEMI_IMPLICIT_EULER, "host"), (4e-4, gpb.RUNGE_KUTTA_4, "open_loop"),
             (2e-3, gpb.RUNGE_KUTTA_2, "pd"), (5e-4, gpb.SEMI_IMPLICIT_EULER, "open_loop"),
             (1e-3, gpb.RUNGE_KUTTA_4, "host"), (7e-4, gpb.RUNGE_KUTTA_2, "open_loop")]
    tau = np.full(vo[-1], 0.3)
    S = Server(ctx, [SlotClass(2, 2, 2, packs=1)], precision=gpb.FP64, chunk_steps=29)
    ids = [int(S.submit(M, i, 1, q0, v0, dt=dt, steps=90 + 7 * i, integrator=integ, control=ctl,
                        tau=tau if ctl == "pd" else None, seed=5 + i, kp=40.0, kd=1.5, keys=0)[0])
           for i, (dt, integ, ctl) in enumerate(cases)]
    S.drain(100000)
    out = [S.result(r) for r in ids]
    S.close()
    for i, (dt, integ, ctl) in enumerate(cases):
        B = Batch(M.subset([i]), ctx)
        B.update(q0[qo[i]:qo[i + 1]], v0[vo[i]:vo[i + 1]])
        B.simulate_steps(90 + 7 * i, dt, integ, gpb.FP64, control=ctl,
                         tau=tau[vo[i]:vo[i + 1]] if ctl == "pd" else None, seed=5 + i, kp=40.0, kd=1.5)
        qb, vb = B.state()
        B.close()
        qs, vs, st, done, _ = out[i]
        assert st == 0 and done == 90 + 7 * i, i
        assert np.array_equal(qb, qs) and np.array_equal(vb, vs), i


@pytest.mark.gpu
def test_admission_respects_capacity_fifo(ctx):
    """One pack of 32 slots, 80 equal requests: they run in submission order, 32 at a time."""
    M, q0, v0, _ = Model.from_config(0, 80, seed=2)
    S = Server(ctx, [SlotClass(2, 2, 2, packs=1)], precision=gpb.FP64, chunk_steps=25)
    ids = S.submit(M, 0, 80, q0, v0, dt=1e-3, steps=50)
    order = []
    peak = 0
    while True:
        st = S.stats()
        if st["pending"] == 0 and st["active"] == 0:
            break
        S.tick()
        peak = max(peak, S.stats()["active"])
        order.extend(S.completed().tolist())
    assert peak <= 32 and len(order) == 80
    assert sorted(order) == ids.tolist()
    first_wave, second = set(ids[:32].tolist()), set(ids[32:64].tolist())
    assert set(order[:32]) == first_wave and set(order[32:64]) == second
    for r in ids:
        q, v, st, done, lat = S.result(r)
        assert st == 0 and done == 50 and lat >= 0.0
    with pytest.raises(gpb.GpbError, match="not finished"):
        S.result(ids[0])
    S.close()


@pytest.mark.gpu
def test_failed_request_is_retired_and_slot_reused(ctx):
    M, q0, v0, _ = Model.from_config(0, 3, seed=4)
    q0 = q0.copy()
    q0[2] = np.nan  # instance 1 starts non-finite
    S = Server(ctx, [SlotClass(2, 2, 2, packs=1)], precision=gpb.FP64, chunk_steps=10)
    ids = S.submit(M, 0, 3, q0, v0, dt=1e-3, steps=30)
    S.drain(100)
    r0, r1, r2 = (S.result(i) for i in ids)
    assert r1[2] != 0 and r1[3] < 30
    assert r0[2] == 0 and r2[2] == 0 and r0[3] == r2[3] == 30
    # the freed slot takes a new request whose result equals a clean run
    M2, q2, v2, _ = Model.from_config(0, 1, seed=9)
    a = S.submit(M2, 0, 1, q2, v2, dt=1e-3, steps=30)
    S.drain(100)
    qa, va, sa, da, _ = S.result(a[0])
    B = Batch(M2, ctx)
    B.update(q2, v2)
    B.simulate_steps(30, 1e-3, 0, gpb.FP64)
    qb, vb = B.state()
    B.close()
    assert sa == 0 and np.array_equal(qa, qb) and np.array_equal(va, vb)
    S.close()


@pytest.mark.gpu
def test_request_fitting_no_class_is_rejected(ctx):
    M, q0, v0, _ = Model.from_config(3, 1, seed=1)
    S = Server(ctx, [SlotClass(2, 2, 2, packs=1)], precision=gpb.FP64)
    with pytest.raises(gpb.GpbError, match="fits no slot class"):
        S.submit(M, 0, 1, q0, v0, dt=1e-3, steps=10)
    S.close()


@pytest.mark.gpu
@pytest.mark.parametrize("algorithm", [gpb.ALGO_CRBA, gpb.ALGO_ABA])
def test_cuboid_requests_alone_mix_and_batch(ctx, algorithm):
    """build_gripper requests (3 GJK/EPA pair queries per evaluation) in a class
    with max_cuboids = 3, mixed with chains: alone == mix, bit for bit, and both
    equal the batch API."""
    from gpb import builders

    n = 12
    Mg = Model.from_mechanisms([builders.build_gripper()] * n)
    qg, vg = builders.gripper_states(np.random.default_rng(8), n)
    Mc, qc, vc, _ = Model.from_config(1, 10, seed=4)
    M = Model.concat([Mg, Mc])
    q0 = np.concatenate([qg.ravel(), qc])
    v0 = np.concatenate([vg.ravel(), vc])
    qo, vo, _ = M.offsets()
    classes = [SlotClass(4, 10, 9, 8, 1, packs=1, max_cuboids=3), SlotClass(48, 48, 48, packs=1)]

    def run(idx, chunk):
        S = Server(ctx, classes, precision=gpb.FP64, chunk_steps=chunk, algorithm=algorithm)
        ids = {}
        for i in idx:
            grip = i < n
            rid = S.submit(M, int(i), 1, q0, v0, dt=1e-5 if grip else 5e-4, steps=60 + 7 * (i % 5),
                           control="host" if grip else "open_loop", seed=3 + i, keys=0)
            ids[i] = int(rid[0])
        S.drain(100000)
        out = {i: S.result(r) for i, r in ids.items()}
        S.close()
        return out

    mix = run(list(range(M.n)), 23)
    for i in (0, 5, 11, 13):
        alone = run([i], 41)[i]
        assert alone[2] == mix[i][2] == 0
        assert np.array_equal(alone[0], mix[i][0]) and np.array_equal(alone[1], mix[i][1]), i
    for i in (2, 9):
        B = Batch(M.subset([i]), ctx)
        B.set_algorithm(algorithm)
        B.update(q0[qo[i]:qo[i + 1]], v0[vo[i]:vo[i + 1]])
        B.simulate_steps(60 + 7 * (i % 5), 1e-5, 0, gpb.FP64)
        qb, vb = B.state()
        B.close()
        assert np.array_equal(qb, mix[i][0]) and np.array_equal(vb, mix[i][1]), i
