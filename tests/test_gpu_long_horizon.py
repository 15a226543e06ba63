"""Long horizons on the GPU against the oracle: energy drift and statistics.

Chaotic mechanisms cannot be compared point by point over long horizons (two
FP64 evaluations that round differently separate exponentially), so:

* the reference's own energy test (src/energy.rs:81-128: a double pendulum under
  semi-implicit Euler for 2 s keeps its energy within 0.1) runs through the GPU,
  whose trajectory and energy match the oracle's;
* 1,024 acrobots of the plain-FP64 configuration (zero torque, semi-implicit
  Euler, dt = 1e-3, 10,000 steps) run on the GPU in FP64 (the drop-in) and in
  the mixed form, and on the oracle.  Per instance: the energy drift
  E(T) − E(0) (kinetic + potential, src/mechanism.rs:334-362) and the final
  state (cos/sin of both angles, both rates).  Each GPU sample is compared with
  the oracle's by a two-sample Kolmogorov–Smirnov test; every test must keep
  p > 1e-3 (with 7 statistics × 2 forms, a false alarm under the null has
  probability below 1.4 %).  In FP64 the energy drift of every instance that
  has not separated from the oracle's trajectory matches it pointwise; the median
  |drift| matches to 15 %.
"""

import math
import os

import numpy as np
import pytest

import gpb
import oracle
from gpb import Batch, Model
from tests.golden import kats

pytestmark = pytest.mark.gpu
G = 9.81
ALPHA = 1e-3


def test_double_pendulum_energy_sie_gpu(ctx):
    """src/energy.rs:81-128 through the GPU: |E(2 s) − E(0)| < 0.1, and the GPU's
    final state and energy equal the oracle's (1e-9)."""
    m, l = 1.0, 1.0
    M = Model.from_mechanisms([kats.double_pendulum(m, (m * l * l, m * l * l, 0), (0, 0, -m * l), (0, 0, -l))])

    def energy(q, v):  # kinetic energy + the reference's double_pendulum_potential_energy (src/energy.rs:9-17)
        ke, _ = oracle.energy(M, 0, q, v)
        return ke + m * G * (-l * math.cos(q[0]) - l * math.cos(q[0]) - l * math.cos(q[0] + q[1]))

    K = gpb.simulate_steps(2.0, 1e-3)
    B = Batch(M, ctx)
    B.update([1.0, 1.0], [0.1, 0.1])
    B.simulate_steps(K, 1e-3, gpb.SEMI_IMPLICIT_EULER)
    q, v = B.state()
    qr, vr, st, _ = oracle.simulate(M, 0, [1.0, 1.0], [0.1, 0.1], 1e-3, K)
    assert st == 0 and np.all(B.status() == 0)
    np.testing.assert_allclose(q, qr, rtol=0, atol=1e-9)
    np.testing.assert_allclose(v, vr, rtol=0, atol=1e-9)
    e0 = energy([1.0, 1.0], [0.1, 0.1])
    assert abs(energy(q, v) - e0) < 1e-1
    assert abs(energy(q, v) - energy(qr, vr)) < 1e-9


def _ks(a, b):
    from scipy.stats import ks_2samp

    return float(ks_2samp(a, b).pvalue)


def _features(q, v):
    q2, v2 = q.reshape(-1, 2), v.reshape(-1, 2)
    return {"cos q1": np.cos(q2[:, 0]), "sin q1": np.sin(q2[:, 0]), "cos q2": np.cos(q2[:, 1]),
            "sin q2": np.sin(q2[:, 1]), "v1": v2[:, 0], "v2": v2[:, 1]}


def test_acrobot_long_horizon_statistics(ctx):
    pytest.importorskip("scipy")
    n, K, dt = 1024, 10_000, 1e-3
    M, q0, v0, _ = Model.from_config(0, n, seed=77)

    def energies(q, v):
        e = np.zeros(n)
        for i in range(n):
            ke, pe = oracle.energy(M, i, q[2 * i:2 * i + 2], v[2 * i:2 * i + 2])
            e[i] = ke + pe
        return e

    e0 = energies(q0, v0)
    # the oracle (the reference's algorithm, FP64, LU) on all host cores
    qo, vo = q0.copy(), v0.copy()
    oracle.simulate_batch(M, qo, vo, dt, K, threads=os.cpu_count() or 1)
    d_ref = energies(qo, vo) - e0
    f_ref = _features(qo, vo)
    B = Batch(M, ctx)
    report = {}
    for name, prec, algo in (("fp64", gpb.FP64, gpb.ALGO_CRBA), ("mixed", gpb.MIXED, gpb.ALGO_ABA)):
        B.set_algorithm(algo)
        B.update(q0, v0)
        B.clear_status()
        B.simulate_steps(K, dt, gpb.SEMI_IMPLICIT_EULER, prec)
        assert np.all(B.status() == 0), name
        q, v = B.state()
        d = energies(q, v) - e0
        p = {"energy drift": _ks(d, d_ref)}
        for k, x in _features(q, v).items():
            p[k] = _ks(x, f_ref[k])
        report[name] = p
        assert min(p.values()) > ALPHA, (name, p)
        # drift magnitudes: the same median (15 %); in FP64, the instances still
        # on the oracle's trajectory (regular motions) drift by the same amount
        assert abs(np.median(np.abs(d)) / np.median(np.abs(d_ref)) - 1.0) < 0.15, name
        if prec == gpb.FP64:
            close = np.max(np.abs(q.reshape(-1, 2) - qo.reshape(-1, 2)), axis=1) < 1e-6
            assert close.sum() > n // 20, int(close.sum())
            assert np.max(np.abs(d - d_ref)[close]) < 1e-6 * max(1.0, np.max(np.abs(e0)))
    B.close()
