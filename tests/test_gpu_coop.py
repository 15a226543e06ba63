"""Block-cooperative packs (gpb_batch_set_coop): four warps share the fill and
the Cholesky factorisation of one pack.  The arithmetic of every tile is the
one-warp path's, so trajectories, status words and completed-step counts must
agree bit for bit."""

import numpy as np
import pytest

import gpb
from gpb import Batch, Model

pytestmark = pytest.mark.gpu


def mixed_batch(seed=5):
    a, qa, va, _ = Model.from_config(1, 1024, seed=seed)      # chains, n ~ U{2..48}
    b, qb, vb, _ = Model.from_config(3, 256, seed=seed + 1)   # quadrupeds: tree, floating base, contacts
    M = Model.concat([a, b])
    q0 = np.concatenate([qa, qb]).copy()
    v0 = np.concatenate([va, vb])
    qo, _, _ = M.offsets()
    for i in (3, 500):  # two instances that fail on their first step
        q0[qo[i]] = np.nan
    return M, q0, v0


def run(ctx, M, q0, v0, coop, precision, integrator, steps=40):
    B = Batch(M, ctx)
    B.set_coop(coop)
    B.update(q0, v0)
    B.simulate_steps(steps, 2e-4, integrator, precision, control="open_loop", seed=3, sigma=1.0)
    q, v = B.state()
    out = q, v, B.status(), B.steps_done()
    B.close()
    return out


@pytest.mark.parametrize("precision", [gpb.FP64, gpb.MIXED])
@pytest.mark.parametrize("integrator", [gpb.SEMI_IMPLICIT_EULER, gpb.RUNGE_KUTTA_2, gpb.RUNGE_KUTTA_4])
def test_coop_matches_one_warp_bit_for_bit(ctx, precision, integrator):
    M, q0, v0 = mixed_batch()
    ref = run(ctx, M, q0, v0, 0, precision, integrator)
    for thr in (16, 30):
        got = run(ctx, M, q0, v0, thr, precision, integrator)
        bad = np.nonzero((ref[2] != got[2]) | (ref[3] != got[3]))[0]
        assert bad.size == 0, (thr, bad[:8], ref[2][bad[:8]], got[2][bad[:8]], ref[3][bad[:8]], got[3][bad[:8]])
        ok = ref[2] == 0
        assert ok.sum() >= M.n - 2
        qo, vo, _ = M.offsets()
        for i in np.nonzero(ok)[0][::7]:
            assert np.array_equal(ref[0][qo[i]:qo[i + 1]], got[0][qo[i]:qo[i + 1]]), i
            assert np.array_equal(ref[1][vo[i]:vo[i + 1]], got[1][vo[i]:vo[i + 1]]), i
        assert np.array_equal(ref[0][np.isfinite(ref[0])], got[0][np.isfinite(got[0])])


def test_coop_knob_validation(ctx):
    M, q0, v0, _ = Model.from_config(0, 4, seed=1)
    B = Batch(M, ctx)
    with pytest.raises(gpb.GpbError, match="min_dof"):
        B.set_coop(65)
    B.set_coop(-1)
    B.close()


def test_autotune_keeps_state_and_results(ctx):
    M, q0, v0 = mixed_batch(seed=8)
    q0 = np.nan_to_num(q0)
    ref = run(ctx, M, q0, v0, 0, gpb.FP64, gpb.SEMI_IMPLICIT_EULER, steps=30)
    B = Batch(M, ctx)
    B.update(q0, v0)
    w, c, lanes = B.autotune(2e-4, gpb.SEMI_IMPLICIT_EULER, gpb.FP64, control="open_loop", seed=3, trial_steps=5)
    assert w in (4, 8) and c in (0, 32, 40) and lanes == 1  # not a chain batch: one lane per instance
    q1, v1 = B.state()
    assert np.array_equal(q1, q0) and np.array_equal(v1, v0) and not B.status().any()
    B.simulate_steps(30, 2e-4, gpb.SEMI_IMPLICIT_EULER, gpb.FP64, control="open_loop", seed=3, sigma=1.0)
    q2, v2 = B.state()
    B.close()
    assert np.array_equal(q2, ref[0]) and np.array_equal(v2, ref[1])
