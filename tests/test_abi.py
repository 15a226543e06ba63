"""The C ABI library without a GPU: loads, exports every declared symbol, and
its host-only entry points (config builders, torque stream, step counting)."""

import ctypes as C
import re

import numpy as np
import pytest

import gpb
import oracle
from conftest import ROOT
from gpb import Model, _abi


def test_exports_every_declared_symbol(built):
    header = (ROOT / "include" / "gpb.h").read_text()
    declared = set(re.findall(r"^\s*(?:int|int64_t|double|const char\*)\s+(gpb_\w+)\s*\(", header, re.M))
    assert len(declared) >= 20
    L = C.CDLL(str(_abi.LIB_PATH))
    missing = [s for s in sorted(declared) if not hasattr(L, s)]
    assert not missing, missing
    bound = {name for name, _, _ in _abi.SIGNATURES}
    assert declared == bound, declared ^ bound
    assert _abi.lib().gpb_abi_version() == 1


def test_torque_stream_matches_oracle_bit_for_bit(built):
    L = _abi.lib()
    vals = []
    for seed in (0, 1, 12345):
        for inst in (0, 7, 65535):
            for block in (0, 1, 199):
                for dof in (0, 5, 47):
                    a = L.gpb_open_loop_tau(seed, inst, block, dof, 1.0)
                    b = oracle.open_loop_tau(seed, inst, block, dof, 1.0)
                    assert a == b, (seed, inst, block, dof, a, b)
                    vals.append(a)
    big = np.array([L.gpb_open_loop_tau(3, i, 0, 0, 1.0) for i in range(4000)])
    assert abs(big.mean()) < 0.06 and abs(big.std() - 1.0) < 0.05


def test_simulate_step_count_matches_reference_loop(built):
    for T, dt in [(10.0, 0.001), (5.0, 1e-2), (2.0, 1e-3), (20.0, 1e-2), (1.1, 1e-3), (0.0, 0.1)]:
        t, k = 0.0, 0
        while t < T:
            t += dt
            k += 1
        assert gpb.simulate_steps(T, dt) == k


@pytest.mark.parametrize("config", [0, 1, 2, 3])
def test_config_builders(built, config):
    n = 96
    M, q0, v0, aux = Model.from_config(config, n, seed=11)
    M2, q1, v1, aux1 = Model.from_config(config, n, seed=11)
    np.testing.assert_array_equal(q0, q1)
    np.testing.assert_array_equal(M.body_inertia, M2.body_inertia)
    assert M.n == n
    qo, vo, co = M.offsets()
    assert qo[-1] == q0.size and vo[-1] == v0.size
    nb = np.diff(M.joint_offset)
    if config == 0:
        assert np.all(nb == 2)
        assert np.all(np.abs(q0) <= np.pi)
        assert abs(np.std(v0) - 0.5) < 0.1
    elif config == 1:
        assert nb.min() >= 2 and nb.max() <= 48
        assert np.all(M.joint_parent == np.concatenate([np.arange(k) for k in nb]))
    elif config == 2:
        assert np.all(nb == 1) and np.all(np.diff(co) == 8)
        m = M.body_inertia[0::10]
        assert np.all((m >= 1000 * 0.2 ** 3) & (m <= 1000.0))
        quats = q0.reshape(n, 7)[:, :4]
        np.testing.assert_allclose(np.linalg.norm(quats, axis=1), 1.0, atol=1e-14)
    else:
        assert np.all(nb == 13) and np.all(np.diff(vo) == 18)
        targets = aux.reshape(n, 18)[:, 6:]
        assert np.all(np.abs(targets) <= 0.5)
    # every instance is a well-posed mechanism for the oracle
    for i in range(0, n, 17):
        qdd, st = oracle.dynamics(M, i, q0[qo[i]:qo[i + 1]], v0[vo[i]:vo[i + 1]])
        assert st == 0 and np.all(np.isfinite(qdd))


def test_model_roundtrip_subset(built):
    M, q0, v0, _ = Model.from_config(1, 20, seed=2)
    S = M.subset([3, 1, 7])
    qo, vo, _ = M.offsets()
    so, sv, _ = S.offsets()
    for k, i in enumerate([3, 1, 7]):
        a, _ = oracle.dynamics(M, i, q0[qo[i]:qo[i + 1]], v0[vo[i]:vo[i + 1]])
        b, _ = oracle.dynamics(S, k, q0[qo[i]:qo[i + 1]], v0[vo[i]:vo[i + 1]])
        np.testing.assert_array_equal(a, b)


def test_mechanism_state_errors_like_reference():
    from gpb import RevoluteJoint, Transform3D, MechanismState
    from tests.golden.kats import body
    with pytest.raises(AssertionError, match="child body is not body 1"):
        MechanismState([RevoluteJoint(Transform3D("a", "world"), (0, 1, 0))], [body("b", 1, (1, 1, 1), (0, 0, 0))])
    with pytest.raises(AssertionError, match="has no parent body of frame nowhere"):
        MechanismState([RevoluteJoint(Transform3D("a", "nowhere"), (0, 1, 0))], [body("a", 1, (1, 1, 1), (0, 0, 0))])
