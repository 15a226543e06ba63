"""gpb_dynamics_static: the dynamics entry point that allocates no device memory.

It serves callers that cannot allocate device memory when they evaluate the
dynamics (a hard real-time loop, or a host that hands out GPU memory through
its own pool): the caller passes device buffers for q, v, τ and q̈, and the
kernel's working memory is a fixed array inside the library.  These tests call
it through the C ABI with device buffers and check it against gpb_dynamics (the
allocating entry point) on three calls in a row: the state of the first call,
a perturbed state, then the first state again — so the later calls run on the
different words the previous call left in the shared array.  The file is named
so that pytest collects it last.
"""

import ctypes as C

import numpy as np
import pytest

import gpb
from gpb import Batch, Model, _abi

pytestmark = pytest.mark.gpu

TOL = 1e-10  # the parity tolerance of the FP64 form (relative to max(|q̈|, 1))


def _dev(a):
    import torch

    return torch.as_tensor(np.ascontiguousarray(a, dtype=np.float64), device="cuda")


@pytest.mark.parametrize("config,n", [(0, 96), (1, 64), (2, 64), (3, 48)])
@pytest.mark.parametrize("precision", [gpb.FP64, gpb.MIXED, gpb.MIXED_REFINED])
def test_static_scratch_matches_allocating_path(ctx, config, n, precision):
    import torch

    M, q0, v0, _ = Model.from_config(config, n, seed=17)
    rng = np.random.default_rng(config)
    qo, vo, _ = M.offsets()
    if config in (2, 3):  # put contacts in play
        q0 = q0.copy()
        for i in range(n):
            q0[qo[i] + 6] = rng.uniform(0.0, 0.4) if config == 2 else rng.uniform(0.38, 0.45)
    tau = rng.normal(size=v0.size)
    # a second state: every joint coordinate and velocity moved (quaternions
    # of floating joints are left as they are, so they stay unit)
    q1, v1, tau1 = q0.copy(), v0 + rng.normal(scale=0.5, size=v0.size), -0.5 * tau
    for i in range(n):
        nq = qo[i + 1] - qo[i]
        if nq == vo[i + 1] - vo[i]:
            q1[qo[i]:qo[i + 1]] += rng.uniform(-0.3, 0.3, nq)
        else:
            q1[qo[i] + 4:qo[i + 1]] += rng.uniform(-0.02, 0.02, nq - 4)
    B = Batch(M, ctx)
    refs = []
    for q, v, t in ((q0, v0, tau), (q1, v1, tau1)):
        B.update(q, v)
        refs.append((q, v, t, B.dynamics_continuous(t, precision=precision)))
    L = _abi.lib()
    stream = torch.cuda.current_stream().cuda_stream
    for call, (q, v, t, ref) in enumerate((refs[0], refs[1], refs[0])):
        qd, vd, td = _dev(q), _dev(v), _dev(t)
        out = torch.full((B.nv,), float("nan"), dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        rc = L.gpb_dynamics_static(B.h, qd.data_ptr(), vd.data_ptr(), td.data_ptr(), precision,
                                   out.data_ptr(), C.c_void_p(stream))
        assert rc == 0, L.gpb_last_error().decode()
        torch.cuda.synchronize()
        got = out.cpu().numpy()
        for i in range(n):
            g, r = got[vo[i]:vo[i + 1]], ref[vo[i]:vo[i + 1]]
            err = np.max(np.abs(g - r)) / max(np.max(np.abs(r)), 1.0)
            assert err <= TOL, (call, i, err)
    assert np.all(B.status() == 0)
    B.close()


def test_static_scratch_rejects_host_buffers(ctx):
    """A host pointer is refused with GPB_E_INVAL before any launch (a kernel
    given it would fault)."""
    M, q0, v0, _ = Model.from_config(0, 8, seed=3)
    B = Batch(M, ctx)
    qd, vd = _dev(q0), _dev(v0)
    out = _dev(np.zeros(v0.size))
    host = np.zeros(v0.size)
    L = _abi.lib()
    rc = L.gpb_dynamics_static(B.h, qd.data_ptr(), host.ctypes.data, None, gpb.FP64, out.data_ptr(), None)
    assert rc == _abi.GPB_E_INVAL
    assert "device or managed memory" in L.gpb_last_error().decode()
    B.close()


def test_static_scratch_rejects_oversized_batch(ctx):
    M, q0, v0, _ = Model.from_config(1, 4096, seed=3)
    B = Batch(M, ctx)
    qd, vd = _dev(q0), _dev(v0)
    out = _dev(np.zeros(v0.size))
    L = _abi.lib()
    rc = L.gpb_dynamics_static(B.h, qd.data_ptr(), vd.data_ptr(), None, gpb.FP64, out.data_ptr(), None)
    assert rc == _abi.GPB_E_RANGE
    msg = L.gpb_last_error().decode()
    assert "static array holds" in msg and str(_abi.GPB_STATIC_SCRATCH_BYTES) in msg
    B.close()
