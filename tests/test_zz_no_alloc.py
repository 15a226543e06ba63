"""gpb_dynamics_static: the dynamics entry point that allocates no device memory.

It serves callers that cannot allocate device memory when they evaluate the
dynamics (a hard real-time loop, or a host that hands out GPU memory through
its own pool): the caller passes device buffers for q, v, τ and q̈, and the
kernel's working memory is a fixed array inside the library.  These tests call
it through the C ABI with device buffers and check it against gpb_dynamics (the
allocating entry point) twice in a row — the second call runs on whatever the
first left in the shared array.  The file is named so that pytest collects it
last.
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
@pytest.mark.parametrize("precision", [gpb.FP64, gpb.MIXED])
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
    B = Batch(M, ctx)
    B.update(q0, v0)
    ref = B.dynamics_continuous(tau, precision=precision)
    qd, vd, td = _dev(q0), _dev(v0), _dev(tau)
    L = _abi.lib()
    stream = torch.cuda.current_stream().cuda_stream
    for call in range(2):
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
