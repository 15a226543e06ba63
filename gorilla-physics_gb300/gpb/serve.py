"""Serving: continuous batching of independent simulation requests
(gpb_server_* of include/gpb.h).

A :class:`Server` keeps a pool of lane slots resident on the GPU.  Requests
(one mechanism each, with its own initial state, step size, horizon,
integrator and control law) queue FIFO per slot class, join the pool between
ticks, run at most ``chunk_steps`` steps per tick and leave when their horizon
is done.  A request's result does not depend on what else shares the pool.
"""

from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _abi
from .batch import Context, _p
from .model import Model


@dataclass
class SlotClass:
    """Capacity of one slot class, and its share of the pool."""
    max_bodies: int
    max_q: int
    max_v: int
    max_contacts: int = 0
    max_halfspaces: int = 0
    weight: float = 0.0  # share of hbm_budget_bytes (0: use `packs`)
    packs: int = 0       # packs of 32 slots
    chunk_steps: int = 0  # steps per tick of this class (0: the server's chunk_steps)
    max_cuboids: int = 0  # cuboid colliders per instance
    planar_only: bool = False  # planar chains only (their packs run the specialised passes)

    def struct(self) -> _abi.GpbSlotClass:
        return _abi.GpbSlotClass(self.max_bodies, self.max_q, self.max_v, self.max_contacts,
                                 self.max_halfspaces, float(self.weight), int(self.packs),
                                 int(self.chunk_steps), int(self.max_cuboids), int(bool(self.planar_only)))


# numpy image of gpb_request (same field order and alignment)
REQUEST_DTYPE = np.dtype([("dt", "f8"), ("steps", "i8"), ("integrator", "i4"), ("control", "i4"),
                          ("seed", "u4"), ("resample_every", "i4"), ("sigma", "f8"), ("kp", "f8"),
                          ("kd", "f8"), ("key", "i4")], align=True)
assert REQUEST_DTYPE.itemsize == C.sizeof(_abi.GpbRequest)


def _opts(classes, precision, chunk_steps, hbm_budget_bytes, max_admit_per_tick, algorithm=_abi.ALGO_CRBA):
    arr = (_abi.GpbSlotClass * len(classes))(*[c.struct() for c in classes])
    o = _abi.GpbServerOpts(precision, chunk_steps, int(hbm_budget_bytes), len(classes),
                           C.cast(arr, C.POINTER(_abi.GpbSlotClass)), max_admit_per_tick, algorithm)
    return o, arr


def plan(classes, hbm_budget_bytes: int = 0, precision: int = _abi.MIXED, chunk_steps: int = 64):
    """(packs per class, device bytes per pack) the server would allocate (host only)."""
    o, keep = _opts(classes, precision, chunk_steps, hbm_budget_bytes, 0)
    n = len(classes)
    packs = np.zeros(n, np.int32)
    nbytes = np.zeros(n, np.int64)
    _abi.check(_abi.lib().gpb_server_plan(C.byref(o), _p(packs, _abi.P_i32), _p(nbytes, _abi.P_i64)),
               "gpb_server_plan")
    return packs, nbytes


class Server:
    def __init__(self, ctx: Context, classes, precision: int = _abi.MIXED, chunk_steps: int = 64,
                 hbm_budget_bytes: int = 0, max_admit_per_tick: int = 0, algorithm: int = _abi.ALGO_CRBA):
        self.ctx = ctx
        o, keep = _opts(classes, precision, chunk_steps, hbm_budget_bytes, max_admit_per_tick, algorithm)
        h = C.c_void_p()
        _abi.check(_abi.lib().gpb_server_create(ctx.h, C.byref(o), C.byref(h)), "gpb_server_create")
        self.h = h
        self._dims = {}  # request id -> (nq, nv)

    def close(self) -> None:
        if self.h:
            _abi.lib().gpb_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def submit(self, model: Model, first: int, count: int, q, v, *, dt, steps,
               integrator: int = _abi.SEMI_IMPLICIT_EULER, control: str = "host", tau=None,
               seed: int = 0, resample_every: int = 10, sigma: float = 1.0, kp: float = 0.0,
               kd: float = 0.0, keys=None) -> np.ndarray:
        """Queues instances first..first+count-1 of `model` as requests.

        q, v (and tau: host torques or PD targets) are the model-wide flat
        arrays; dt, steps, seed and keys may be scalars or per-request arrays.
        `keys` are the instances' numbers in the open-loop draw (default 0, the
        number of an instance run as a batch of one).  Returns the request ids.
        """
        qo, vo, _ = model.offsets()
        q = np.ascontiguousarray(q, np.float64)
        v = np.ascontiguousarray(v, np.float64)
        qs = q[qo[first]:qo[first + count]]
        vs = v[vo[first]:vo[first + count]]
        ts = None
        if tau is not None:
            ts = np.ascontiguousarray(np.asarray(tau, np.float64)[vo[first]:vo[first + count]])
        mode = {"host": _abi.CONTROL_HOST_TAU, "open_loop": _abi.CONTROL_OPEN_LOOP,
                "pd": _abi.CONTROL_PD}[control]
        bc = lambda x, t: np.broadcast_to(np.asarray(x, t), (count,))
        dts, ks, seeds = bc(dt, np.float64), bc(steps, np.int64), bc(seed, np.uint32)
        keys = bc(0 if keys is None else keys, np.int32)
        reqs = np.zeros(max(count, 1), REQUEST_DTYPE)
        reqs["dt"][:count], reqs["steps"][:count], reqs["seed"][:count] = dts, ks, seeds
        reqs["key"][:count] = keys
        reqs["integrator"], reqs["control"], reqs["resample_every"] = integrator, mode, resample_every
        reqs["sigma"], reqs["kp"], reqs["kd"] = sigma, kp, kd
        ids = np.zeros(max(count, 1), np.uint64)
        _abi.check(_abi.lib().gpb_server_submit(
            self.h, C.byref(model.struct()), first, count, _p(qs), _p(vs), _p(ts),
            reqs.ctypes.data_as(C.POINTER(_abi.GpbRequest)),
            ids.ctypes.data_as(C.POINTER(C.c_uint64))), "gpb_server_submit")
        ids = ids[:count]
        nq = np.diff(qo)[first:first + count]
        nv = np.diff(vo)[first:first + count]
        for i, a, b in zip(ids.tolist(), nq.tolist(), nv.tolist()):
            self._dims[i] = (a, b)
        return ids

    def tick(self) -> int:
        """One admission + chunk + retirement round; returns requests finished in it."""
        n = C.c_int32()
        _abi.check(_abi.lib().gpb_server_tick(self.h, C.byref(n)), "gpb_server_tick")
        return n.value

    def completed(self, max_ids: int = 1 << 16) -> np.ndarray:
        """Ids of finished requests not listed before."""
        out = np.zeros(max_ids, np.uint64)
        n = C.c_int32()
        _abi.check(_abi.lib().gpb_server_completed(self.h, out.ctypes.data_as(C.POINTER(C.c_uint64)),
                                                   max_ids, C.byref(n)), "gpb_server_completed")
        return out[:n.value]

    def result(self, rid: int):
        """(q, v, status, steps_done, latency_s) of a finished request (then forgotten)."""
        nq, nv = self._dims.get(int(rid), (0, 0))  # unknown ids: the library reports the error
        q = np.zeros(max(nq, 1))
        v = np.zeros(max(nv, 1))
        st = C.c_int32()
        sd = C.c_int64()
        lat = C.c_double()
        _abi.check(_abi.lib().gpb_server_result(self.h, C.c_uint64(int(rid)), _p(q), _p(v), C.byref(st),
                                                C.byref(sd), C.byref(lat)), "gpb_server_result")
        self._dims.pop(int(rid), None)
        return q[:nq], v[:nv], st.value, sd.value, lat.value

    def forget(self, ids) -> None:
        """Drops the results of finished requests without reading them."""
        ids = np.ascontiguousarray(ids, np.uint64)
        for i in ids.tolist():
            self._dims.pop(i, None)
        _abi.check(_abi.lib().gpb_server_forget(self.h, ids.ctypes.data_as(C.POINTER(C.c_uint64)), ids.size),
                   "gpb_server_forget")

    def stats(self) -> dict:
        s = _abi.GpbServerStats()
        _abi.check(_abi.lib().gpb_server_stats_get(self.h, C.byref(s)), "gpb_server_stats_get")
        return {n: getattr(s, n) for n, _ in s._fields_}

    def drain(self, max_ticks: int = 1 << 30) -> None:
        """Ticks until nothing is pending or running."""
        for _ in range(max_ticks):
            st = self.stats()
            if st["pending"] == 0 and st["active"] == 0:
                return
            self.tick()
        raise RuntimeError("Server.drain: requests still running after max_ticks")
