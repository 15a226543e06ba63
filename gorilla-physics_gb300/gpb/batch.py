"""Batched stepping on the GPU: the drop-in for gorilla-physics' `step` /
`simulate` over a slice of mechanism states (src/simulate.rs:20-112).

``Batch`` owns one ``gpb_batch`` (all instances resident in HBM).  Its
``step`` / ``simulate`` / ``dynamics_continuous`` call the CUDA kernels through
the C ABI; there is no CPU path.
"""

from __future__ import annotations

import ctypes as C
import weakref
from typing import Sequence

import numpy as np

from . import _abi
from .model import MechanismState, Model

Integrator = type("Integrator", (), {
    "SemiImplicitEuler": _abi.SEMI_IMPLICIT_EULER,
    "RungeKutta2": _abi.RUNGE_KUTTA_2,
    "RungeKutta4": _abi.RUNGE_KUTTA_4,
    "VelocityStepping": _abi.VELOCITY_STEPPING,
})
Precision = type("Precision", (), {"FP64": _abi.FP64, "MIXED": _abi.MIXED})


def _p(a: np.ndarray | None, t=_abi.P_f64):
    return None if a is None else a.ctypes.data_as(t)


class Context:
    """One CUDA device + stream (gpb_ctx)."""

    def __init__(self, device: int = 0):
        L = _abi.lib()
        h = C.c_void_p()
        _abi.check(L.gpb_create(device, C.byref(h)), "gpb_create")
        self.h = h
        self.device = device
        self._batches = weakref.WeakSet()

    def close(self) -> None:
        """Destroys every batch still alive on this context, then the context."""
        if self.h:
            for b in list(self._batches):
                b.close()
            _abi.lib().gpb_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def launches(self) -> int:
        return int(_abi.lib().gpb_launch_count(self.h))

    def synchronize(self) -> None:
        _abi.check(_abi.lib().gpb_synchronize(self.h), "gpb_synchronize")


class Batch:
    """Many mechanism states stepped together on one GPU.

    ``Batch(model_or_states, ctx)`` builds the device tables; the state starts
    at zero (joint zero, identity pose) like ``MechanismState::new``.
    """

    def __init__(self, mechanisms: Model | Sequence[MechanismState], ctx: Context | None = None):
        self.ctx = ctx or Context()
        if isinstance(mechanisms, Model):
            self.model = mechanisms
            init = None
        else:
            self.model = Model.from_mechanisms(mechanisms)
            init = mechanisms
        L = _abi.lib()
        if not self.ctx.h:
            raise ValueError("the context is closed")
        h = C.c_void_p()
        _abi.check(L.gpb_batch_create(self.ctx.h, C.byref(self.model.struct()), C.byref(h)),
                   "gpb_batch_create")
        self.h = h
        self.ctx._batches.add(self)
        n = self.model.n
        self.q_offset = np.zeros(n + 1, np.int64)
        self.v_offset = np.zeros(n + 1, np.int64)
        nq, nv = C.c_int64(), C.c_int64()
        _abi.check(L.gpb_batch_layout(self.h, _p(self.q_offset, _abi.P_i64),
                                      _p(self.v_offset, _abi.P_i64), C.byref(nq), C.byref(nv)),
                   "gpb_batch_layout")
        self.nq, self.nv = nq.value, nv.value
        self.nc = int(self.model.contact_offset[-1]) if n else 0
        if init is not None:
            self.update(np.concatenate([m.q for m in init] or [np.zeros(0)]),
                        np.concatenate([m.v for m in init] or [np.zeros(0)]))

    @property
    def n(self) -> int:
        return self.model.n

    def close(self) -> None:
        if getattr(self, "h", None):
            if self.ctx.h:  # a closed context already destroyed this batch
                _abi.lib().gpb_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- state ----------------------------------------------------------------
    def update(self, q, v) -> None:
        """MechanismState::update for every instance (flattened q / v)."""
        q = np.ascontiguousarray(q, dtype=np.float64).ravel()
        v = np.ascontiguousarray(v, dtype=np.float64).ravel()
        if q.size != self.nq or v.size != self.nv:
            raise ValueError(f"expected {self.nq} q and {self.nv} v values, got {q.size}, {v.size}")
        _abi.check(_abi.lib().gpb_set_state(self.h, _p(q), _p(v)), "gpb_set_state")

    def state(self) -> tuple[np.ndarray, np.ndarray]:
        q = np.zeros(max(self.nq, 1))
        v = np.zeros(max(self.nv, 1))
        _abi.check(_abi.lib().gpb_get_state(self.h, _p(q), _p(v)), "gpb_get_state")
        return q[:self.nq], v[:self.nv]

    @property
    def q(self) -> np.ndarray:
        return self.state()[0]

    @property
    def v(self) -> np.ndarray:
        return self.state()[1]

    def status(self) -> np.ndarray:
        s = np.zeros(max(self.n, 1), np.int32)
        _abi.check(_abi.lib().gpb_batch_status(self.h, _p(s, _abi.P_i32)), "gpb_batch_status")
        return s[:self.n]

    def steps_done(self) -> np.ndarray:
        """Steps each instance completed in the last simulate/step call."""
        s = np.zeros(max(self.n, 1), np.int64)
        _abi.check(_abi.lib().gpb_batch_steps_done(self.h, _p(s, _abi.P_i64)), "gpb_batch_steps_done")
        return s[:self.n]

    def clear_status(self) -> None:
        _abi.check(_abi.lib().gpb_batch_clear_status(self.h), "gpb_batch_clear_status")

    def set_gravity(self, g: float) -> None:
        """Gravitational acceleration along −z (default 9.81; 0 = off)."""
        _abi.check(_abi.lib().gpb_batch_set_gravity(self.h, g), "gpb_batch_set_gravity")

    def free_velocity(self, dt: float, tau=None, precision: int = _abi.FP64) -> np.ndarray:
        """Articulated::free_velocity (src/hybrid/articulated/mod.rs:124-199): v + dt·M⁻¹(τ − c)."""
        t = None if tau is None else np.ascontiguousarray(tau, dtype=np.float64).ravel()
        out = np.zeros(max(self.nv, 1))
        _abi.check(_abi.lib().gpb_free_velocity(self.h, dt, _p(t), precision, _p(out)), "gpb_free_velocity")
        return out[:self.nv]

    def set_algorithm(self, algorithm: int) -> None:
        """ALGO_CRBA (the reference's route, default) or ALGO_ABA (articulated-body algorithm)."""
        _abi.check(_abi.lib().gpb_batch_set_algorithm(self.h, algorithm), "gpb_batch_set_algorithm")

    def set_coop(self, min_dof: int) -> None:
        """Block-cooperative packs from `min_dof` DOF up (-1 default, 0 off)."""
        _abi.check(_abi.lib().gpb_batch_set_coop(self.h, min_dof), "gpb_batch_set_coop")

    def set_mapping(self, lanes_per_instance: int) -> None:
        """Lanes per instance of GPB_FP64 steps: 1 (default) or 2..32 (body-parallel chains)."""
        _abi.check(_abi.lib().gpb_batch_set_mapping(self.h, lanes_per_instance), "gpb_batch_set_mapping")

    def set_launch(self, warps_per_sm: int) -> None:
        """Resident warps per SM of the step kernel (0 = occupancy limit)."""
        _abi.check(_abi.lib().gpb_batch_set_launch(self.h, warps_per_sm), "gpb_batch_set_launch")

    # -- the hot path -----------------------------------------------------------
    def dynamics_continuous(self, tau=None, precision: int = _abi.FP64,
                            contact_forces: bool = False):
        """q̈ at the current state (src/dynamics.rs:322-364); optionally the contact forces."""
        t = None if tau is None else np.ascontiguousarray(tau, dtype=np.float64).ravel()
        qdd = np.zeros(max(self.nv, 1))
        cf = np.zeros(max(3 * self.nc, 1)) if contact_forces else None
        _abi.check(_abi.lib().gpb_dynamics(self.h, _p(t), precision, _p(qdd), _p(cf)),
                   "gpb_dynamics")
        if contact_forces:
            return qdd[:self.nv], cf[:3 * self.nc]
        return qdd[:self.nv]

    def step(self, dt: float, tau=None, integrator: int = _abi.SEMI_IMPLICIT_EULER,
             precision: int = _abi.FP64) -> None:
        """One step (src/simulate.rs:20-83) of every instance; τ = None means zero."""
        t = None if tau is None else np.ascontiguousarray(tau, dtype=np.float64).ravel()
        _abi.check(_abi.lib().gpb_step(self.h, dt, _p(t), integrator, precision), "gpb_step")

    def simulate_steps(self, K: int, dt: float, integrator: int = _abi.SEMI_IMPLICIT_EULER,
                       precision: int = _abi.FP64, control: str = "host", tau=None,
                       seed: int = 0, resample_every: int = 10, sigma: float = 1.0,
                       kp: float = 0.0, kd: float = 0.0, step0: int = 0, record_every: int = 0):
        """K steps with the device-side control law ('host' τ, 'open_loop', 'pd').

        Returns the history [K // record_every, nq + nv] when record_every > 0.
        """
        mode = {"host": _abi.CONTROL_HOST_TAU, "open_loop": _abi.CONTROL_OPEN_LOOP,
                "pd": _abi.CONTROL_PD}[control]
        t = None if tau is None else np.ascontiguousarray(tau, dtype=np.float64).ravel()
        ctl = _abi.GpbControl(mode, seed, resample_every, sigma, kp, kd, _p(t))
        hist = None
        if record_every > 0:
            hist = np.zeros(max((K // record_every) * (self.nq + self.nv), 1))
        _abi.check(_abi.lib().gpb_simulate(self.h, dt, K, step0, integrator, precision,
                                           C.byref(ctl), record_every, _p(hist)), "gpb_simulate")
        if hist is not None:
            return hist[:(K // record_every) * (self.nq + self.nv)].reshape(
                K // record_every, self.nq + self.nv)
        return None

    def autotune(self, dt: float, integrator: int = _abi.SEMI_IMPLICIT_EULER,
                 precision: int = _abi.FP64, control: str = "host", tau=None, seed: int = 0,
                 resample_every: int = 10, sigma: float = 1.0, kp: float = 0.0, kd: float = 0.0,
                 trial_steps: int = 20) -> tuple[int, int, int]:
        """Times the launch shapes on this batch's own step and keeps the fastest.

        Returns (warps_per_sm, coop_min_dof, lanes_per_instance); the state is
        left unchanged."""
        mode = {"host": _abi.CONTROL_HOST_TAU, "open_loop": _abi.CONTROL_OPEN_LOOP,
                "pd": _abi.CONTROL_PD}[control]
        t = None if tau is None else np.ascontiguousarray(tau, dtype=np.float64).ravel()
        ctl = _abi.GpbControl(mode, seed, resample_every, sigma, kp, kd, _p(t))
        w, c, lanes = C.c_int32(), C.c_int32(), C.c_int32()
        _abi.check(_abi.lib().gpb_batch_autotune(self.h, dt, integrator, precision, C.byref(ctl), trial_steps,
                                                 C.byref(w), C.byref(c), C.byref(lanes)), "gpb_batch_autotune")
        return w.value, c.value, lanes.value


def simulate_steps(final_time: float, dt: float) -> int:
    """Step count of `while t < final_time { t += dt }` (src/simulate.rs:97-109)."""
    return int(_abi.lib().gpb_simulate_steps(final_time, dt))


def simulate(batch: Batch, final_time: float, dt: float, tau=None,
             integrator: int = _abi.SEMI_IMPLICIT_EULER, precision: int = _abi.FP64):
    """`simulate` (src/simulate.rs:87-112) for every instance with constant τ.

    Returns (qs, vs): arrays [steps + 1, nq] and [steps + 1, nv] like the
    reference's per-step history (initial state first).
    """
    K = simulate_steps(final_time, dt)
    q0, v0 = batch.state()
    hist = batch.simulate_steps(K, dt, integrator, precision, "host", tau=tau, record_every=1)
    if hist is None:
        hist = np.zeros((0, batch.nq + batch.nv))
    qs = np.vstack([q0[None, :], hist[:, :batch.nq]])
    vs = np.vstack([v0[None, :], hist[:, batch.nq:]])
    return qs, vs
