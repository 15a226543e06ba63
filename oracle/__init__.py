"""TEST INFRASTRUCTURE — the CPU oracle (FP64 restatement of gorilla-physics'
continuous step).  Only tests/, __graft_entry__.smoke() and bench.py's CPU
baseline may use it, and only as the checker / baseline, never as a product
path.

Functions take a ``gpb.Model`` and one instance's flattened q / v / τ.
"""

from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REPO = HERE.parent
LIB = HERE / "liboracle.so"
SRC = HERE / "gpb_oracle.cpp"
# The seeded workload generator (the benchmark configurations' mechanisms and
# initial states) is the package's own source file, compiled here for the CPU so
# that the reference arm of the benchmark builds its inputs without loading the
# CUDA library; tests check that both builds produce identical tables.
CONFIGS_SRC = REPO / "gorilla-physics_gb300" / "csrc" / "gpb_configs.cpp"
SOURCES = (SRC, HERE / "collision.cpp", HERE / "socp.cpp", CONFIGS_SRC)

P_f64 = C.POINTER(C.c_double)
P_i64 = C.POINTER(C.c_int64)
P_i32 = C.POINTER(C.c_int32)

LU, CHOLESKY = 0, 1


def build(force: bool = False) -> Path:
    """g++ -O2 -ffp-contract=off (x86 and Arm agree bit for bit)."""
    deps = [*SOURCES, HERE / "collision.h", HERE / "socp.h", REPO / "include/gpb.h",
            CONFIGS_SRC.parent / "gpb_rng.h", Path(__file__)]
    if force or not LIB.exists() or LIB.stat().st_mtime < max(p.stat().st_mtime for p in deps):
        tmp = LIB.with_suffix(".so.tmp")
        subprocess.run(["g++", "-std=c++17", "-O2", "-fPIC", "-shared", "-ffp-contract=off",
                        "-I", str(REPO / "include"), "-I", str(CONFIGS_SRC.parent), *map(str, SOURCES),
                        "-o", str(tmp), "-lpthread"],
                       check=True)
        os.replace(tmp, LIB)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(str(LIB))
        vp = C.c_void_p
        L.oracle_dims.argtypes = [vp, C.c_int64, P_i32, P_i32, P_i32]
        L.oracle_dynamics.argtypes = [vp, C.c_int64, P_f64, P_f64, P_f64, C.c_int, P_f64, P_f64]
        L.oracle_mass_matrix.argtypes = [vp, C.c_int64, P_f64, P_f64]
        L.oracle_free_velocity.argtypes = [vp, C.c_int64, P_f64, P_f64, P_f64, C.c_double, C.c_int, P_f64]
        L.oracle_collide_cuboids.argtypes = [C.c_int64, P_f64, P_f64, P_f64, P_f64, C.c_int, P_i32,
                                             P_f64, P_f64, P_i32]
        L.oracle_vs_step.argtypes = [vp, C.c_int64, P_f64, P_f64, P_f64, C.c_double, C.c_int, P_i32,
                                     P_f64, P_f64, P_f64, P_f64, P_f64]
        L.oracle_socp_solve.argtypes = [C.c_int, P_f64, P_f64, C.c_double, P_f64, P_f64]
        L.oracle_energy.argtypes = [vp, C.c_int64, P_f64, P_f64, P_f64, P_f64]
        L.oracle_step.argtypes = [vp, C.c_int64, P_f64, P_f64, P_f64, C.c_double, C.c_int, C.c_int]
        L.oracle_open_loop_tau.argtypes = [C.c_uint32, C.c_int64, C.c_int64, C.c_int32, C.c_double]
        L.oracle_open_loop_tau.restype = C.c_double
        L.oracle_simulate.argtypes = [vp, C.c_int64, P_f64, P_f64, C.c_double, C.c_int64,
                                      C.c_int64, C.c_int, C.c_int, C.c_int, C.c_uint32, C.c_int,
                                      C.c_double, C.c_double, C.c_double, P_f64, C.c_int64, P_f64]
        L.gpb_config_sizes.argtypes = [C.c_int, C.c_int64, C.c_uint32] + [P_i64] * 5
        L.gpb_config_build.argtypes = [C.c_int, C.c_int64, C.c_uint32, C.c_int, P_i32, P_i32, P_i32, P_f64,
                                       P_f64, P_f64, P_f64, P_i32, P_i32, P_f64, P_i32, P_f64, P_i32,
                                       P_f64, P_f64, P_f64]
        L.oracle_simulate_batch.argtypes = [vp, C.c_int64, C.c_int64, P_i64, P_i64, P_f64, P_f64,
                                            C.c_double, C.c_int64, C.c_int64, C.c_int, C.c_int,
                                            C.c_int, C.c_uint32, C.c_int, C.c_double, C.c_double,
                                            C.c_double, P_f64, C.c_int]
        _lib = L
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data_as(P_f64)


def _m(model):
    return C.cast(C.pointer(model.struct()), C.c_void_p)


def dims(model, i):
    nq, nv, nc = C.c_int32(), C.c_int32(), C.c_int32()
    rc = lib().oracle_dims(_m(model), i, C.byref(nq), C.byref(nv), C.byref(nc))
    if rc:
        raise ValueError(f"oracle: malformed instance {i}")
    return nq.value, nv.value, nc.value


def _checked(model, i, q, v, tau=None):
    nq, nv, nc = dims(model, i)
    q = np.ascontiguousarray(q, float).ravel()
    v = np.ascontiguousarray(v, float).ravel()
    t = None if tau is None else np.ascontiguousarray(tau, float).ravel()
    if q.size != nq or v.size != nv or (t is not None and t.size != nv):
        raise ValueError(f"instance {i}: expected {nq} q / {nv} v values, got {q.size} / {v.size}"
                         + ("" if t is None else f" / tau {t.size}"))
    return nq, nv, nc, q, v, t


def dynamics(model, i, q, v, tau=None, solver=LU, contact_forces=False):
    """q̈ (and contact forces) of instance i; returns (qdd, status[, cforce])."""
    nq, nv, nc, q, v, t = _checked(model, i, q, v, tau)
    qdd = np.zeros(max(nv, 1))
    cf = np.zeros(max(3 * nc, 1))
    st = lib().oracle_dynamics(_m(model), i, _p(q), _p(v), _p(t), solver, _p(qdd), _p(cf))
    if contact_forces:
        return qdd[:nv], st, cf[:3 * nc]
    return qdd[:nv], st


def free_velocity(model, i, q, v, tau=None, dt=1e-3, gravity=True):
    """Articulated::free_velocity of instance i (src/hybrid/articulated/mod.rs:124-199)."""
    _, _, _, q, v, tau = _checked(model, i, q, v, tau)
    out = np.zeros(max(v.size, 1))
    st = lib().oracle_free_velocity(_m(model), i, _p(q), _p(v), _p(tau), dt, int(bool(gravity)), _p(out))
    return out[:v.size], st


COL_HIT, COL_NONE = 1, 0


def collide_cuboids(pose_a, dims_a, pose_b, dims_b, translate=True, stats=False):
    """CollisionDetector::new(A, B).gjk() / .epa() (src/collision/mod.rs:48-87) for
    n pairs: poses (n, 7) = (qx, qy, qz, qw, tx, ty, tz), dims (n, 3) = (w, d, h).
    Returns (result codes (n,), cp_a (n, 3), cp_b (n, 3)[, stats (n, 7): GJK
    iterations, EPA expansions, vertices, faces, edges, heap size, FP64 operations])."""
    f = lambda a, k: np.ascontiguousarray(np.asarray(a, float).reshape(-1, k))
    pa, da, pb, db = f(pose_a, 7), f(dims_a, 3), f(pose_b, 7), f(dims_b, 3)
    n = pa.shape[0]
    res = np.zeros(n, np.int32)
    ca, cb = np.zeros((n, 3)), np.zeros((n, 3))
    stt = np.zeros((n, 7), np.int32)
    lib().oracle_collide_cuboids(n, _p(pa), _p(da), _p(pb), _p(db), int(bool(translate)),
                                 res.ctypes.data_as(P_i32), _p(ca), _p(cb), stt.ctypes.data_as(P_i32))
    return (res, ca, cb, stt) if stats else (res, ca, cb)


VELOCITY_STEPPING = 3


def vs_step(model, i, q, v, dt, tau=None, max_contacts=64):
    """One velocity-stepping step of instance i with its program (src/dynamics.rs:367-430,
    652-742).  Returns dict(q, v, status, nc, J, M, vfree, lam, vnext)."""
    _, nv, _, q, v, t = _checked(model, i, q, v, tau)
    q, v = q.copy(), v.copy()
    nc = C.c_int32()
    m = 3 * max_contacts
    J = np.zeros(max(m * nv, 1))
    Mm = np.zeros(max(nv * nv, 1))
    vf, vn = np.zeros(max(nv, 1)), np.zeros(max(nv, 1))
    lam = np.zeros(max(m, 1))
    st = lib().oracle_vs_step(_m(model), i, _p(q), _p(v), _p(t), dt, max_contacts, C.byref(nc), _p(J),
                              _p(Mm), _p(vf), _p(lam), _p(vn))
    k = nc.value
    return dict(q=q, v=v, status=st, nc=k, J=J[:3 * k * nv].reshape(3 * k, nv), M=Mm[:nv * nv].reshape(nv, nv),
                vfree=vf[:nv], lam=lam[:3 * k], vnext=vn[:nv])


def socp_solve(G, g, mu=0.95):
    """The velocity-stepping friction-cone program (src/dynamics.rs:652-742):
    minimise ½λᵀGλ + gᵀλ with ‖(λ_t, λ_b)‖ ≤ μ λ_n per contact.  Returns
    (λ, status, (iterations, residual, gap))."""
    G = np.ascontiguousarray(G, float)
    g = np.ascontiguousarray(g, float).ravel()
    nc = g.size // 3
    lam = np.zeros(max(g.size, 1))
    info = np.zeros(3)
    st = lib().oracle_socp_solve(nc, _p(G), _p(g), mu, _p(lam), _p(info))
    return lam[:g.size], st, tuple(info)


def mass_matrix(model, i, q):
    nq, nv, _ = dims(model, i)
    H = np.zeros((max(nv, 1), max(nv, 1)))
    lib().oracle_mass_matrix(_m(model), i, _p(np.ascontiguousarray(q, float)), _p(H))
    return H[:nv, :nv]


def energy(model, i, q, v):
    ke, pe = C.c_double(), C.c_double()
    lib().oracle_energy(_m(model), i, _p(np.ascontiguousarray(q, float)),
                        _p(np.ascontiguousarray(v, float)), C.byref(ke), C.byref(pe))
    return ke.value, pe.value


def step(model, i, q, v, dt, tau=None, integrator=0, solver=LU):
    _, _, _, q, v, t = _checked(model, i, q, v, tau)
    q, v = q.copy(), v.copy()
    st = lib().oracle_step(_m(model), i, _p(q), _p(v), _p(t), dt, integrator, solver)
    return q, v, st


def open_loop_tau(seed, inst, block, dof, sigma=1.0):
    return lib().oracle_open_loop_tau(seed, inst, block, dof, sigma)


CONTROL = {"host": 0, "open_loop": 1, "pd": 2}


def simulate(model, i, q, v, dt, K, integrator=0, solver=LU, control="host", ctl=None, seed=0,
             resample_every=10, sigma=1.0, kp=0.0, kd=0.0, step0=0, record_every=0):
    """K steps of instance i; returns (q, v, status, history)."""
    nq, nv, _, q, v, c = _checked(model, i, q, v, ctl)
    q, v = q.copy(), v.copy()
    hist = np.zeros(max((K // record_every) * (nq + nv), 1)) if record_every > 0 else None
    st = lib().oracle_simulate(_m(model), i, _p(q), _p(v), dt, K, step0, integrator, solver,
                               CONTROL[control], seed, resample_every, sigma, kp, kd, _p(c),
                               record_every, _p(hist))
    if hist is not None:
        hist = hist[:(K // record_every) * (nq + nv)].reshape(K // record_every, nq + nv)
    return q, v, st, hist


def simulate_batch(model, q_all, v_all, dt, K, integrator=0, solver=LU, control="host",
                   ctl_all=None, seed=0, resample_every=10, sigma=1.0, kp=0.0, kd=0.0, step0=0,
                   begin=0, end=None, threads=1):
    """K steps of instances [begin, end) in place on `threads` host threads."""
    qo, vo, _ = model.offsets()
    end = model.n if end is None else end
    c = None if ctl_all is None else np.ascontiguousarray(ctl_all, float)
    rc = lib().oracle_simulate_batch(_m(model), begin, end, qo.ctypes.data_as(P_i64),
                                     vo.ctypes.data_as(P_i64), _p(q_all), _p(v_all), dt, K, step0,
                                     integrator, solver, CONTROL[control], seed, resample_every,
                                     sigma, kp, kd, _p(c), threads)
    if rc:
        raise ValueError("oracle: malformed model")


def from_config(config, n, seed=0, contact_model=1):
    """The benchmark configuration's seeded mechanisms and initial state, built
    by the CPU compilation of the workload generator (no CUDA library is
    loaded).  Returns (model, q0, v0, aux) like gpb.Model.from_config."""
    from gpb.model import Model  # the table container only

    L = lib()
    sz = [C.c_int64() for _ in range(5)]
    rc = L.gpb_config_sizes(config, n, seed, *[C.byref(x) for x in sz])
    if rc:
        raise ValueError(f"oracle.from_config: bad configuration {config}")
    nj, nc, nh, nq, nv = (x.value for x in sz)
    a = dict(joint_offset=np.zeros(n + 1, np.int32), joint_type=np.zeros(nj, np.int32),
             joint_parent=np.zeros(nj, np.int32), joint_iso=np.zeros(7 * nj), joint_axis=np.zeros(3 * nj),
             joint_spring=np.zeros(2 * nj), body_inertia=np.zeros(10 * nj),
             contact_offset=np.zeros(n + 1, np.int32), contact_body=np.zeros(max(nc, 1), np.int32),
             contact_params=np.zeros(max(6 * nc, 1)), halfspace_offset=np.zeros(n + 1, np.int32),
             halfspace_params=np.zeros(max(8 * nh, 1)), contact_model=np.zeros(n, np.int32))
    q0, v0, aux = np.zeros(max(nq, 1)), np.zeros(max(nv, 1)), np.zeros(max(nv, 1))
    i32 = lambda x: x.ctypes.data_as(P_i32)
    f64 = lambda x: x.ctypes.data_as(P_f64)
    rc = L.gpb_config_build(config, n, seed, contact_model, i32(a["joint_offset"]), i32(a["joint_type"]),
                            i32(a["joint_parent"]), f64(a["joint_iso"]), f64(a["joint_axis"]),
                            f64(a["joint_spring"]), f64(a["body_inertia"]), i32(a["contact_offset"]),
                            i32(a["contact_body"]), f64(a["contact_params"]), i32(a["halfspace_offset"]),
                            f64(a["halfspace_params"]), i32(a["contact_model"]), f64(q0), f64(v0), f64(aux))
    if rc:
        raise ValueError(f"oracle.from_config: build failed ({rc})")
    a["contact_body"] = a["contact_body"][:nc]
    a["contact_params"] = a["contact_params"][:6 * nc]
    a["halfspace_params"] = a["halfspace_params"][:8 * nh]
    return Model(**a), q0[:nq], v0[:nv], aux[:nv]
