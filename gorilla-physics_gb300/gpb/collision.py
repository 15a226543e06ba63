"""Cuboid–cuboid collision queries on the GPU.

``collide_cuboids`` replaces ``CollisionDetector::new(&A, &B)`` followed by
``gjk()`` and ``epa()`` (src/collision/mod.rs:48-87) for many independent pairs
at once; the same routine runs inside the step for mechanisms whose bodies
carry cuboid colliders (src/contact.rs:191-242).
"""

from __future__ import annotations

import ctypes as C

import numpy as np

from . import _abi

HIT, NONE, PANIC, OVERFLOW = 1, 0, -1, -2


def _f64(a, k):
    return np.ascontiguousarray(np.asarray(a, float).reshape(-1, k))


def collide_cuboids(ctx, pose_a, size_a, pose_b, size_b):
    """n pairs: poses (n, 7) = (qx, qy, qz, qw, tx, ty, tz), sizes (n, 3) = (w, d, h).

    Returns (result (n,) int32, cp_a (n, 3), cp_b (n, 3)); result 1 = in
    collision (cp_b − cp_a is the penetration), 0 = apart, -1 = a case where the
    reference panics, -2 = past the kernel's storage bounds."""
    pa, sa, pb, sb = _f64(pose_a, 7), _f64(size_a, 3), _f64(pose_b, 7), _f64(size_b, 3)
    n = pa.shape[0]
    if not (sa.shape[0] == pb.shape[0] == sb.shape[0] == n):
        raise ValueError("collide_cuboids: pose / size arrays of different lengths")
    res = np.zeros(n, np.int32)
    ca, cb = np.zeros((n, 3)), np.zeros((n, 3))
    p = lambda a: a.ctypes.data_as(_abi.P_f64)
    _abi.check(_abi.lib().gpb_collide_cuboids(ctx.h, n, p(pa), p(sa), p(pb), p(sb),
                                              res.ctypes.data_as(_abi.P_i32), p(ca), p(cb)),
               "gpb_collide_cuboids")
    return res, ca, cb


def collide_cuboids_device(ctx, n, pose_a, size_a, pose_b, size_b, result, cp_a, cp_b, stream=None):
    """The same on device buffers (integer device addresses, e.g. torch
    ``data_ptr()``); only enqueues the kernel on `stream` (None = the context's)."""
    _abi.check(_abi.lib().gpb_collide_cuboids_device(ctx.h, int(n), pose_a, size_a, pose_b, size_b,
                                                     result, cp_a, cp_b, stream), "gpb_collide_cuboids_device")
