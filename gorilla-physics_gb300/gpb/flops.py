"""Algorithmic work of one instance-step (the roofline numerator).

Counting convention: add, sub, mul, div, sqrt, sin, cos = 1 flop; a fused
multiply-add = 2.  The counts are those of the minimal world-frame
CRBA + RNEA + Cholesky algorithm (the work any implementation of
dynamics_continuous must do), per body:

  revolute / prismatic body  400   FK 38, motion subspace 9, twist 12,
                                   Coriolis bias 33, inertia to world 115,
                                   Newton–Euler 120, inward sweep 69, update 4
  floating body             1040   (6-column motion subspace and projections,
                                   quaternion integration)
  fixed body                 300
  contact point               95   if in contact, 40 otherwise (test only)
plus the mass-matrix fill (11 per ancestor pair of DOFs), the Cholesky
factorisation ((n−1)n(n+1)/3 + n(n−1)/2 + 2n) and the two triangular solves (2n²).
RK2 / RK4 evaluate the dynamics 2 / 4 times.
"""

from __future__ import annotations

import numpy as np

PER_BODY = {0: 300, 1: 400, 2: 400, 3: 1040}
CONTACT = 95


def cholesky_flops(n: int) -> int:
    return (n - 1) * n * (n + 1) // 3 + n * (n - 1) // 2 + 2 * n


def instance_flops(joint_type: np.ndarray, joint_parent: np.ndarray, n_contacts: int) -> int:
    """One dynamics evaluation of one mechanism."""
    nv_j = np.choose(joint_type, [0, 1, 1, 6])
    n = int(nv_j.sum())
    f = int(sum(PER_BODY[int(t)] for t in joint_type))
    # ancestor-or-self DOF pairs for the fill
    pairs = 0
    for b in range(len(joint_type)):
        a, anc = b, 0
        while True:
            anc += int(nv_j[a])
            p = int(joint_parent[a])
            if p == 0:
                break
            a = p - 1
        pairs += int(nv_j[b]) * (anc - int(nv_j[b])) + int(nv_j[b]) * (int(nv_j[b]) + 1) // 2
    f += 11 * pairs + cholesky_flops(n) + 2 * n * n + n + CONTACT * n_contacts
    return f


def model_flops(model, integrator: int = 0) -> np.ndarray:
    """Per-instance flops of one integrator step for every instance of a Model."""
    evals = {0: 1, 1: 2, 2: 4}[integrator]
    out = np.zeros(model.n, np.int64)
    jo, co = model.joint_offset, model.contact_offset
    cache: dict = {}
    for i in range(model.n):
        t = model.joint_type[jo[i]:jo[i + 1]]
        p = model.joint_parent[jo[i]:jo[i + 1]]
        key = (t.tobytes(), p.tobytes(), int(co[i + 1] - co[i]))
        if key not in cache:
            cache[key] = instance_flops(t, p, key[2])
        out[i] = evals * cache[key]
    return out
