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


# ---------------------------------------------------------------------------
# Articulated-body algorithm (GPB_ALGO_ABA), counted from its three passes as
# implemented (same convention).  Per body, FP64 form:
#   revolute about a principal axis with identity init rotation  620
#     (pass 1: sin/cos 2, transforms 42, bias acceleration 30, v ×* I v 72;
#      pass 2: U, D, u 13, I^A − U D⁻¹ Uᵀ 48, I^a c + U D⁻¹ u 84, congruence to
#      the parent 183 (planar rotation 84, shift 99), accumulation 21, force to
#      the parent 48; pass 3: 67)
#   other revolute 845, prismatic 800 (full 3×3 rotation of the congruence,
#   Rodrigues, U = I^A S with a general axis), floating root 440 (6×6
#   Cholesky and solve), fixed 650
#   contact point 130, plus 60 per body of a mechanism with contacts whose
#   parent is not the world (FP64 world poses; a body on the world takes its
#   joint transform as its pose)
# GPB_MIXED runs the articulated-inertia recursion, the 1-DOF q̈ solve and a
# floating joint's 6×6 factor and solve in double-float on the FP32 pipes;
# what stays FP64 is the state update, u, the reduction of q before sin/cos
# and the open-loop torque draw: 23 per planar revolute body (ncu on 65,536
# serial chains: 575 FP64 flops per instance-step), 50 other revolute
# (Rodrigues), 30 prismatic, 10 fixed, and 165 per floating joint (its
# quaternion to rotation 31, joint offset 18, FP64↔double-float conversions
# of its bias force and q̈ 12, velocity sums 6, the quaternion and position
# update 98).  A mechanism with contacts keeps in FP64 only the contact
# differences that cancel:
#   contact point 18 (penetration test 6; for a point in contact, 24 more for
#   the contact-point velocity v + ω × r and its split into ż and v_t: half
#   of the points in contact on average), plus 23 per body with points (the
#   half-space's body-frame normal and the origin's signed distance);
#   per body whose parent is not the world, 120 (FP64 world pose 63, FP64
#   body-velocity recursion 51, FP64 joint rotation 6).
# ncu on 32,768 cubes in flight (the first 20 steps, mostly before landing):
# 284 FP64 flops per cube-step (96 DFMA, 46 DADD, 46 DMUL per cube); this
# count gives 236 with no point in contact and 332 with half of them.
# ---------------------------------------------------------------------------

ABA_FP64 = {"rev_planar": 620, "rev": 845, "pri": 800, "float": 440, "fixed": 650}
ABA_MIXED_FP64 = {"rev_planar": 23, "rev": 50, "pri": 30, "float": 165, "fixed": 10}
ABA_CONTACT = 130
ABA_POSE = 60
ABA_MIXED_CONTACT = 18
ABA_MIXED_CONTACT_BODY = 23
ABA_MIXED_POSE = 120


def _aba_kinds(model, i):
    jo = model.joint_offset
    kinds = []
    for j in range(jo[i], jo[i + 1]):
        t = int(model.joint_type[j])
        if t == 1:
            iso = model.joint_iso[7 * j:7 * j + 4]
            ax = model.joint_axis[3 * j:3 * j + 3]
            planar = (iso[0] == 0 and iso[1] == 0 and iso[2] == 0 and iso[3] == 1 and
                      np.count_nonzero(ax) == 1 and abs(ax[np.nonzero(ax)[0][0]]) == 1.0)
            kinds.append("rev_planar" if planar else "rev")
        else:
            kinds.append({0: "fixed", 2: "pri", 3: "float"}[t])
    return kinds


def aba_model_flops(model, mixed: bool = False, integrator: int = 0) -> np.ndarray:
    """Per-instance FP64 flops of one integrator step with the articulated-body
    algorithm (all of it for GPB_FP64; the FP64 share for GPB_MIXED)."""
    evals = {0: 1, 1: 2, 2: 4}[integrator]
    table = ABA_MIXED_FP64 if mixed else ABA_FP64
    out = np.zeros(model.n, np.int64)
    co, jo, ho = model.contact_offset, model.joint_offset, model.halfspace_offset
    cache: dict = {}
    for i in range(model.n):
        kinds = tuple(_aba_kinds(model, i))
        nc = int(co[i + 1] - co[i])
        off_world = int(np.count_nonzero(model.joint_parent[jo[i]:jo[i + 1]]))
        # bodies carrying points (contact_body is 1-based) × half-spaces
        with_points = len(set(model.contact_body[co[i]:co[i + 1]].tolist())) * int(ho[i + 1] - ho[i])
        key = (kinds, nc, off_world, with_points)
        if key not in cache:
            f = sum(table[k] for k in kinds)
            if nc and mixed:
                f += ABA_MIXED_CONTACT * nc + ABA_MIXED_CONTACT_BODY * with_points + ABA_MIXED_POSE * off_world
            elif nc:
                f += ABA_CONTACT * nc + ABA_POSE * off_world
            cache[key] = f
        out[i] = evals * cache[key]
    return out
