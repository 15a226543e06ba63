"""The body-parallel mapping's algorithm (gorilla-physics_gb300/csrc/gpb_group.cuh)
restated in numpy and checked against the oracle on the CPU, independently of
the GPU:

* world poses as an exclusive Kogge–Stone prefix product over G lanes of S
  consecutive bodies each (a serial pass over the lane's bodies, then the scan
  of the lane totals);
* body velocities and bias accelerations as one scan of pairs with
  (V1, A1) ⊕ (V2, A2) = (V1 + V2, A1 + A2 + V1 ×m V2);
* composite inertias and joint forces as suffix sums;
* on a chain H_ij = (Ic_i S_i) · S_j for j ≤ i;
* the Cholesky factor by 4-column panels (identity padding to whole panels)
  and the two triangular solves by the same panels.

q̈ must match the oracle's FP64 dynamics (the reference's algorithm) within
1e-10 · max(|q̈|, 1), and H the oracle's mass matrix within 1e-12 · max|H|,
for every lane count the mapping accepts.
"""

import numpy as np
import pytest

import oracle
from tests.test_gpu_group import random_chains

G_ACC = 9.81


def quat_to_mat(x, y, z, w):
    return np.array([[w * w + x * x - y * y - z * z, 2 * (x * y - w * z), 2 * (x * z + w * y)],
                     [2 * (x * y + w * z), w * w - x * x + y * y - z * z, 2 * (y * z - w * x)],
                     [2 * (x * z - w * y), 2 * (y * z + w * x), w * w - x * x - y * y + z * z]])


def rot(axis, angle):
    a = np.asarray(axis, float)
    K = np.array([[0, -a[2], a[1]], [a[2], 0, -a[0]], [-a[1], a[0], 0]])
    return np.cos(angle) * np.eye(3) + np.sin(angle) * K + (1 - np.cos(angle)) * np.outer(a, a)


def compose(a, b):  # a ∘ b: first b, then a
    return a[0] @ b[0], a[1] + a[0] @ b[1]


def crm(x, y):  # (ω, v) ×m (ω', v')
    return np.concatenate([np.cross(x[:3], y[:3]), np.cross(x[:3], y[3:]) + np.cross(x[3:], y[:3])])


def crf(x, f):  # (ω, v) ×* (n, f)
    return np.concatenate([np.cross(x[:3], f[:3]) + np.cross(x[3:], f[3:]), np.cross(x[:3], f[3:])])


def imul(I, s):  # I = (J 3×3, c = m·com, m); (J ω + c × v, m v − c × ω)
    J, c, m = I
    return np.concatenate([J @ s[:3] + np.cross(c, s[3:]), m * s[3:] - np.cross(c, s[:3])])


def to_world(J, c, m, R, p):
    """Body inertia about the body origin → about the world origin (parallel axis)."""
    cw = R @ c
    Jw = R @ J @ R.T + m * (p @ p * np.eye(3) - np.outer(p, p)) + 2 * (cw @ p) * np.eye(3) \
        - np.outer(cw, p) - np.outer(p, cw)
    return Jw, cw + m * p, m


def excl_scan(vals, G, S, comb, ident):
    """Exclusive prefix of vals (one per body) the way the kernel computes it:
    each lane t combines its S bodies serially, the lane totals are scanned by
    Kogge–Stone over G lanes, and each body gets (lanes before) ⊕ (its lane's
    bodies up to it).  Returns the inclusive value per body."""
    nb = len(vals)
    local = []
    tot = []
    for t in range(G):
        acc = None
        for s in range(S):
            b = t * S + s
            v = vals[b] if b < nb else ident
            acc = v if acc is None else comb(acc, v)
            local.append(acc)
        tot.append(acc)
    x = list(tot)
    d = 1
    while d < G:
        x = [comb(x[t - d], x[t]) if t >= d else x[t] for t in range(G)]
        d *= 2
    out = []
    for t in range(G):
        e = x[t - 1] if t > 0 else ident
        for s in range(S):
            out.append(comb(e, local[t * S + s]))
    return out[:nb]


def group_dynamics(M, i, q, v, tau, G, S):
    """q̈ and H of instance i (a serial chain) by the body-parallel algorithm."""
    j0, j1 = M.joint_offset[i], M.joint_offset[i + 1]
    nb = j1 - j0
    types = M.joint_type[j0:j1]
    iso = M.joint_iso.reshape(-1, 7)[j0:j1]
    axes = M.joint_axis.reshape(-1, 3)[j0:j1]
    inert = M.body_inertia.reshape(-1, 10)[j0:j1]
    spring = M.joint_spring.reshape(-1, 2)[j0:j1]
    dof = [k for k in range(nb) if types[k] in (1, 2)]
    vo = {k: n for n, k in enumerate(dof)}
    n = len(dof)
    # joint transforms
    X = []
    for k in range(nb):
        Ri = quat_to_mat(*iso[k, :4])
        ti = iso[k, 4:].copy()
        if types[k] == 1:
            X.append((Ri @ rot(axes[k], q[vo[k]]), ti))
        elif types[k] == 2:
            X.append((Ri, ti + Ri @ axes[k] * q[vo[k]]))
        else:
            X.append((Ri, ti))
    W = excl_scan(X, G, S, compose, (np.eye(3), np.zeros(3)))
    # motion subspaces and the (V, A) pair scan
    Sw = []
    for k in range(nb):
        if types[k] in (1, 2):
            aw = W[k][0] @ axes[k]
            Sw.append(np.concatenate([aw, np.cross(W[k][1], aw)]) if types[k] == 1
                      else np.concatenate([np.zeros(3), aw]))
        else:
            Sw.append(np.zeros(6))
    vj = [Sw[k] * (v[vo[k]] if k in vo else 0.0) for k in range(nb)]
    VA = excl_scan([(x, np.zeros(6)) for x in vj], G, S,
                   lambda a, b: (a[0] + b[0], a[1] + b[1] + crm(a[0], b[0])), (np.zeros(6), np.zeros(6)))
    grav = np.array([0, 0, 0, 0, 0, G_ACC])
    # per body: world inertia, Newton–Euler force
    Iw, f = [], []
    for k in range(nb):
        m = inert[k, 0]
        c = inert[k, 1:4]
        J = np.array([[inert[k, 4], inert[k, 7], inert[k, 8]], [inert[k, 7], inert[k, 5], inert[k, 9]],
                      [inert[k, 8], inert[k, 9], inert[k, 6]]])
        I = to_world(J, c, m, *W[k])
        V, A = VA[k][0], VA[k][1] + grav
        Iw.append(I)
        f.append(imul(I, A) + crf(V, imul(I, V)))
    # suffix sums (the reverse scan)
    rev = excl_scan([(I[0], I[1], I[2], ff) for I, ff in zip(Iw[::-1], f[::-1])], G, S,
                    lambda a, b: (a[0] + b[0], a[1] + b[1], a[2] + b[2], a[3] + b[3]),
                    (np.zeros((3, 3)), np.zeros(3), 0.0, np.zeros(6)))[::-1]
    H = np.zeros((n, n))
    rhs = np.zeros(n)
    Fi = {}
    for k in dof:
        Ic = rev[k][:3]
        Fi[k] = imul(Ic, Sw[k])
        r = tau[vo[k]]
        if types[k] == 2 and spring[k, 0] != 0.0:
            r += -spring[k, 0] * (q[vo[k]] - spring[k, 1])
        rhs[vo[k]] = r - Sw[k] @ rev[k][3]
    for a in dof:
        for b in dof:
            if vo[b] <= vo[a]:
                H[vo[a], vo[b]] = H[vo[b], vo[a]] = Fi[a] @ Sw[b]
    # Cholesky by 4-column panels, identity padding, and the panel solves
    n4 = (n + 3) // 4 * 4
    A = np.eye(n4)
    A[:n, :n] = H
    x = np.zeros(n4)
    x[:n] = rhs
    dinv = np.zeros(n4)
    for k in range(0, n4, 4):
        L = np.tril(A[k:k + 4, k:k + 4])
        for c in range(4):
            d = L[c, c] - L[c, :c] @ L[c, :c]
            r = 1.0 / np.sqrt(d)
            L[c, c] = d * r
            for a in range(c + 1, 4):
                L[a, c] = (L[a, c] - L[a, :c] @ L[c, :c]) * r
            dinv[k + c] = r
        A[k:k + 4, k:k + 4] = L
        for i2 in range(k + 4, n4):
            lrow = np.zeros(4)
            for c in range(4):
                lrow[c] = (A[i2, k + c] - lrow[:c] @ L[c, :c]) * dinv[k + c]
            A[i2, k:k + 4] = lrow
        B = A[k + 4:, k:k + 4]
        A[k + 4:, k + 4:] -= np.tril(B @ B.T)
    z = np.zeros(n4)
    for k in range(0, n4, 4):
        y = np.zeros(4)
        for a in range(4):
            y[a] = (x[k + a] - A[k + a, k:k + a] @ y[:a]) * dinv[k + a]
        x[k + 4:] -= A[k + 4:, k:k + 4] @ y
        z[k:k + 4] = y
    out = np.zeros(n4)
    for k in range(n4 - 4, -1, -4):
        w = np.zeros(4)
        for a in range(3, -1, -1):
            w[a] = (z[k + a] - A[k + a + 1:k + 4, k + a] @ w[a + 1:]) * dinv[k + a]
        z[:k] -= A[k:k + 4, :k].T @ w
        out[k:k + 4] = w
    return out[:n], H


def lane_shapes(nb):
    return [(g, 1 if g >= nb else 2) for g in (2, 4, 8, 16, 32) if 2 * g >= nb] + [(128, 1)]


@pytest.mark.parametrize("nb_lo,nb_hi", [(1, 4), (5, 12), (13, 30)])
def test_group_algorithm_matches_oracle(nb_lo, nb_hi):
    rng = np.random.default_rng(17 + nb_lo)
    M = random_chains(rng, 6, nb_lo, nb_hi)
    qo, vo, _ = M.offsets()
    for i in range(M.n):
        q = rng.uniform(-np.pi, np.pi, qo[i + 1] - qo[i])
        v = rng.normal(size=vo[i + 1] - vo[i])
        tau = rng.normal(size=vo[i + 1] - vo[i])
        ref, st = oracle.dynamics(M, i, q, v, tau, solver=oracle.CHOLESKY)
        assert st == 0
        Href = oracle.mass_matrix(M, i, q)
        nb = M.joint_offset[i + 1] - M.joint_offset[i]
        for G, S in lane_shapes(nb):
            qdd, H = group_dynamics(M, i, q, v, tau, G, S)
            assert np.max(np.abs(H - Href)) <= 1e-12 * max(np.max(np.abs(Href)), 1.0), (i, G)
            assert np.max(np.abs(qdd - ref)) <= 1e-10 * max(np.max(np.abs(ref)), 1.0), (i, G)
