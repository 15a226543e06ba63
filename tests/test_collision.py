"""Cuboid–cuboid collision (GJK + EPA, src/collision/{gjk,epa,polytope,mod}.rs).

CPU: the oracle's restatement against the reference's own collision tests —
the fixed samples with their analytic answers and tolerances, and the
randomised tests' success rates on seeded draws of the same distributions.

GPU (-m gpu): the library's collision routine (gpb_collide_cuboids, the code
the step runs for cuboid colliders) against the oracle on the same inputs.  The
routine is a discrete algorithm computed in the reference's order of
operations with IEEE-rounded operations, and the oracle is compiled without
floating-point contraction, so the outcome codes and contact points must be
identical bit for bit.
"""

import zlib

import numpy as np
import pytest

import oracle
from tests.golden import cuboids as cb

HIT = oracle.COL_HIT


def _one(A, da, B, db, translate):
    r, ca, cbp = oracle.collide_cuboids(A, da, B, db, translate=translate)
    return int(r[0]), ca[0], cbp[0]


def _move(pose_vec, delta):
    p = np.array(pose_vec, float)
    p[4:7] += delta
    return p


@pytest.mark.parametrize("case", cb.SAMPLES, ids=[c[0] for c in cb.SAMPLES])
def test_oracle_reference_samples(built, case):
    name, A, da, B, db, tr, checks = case
    r, ca, cbp = _one(A, da, B, db, tr)
    assert r >= 0, f"{name}: collision query failed ({r})"
    depth = np.linalg.norm(ca - cbp)
    for chk in checks:
        kind = chk[0]
        if kind == "hit":
            assert (r == HIT) == chk[1], name
        elif kind == "depth":
            assert abs(depth - chk[1]) <= chk[2], (name, depth)
        elif kind == "depth_if_hit":
            assert r != HIT or abs(depth - chk[1]) <= chk[2], (name, depth)
        elif kind == "depth_gt":
            assert depth > chk[1], name
        elif kind == "cp":
            p = ca if chk[1] == "a" else cbp
            assert abs(p[chk[2]] - chk[3]) <= chk[4], (name, chk, p)
        elif kind == "same":
            assert abs(ca[chk[1]] - cbp[chk[1]]) <= chk[2], (name, chk, ca, cbp)
        elif kind == "separates":
            # moving B by (cp_a − cp_b)(1 + s) separates the shapes (epa.rs:459-463)
            rr, _, _ = _one(A, da, _move(B, (ca - cbp) * (1 + chk[1])), db, tr)
            assert rr == 0, name


def test_oracle_ignored_sample_fails_like_the_reference(built):
    """epa_sample2 is #[ignore]d upstream because it does not pass; the
    restatement reaches one of the reference's panics on it."""
    r, _, _ = _one(cb.pose(cb.I, (0, 0, 0)), (1, 1, 1), cb.pose(cb.I, (1 - 1e-3, 0, 0)), (1, 1, 1), False)
    assert r < 0


def test_oracle_gjk_random(built):
    """gjk_face_shallow_penetration / gjk_no_penetration / gjk_small_separation
    (5000 draws each in the reference; both argument orders)."""
    rng = np.random.default_rng(20250101)
    n = 5000
    pa, da, pb, db = cb.shallow_face_pairs(rng, n)
    for A, dA, B, dB in ((pa, da, pb, db), (pb, db, pa, da)):
        r, _, _ = oracle.collide_cuboids(A, dA, B, dB, translate=False)
        assert np.all(r == HIT)
    for gen in (cb.separated_pairs, cb.small_separation_pairs):
        pa, da, pb, db = gen(rng, n)
        for A, dA, B, dB in ((pa, da, pb, db), (pb, db, pa, da)):
            r, _, _ = oracle.collide_cuboids(A, dA, B, dB, translate=False)
            assert np.all(r == 0), gen.__name__


def test_oracle_epa_face_face_shallow_penetration(built):
    """epa.rs:365-435: the contact points lie on the surfaces, and moving either
    shape by (1 ± 1e-2) times the penetration separates / keeps it in contact in
    more than 99.5 % of the draws (the reference's own bar)."""
    rng = np.random.default_rng(7)
    n = 2000
    pa, da, pb, db = cb.epa_face_pairs(rng, n)
    r, ca, cbp = oracle.collide_cuboids(pa, da, pb, db)
    assert np.all(r == HIT)
    pen = ca - cbp
    sep = col = 0
    for s, want, sign_b in ((1 + 1e-2, 0, 1), (1 - 1e-2, HIT, 1), (1 + 1e-2, 0, -1), (1 - 1e-2, HIT, -1)):
        if sign_b > 0:
            B2 = pb.copy()
            B2[:, 4:7] += pen * s
            rr, _, _ = oracle.collide_cuboids(pa, da, B2, db)
        else:
            A2 = pa.copy()
            A2[:, 4:7] -= pen * s
            rr, _, _ = oracle.collide_cuboids(A2, da, pb, db)
        if want == 0:
            sep += int(np.sum(rr == 0))
        else:
            col += int(np.sum(rr == HIT))
    assert sep / (2 * n) > 0.995 and col / (2 * n) > 0.995, (sep, col)
    # point_on_surface (cuboid.rs:108-149): within 1e-3 of a face, inside the box
    from scipy.spatial.transform import Rotation
    for P, D, C in ((pa, da, ca), (pb, db, cbp)):
        Rm = Rotation.from_quat(P[:, :4]).as_matrix()
        loc = np.einsum("nji,nj->ni", Rm, C - P[:, 4:7])
        half = D / 2
        assert np.all(np.abs(loc) <= half + 1e-3)
        assert np.all(np.min(half - np.abs(loc), axis=1) < 1e-3)


def test_oracle_storage_high_water_marks(built):
    """The kernel's fixed storage (48 vertices, 160 faces, 32 edges, 64 GJK
    iterations) is far above what these distributions reach."""
    rng = np.random.default_rng(3)
    worst = np.zeros(7, int)
    for gen in (cb.shallow_face_pairs, cb.epa_face_pairs, cb.deep_pairs):
        pa, da, pb, db = gen(rng, 20000)
        r, _, _, st = oracle.collide_cuboids(pa, da, pb, db, stats=True)
        assert np.all(r >= 0)
        worst = np.maximum(worst, st.max(0))
    gjk, _, verts, tris, edges, _, _ = worst
    assert gjk < 64 and verts < 48 and tris < 160 and edges < 32, worst


# ---------------------------------------------------------------------------
# GPU: bit-identical to the oracle

def _gpu_vs_oracle(ctx, pa, da, pb, db):
    import gpb
    r, ca, cbp = gpb.collide_cuboids(ctx, pa, da, pb, db)
    ro, cao, cbo = oracle.collide_cuboids(pa, da, pb, db)
    assert np.array_equal(r >= 0, ro >= 0) and np.array_equal(np.where(r < 0, -1, r), np.where(ro < 0, -1, ro))
    hit = r == HIT
    assert np.array_equal(ca[hit], cao[hit]) and np.array_equal(cbp[hit], cbo[hit])
    return r


@pytest.mark.gpu
def test_gpu_reference_samples_bitwise(ctx):
    rows = [c for c in cb.SAMPLES]
    pa = np.array([c[1] for c in rows], float)
    da = np.array([c[2] for c in rows], float)
    pb = np.array([c[3] for c in rows], float)
    db = np.array([c[4] for c in rows], float)
    r = _gpu_vs_oracle(ctx, pa, da, pb, db)
    assert np.all(r >= 0)


@pytest.mark.gpu
@pytest.mark.parametrize("gen", ["shallow_face_pairs", "separated_pairs", "small_separation_pairs",
                                 "epa_face_pairs", "deep_pairs"])
def test_gpu_random_pairs_bitwise(ctx, gen):
    rng = np.random.default_rng(zlib.crc32(gen.encode()))
    pa, da, pb, db = getattr(cb, gen)(rng, 20000)
    r = _gpu_vs_oracle(ctx, pa, da, pb, db)
    assert np.all(r >= 0)
    # and in the other argument order
    _gpu_vs_oracle(ctx, pb, db, pa, da)


@pytest.mark.gpu
def test_gpu_degenerate_cases(ctx):
    """Exactly touching / coincident / identical boxes: the same outcome code
    (including the reference's panics) and points as the oracle."""
    I = cb.I
    rows = [
        (cb.pose(I, (0, 0, 0)), (1, 1, 1), cb.pose(I, (1, 0, 0)), (1, 1, 1)),        # faces touch
        (cb.pose(I, (0, 0, 0)), (1, 1, 1), cb.pose(I, (0, 0, 0)), (1, 1, 1)),        # identical
        (cb.pose(I, (0, 0, 0)), (1, 1, 1), cb.pose(I, (1 - 1e-3, 0, 0)), (1, 1, 1)),  # epa_sample2
        (cb.pose(I, (0, 0, 0)), (2, 2, 2), cb.pose(I, (1, 1, 1)), (2, 2, 2)),        # corner overlap
        (cb.pose(I, (5, 5, 5)), (1, 2, 3), cb.pose(I, (5.5, 5.5, 5.5)), (3, 2, 1)),
    ]
    pa = np.array([r[0] for r in rows], float)
    da = np.array([r[1] for r in rows], float)
    pb = np.array([r[2] for r in rows], float)
    db = np.array([r[3] for r in rows], float)
    _gpu_vs_oracle(ctx, pa, da, pb, db)
