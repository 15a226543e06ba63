"""TEST INFRASTRUCTURE — algorithmic work of the cuboid collision workloads.

Counts, with the oracle's instrumented restatement of GJK + EPA (every add,
sub, mul, div and sqrt of the restated algorithm is 1), the mean FP64
operations per collision query of the seeded workloads that bench.py's
--cuboids mode times, and writes them to profiles/collision_work.json; the
bench divides them by its measured kernel times for the roofline fraction.

    python oracle/collision_work.py
"""

from __future__ import annotations

import json
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT / "gorilla-physics_gb300"))
sys.path.insert(0, str(ROOT))

import oracle  # noqa: E402
from gpb import Model, builders  # noqa: E402

SEED = 2026   # bench.py --seed default
SAMPLE = 65536


def pair_work(kind):
    rng = np.random.default_rng(SEED)
    pa, da, pb, db = builders.cuboid_pairs(rng, SAMPLE, kind)
    r, _, _, st = oracle.collide_cuboids(pa, da, pb, db, stats=True)
    return {"mean_flops": float(st[:, 6].mean()), "hit_fraction": float(np.mean(r == 1)),
            "sample": f"{SAMPLE} pairs of builders.cuboid_pairs(default_rng({SEED}), {SAMPLE}, {kind!r})"}


def gripper_work():
    """FP64 operations of the three jaw/cube pair queries of one dynamics
    evaluation at the bench's initial gripper states."""
    rng = np.random.default_rng(SEED)
    n = 8192
    q, _ = builders.gripper_states(rng, n)
    M = Model.from_mechanisms([builders.build_gripper()])
    iso = M.joint_iso.reshape(-1, 7)
    axis = M.joint_axis.reshape(-1, 3)
    size = M.body_cuboid.reshape(-1, 3)
    # body poses: lift (prismatic −z from (0,0,2)), jaws (prismatic ∓x from the
    # lift), cube (floating from (0,0,0.25)); no rotation except the cube's
    lift = np.stack([np.zeros(n), np.zeros(n), 2.0 - q[:, 0]], 1)
    left = lift + iso[1, 4:7] + axis[1] * q[:, 1:2]
    right = lift + iso[2, 4:7] + axis[2] * q[:, 2:3]
    cube_t = iso[3, 4:7] + q[:, 7:10]
    ident = np.tile([0.0, 0.0, 0.0, 1.0], (n, 1))
    poses = {1: np.concatenate([ident, left], 1), 2: np.concatenate([ident, right], 1),
             3: np.concatenate([q[:, 3:7], cube_t], 1)}
    total = np.zeros(n)
    hits = 0
    for a, b in ((1, 2), (1, 3), (2, 3)):
        r, _, _, st = oracle.collide_cuboids(poses[a], np.tile(size[a], (n, 1)), poses[b],
                                             np.tile(size[b], (n, 1)), stats=True)
        total += st[:, 6]
        hits += int(np.sum(r == 1))
    return {"mean_flops_per_evaluation": float(total.mean()), "pair_queries_per_evaluation": 3,
            "hits_per_evaluation": hits / n,
            "sample": f"{n} states of builders.gripper_states(default_rng({SEED}), {n})"}


def main():
    out = {"unit": "FP64 operations (add, sub, mul, div, sqrt = 1) of the restated GJK + EPA",
           "pairs_shallow": pair_work("shallow"), "pairs_deep": pair_work("deep"),
           "gripper": gripper_work(),
           "generated_by": "python oracle/collision_work.py"}
    path = ROOT / "profiles" / "collision_work.json"
    path.write_text(json.dumps(out, indent=1) + "\n")
    print(json.dumps(out, indent=1))


if __name__ == "__main__":
    main()
