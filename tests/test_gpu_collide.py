"""jg_collide_pairs (batched NarrowPhase.MprEpa) against the oracle's MprEpa.

Contact normal, depth and points within 1e-4 (relative to max(1, |x|)) for at least
99.9 % of colliding pairs.  Pairs the MPR settles alone (penetration <= the EPA threshold
0.02) run the same FP32 arithmetic on both sides; deeper pairs run EPA, whose face data is
FP64 on both sides (as in the reference's ConvexPolytope), so those agree as closely.
"""
import numpy as np
import pytest

import oracle_lib as O
from jitterphysics2_gb300 import abi, scenes
from jitterphysics2_gb300.world import world_for_scene

pytestmark = pytest.mark.gpu


def overlap_scene(seed=21, n=400):
    return scenes.mixed_pile(n=n, box=(8.0, 8.0, 8.0), y0=-4.0, cells=8, seed=seed)


def candidate_pairs(sc, rng, limit=6000):
    sh, b = sc["shapes"], sc["bodies"]
    pos = b["position"][sh["body"]].astype(np.float64)
    tri = sh["kind"] == abi.SHAPE_TRIANGLE
    tv = sc["triangles"]
    tc = (tv["a"] + tv["b"] + tv["c"]) / 3.0
    pos[tri] = tc[sh["data_offset"][tri]]
    dyn = np.nonzero(sh["body"] >= 2)[0]
    pairs = []
    for i in dyn:
        d = np.linalg.norm(pos - pos[i], axis=1)
        near = np.nonzero((d < 2.2) & (np.arange(len(sh)) != i))[0]
        for j in near:
            if j < i and sh["body"][j] >= 2:
                continue  # body-body pairs once
            pairs.append((min(i, j), max(i, j)) if sh["body"][j] >= 2 else (j, i))
        if pos[i, 1] < 1.5:
            pairs.append((0, i))
    pairs = np.array(sorted(set(pairs)), np.int32)
    if len(pairs) > limit:
        pairs = pairs[rng.choice(len(pairs), limit, replace=False)]
    return pairs


def rel_err(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return np.abs(a - b).max(axis=-1) / np.maximum(1.0, np.abs(b).max(axis=-1))


def compare(sc, w, pairs):
    hit, pA, pB, nrm, pen = w.collide_pairs(pairs)
    o = O.OracleWorld(sc)
    res = [o.collide(int(a), int(b)) for a, b in pairs]
    ohit = np.array([r[0] for r in res])
    op = np.array([r[4] for r in res])
    errs = np.stack([rel_err(nrm, np.array([r[3] for r in res])), rel_err(pA, np.array([r[1] for r in res])),
                     rel_err(pB, np.array([r[2] for r in res])),
                     np.abs(pen - op) / np.maximum(1.0, np.abs(op))], 1).max(axis=1)
    # the hit decision is the same MPR arithmetic
    assert np.mean(hit == ohit) > 0.999, np.nonzero(hit != ohit)[0][:10]
    both = hit & ohit
    return both & (op <= 0.02), both & (op > 0.02), errs, pen, op


def test_collide_pairs_matches_oracle_on_resting_contacts():
    # a settled pile: shallow contacts that the MPR settles without EPA
    sc = scenes.mixed_pile(n=400, box=(20.0, 3.0, 20.0), y0=0.0, cells=8, seed=7, lattice=3.0)
    w = world_for_scene(sc)
    for _ in range(250):
        w.step(sc["dt"])
    sc = dict(sc)
    sc["bodies"] = w.bodies()
    pairs = candidate_pairs(sc, np.random.default_rng(1))
    shallow, deep, errs, _, _ = compare(sc, w, pairs)
    assert shallow.sum() > 300, shallow.sum()
    assert np.mean(errs[shallow] < 1e-4) >= 0.999, np.sort(errs[shallow])[-10:]


def test_collide_pairs_matches_oracle_on_deep_overlaps():
    # bodies dropped into a small box: deep overlaps, body-body, ground and triangle pairs
    sc = overlap_scene()
    pairs = candidate_pairs(sc, np.random.default_rng(0))
    w = world_for_scene(sc)
    shallow, deep, errs, pen, op = compare(sc, w, pairs)
    assert deep.sum() > 500, deep.sum()
    bad = np.nonzero(deep & (errs >= 1e-4))[0]
    assert np.mean(errs[deep] < 1e-4) >= 0.999, (np.mean(errs[deep] < 1e-4), [(tuple(pairs[i]), errs[i]) for i in bad[:10]])


def test_collide_pairs_rejects_bad_input():
    from jitterphysics2_gb300.abi import JitterError
    sc = overlap_scene(n=20)
    w = world_for_scene(sc)
    with pytest.raises(JitterError):
        w.collide_pairs(np.array([[0, len(sc["shapes"])]], np.int32))
    hit, *_ = w.collide_pairs(np.zeros((0, 2), np.int32))
    assert len(hit) == 0
