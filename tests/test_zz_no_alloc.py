"""jg_collide_pairs_noalloc (fixed device scratch, no allocation in the call) against
jg_collide_pairs (scratch grown with cudaMalloc) on the same pairs: identical bits, on two
calls in a row with different batches, and after a step moved the bodies.  Collected last
so that it also runs after every other GPU test in the same process."""
import numpy as np
import pytest

from jitterphysics2_gb300 import abi, scenes
from jitterphysics2_gb300.abi import JitterError
from jitterphysics2_gb300.world import world_for_scene

pytestmark = pytest.mark.gpu


def pile_pairs(sc, rng, count):
    # shape pairs whose bodies are near each other, plus pairs with the ground box
    sh, b = sc["shapes"], sc["bodies"]
    dyn = np.nonzero(sh["body"] >= 2)[0]
    pos = b["position"][sh["body"]]
    out = []
    for i in dyn:
        d = np.linalg.norm(pos[dyn] - pos[i], axis=1)
        for j in dyn[(d < 2.5) & (dyn > i)]:
            out.append((i, j))
        out.append((0, i))
    out = np.array(out, np.int32)
    return out[rng.choice(len(out), min(count, len(out)), replace=False)]


def same(a, b):
    return all(np.array_equal(x, y) for x, y in zip(a, b))


def test_noalloc_matches_allocating_query_on_consecutive_calls():
    sc = scenes.mixed_pile(n=300, box=(8.0, 8.0, 8.0), y0=-4.0, cells=8, seed=31)
    w = world_for_scene(sc)
    rng = np.random.default_rng(5)
    first = pile_pairs(sc, rng, 3000)
    second = pile_pairs(sc, rng, 1200)
    assert len(first) > 1000 and len(second) > 500
    for pairs in (first, second):
        ref = w.collide_pairs(pairs)
        got = w.collide_pairs(pairs, noalloc=True)
        assert ref[0].sum() > 100
        assert same(ref, got)
    # bodies moved by a step: the query sees the new poses
    w.step(sc["dt"])
    assert same(w.collide_pairs(first), w.collide_pairs(first, noalloc=True))


def test_noalloc_rejects_batches_above_its_scratch():
    sc = scenes.mixed_pile(n=20, box=(8.0, 8.0, 8.0), y0=-4.0, cells=8, seed=32)
    w = world_for_scene(sc)
    pairs = np.zeros((abi.COLLIDE_NOALLOC_MAX_PAIRS + 1, 2), np.int32)
    pairs[:, 1] = len(sc["shapes"]) - 1
    with pytest.raises(JitterError) as e:
        w.collide_pairs(pairs, noalloc=True)
    assert e.value.code == abi.JG_ERR_CAPACITY
    # the largest batch it takes still runs and agrees with the allocating call
    ok = pairs[:abi.COLLIDE_NOALLOC_MAX_PAIRS]
    assert same(w.collide_pairs(ok), w.collide_pairs(ok, noalloc=True))
