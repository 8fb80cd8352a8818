"""The oracle's persistent contact cache pinned to the reference's
PersistentContactManifoldSelectionTests (Regression/PersistentContactManifoldSelectionTests.cs):
a four-point manifold registers the same four contacts in any order and keeps the points
BuildManifold chose, and a full cache given a point it already holds reuses that slot.
Contact positions are compared as RelativePosition1 + body 1's position (set equality,
squared tolerance 1e-8, and 1e-10 for the reuse case, the reference's values).
"""
import numpy as np
import pytest

import oracle_lib as O
from jitterphysics2_gb300 import abi, scenes


def _boxes():
    """Two 2x2x2 boxes, B 1.9 above A and turned a quarter of pi about y."""
    b = scenes._body(2)
    b["inv_mass"] = 1.0
    b["inv_inertia"] = (1, 0, 0, 1, 0, 1)
    b["position"][1] = (0, 1.9, 0)
    b["orientation"][1] = (0, np.sin(np.pi / 8), 0, np.cos(np.pi / 8))
    s = np.zeros(2, abi.SHAPE_DTYPE)
    s["kind"] = abi.SHAPE_BOX
    s["body"] = (0, 1)
    s["dims"][:, :3] = 1.0
    return dict(bodies=b, shapes=s, hull=np.zeros((0, 3), np.float32), triangles=np.zeros(0, abi.TRIANGLE_DTYPE))


def _manifold(sc):
    b = sc["bodies"]
    box = O.box(1.0, 1.0, 1.0)
    hit, pA, pB, n, _, _ = O.collide(box, box, b["orientation"][0], b["orientation"][1], b["position"][0],
                                     b["position"][1], mode=1)
    assert hit
    A, B = O.manifold(box, box, b["orientation"][0], b["orientation"][1], b["position"][0], b["position"][1], pA, pB, n)
    return A, B, n


def _positions(o):
    body1 = o.bodies()["position"][0].astype(np.float64)
    return [np.asarray(c["rel_pos1"], np.float64) + body1 for c in o.contacts()]


def _same_set(expected, actual, eps2):
    assert len(actual) == len(expected)
    used = [False] * len(actual)
    for e in expected:
        k = next(i for i, a in enumerate(actual) if not used[i] and np.sum((a - e) ** 2) <= eps2)
        used[k] = True


def test_four_point_manifold_registers_the_same_contacts_in_any_order():
    sc = _boxes()
    A, B, n = _manifold(sc)
    assert len(A) == 4
    first, rotated = O.OracleWorld(sc), O.OracleWorld(sc)
    first.register_manifold(0, 1, A, B, n)
    order = [(i + 2) % 4 for i in range(4)]
    rotated.register_manifold(0, 1, A[order], B[order], n)
    pa, pb = _positions(first), _positions(rotated)
    assert len(pa) == 4
    _same_set(pa, pb, 1e-8)


def test_registering_keeps_the_points_the_manifold_chose():
    sc = _boxes()
    A, B, n = _manifold(sc)
    o = O.OracleWorld(sc)
    o.register_manifold(0, 1, A, B, n)
    _same_set(list(A), _positions(o), 1e-8)


def test_a_full_cache_reuses_the_matching_slot():
    sc = _boxes()
    b = sc["bodies"]
    b["position"][1] = (0, 0, 0)
    b["orientation"][1] = (0, 0, 0, 1)
    o = O.OracleWorld(sc)
    n = np.array([0.0, 1.0, 0.0])
    pts = np.array([(-1, 0, -1), (1, 0, -1), (1, 0, 1), (-1, 0, 1)], np.float64)
    for q in pts:
        o.register_contact(0, 1, q, q - 0.1 * n, n)
    before = _positions(o)
    o.register_contact(0, 1, pts[1], pts[1] - 0.1 * n, n)
    after = _positions(o)
    assert len(after) == 4
    _same_set(before, after, 1e-10)
