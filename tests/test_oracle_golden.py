"""Pins the CPU oracle to the reference's own known-answer tests for the hot path.

Each test restates one test of src/JitterTests (cited per test) against the oracle, in
both precisions where the reference runs both (CI matrix single/double,
.github/workflows/jitter-tests.yml).  Values with explicit expectations in the
reference (SAT depths, manifold corners, the analytic penalty bias, exact orientation
signs) are checked with the reference's tolerances.
"""
import itertools
from fractions import Fraction

import numpy as np
import pytest

import oracle_lib as O
from jitterphysics2_gb300 import abi, scenes

IDQ = np.array([0.0, 0.0, 0.0, 1.0])


def qaxis(axis, angle):
    axis = np.asarray(axis, np.float64)
    axis = axis / np.linalg.norm(axis)
    s = np.sin(angle / 2)
    return np.array([axis[0] * s, axis[1] * s, axis[2] * s, np.cos(angle / 2)])


def rotate(q, v):
    x, y, z, w = q
    R = np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                  [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                  [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])
    return R @ np.asarray(v)


def qmul(a, b):
    ax, ay, az, aw = a
    bx, by, bz, bw = b
    return np.array([aw * bx + bw * ax + ay * bz - az * by, aw * by + bw * ay + az * bx - ax * bz,
                     aw * bz + bw * az + ax * by - ay * bx, aw * bw - (ax * bx + ay * by + az * bz)])


def box_sat_depth(ha, hb, q, p):
    """Minimum penetration over the 15 SAT axes of two boxes, A at the origin
    (ConvexPolytopeTests.MinimumBoxDepth, ConvexPolytopeTests.cs:176-196)."""
    axA = np.eye(3)
    axB = np.stack([rotate(q, e) for e in np.eye(3)])
    axes = list(axA) + list(axB) + [np.cross(a, b) for a in axA for b in axB]

    def sup(h, R, d, off):
        return off + R @ (np.sign(np.where(R.T @ d == 0, 1, R.T @ d)) * h)

    RA, RB = np.eye(3), axB.T
    best = np.inf
    for a in axes:
        if a @ a < 1e-12:
            continue
        a = a / np.linalg.norm(a)
        pos = sup(ha, RA, a, 0) - sup(hb, RB, -a, p)
        neg = sup(ha, RA, -a, 0) - sup(hb, RB, a, p)
        best = min(best, pos @ a, neg @ -a)
    return best


@pytest.mark.parametrize("real", ["f", "d"])
def test_collision_duplicate_support_matches_box_sat(real):
    # ConvexPolytopeTests.Collision_DuplicateSupportRegressionMatchesBoxSat (ConvexPolytopeTests.cs:164-174)
    a, b = O.box(2, 0.25, 1), O.box(0.5, 0.5, 0.5)
    q = np.array([-0.34783155, 0.69148487, -0.5953642, -0.21541446])
    pos = np.array([0.53918016, 0.12698002, -1.1122025])
    exp = box_sat_depth(np.array([2, 0.25, 1]), np.array([0.5, 0.5, 0.5]), q, pos)
    hit, _, _, n, depth, _ = O.collide(a, b, IDQ, q, np.zeros(3), pos, mode=1, real=real)
    assert hit
    assert abs(depth - exp) <= 1e-4
    assert np.all(np.isfinite(n))


@pytest.mark.parametrize("real", ["f", "d"])
@pytest.mark.parametrize("case", ["collinear", "oblique"])
def test_mprepa_regressions_match_box_sat(real, case):
    # ConvexPolytopeTests.MprEpa_CollinearSupportRegressionMatchesBoxSat / ObliqueBox (ConvexPolytopeTests.cs:198-233)
    if case == "collinear":
        h = np.array([0.3, 1.2, 0.7])
        q = np.array([0, 0.99999815, 0, -0.0019342888]) if real == "f" else np.array([0, 0.999998129169539, 0, -0.0019343364293572605])
        pos = np.array([0, 0.43866748, 0]) if real == "f" else np.array([0, 0.43866746976909576, 0])
    else:
        h = np.array([2, 0.25, 1])
        q = np.array([-0.28864738, -0.1558499, 0.15853547, -0.931268]) if real == "f" else \
            np.array([-0.28864726319747464, -0.15584983931147614, 0.15853538827229016, -0.9312680149669853])
        pos = np.array([-0.7871254, 0.20686495, -0.014221248]) if real == "f" else \
            np.array([-0.7871254097758174, 0.20686499835933464, -0.014221211987464191])
    a = O.box(*h)
    exp = box_sat_depth(h, h, q, pos)
    hit, pA, pB, n, depth, _ = O.collide(a, a, IDQ, q, np.zeros(3), pos, mode=0, real=real)
    assert hit
    assert abs(depth - exp) <= 1e-4
    # depth matches the Minkowski support along the normal
    sa = O.support(a, n, real)
    sb = rotate(q, O.support(a, rotate(np.array([-q[0], -q[1], -q[2], q[3]]), -n), real)) + pos
    assert abs((sa - sb) @ n - depth) <= 1e-4


@pytest.mark.parametrize("real", ["f", "d"])
@pytest.mark.parametrize("shape_name", ["cube", "cylinder", "flat box"])
@pytest.mark.parametrize("threshold", [0.0, 0.02])
def test_mprepa_floor_contacts_remain_exact(real, shape_name, threshold):
    # ConvexPolytopeTests.MprEpa_FloorContactsRemainExact (ConvexPolytopeTests.cs:235-263)
    shp = {"cube": O.box(0.5, 0.5, 0.5), "cylinder": O.cylinder(0.5, 1.0), "flat box": O.box(1.5, 0.1, 0.7)}[shape_name]
    floor = O.box(20, 0.5, 20)
    top = O.support(shp, [0, 1, 0], real)[1]
    wrong = []
    for depth in (0.001, 0.005, 0.01, 0.025, 0.05, 0.1):
        for yaw in range(0, 90, 3):
            q = qaxis([0, 1, 0], yaw * np.pi / 180)
            for x in range(-2, 3):
                for z in range(-2, 3):
                    pos = np.array([x * 0.37, top - depth, z * 0.53])
                    hit, _, _, n, actual, _ = O.collide(shp, floor, q, IDQ, pos, np.array([0, -0.5, 0]), threshold, 0, real)
                    if hit and np.isfinite(actual) and abs(actual - depth) <= 1e-4 and abs(n[1]) >= 0.9999:
                        continue
                    wrong.append((depth, yaw, x, z, actual, n))
    assert not wrong, wrong[:3]


@pytest.mark.parametrize("real", ["f", "d"])
def test_mprepa_depth_always_matches_its_normal(real):
    # ConvexPolytopeTests.MprEpa_DepthAlwaysMatchesItsNormal (ConvexPolytopeTests.cs:265-317); the
    # reference draws from .NET Random(11), here a seeded numpy generator draws the same distribution.
    shapes = [O.box(0.5, 0.5, 0.5), O.box(2, 0.25, 1), O.cylinder(0.5, 1.0), O.capsule(0.3, 0.5), O.sphere(0.5)]
    rng = np.random.default_rng(11)

    def rdir():
        v = rng.random(3) - 0.5
        return v / np.linalg.norm(v)

    overlapping, wrong = 0, []
    for i in range(4000):
        a, b = shapes[rng.integers(5)], shapes[rng.integers(5)]
        q = qaxis([0, 1, 0], rng.random() * 6) if i % 3 == 0 else qaxis(rdir(), rng.random() * 6)
        d = np.array([0, 1.0, 0]) if i % 3 == 0 else rdir()
        pos = d * (0.4 + rng.random() * 1.4)
        if i % 2 == 1:
            outside, inside = 6.0, 0.0
            for _ in range(40):
                mid = (outside + inside) * 0.5
                if O.collide(a, b, IDQ, q, np.zeros(3), d * mid, 1e9, 0, real)[0]:
                    inside = mid
                else:
                    outside = mid
            pos = d * (inside - rng.random() * 0.03)
        hit, _, _, n, pen, _ = O.collide(a, b, IDQ, q, np.zeros(3), pos, 0.02, 0, real)
        if not hit:
            continue
        overlapping += 1
        qc = np.array([-q[0], -q[1], -q[2], q[3]])
        sv = O.support(a, n, real) - (rotate(q, O.support(b, rotate(qc, -n), real)) + pos)
        if abs(sv @ n - pen) > 1e-3:
            wrong.append((i, pen, sv @ n))
    assert overlapping > 1000
    assert not wrong, wrong[:3]


# ---- CollisionManifold (Regression/CollisionManifoldTests.cs) --------------------------------
@pytest.mark.parametrize("real", ["f", "d"])
@pytest.mark.parametrize("radius,sphere_first", [(0.5, False), (0.5, True), (1.0, False), (1.0, True)])
def test_manifold_sphere_on_floor_keeps_original(real, radius, sphere_first):
    # SphereAgainstFloor_PreservesOriginalContact (CollisionManifoldTests.cs:101-126)
    floor, sph = O.box(100, 100, 100), O.sphere(radius)
    fpos, spos = np.array([0, -100, 0.0]), np.array([3, radius - 0.005, -2])
    fpt, spt = np.array([3, 0, -2.0]), np.array([3, -0.005, -2])
    if sphere_first:
        A, B = O.manifold(sph, floor, IDQ, IDQ, spos, fpos, spt, fpt, [0, -1, 0], real)
        exp_a, exp_b = spt, fpt
    else:
        A, B = O.manifold(floor, sph, IDQ, IDQ, fpos, spos, fpt, spt, [0, 1, 0], real)
        exp_a, exp_b = fpt, spt
    assert len(A) == 1
    assert np.abs(A[0] - exp_a).max() < 1e-5 and np.abs(B[0] - exp_b).max() < 1e-5


@pytest.mark.parametrize("real", ["f", "d"])
@pytest.mark.parametrize("radius", [0.5, 1.0])
def test_manifold_cylinder_on_floor(real, radius):
    # CylinderAgainstFloor_PreservesEndpointsAndOriginalContact (CollisionManifoldTests.cs:128-153)
    floor, cyl = O.box(100, 100, 100), O.cylinder(radius, 2.0)
    fpos, cpos = np.array([0, -100, 0.0]), np.array([10, radius - 0.005, 0])
    cq = qaxis([0, 0, 1], np.pi / 2)
    hit, pA, pB, n, _, _ = O.collide(floor, cyl, IDQ, cq, fpos, cpos, 0.02, 0, real)
    assert hit
    A, B = O.manifold(floor, cyl, IDQ, cq, fpos, cpos, pA, pB, n, real)
    assert len(A) == 3
    assert abs(abs(A[0][0] - cpos[0]) - 1) < 1e-5 and abs(abs(A[1][0] - cpos[0]) - 1) < 1e-5
    assert abs(A[0][0] - A[1][0]) > 1e-5
    assert np.abs(A[2] - pA).max() < 1e-5 and np.abs(B[2] - pB).max() < 1e-5


@pytest.mark.parametrize("real", ["f", "d"])
def test_manifold_equal_face_boxes_four_corners(real):
    # EqualFaceBoxes_ProduceFourCornerContacts (CollisionManifoldTests.cs:155-180)
    b = O.box(1, 1, 1)
    pb = np.array([0, 1.9, 0])
    hit, pA, pB, n, pen, _ = O.collide(b, b, IDQ, IDQ, np.zeros(3), pb, 0, 1, real)
    assert hit
    A, B = O.manifold(b, b, IDQ, IDQ, np.zeros(3), pb, pA, pB, n, real)
    assert len(A) == 4
    for a, bb in zip(A, B):
        assert abs(a[1] - 1.0) < 1e-4 and abs(bb[1] - 0.9) < 1e-4
        assert abs(abs(a[0]) - 1) < 1e-4 and abs(abs(a[2]) - 1) < 1e-4
        assert abs((a - bb) @ n - pen) < 1e-4
    d = np.linalg.norm(A[:, None] - A[None], axis=2) + np.eye(4)
    assert d.min() > 1e-4


@pytest.mark.parametrize("real", ["f", "d"])
@pytest.mark.parametrize("prism_first", [False, True])
def test_manifold_triangular_prism(real, prism_first):
    # TriangularFaceAgainstFloor_PreservesTriangleAndOriginalContact (CollisionManifoldTests.cs:182-209)
    floor = O.box(2, 1, 2)
    prism = O.hull([[-1, -1, -1], [1, -1, -1], [0, -1, 1], [-1, 1, -1], [1, 1, -1], [0, 1, 1]])
    fpos, ppos = np.array([0, -1, 0.0]), np.array([0, 0.995, 0])
    fpt, ppt = np.zeros(3), np.array([0, -0.005, 0])
    if prism_first:
        A, B = O.manifold(prism, floor, IDQ, IDQ, ppos, fpos, ppt, fpt, [0, -1, 0], real)
        floor_pts, last_a, last_b = B, ppt, fpt
    else:
        A, B = O.manifold(floor, prism, IDQ, IDQ, fpos, ppos, fpt, ppt, [0, 1, 0], real)
        floor_pts, last_a, last_b = A, fpt, ppt
    assert len(A) == 4
    expected = [np.array(v, float) for v in ([-1, 0, -1], [1, 0, -1], [0, 0, 1], [0, 0, 0])]
    used = set()
    for e in expected:
        m = [i for i in range(4) if i not in used and np.sum((floor_pts[i] - e) ** 2) <= 1e-10]
        assert m, (e, floor_pts)
        used.add(m[0])
    assert np.abs(A[3] - last_a).max() < 1e-5 and np.abs(B[3] - last_b).max() < 1e-5


@pytest.mark.parametrize("real", ["f", "d"])
def test_manifold_rotated_boxes_cover_all_quadrants(real):
    # RotatedFaceBoxes_IncludeIntersectionVertices / _ReductionSpansAllQuadrants
    # (CollisionManifoldTests.cs:211-273)
    b = O.box(1, 1, 1)
    qb = qaxis([0, 1, 0], np.pi / 4)
    pb = np.array([0, 1.9, 0])
    hit, pA, pB, n, pen, _ = O.collide(b, b, IDQ, qb, np.zeros(3), pb, 0, 1, real)
    assert hit
    A, B = O.manifold(b, b, IDQ, qb, np.zeros(3), pb, pA, pB, n, real)
    assert len(A) == 4
    eps = 2e-4
    quads = set()
    qc = np.array([-qb[0], -qb[1], -qb[2], qb[3]])
    for a, bb in zip(A, B):
        assert abs(a[1] - 1) < eps and abs((a - bb) @ n - pen) < eps
        assert abs(a[0]) <= 1 + eps and abs(a[2]) <= 1 + eps
        lb = rotate(qc, bb - pb)
        assert abs(lb[1] + 1) < eps and abs(lb[0]) <= 1 + eps and abs(lb[2]) <= 1 + eps
        assert abs(a[0]) > 0.05 and abs(a[2]) > 0.05
        quads.add((a[0] > 0, a[2] > 0))
    assert len(quads) == 4


@pytest.mark.parametrize("real", ["f", "d"])
def test_manifold_world_offset_invariance(real):
    # RotatedFaceBoxes_AtLargeWorldOffset_MatchNearOriginContacts (CollisionManifoldTests.cs:275-321)
    b = O.box(1, 1, 1)
    qb = qaxis([0, 1, 0], np.pi / 4)
    pb = np.array([0, 1.9, 0])
    off = np.array([10000.0, -20000.0, 30000.0])
    hit, pA, pB, n, _, _ = O.collide(b, b, IDQ, qb, np.zeros(3), pb, 0, 1, real)
    A0, B0 = O.manifold(b, b, IDQ, qb, np.zeros(3), pb, pA, pB, n, real)
    A1, B1 = O.manifold(b, b, IDQ, qb, off, off + pb, pA + off, pB + off, n, real)
    assert len(A0) == len(A1)
    for S0, S1 in ((A0, A1 - off), (B0, B1 - off)):
        for p0 in S0:
            assert np.min(np.sum((S1 - p0) ** 2, axis=1)) <= 1e-6


@pytest.mark.parametrize("real", ["f", "d"])
@pytest.mark.parametrize("box_first", [True, False])
def test_manifold_box_and_ridge(real, box_first):
    # BoxFaceAndRidge / RidgeAndBoxFace (CollisionManifoldTests.cs:323-390)
    bx = O.box(2, 2, 2)
    ridge = O.hull([[-2, -1, 0], [2, -1, 0], [-2, 1, -1], [2, 1, -1], [-2, 1, 1], [2, 1, 1]])
    if box_first:
        A, B = O.manifold(bx, ridge, IDQ, IDQ, np.zeros(3), np.array([0, 2.9, 0]), [0, 2.0, 0], [0, 1.9, 0], [0, 1, 0], real)
        ya, yb = 2.0, 1.9
    else:
        A, B = O.manifold(ridge, bx, IDQ, IDQ, np.array([0, 2.9, 0]), np.zeros(3), [0, 1.9, 0], [0, 2.0, 0], [0, -1, 0], real)
        ya, yb = 1.9, 2.0
    assert len(A) == 3
    for i in range(2):
        assert abs(A[i][1] - ya) < 1e-4 and abs(B[i][1] - yb) < 1e-4
        assert abs(abs(A[i][0]) - 2) < 1e-4 and abs(A[i][2]) < 1e-4 and abs(B[i][2]) < 1e-4
    assert np.allclose(A[2], [0, ya, 0]) and np.allclose(B[2], [0, yb, 0])


# ---- exact predicates (Behavior/ExactPredicateTests.cs + DyadicReference.cs) ------------------
def exact_sign(a, b, c, p):
    A = [[Fraction(float(x)) for x in v] for v in (a, b, c, p)]
    u = [A[0][i] - A[1][i] for i in range(3)]
    v = [A[0][i] - A[2][i] for i in range(3)]
    d = [A[3][i] - A[0][i] for i in range(3)]
    n = [u[1] * v[2] - u[2] * v[1], u[2] * v[0] - u[0] * v[2], u[0] * v[1] - u[1] * v[0]]
    s = n[0] * d[0] + n[1] * d[1] + n[2] * d[2]
    return (s > 0) - (s < 0)


@pytest.mark.parametrize("real", ["f", "d"])
def test_exact_orientation_matches_rational_arithmetic(real):
    lib = O.load()
    rng = np.random.default_rng(3)
    dt = np.float32 if real == "f" else np.float64
    cases = []
    for _ in range(300):
        a, b, c = (rng.normal(size=3) * 10 ** rng.uniform(-3, 3, size=3)).astype(dt), rng.normal(size=3).astype(dt), rng.normal(size=3).astype(dt)
        t, s = rng.random(), rng.random()
        p = (a + t * (b - a) + s * (c - a)).astype(dt)   # on the plane up to rounding: the hard cases
        cases.append((a, b, c, p))
        cases.append((a, b, c, rng.normal(size=3).astype(dt)))
    cases.append((np.array([0, 0, 0], dt), np.array([1, 0, 0], dt), np.array([0, 1, 0], dt), np.array([0.5, 0.5, 0], dt)))
    for a, b, c, p in cases:
        args = [np.ascontiguousarray(x, np.float64) for x in (a, b, c, p)]
        got = getattr(lib, "jor_exact_side_" + real)(*[O.p(x) for x in args])
        assert got == exact_sign(a, b, c, p)
        sign = np.zeros(1, np.int32)
        if getattr(lib, "jor_filter_side_" + real)(*[O.p(x) for x in args], O.p(sign)):
            assert sign[0] == got  # the filter only reports proven signs (PlaneFilter.cs:56-70)


@pytest.mark.parametrize("real", ["f", "d"])
def test_stable_math_tracks_libm(real):
    lib = O.load()
    tol = 2e-6 if real == "f" else 1e-12
    for a in np.linspace(-20, 20, 2001):
        s, c = np.zeros(1), np.zeros(1)
        getattr(lib, "jor_stable_sincos_" + real)(a, O.p(s), O.p(c))
        assert abs(s[0] - np.sin(a)) < tol * max(1, abs(a)) and abs(c[0] - np.cos(a)) < tol * max(1, abs(a))
    for y, x in itertools.product(np.linspace(-3, 3, 41), np.linspace(-3, 3, 41)):
        # the reference truncates the atan series at order 17: ~3e-9 at |x| = tan(pi/8)
        assert abs(getattr(lib, "jor_stable_atan2_" + real)(y, x) - np.arctan2(y, x)) < max(10 * tol, 1e-8)


# ---- contact solver (Regression/ContactSubstepTests.cs, Behavior/ContactLifecycleTests.cs) ----
def _two_body_scene(b1, b2):
    bodies = scenes._body(2)
    for i, b in enumerate((b1, b2)):
        for k, v in b.items():
            bodies[k][i] = v
    shapes = np.zeros(2, abi.SHAPE_DTYPE)
    shapes["kind"] = abi.SHAPE_SPHERE
    shapes["dims"][:, 0] = 0.5
    shapes["body"] = [0, 1]
    return dict(bodies=bodies, shapes=shapes, hull=np.zeros((0, 3), np.float32),
                triangles=np.zeros(0, abi.TRIANGLE_DTYPE), joints=[], params={})


@pytest.mark.parametrize("real", ["f", "d"])
def test_penalty_bias_follows_rotation_within_step(real):
    # ContactSubstepTests.RotationWithinStep_UpdatesPenetrationWithoutAddingNormalTorque (ContactSubstepTests.cs:13-47)
    tol = 1e-5 if real == "f" else 1e-12
    null = dict(motion_type=abi.MOTION_STATIC, inv_mass=0.0, inv_inertia=np.zeros(6), friction=0.0)
    inv_i = 1.0 / (0.4 * (4 / 3 * np.pi * 0.125) * 0.25)
    sph = dict(position=(0, 0.45, 0), velocity=(0, -1, 0), inv_mass=1 / (4 / 3 * np.pi * 0.125),
               inv_inertia=(inv_i, 0, 0, inv_i, 0, inv_i), friction=0.0)
    w = O.OracleWorld(_two_body_scene(null, sph), real=real)
    w.register_contact(0, 1, [0, 0, 0], [0, -0.05, 0], [0, 1, 0])
    q = qaxis([0, 0, 1], 0.3).astype(np.float32)
    w.fn("jor_world_set_orientation")(w.h, 1, O.p(q))
    w.fn("jor_world_prepare")(w.h, 0.01, 3)
    c = w.contacts()[0]
    pen = 0.5 * np.cos(0.3) - 0.45
    expected = 0.2 * 100.0 * (pen - 0.01)
    assert abs(c["penalty_bias"] - expected) < 5 * tol + 1e-6
    assert np.abs(c["rel_pos2"] + np.array([0, 0.5, 0])).max() < tol
    w.fn("jor_world_iterate")(w.h, 1)
    b = w.bodies()
    assert abs(b["velocity"][1][1] - expected) < 5 * tol + 1e-6
    assert np.linalg.norm(b["angular_velocity"][1]) < 1e-5


@pytest.mark.parametrize("real", ["f", "d"])
@pytest.mark.parametrize("bias", [False, True])
def test_contact_iteration_conserves_momentum(real, bias):
    # ContactLifecycleTests.ContactIteration_ConservesLinearAndAngularMomentum (ContactLifecycleTests.cs:15-73)
    tol = 1e-5 if real == "f" else 1e-12
    q1 = qmul(qaxis([1, 0, 0], 0.4), qaxis([0, 0, 1], 0.7))
    q2 = qmul(qaxis([0, 1, 0], 0.6), qaxis([1, 0, 0], 0.3))
    b1 = dict(position=(-0.6, 0.3, 0.4), orientation=q1, velocity=(2, 3, -1), angular_velocity=(0.2, -0.4, 0.1),
              inv_mass=0.5, inv_inertia=(1 / 3, 0, 0, 1 / 5, 0, 1 / 7), friction=0.75)
    b2 = dict(position=(0.8, -0.2, -0.5), orientation=q2, velocity=(-1, -2, 0.5), angular_velocity=(-0.3, 0.1, 0.5),
              inv_mass=1 / 3, inv_inertia=(1 / 4, 0, 0, 1 / 6, 0, 1 / 9), friction=0.75)
    w = O.OracleWorld(_two_body_scene(b1, b2), real=real)
    n = np.array([0.3, 1, -0.4]) / np.linalg.norm([0.3, 1, -0.4])
    w.register_contact(0, 1, [0.1, 0.4, 0.5], [0.1, 0.4, 0.5], n)
    w.fn("jor_world_prepare")(w.h, 0.01, 1)
    w.fn("jor_world_set_penalty")(w.h, 0, 0, 1.0)

    def inertia(i):
        out = np.zeros(6)
        w.fn("jor_world_inertia_world")(w.h, i, O.p(out))
        m = np.array([[out[0], out[1], out[2]], [out[1], out[3], out[4]], [out[2], out[4], out[5]]])
        return np.linalg.inv(m)

    I1, I2 = inertia(0), inertia(1)
    # the scene's inverse masses are stored as float32: use the masses they encode
    m1, m2 = 1.0 / float(np.float32(0.5)), 1.0 / float(np.float32(1 / 3))

    def momenta():
        b = w.bodies_d()
        x, v, av = b["position"], b["velocity"], b["angular_velocity"]
        lin = m1 * v[0] + m2 * v[1]
        ang = np.cross(x[0], m1 * v[0]) + np.cross(x[1], m2 * v[1]) + I1 @ av[0] + I2 @ av[1]
        return lin, ang

    L0, A0 = momenta()
    w0 = w.bodies_d()["angular_velocity"][0].copy()
    for _ in range(8):
        w.fn("jor_world_iterate")(w.h, 1 if bias else 0)
        L, A = momenta()
        assert np.abs(L - L0).max() < 10 * tol * 10 and np.abs(A - A0).max() < 10 * tol * 10
    c = w.contacts()[0]
    assert c["accumulated"][0] > tol
    assert abs(c["accumulated"][1]) + abs(c["accumulated"][2]) > tol
    assert np.abs(w.bodies_d()["angular_velocity"][0] - w0).max() > tol


# ---- behaviour (Behavior/StackingTests.cs) ----------------------------------------------------
def test_box_stack_stays_upright():
    # StackingTests: a 12-box stack stays standing (StackingTests.cs:22-40)
    n = 12
    bodies = scenes._body(n + 1)
    shapes = np.zeros(n + 1, abi.SHAPE_DTYPE)
    scenes.ground(bodies, shapes, 0, 0)
    shapes["kind"][1:] = abi.SHAPE_BOX
    shapes["dims"][1:, :3] = 0.5
    shapes["body"] = np.arange(n + 1)
    bodies["position"][1:] = np.stack([np.zeros(n), 0.5 + np.arange(n) * 0.999, np.zeros(n)], 1)
    scenes.set_mass(bodies, shapes, None, 1, 1)
    bodies["inv_mass"][1:] = bodies["inv_mass"][1]
    bodies["inv_inertia"][1:] = bodies["inv_inertia"][1]
    scene = dict(bodies=bodies, shapes=shapes, hull=np.zeros((0, 3), np.float32),
                 triangles=np.zeros(0, abi.TRIANGLE_DTYPE), joints=[], params=dict(substeps=4, solver_iterations=8))
    w = O.OracleWorld(scene)
    top0 = w.bodies()["position"][n].copy()
    for _ in range(600):
        w.step(0.01)
    top = w.bodies()["position"][n]
    assert np.linalg.norm(top - top0) < 1.0


@pytest.mark.parametrize("substeps", [1, 3])
def test_resting_cylinder_does_not_start_rolling(substeps):
    # ContactSubstepTests.RestingCylinder_DoesNotStartRollingWithAuxiliaryContacts
    # (Regression/ContactSubstepTests.cs:144-172): a cylinder (height 2, radius 0.5) on its
    # side, 0.005 into a static floor, no damping, 4 + 2 iterations, auxiliary contacts on
    bodies = scenes._body(2)
    shapes = np.zeros(2, abi.SHAPE_DTYPE)
    scenes.ground(bodies, shapes, 0, 0, size=(200.0, 200.0, 200.0), y=-100.0)
    shapes["kind"][1] = abi.SHAPE_CYLINDER
    shapes["body"][1] = 1
    shapes["dims"][1, :2] = (0.5, 2.0)
    scenes.set_mass(bodies, shapes, None, 1, 1)
    bodies["position"][1] = (10.0, 0.495, 0.0)
    bodies["orientation"][1] = (0.0, 0.0, np.sin(np.pi / 4), np.cos(np.pi / 4))
    bodies["linear_damping"] = bodies["angular_damping"] = 1.0
    bodies["restitution"] = 0.0
    sc = dict(bodies=bodies, shapes=shapes, hull=np.zeros((0, 3), np.float32), triangles=np.zeros(0, abi.TRIANGLE_DTYPE),
              params=dict(substeps=substeps, solver_iterations=4, relax_iterations=2))
    w = O.OracleWorld(sc)
    for _ in range(1000):
        w.step(0.01)
    b = w.bodies()
    assert np.linalg.norm(b["velocity"][1]) < 0.02
    assert np.linalg.norm(b["angular_velocity"][1]) < 0.04
    assert abs(b["position"][1][1] - 0.495) < 0.001


def test_cached_contact_offsets_are_current_after_each_step():
    # ContactSubstepTests.CachedContact_KeepsOffsetsFixedUntilSolvingFinishes
    # (Regression/ContactSubstepTests.cs:48-92), its after-step half: detection rejected
    # (steps without narrowphase), a spinning sphere's registered contact keeps one cached
    # point whose body-2 offset is the current rotation of the registered point
    null = dict(motion_type=abi.MOTION_STATIC, inv_mass=0.0, inv_inertia=np.zeros(6), position=(0, -1, 0))
    inv_i = 1.0 / (0.4 * (4 / 3 * np.pi * 0.125) * 0.25)
    ball = dict(angular_velocity=(0, 0, 1), inv_mass=1 / (4 / 3 * np.pi * 0.125), inv_inertia=(inv_i, 0, 0, inv_i, 0, inv_i),
                linear_damping=1.0, angular_damping=1.0, flags=abi.BODY_ACTIVE | abi.BODY_NO_GRAVITY)
    sc = _two_body_scene(null, ball)
    sc["params"] = dict(substeps=3, gravity=(0.0, 0.0, 0.0))
    w = O.OracleWorld(sc)
    point = np.array([0.0, -0.5, 0.0])
    w.register_contact(0, 1, point, point, [0, 1, 0])
    for _ in range(2):
        w.step(0.01, narrow=False)
        q = w.bodies()["orientation"][1].astype(np.float64)
        x, y, z, s = q
        R = np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * s), 2 * (x * z + y * s)],
                      [2 * (x * y + z * s), 1 - 2 * (x * x + z * z), 2 * (y * z - x * s)],
                      [2 * (x * z - y * s), 2 * (y * z + x * s), 1 - 2 * (x * x + y * y)]])
        c = w.contacts()
        assert len(c) == 1
        assert np.abs(c[0]["rel_pos2"] - R @ point).max() < 1e-5


# ---- locked motion axes (Behavior/AllowedMotionTests.cs) -------------------------------------
LIN_X, LIN_Y, LIN_Z, ANG = 1, 2, 4, 56


def _locked_body_scene(allowed, **fields):
    """AllowedMotionTests' world and body: no gravity, one substep, no damping, inverse
    mass 0.5 and zero inverse inertia, plus a static body 0 at the origin."""
    bodies = scenes._body(2)
    bodies["motion_type"][0] = abi.MOTION_STATIC
    bodies["inv_mass"][0] = 0.0
    bodies["inv_inertia"][0] = 0.0
    bodies["inv_mass"][1] = 0.5
    bodies["inv_inertia"][1] = 0.0
    bodies["linear_damping"] = bodies["angular_damping"] = 1.0
    bodies["flags"][1] = abi.BODY_ACTIVE | ((63 ^ allowed) << abi.BODY_LOCKS_SHIFT)
    bodies["friction"] = 0.0
    for k, v in fields.items():
        bodies[k][1] = v
    shapes = np.zeros(2, abi.SHAPE_DTYPE)
    shapes["kind"] = abi.SHAPE_SPHERE
    shapes["dims"][:, 0] = 0.5
    shapes["body"] = [0, 1]
    return dict(bodies=bodies, shapes=shapes, hull=np.zeros((0, 3), np.float32),
                triangles=np.zeros(0, abi.TRIANGLE_DTYPE), joints=[],
                params=dict(substeps=1, solver_iterations=1, relax_iterations=0, gravity=(0.0, 0.0, 0.0)))


def test_forces_and_gravity_respect_locked_axes_across_substeps():
    # AllowedMotionTests.ForcesAndGravity_RespectWorldAxesAcrossSubsteps (:143-167): the force
    # and gravity become velocity deltas at the end of a step and act in the next one
    sc = _locked_body_scene(63 ^ LIN_Y, position=(1, 2, 3), orientation=(0, 0, np.sin(0.6), np.cos(0.6)),
                            force=(2, 4, 6))
    sc["bodies"]["flags"][1] &= ~abi.BODY_NO_GRAVITY
    sc["params"].update(substeps=4, gravity=(3.0, 4.0, 5.0))
    w = O.OracleWorld(sc)
    dt = 1.0 / 60.0
    w.step(dt)
    w.step(dt)
    b = w.bodies()
    assert b["velocity"][1][0] == pytest.approx(4 * dt, abs=1e-5)
    assert b["velocity"][1][1] == 0.0
    assert b["velocity"][1][2] == pytest.approx(8 * dt, abs=1e-5)
    assert b["position"][1][1] == 2.0


def test_oblique_contact_uses_the_directional_mass():
    # AllowedMotionTests.ObliqueContact_UsesDirectionalMassInOneIteration (:215-240)
    sc = _locked_body_scene(LIN_Y | ANG, velocity=(0, -3, 0))
    w = O.OracleWorld(sc)
    n = np.array([1.0, 1.0, 0.0]) / np.sqrt(2.0)
    w.register_contact(0, 1, [0, 0, 0], [0, 0, 0], n)
    w.fn("jor_world_prepare")(w.h, 0.01, 1)
    w.fn("jor_world_iterate")(w.h, 0)
    assert np.abs(w.bodies()["velocity"][1]).max() < 1e-5
    c = w.contacts()[0]
    assert c["mass"][0] == pytest.approx(4.0, abs=1e-5)
    assert c["mass"][2] == 0.0


def test_completely_blocked_contact_stays_finite():
    # AllowedMotionTests.CompletelyBlockedContact_RemainsFinite (:242-268)
    sc = _locked_body_scene(0)
    w = O.OracleWorld(sc)
    w.register_contact(0, 1, [0, 0, 0], [0, 0, 0], [0, 1, 0])
    w.fn("jor_world_set_penalty")(w.h, 0, 0, 1.0)
    w.fn("jor_world_prepare")(w.h, 0.01, 1)
    for _ in range(3):
        w.fn("jor_world_iterate")(w.h, 1)
    b = w.bodies()
    np.testing.assert_array_equal(b["velocity"][1], 0.0)
    np.testing.assert_array_equal(b["angular_velocity"][1], 0.0)
    c = w.contacts()[0]
    assert c["accumulated"][0] == 0.0 and c["accumulated"][1] == 0.0


def test_a_force_changes_velocity_two_steps_later():
    # ForceImpulseTests.AddForce_ChangesVelocityAfterStep (Behavior/ForceImpulseTests.cs:126-143)
    sc = _locked_body_scene(63)
    sc["bodies"]["inv_mass"][1] = 1.0
    sc["bodies"]["position"][0] = (0, -100, 0)     # the body alone, as in the reference's world
    w = O.OracleWorld(sc)
    w.step(1.0 / 60.0)
    b = w.bodies()
    b["force"][1] = (100, 0, 0)
    w.set_bodies(b)
    w.step(1.0 / 60.0)
    assert w.bodies()["velocity"][1][0] == 0.0
    w.step(1.0 / 60.0)
    assert w.bodies()["velocity"][1][0] > 0.0


POINTONPLANE = 7    # restated in the oracle ahead of its device row


@pytest.mark.parametrize("kind", ["DistanceLimit", "BallSocket", "PointOnPlane"])
def test_joint_stops_the_permitted_velocity_in_one_iteration(kind):
    # AllowedMotionTests.Joint_StopsPermittedVelocityInOneIteration (:316-372), the kinds the
    # oracle has: one step, one iteration, a body free to move along y only
    axis = np.array([1.0, 2.0, 3.0]) / np.sqrt(14.0)
    pos = axis if kind == "DistanceLimit" else np.zeros(3)
    sc = _locked_body_scene(LIN_Y | ANG, velocity=(0, -3, 0), position=pos)
    sc["shapes"] = sc["shapes"][1:]   # the static body has no shape: nothing collides
    w = O.OracleWorld(sc)
    if kind == "DistanceLimit":
        j = w.add_joint(abi.CONSTRAINT_DISTANCELIMIT, 0, 1, (0, 0, 0) + tuple(pos) + (1e-6, -1e-6))
    elif kind == "PointOnPlane":
        j = w.add_joint(POINTONPLANE, 0, 1, tuple(axis) + (0, 0, 0, 0, 0, 0, 1e-6, -1e-6))
    else:
        j = w.add_joint(abi.CONSTRAINT_BALLSOCKET, 0, 1, (0, 0, 0))
    w.joint_params(j, 0.0, 0.0)
    w.step(0.01)
    v = w.bodies()["velocity"][1]
    assert v[0] == 0.0 and v[2] == 0.0 and abs(v[1]) < 1e-5


@pytest.mark.parametrize("linear_locks", [False, True])
def test_solve_mode_flags_mask_each_body_update(linear_locks):
    # AllowedMotionTests.AllSolveModes... (:262-314): every ContactData.Mode combination updates
    # exactly the bodies and parts it names
    n = np.array([1.0, 1.0, 0.0]) / np.sqrt(2.0) if linear_locks else np.array([1.0, 0.0, 0.0])
    for bits in range(16):
        bodies = scenes._body(2)
        bodies["inv_mass"] = (0.5, 0.25)
        bodies["inv_inertia"] = 0.0
        bodies["linear_damping"] = bodies["angular_damping"] = 1.0
        bodies["friction"] = bodies["restitution"] = 0.0
        if linear_locks:
            bodies["flags"] = abi.BODY_ACTIVE | (LIN_Y << abi.BODY_LOCKS_SHIFT)
        bodies["velocity"][0] = (1, 0, 0)
        shapes = np.zeros(2, abi.SHAPE_DTYPE)
        shapes["kind"] = abi.SHAPE_SPHERE
        shapes["dims"][:, 0] = 0.5
        shapes["body"] = [0, 1]
        sc = dict(bodies=bodies, shapes=shapes, hull=np.zeros((0, 3), np.float32), triangles=np.zeros(0, abi.TRIANGLE_DTYPE))
        w = O.OracleWorld(sc)
        w.register_contact(0, 1, [0, 0, 0], [0, 0, 0], n)
        w.fn("jor_world_set_arbiter_mode")(w.h, 0, bits)
        w.fn("jor_world_prepare")(w.h, 0.01, 1)
        w.fn("jor_world_iterate")(w.h, 0)
        b = w.bodies()
        lin1, lin2 = bool(bits & 1), bool(bits & 4)
        inv = (0.5 if lin1 else 0.0) + (0.25 if lin2 else 0.0)
        imp = 1.0 / inv if inv > 0 else 0.0
        e1 = np.array([1.0 - (0.5 * imp if lin1 else 0.0), 0, 0])
        e2 = np.array([0.25 * imp if lin2 else 0.0, 0, 0])
        assert np.abs(b["velocity"][0] - e1).max() < 1e-5, bits
        assert np.abs(b["velocity"][1] - e2).max() < 1e-5, bits
        np.testing.assert_array_equal(b["angular_velocity"][:2], 0.0)


def test_point_on_plane_pulls_a_body_onto_its_plane():
    # AdditionalConstraintBehaviorTests.PointOnPlane_ReducesDistanceToPlane (:86-113): a unit
    # sphere 3 above the plane y = 0 of a static body, no gravity, 4 substeps, 2 seconds
    bodies = scenes._body(2)
    shapes = np.zeros(2, abi.SHAPE_DTYPE)
    shapes["kind"] = abi.SHAPE_SPHERE
    shapes["dims"][:, 0] = 1.0
    shapes["body"] = [0, 1]
    scenes.set_mass(bodies, shapes, None, 1, 1)
    bodies["motion_type"][0] = abi.MOTION_STATIC
    bodies["inv_mass"][0] = 0.0
    bodies["inv_inertia"][0] = 0.0
    bodies["position"][1] = (1, 3, 2)
    sc = dict(bodies=bodies, shapes=shapes, hull=np.zeros((0, 3), np.float32), triangles=np.zeros(0, abi.TRIANGLE_DTYPE),
              params=dict(substeps=4, gravity=(0.0, 0.0, 0.0)))
    w = O.OracleWorld(sc)
    w.add_joint(POINTONPLANE, 0, 1, (0, 1, 0, 0, 0, 0, 1, 3, 2, 1e-6, -1e-6))
    for _ in range(200):
        w.step(0.01)
    y = abs(float(w.bodies()["position"][1][1]))
    assert y < 3.0 and y < 0.2


def test_hinge_limit_reduces_rotation():
    # AdditionalConstraintBehaviorTests.HingeAngle_LimitReducesRotationComparedToUnconstrained
    # (:115-155): a unit sphere spun at 8 rad/s about y for 10 steps, with and without a
    # hinge about y limited to +-10 degrees
    def run(constrained):
        bodies = scenes._body(2)
        shapes = np.zeros(1, abi.SHAPE_DTYPE)
        shapes["kind"] = abi.SHAPE_SPHERE
        shapes["dims"][0, 0] = 1.0
        shapes["body"] = 1
        scenes.set_mass(bodies, shapes, None, 1, 0)
        bodies["motion_type"][0] = abi.MOTION_STATIC
        bodies["inv_mass"][0] = 0.0
        bodies["inv_inertia"][0] = 0.0
        bodies["position"][0] = (0, -50, 0)
        bodies["angular_velocity"][1] = (0, 8, 0)
        sc = dict(bodies=bodies, shapes=shapes, hull=np.zeros((0, 3), np.float32),
                  triangles=np.zeros(0, abi.TRIANGLE_DTYPE), params=dict(substeps=4, gravity=(0.0, 0.0, 0.0)))
        w = O.OracleWorld(sc)
        if constrained:
            w.add_joint(abi.CONSTRAINT_HINGEANGLE, 0, 1, (0, 1, 0, -np.radians(10), np.radians(10)))
        for _ in range(10):
            w.step(0.01)
        return 2.0 * np.arccos(np.clip(abs(float(w.bodies()["orientation"][1][3])), 0.0, 1.0))

    free, held = run(False), run(True)
    assert free > 0.4 and held < free and held < 0.4


ANGULARMOTOR = 8    # restated in the oracle ahead of its device row


def test_angular_motor_drives_toward_its_target():
    # AdditionalConstraintBehaviorTests.AngularMotor_DrivesAngularVelocityTowardTarget (:30-52):
    # target 3 rad/s about y, at most 100 N m, one second, 4 substeps, no gravity
    bodies = scenes._body(2)
    shapes = np.zeros(1, abi.SHAPE_DTYPE)
    shapes["kind"] = abi.SHAPE_SPHERE
    shapes["dims"][0, 0] = 1.0
    shapes["body"] = 1
    scenes.set_mass(bodies, shapes, None, 1, 0)
    bodies["motion_type"][0] = abi.MOTION_STATIC
    bodies["inv_mass"][0] = 0.0
    bodies["inv_inertia"][0] = 0.0
    bodies["position"][0] = (0, -50, 0)
    sc = dict(bodies=bodies, shapes=shapes, hull=np.zeros((0, 3), np.float32),
              triangles=np.zeros(0, abi.TRIANGLE_DTYPE), params=dict(substeps=4, gravity=(0.0, 0.0, 0.0)))
    w = O.OracleWorld(sc)
    w.add_joint(ANGULARMOTOR, 0, 1, (0, 1, 0, 0, 1, 0, 3.0, 100.0))
    for _ in range(100):
        w.step(0.01)
    assert w.bodies()["angular_velocity"][1][1] == pytest.approx(3.0, abs=0.3)


LINEARMOTOR = 9     # restated in the oracle ahead of its device row


def test_linear_motor_drives_toward_its_target():
    # AdditionalConstraintBehaviorTests.LinearMotor_DrivesBodyTowardTargetVelocity (:7-28):
    # target 2 m/s along x, at most 100 N, one second, 4 substeps, no gravity
    bodies = scenes._body(2)
    shapes = np.zeros(1, abi.SHAPE_DTYPE)
    shapes["kind"] = abi.SHAPE_SPHERE
    shapes["dims"][0, 0] = 1.0
    shapes["body"] = 1
    scenes.set_mass(bodies, shapes, None, 1, 0)
    bodies["motion_type"][0] = abi.MOTION_STATIC
    bodies["inv_mass"][0] = 0.0
    bodies["inv_inertia"][0] = 0.0
    bodies["position"][0] = (0, -50, 0)
    sc = dict(bodies=bodies, shapes=shapes, hull=np.zeros((0, 3), np.float32),
              triangles=np.zeros(0, abi.TRIANGLE_DTYPE), params=dict(substeps=4, gravity=(0.0, 0.0, 0.0)))
    w = O.OracleWorld(sc)
    w.add_joint(LINEARMOTOR, 0, 1, (1, 0, 0, 1, 0, 0, 2.0, 100.0))
    for _ in range(100):
        w.step(0.01)
    assert w.bodies()["velocity"][1][0] == pytest.approx(2.0, abs=0.2)
