"""Direct GPU parity checks of rows the pile tests cover only in aggregate, through the C ABI:

- the broadphase pair list of a step against the oracle's exact pair set
  (DynamicTree.EnumerateOverlapsCallback, DynamicTree.cs:266-286, with World.cs:447-455):
  index work, so the two sets must be equal;
- the reference's CollisionManifold known-answer cases (CollisionManifoldTests.cs:101-390)
  run through the device's manifold function (jg_manifold_pairs), against the oracle's
  BuildManifold and the cases' expected points;
- the persistent contact cache over consecutive steps from identical states, slot by slot:
  AddContact merging into full caches (Contact.cs:329-416) and the usage masks that
  UpdatePosition leaves (Contact.cs:238-264);
- the gyroscopic integration branch (World.Step.cs:1075-1104) against the oracle, bit for bit;
- bodies resting on the heightfield's internal edges, where the triangle-edge filter
  (TriangleEdgeCollisionFilter.cs:243-420) decides the contacts, against the oracle.
"""
import numpy as np
import pytest

import oracle_lib as O
from jitterphysics2_gb300 import abi, scenes
from jitterphysics2_gb300.world import world_for_scene
from test_gpu_parity import _settled_pile, compare_contact_caches

pytestmark = pytest.mark.gpu
IDQ = np.array([0, 0, 0, 1.0])


def qaxis(axis, angle):
    a = np.asarray(axis, float) / np.linalg.norm(axis)
    return np.array([*(a * np.sin(angle / 2)), np.cos(angle / 2)])


def two_shape_scene(a, b, qa, qb, pa, pb):
    """A world of two bodies holding shapes a and b (oracle_lib shape records, with hull
    points for point clouds) at the given poses."""
    bodies = scenes._body(2)
    shapes = np.zeros(2, abi.SHAPE_DTYPE)
    hull = []
    for i, (s, q, p) in enumerate(((a, qa, pa), (b, qb, pb))):
        rec, pts = (s[0], s[1]) if isinstance(s, tuple) else (s, None)
        shapes[i] = rec[0]
        shapes["body"][i] = i
        if pts is not None:
            shapes["data_offset"][i] = sum(len(h) for h in hull)
            hull.append(np.asarray(pts, np.float32))
        bodies["position"][i] = np.asarray(p, np.float32)
        bodies["orientation"][i] = np.asarray(q, np.float32)
        bodies["inv_mass"][i] = 1.0
        bodies["inv_inertia"][i] = (1, 0, 0, 1, 0, 1)
    return dict(bodies=bodies, shapes=shapes, hull=np.concatenate(hull) if hull else np.zeros((0, 3), np.float32),
                triangles=np.zeros(0, abi.TRIANGLE_DTYPE), joints=[], params=dict(gravity=(0.0, 0.0, 0.0)), dt=0.01)


def f32(x):
    return np.asarray(x, np.float32).astype(np.float64)


def gpu_and_oracle_manifold(a, b, qa, qb, pa, pb, pA, pB, n):
    qa, qb, pa, pb, pA, pB, n = (f32(x) for x in (qa, qb, pa, pb, pA, pB, n))
    w = world_for_scene(two_shape_scene(a, b, qa, qb, pa, pb))
    (GA, GB), = w.manifold_pairs(np.array([[0, 1]], np.int32), np.concatenate([pA, pB, n])[None])
    w.close()
    OA, OB = O.manifold(a, b, qa, qb, pa, pb, pA, pB, n, "f")
    assert len(GA) == len(OA), (GA, OA)
    assert np.abs(GA - OA).max(initial=0) <= 1e-6 and np.abs(GB - OB).max(initial=0) <= 1e-6, (GA, OA)
    return GA.astype(np.float64), GB.astype(np.float64)


def gpu_collide(a, b, qa, qb, pa, pb):
    w = world_for_scene(two_shape_scene(a, b, f32(qa), f32(qb), f32(pa), f32(pb)))
    hit, pA, pB, n, pen = w.collide_pairs(np.array([[0, 1]], np.int32))
    w.close()
    return bool(hit[0]), pA[0], pB[0], n[0], float(pen[0])


@pytest.mark.parametrize("radius,sphere_first", [(0.5, False), (1.0, True)])
def test_manifold_sphere_on_floor_on_the_device(radius, sphere_first):
    # SphereAgainstFloor_PreservesOriginalContact (CollisionManifoldTests.cs:101-126)
    floor, sph = O.box(100, 100, 100), O.sphere(radius)
    fpos, spos = np.array([0, -100, 0.0]), np.array([3, radius - 0.005, -2])
    fpt, spt = np.array([3, 0, -2.0]), np.array([3, -0.005, -2])
    if sphere_first:
        A, B = gpu_and_oracle_manifold(sph, floor, IDQ, IDQ, spos, fpos, spt, fpt, [0, -1, 0])
        exp_a, exp_b = spt, fpt
    else:
        A, B = gpu_and_oracle_manifold(floor, sph, IDQ, IDQ, fpos, spos, fpt, spt, [0, 1, 0])
        exp_a, exp_b = fpt, spt
    assert len(A) == 1 and np.abs(A[0] - exp_a).max() < 1e-5 and np.abs(B[0] - exp_b).max() < 1e-5


def test_manifold_cylinder_on_floor_on_the_device():
    # CylinderAgainstFloor_PreservesEndpointsAndOriginalContact (CollisionManifoldTests.cs:128-153)
    floor, cyl = O.box(100, 100, 100), O.cylinder(0.5, 2.0)
    fpos, cpos, cq = np.array([0, -100, 0.0]), np.array([10, 0.495, 0]), qaxis([0, 0, 1], np.pi / 2)
    hit, pA, pB, n, _ = gpu_collide(floor, cyl, IDQ, cq, fpos, cpos)
    assert hit
    A, B = gpu_and_oracle_manifold(floor, cyl, IDQ, cq, fpos, cpos, pA, pB, n)
    assert len(A) == 3
    assert abs(abs(A[0][0] - cpos[0]) - 1) < 1e-5 and abs(abs(A[1][0] - cpos[0]) - 1) < 1e-5
    assert abs(A[0][0] - A[1][0]) > 1e-5
    assert np.abs(A[2] - pA).max() < 1e-5 and np.abs(B[2] - pB).max() < 1e-5


def test_manifold_equal_face_boxes_on_the_device():
    # EqualFaceBoxes_ProduceFourCornerContacts (CollisionManifoldTests.cs:155-180)
    b, pb = O.box(1, 1, 1), np.array([0, 1.9, 0])
    hit, pA, pB, n, pen = gpu_collide(b, b, IDQ, IDQ, np.zeros(3), pb)
    assert hit
    A, B = gpu_and_oracle_manifold(b, b, IDQ, IDQ, np.zeros(3), pb, pA, pB, n)
    assert len(A) == 4
    for a, bb in zip(A, B):
        assert abs(a[1] - 1.0) < 1e-4 and abs(bb[1] - 0.9) < 1e-4
        assert abs(abs(a[0]) - 1) < 1e-4 and abs(abs(a[2]) - 1) < 1e-4
        assert abs((a - bb) @ n - pen) < 1e-4


@pytest.mark.parametrize("prism_first", [False, True])
def test_manifold_triangular_prism_on_the_device(prism_first):
    # TriangularFaceAgainstFloor_PreservesTriangleAndOriginalContact (CollisionManifoldTests.cs:182-209)
    floor = O.box(2, 1, 2)
    prism = O.hull([[-1, -1, -1], [1, -1, -1], [0, -1, 1], [-1, 1, -1], [1, 1, -1], [0, 1, 1]])
    fpos, ppos = np.array([0, -1, 0.0]), np.array([0, 0.995, 0])
    fpt, ppt = np.zeros(3), np.array([0, -0.005, 0])
    if prism_first:
        A, B = gpu_and_oracle_manifold(prism, floor, IDQ, IDQ, ppos, fpos, ppt, fpt, [0, -1, 0])
        floor_pts, last_a, last_b = B, ppt, fpt
    else:
        A, B = gpu_and_oracle_manifold(floor, prism, IDQ, IDQ, fpos, ppos, fpt, ppt, [0, 1, 0])
        floor_pts, last_a, last_b = A, fpt, ppt
    assert len(A) == 4
    used = set()
    for e in ([-1, 0, -1], [1, 0, -1], [0, 0, 1], [0, 0, 0]):
        m = [i for i in range(4) if i not in used and np.sum((floor_pts[i] - e) ** 2) <= 1e-10]
        assert m, (e, floor_pts)
        used.add(m[0])
    assert np.abs(A[3] - last_a).max() < 1e-5 and np.abs(B[3] - last_b).max() < 1e-5


def test_manifold_rotated_boxes_on_the_device():
    # RotatedFaceBoxes_IncludeIntersectionVertices / _ReductionSpansAllQuadrants (CollisionManifoldTests.cs:211-273)
    b, qb, pb = O.box(1, 1, 1), qaxis([0, 1, 0], np.pi / 4), np.array([0, 1.9, 0])
    hit, pA, pB, n, pen = gpu_collide(b, b, IDQ, qb, np.zeros(3), pb)
    assert hit
    A, B = gpu_and_oracle_manifold(b, b, IDQ, qb, np.zeros(3), pb, pA, pB, n)
    assert len(A) == 4
    quads = set()
    for a, bb in zip(A, B):
        assert abs(a[1] - 1) < 2e-4 and abs((a - bb) @ n - pen) < 2e-4
        assert abs(a[0]) > 0.05 and abs(a[2]) > 0.05
        quads.add((a[0] > 0, a[2] > 0))
    assert len(quads) == 4


@pytest.mark.parametrize("box_first", [True, False])
def test_manifold_box_and_ridge_on_the_device(box_first):
    # BoxFaceAndRidge / RidgeAndBoxFace (CollisionManifoldTests.cs:323-390)
    bx = O.box(2, 2, 2)
    ridge = O.hull([[-2, -1, 0], [2, -1, 0], [-2, 1, -1], [2, 1, -1], [-2, 1, 1], [2, 1, 1]])
    if box_first:
        A, B = gpu_and_oracle_manifold(bx, ridge, IDQ, IDQ, np.zeros(3), [0, 2.9, 0], [0, 2.0, 0], [0, 1.9, 0], [0, 1, 0])
        ya, yb = 2.0, 1.9
    else:
        A, B = gpu_and_oracle_manifold(ridge, bx, IDQ, IDQ, [0, 2.9, 0], np.zeros(3), [0, 1.9, 0], [0, 2.0, 0], [0, -1, 0])
        ya, yb = 1.9, 2.0
    assert len(A) == 3
    for i in range(2):
        assert abs(A[i][1] - ya) < 1e-4 and abs(B[i][1] - yb) < 1e-4
        assert abs(abs(A[i][0]) - 2) < 1e-4 and abs(A[i][2]) < 1e-4
    assert np.allclose(A[2], [0, ya, 0]) and np.allclose(B[2], [0, yb, 0])


def test_broadphase_pair_set_equals_the_oracles():
    # a formed pile over the heightfield: body-body, body-ground and body-triangle pairs
    sc = scenes.mixed_pile(n=2000, box=(30.0, 10.0, 30.0), y0=0.0, cells=16, seed=23, lattice=2.0)
    w = world_for_scene(sc)
    for _ in range(120):
        w.step(sc["dt"])
    sc2 = dict(sc)
    sc2["bodies"] = w.bodies()
    g = world_for_scene(sc2)
    g.step(sc["dt"])
    norm = lambda p: {(int(min(a, b)), int(max(a, b))) for a, b in p}
    gp, op = norm(g.pairs()), norm(O.OracleWorld(sc2).pairs())
    assert len(gp) > 3000
    tri = {p for p in gp if sc["shapes"]["kind"][p[0]] == abi.SHAPE_TRIANGLE or sc["shapes"]["kind"][p[1]] == abi.SHAPE_TRIANGLE}
    assert len(tri) > 50
    assert gp == op, (len(gp), len(op), sorted(gp - op)[:5], sorted(op - gp)[:5])


def test_contact_cache_follows_the_oracle_over_steps():
    """Six consecutive steps, each replayed by the oracle from the GPU's state before it in
    the GPU's order: the caches agree slot by slot (usage masks after the break test,
    contact points, normals, accumulated impulses) while full caches take new points."""
    sc, w = _settled_pile(n=400, steps=200, seed=19)
    full = replaced = 0
    for _ in range(6):
        b0, c0 = w.bodies(), w.contacts()
        w.step(sc["dt"])
        c1 = w.contacts()
        o = O.OracleWorld(sc, external_order=True)
        o.set_bodies(b0)
        o.set_contacts(c0)
        o.narrowphase()
        for c in c1:
            o.set_arbiter_color(c["shape1"], c["shape2"], c["color"])
        o.step(sc["dt"], narrow=False)
        oc = o.contacts()
        stats = compare_contact_caches(c1, oc)
        assert stats["common_keys"] >= 0.999 * stats["keys"] and stats["slot_mismatch"] <= 0.001 * stats["keys"], stats
        assert stats["normal_ok"] >= 0.999 and stats["point_ok"] >= 0.999, stats
        G = {(int(r["shape1"]), int(r["shape2"]), int(r["slot"])): r for r in c1}
        Om = {(int(r["shape1"]), int(r["shape2"]), int(r["slot"])): r for r in oc}
        keys = set(G) & set(Om)
        mask_ok = np.mean([G[k]["usage_mask"] == Om[k]["usage_mask"] for k in keys])
        imp = np.array([np.abs(G[k]["accumulated"] - Om[k]["accumulated"]).max() / max(1.0, np.abs(Om[k]["accumulated"]).max())
                        for k in keys])
        assert mask_ok >= 0.999 and np.mean(imp < 1e-3) >= 0.999, (mask_ok, np.sort(imp)[-5:])
        full += sum(1 for r in c0 if (r["usage_mask"] & 15) == 15)
        before = {(int(r["shape1"]), int(r["shape2"]), int(r["slot"])): r["pos1_local"] for r in c0}
        replaced += sum(1 for k in keys if k in before and np.abs(before[k] - G[k]["pos1_local"]).max() > 1e-3)
    assert full > 100 and replaced > 10, (full, replaced)


def test_gyroscopic_integration_matches_the_oracle_bitwise():
    # asymmetric boxes spinning about a non-principal axis in free space, gyroscopic term on
    n = 24
    bodies = scenes._body(n)
    shapes = np.zeros(n, abi.SHAPE_DTYPE)
    rng = np.random.default_rng(5)
    for i in range(n):
        shapes[i]["kind"], shapes[i]["body"] = abi.SHAPE_BOX, i
        shapes[i]["dims"][:3] = rng.uniform(0.1, 1.0, 3)
        scenes.set_mass(bodies, shapes, np.zeros((0, 3), np.float32), i, i)
        bodies["position"][i] = (4.0 * i, 10.0, 0.0)
        bodies["angular_velocity"][i] = rng.uniform(-8, 8, 3)
    bodies["orientation"][:] = scenes.random_quaternions(rng, n)
    bodies["flags"] |= abi.BODY_GYROSCOPIC | abi.BODY_NO_GRAVITY
    bodies["angular_damping"] = 1.0
    sc = dict(bodies=bodies, shapes=shapes, hull=np.zeros((0, 3), np.float32), triangles=np.zeros(0, abi.TRIANGLE_DTYPE),
              joints=[], params=dict(substeps=4, solver_iterations=8, relax_iterations=4), dt=0.01)
    g, o = world_for_scene(sc), O.OracleWorld(sc)
    for _ in range(50):
        g.step(sc["dt"])
        o.step(sc["dt"])
    gb, ob = g.bodies(), o.bodies()
    start = np.linalg.norm(bodies["angular_velocity"], axis=1)
    assert np.abs(np.linalg.norm(gb["angular_velocity"], axis=1) - start).max() > 1e-3  # the term acted
    assert np.array_equal(gb["angular_velocity"], ob["angular_velocity"])
    assert np.array_equal(gb["orientation"], ob["orientation"])


def test_bodies_on_heightfield_edges_match_the_oracle():
    """Small spheres and boxes resting across the heightfield's internal edges and vertices,
    where the triangle-edge filter decides every contact: the step's contact cache against
    the oracle's."""
    sc = dict(scenes.mixed_pile(n=10, box=(20.0, 4.0, 20.0), y0=0.0, cells=16, seed=29))
    tris = sc["triangles"]
    rng = np.random.default_rng(7)
    # points on shared edges: midpoints of each triangle's edges, the heightfield is static at the origin
    mids = np.concatenate([(tris["a"] + tris["b"]) / 2, (tris["b"] + tris["c"]) / 2, (tris["c"] + tris["a"]) / 2])
    pick = mids[rng.choice(len(mids), 600, replace=False)]
    n = len(pick)
    bodies = scenes._body(n + 2)
    bodies[:2] = sc["bodies"][:2]
    nt = len(tris)
    shapes = np.zeros(1 + nt + n, abi.SHAPE_DTYPE)
    shapes[:1 + nt] = sc["shapes"][:1 + nt]
    for i in range(n):
        si, bi = 1 + nt + i, 2 + i
        shapes[si]["body"] = bi
        if i % 2:
            shapes[si]["kind"], shapes[si]["dims"][0] = abi.SHAPE_SPHERE, 0.15
            bodies["position"][bi] = pick[i] + (0, 0.145, 0)
        else:
            shapes[si]["kind"], shapes[si]["dims"][:3] = abi.SHAPE_BOX, 0.12
            bodies["position"][bi] = pick[i] + (0, 0.1, 0)
        scenes.set_mass(bodies, shapes, np.zeros((0, 3), np.float32), bi, si)
    sc2 = dict(sc, bodies=bodies, shapes=shapes, hull=np.zeros((0, 3), np.float32))
    g = world_for_scene(sc2)
    g.step(sc2["dt"])
    gc = g.contacts()
    o = O.OracleWorld(sc2)
    o.narrowphase()
    oc = o.contacts()
    tri_contacts = sum(1 for r in gc if sc2["shapes"]["kind"][r["shape1"]] == abi.SHAPE_TRIANGLE or
                       sc2["shapes"]["kind"][r["shape2"]] == abi.SHAPE_TRIANGLE)
    assert tri_contacts > 300, tri_contacts
    stats = compare_contact_caches(gc, oc)
    assert stats["common_keys"] >= 0.999 * stats["keys"], stats
    assert stats["slot_mismatch"] <= 0.001 * stats["keys"], stats
    assert stats["normal_ok"] >= 0.999 and stats["point_ok"] >= 0.999, stats
