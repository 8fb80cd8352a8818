"""Speculative contacts in the oracle (CPU): the sweep and the detect branch that uses it.

Pinned to the reference's own cases: CollisionTests.SweepTest (the sweep's time of impact,
points and normal for a turned sphere and box),
ContactLifecycleTests.SeparatedContact_UsesOriginalSpeculativeThreshold (the speculative
bias of a separated contact) and BroadPhaseUpdateTests (a speculative box grows by dt |v| of
its linear velocity alone; a bullet stops at a thin wall in its first step).

NarrowPhase.Sweep (NarrowPhase.cs:1100-1222) on SimplexSolverAB (SimplexSolverAB.cs) is
checked against closed-form times of impact; the detect branch (World.Detect.cs:168-196)
and the swept bounding boxes (RigidBodyShape.cs:37-57) against the behaviour they exist
for: a fast body does not pass through a thin slab between two steps.  The sweep stops
within 1e-4 of contact (its collideEpsilon), so a time of impact is exact to
1e-4 / closing speed plus rounding.
"""
import numpy as np
import pytest

import oracle_lib as O
from jitterphysics2_gb300 import abi, scenes

I = (0.0, 0.0, 0.0, 1.0)


def _quat(axis, angle):
    a = np.asarray(axis, np.float64) / np.linalg.norm(axis)
    return (*(a * np.sin(angle / 2)), np.cos(angle / 2))


@pytest.mark.parametrize("real", ["f", "d"])
def test_two_spheres_meet_at_the_closed_form_time(real):
    hit, pA, pB, n, toi = O.sweep(O.sphere(1.0), O.sphere(1.0), I, I, (0, 0, 0), (10, 0, 0), (0, 0, 0), (-20, 0, 0),
                                  real=real)
    assert hit
    assert toi == pytest.approx(0.4, abs=1e-6)
    # points at the bodies' current poses, normal from A to B
    np.testing.assert_allclose(pA, (1, 0, 0), atol=1e-6)
    np.testing.assert_allclose(pB, (9, 0, 0), atol=1e-6)
    np.testing.assert_allclose(n, (1, 0, 0), atol=1e-6)
    assert np.dot(n, pA - pB) < 0  # a speculative (negative) penetration


def test_both_bodies_moving_sweep_the_relative_velocity():
    hit, pA, pB, n, toi = O.sweep(O.sphere(1.0), O.sphere(1.0), I, I, (0, 0, 0), (10, 0, 0), (5, 0, 0), (-15, 0, 0))
    assert hit and toi == pytest.approx(0.4, abs=1e-6)
    np.testing.assert_allclose(pA, (1, 0, 0), atol=1e-6)
    np.testing.assert_allclose(pB, (9, 0, 0), atol=1e-6)


def test_separating_bodies_report_no_hit():
    hit, _, _, _, toi = O.sweep(O.sphere(1.0), O.sphere(1.0), I, I, (0, 0, 0), (10, 0, 0), (0, 0, 0), (20, 0, 0))
    assert not hit and np.isinf(toi)
    # moving sideways past each other: the closing speed along the separating axis is zero
    hit, _, _, _, toi = O.sweep(O.sphere(1.0), O.sphere(1.0), I, I, (0, 0, 0), (10, 0, 0), (0, 0, 0), (0, 30, 0))
    assert not hit and np.isinf(toi)


def test_overlapping_bodies_hit_at_time_zero():
    hit, _, _, n, toi = O.sweep(O.sphere(1.0), O.sphere(1.0), I, I, (0, 0, 0), (1, 0, 0), (0, 0, 0), (-20, 0, 0))
    assert hit and toi == 0.0
    np.testing.assert_array_equal(n, (0, 0, 0))


def test_box_falling_on_a_box_meets_at_the_gap_over_the_speed():
    hit, pA, pB, n, toi = O.sweep(O.box(0.5, 0.5, 0.5), O.box(0.5, 0.5, 0.5), I, I, (0, 0, 0), (0.1, 5, 0.2),
                                  (0, 0, 0), (0, -10, 0))
    assert hit
    assert toi == pytest.approx(0.4, abs=1e-4 / 10 + 1e-6)
    np.testing.assert_allclose(n, (0, 1, 0), atol=1e-3)
    assert pA[1] == pytest.approx(0.5, abs=1e-4) and pB[1] == pytest.approx(4.5, abs=1e-4)


@pytest.mark.parametrize("seed", range(5))
def test_sweep_does_not_depend_on_the_frame_of_a(seed):
    # a sphere looks the same in every orientation: rotating body A must not move the hit
    rng = np.random.Generator(np.random.PCG64(seed))
    qa = _quat(rng.normal(size=3), rng.uniform(0, np.pi))
    qb = _quat(rng.normal(size=3), rng.uniform(0, np.pi))
    pb = (rng.uniform(-1, 1), 6.0, rng.uniform(-1, 1))
    vb = (rng.uniform(-2, 2), -30.0, rng.uniform(-2, 2))
    ref = O.sweep(O.sphere(0.7), O.box(0.4, 0.3, 0.5), I, qb, (0, 0, 0), pb, (0, 0, 0), vb, real="d")
    rot = O.sweep(O.sphere(0.7), O.box(0.4, 0.3, 0.5), qa, qb, (0, 0, 0), pb, (0, 0, 0), vb, real="d")
    assert ref[0] and rot[0]
    assert rot[4] == pytest.approx(ref[4], abs=1e-5)
    np.testing.assert_allclose(rot[3], ref[3], atol=2e-3)


def _run(sc, steps, **params):
    w = O.OracleWorld(sc, **params)
    spec = 0
    for _ in range(steps):
        w.step(sc["dt"])
        spec += w.counters()["speculative"]
    return w, spec


def test_speculative_bodies_stop_on_a_thin_slab_and_others_pass_through():
    w, spec = _run(scenes.bullets(n=64, speculative=True), 30)
    y = w.bodies()["position"][1:, 1]
    assert spec > 0 and (y > 0.05).all(), y.min()
    w, spec = _run(scenes.bullets(n=64, speculative=False), 30)
    y = w.bodies()["position"][1:, 1]
    assert spec == 0 and (y < -1.0).sum() > 50


def test_speculative_contacts_change_linear_velocity_only():
    # first step: every hit is speculative (no body starts inside the slab), registered with
    # SolveMode.Angular removed, so no bullet picks up angular velocity
    sc = scenes.bullets(n=64)
    w, spec = _run(sc, 1)
    b = w.bodies()
    assert spec > 10
    assert np.abs(b["angular_velocity"]).max() == 0.0
    slowed = b["velocity"][1:, 1] > sc["bodies"]["velocity"][1:, 1] + 1.0
    assert slowed.sum() == spec


def test_no_speculative_contact_below_the_velocity_threshold():
    sc = scenes.bullets(n=64)
    w, spec = _run(sc, 30, speculative_threshold=200.0)
    assert spec == 0
    assert (w.bodies()["position"][1:, 1] < -1.0).sum() > 50


def test_swept_boxes_find_the_slab_pairs():
    # a speculative body's box grows by dt |v| on every side: the slab pairs are exactly
    # the bullets whose grown box reaches the slab's top face (y = 0.05)
    dt = 1.0 / 60.0
    for spec in (False, True):
        sc = scenes.bullets(n=64, speculative=spec)
        o = O.OracleWorld(sc)
        o.narrowphase(dt=dt)
        got = {int(j) for i, j in o.pairs() if i == 0}
        want = set()
        for k in range(1, 65):
            s, b = sc["shapes"][k:k + 1], sc["bodies"][k]
            lo, _ = O.aabb(s, b["orientation"], b["position"])
            grow = dt * np.float32(np.linalg.norm(b["velocity"].astype(np.float64))) if spec else 0.0
            if lo[1] - grow <= 0.05:
                want.add(k)
        assert got == want
        assert (len(got) > 10) == spec


@pytest.mark.parametrize("real", ["f", "d"])
def test_reference_sweep_case(real):
    # CollisionTests.SweepTest (Behavior/CollisionTests.cs:143-169): a sphere (r 0.5) and a
    # box (size 1) both turned 45 degrees about z, closing along the diagonal at speed 3
    rot = (0.0, 0.0, np.sin(np.pi / 8), np.cos(np.pi / 8))
    sweep = np.array([1.0, 1.0, 0.0]) / np.sqrt(2.0)
    hit, pA, pB, n, lam = O.sweep(O.sphere(0.5), O.box(0.5, 0.5, 0.5), rot, rot, (1, 1, 3), (11, 11, 3),
                                  sweep, -2.0 * sweep, real=real)
    assert hit
    lam_x = (np.sqrt(200.0) - 1.0) / 3.0
    point = np.array([1.0, 1.0, 3.0]) + sweep * (0.5 + lam_x)
    assert np.sum((n - sweep) ** 2) < 1e-4
    assert np.sum((pA - (point - sweep * lam)) ** 2) < 1e-4
    assert np.sum((pB - (point + 2.0 * sweep * lam)) ** 2) < 1e-4
    assert abs(lam - lam_x) < 1e-4


@pytest.mark.parametrize("gap, target", [(0.1, -0.9), (0.005, 10.0)])
def test_separated_contact_uses_the_speculative_threshold(gap, target):
    # ContactLifecycleTests.SeparatedContact_UsesOriginalSpeculativeThreshold
    # (Behavior/ContactLifecycleTests.cs:109-146): a contact 0.1 apart at dt 0.1 is
    # speculative (bias = -gap / dt * 0.9); one 0.005 apart keeps its restitution bias
    from test_oracle_golden import _two_body_scene
    null = dict(motion_type=abi.MOTION_STATIC, inv_mass=0.0, inv_inertia=np.zeros(6), friction=0.0, restitution=1.0)
    inv_i = 1.0 / (0.4 * 1.0 * 0.25 * 0.25)
    ball = dict(position=(gap, 0, 0), velocity=(-10, 0, 0), inv_mass=1.0, inv_inertia=(inv_i, 0, 0, inv_i, 0, inv_i),
                friction=0.0, restitution=1.0)
    w = O.OracleWorld(_two_body_scene(null, ball))
    w.register_contact(0, 1, [0, 0, 0], [gap, 0, 0], [1, 0, 0])
    assert w.contacts()[0]["bias"] == pytest.approx(10.0)
    w.fn("jor_world_prepare")(w.h, 0.1, 1)
    c = w.contacts()[0]
    assert c["bias"] == pytest.approx(target, abs=1e-5) and c["penalty_bias"] == 0.0
    w.fn("jor_world_iterate")(w.h, 1)
    assert w.bodies()["velocity"][1][0] == pytest.approx(target, abs=1e-5)
    w.fn("jor_world_iterate")(w.h, 0)
    assert w.bodies()["velocity"][1][0] == pytest.approx(target, abs=1e-5)


def _one_body(shape_kind, dims, speculative, velocity, angular=(0, 0, 0), position=(0, 0, 0)):
    b = np.zeros(1, abi.BODY_DTYPE)
    b["orientation"][0, 3] = 1.0
    b["inv_mass"] = 1.0
    b["inv_inertia"] = (1, 0, 0, 1, 0, 1)
    b["linear_damping"] = b["angular_damping"] = 1.0
    b["flags"] = abi.BODY_ACTIVE | abi.BODY_NO_GRAVITY | (abi.BODY_SPECULATIVE if speculative else 0)
    b["position"] = position
    b["velocity"] = velocity
    b["angular_velocity"] = angular
    s = np.zeros(1, abi.SHAPE_DTYPE)
    s["kind"] = shape_kind
    s["dims"][0, :len(dims)] = dims
    return dict(bodies=b, shapes=s, hull=np.zeros((0, 3), np.float32), triangles=np.zeros(0, abi.TRIANGLE_DTYPE))


@pytest.mark.parametrize("linear", [False, True])
def test_speculative_bounds_use_only_linear_velocity(linear):
    # BroadPhaseUpdateTests.SpeculativeBoundsUseOnlyLinearVelocity
    # (Behavior/BroadPhaseUpdateTests.cs:7-36): BoxShape(4, 0.2, 0.2) spinning at 1000 rad/s,
    # speed 5 or 0, dt 0.02: padding 0.1 or none; without the flag the tight box
    v = (3.0, 4.0, 0.0) if linear else (0.0, 0.0, 0.0)
    tight = O.OracleWorld(_one_body(abi.SHAPE_BOX, (2.0, 0.1, 0.1), False, v, (0, 0, 1000))).shape_box(0, 0.02)
    grown = O.OracleWorld(_one_body(abi.SHAPE_BOX, (2.0, 0.1, 0.1), True, v, (0, 0, 1000))).shape_box(0, 0.02)
    pad = 0.1 if linear else 0.0
    assert np.linalg.norm(grown[0] - (tight[0] - pad)) < 1e-5
    assert np.linalg.norm(grown[1] - (tight[1] + pad)) < 1e-5
    np.testing.assert_allclose(tight[0], (-2.0, -0.1, -0.1), atol=1e-6)


def test_speculative_bullet_stops_at_a_thin_wall_in_one_step():
    # BroadPhaseUpdateTests.SpeculativeVelocityChangeUpdatesBroadphaseBeforeFirstStep
    # (Behavior/BroadPhaseUpdateTests.cs:58-90): a 0.1 sphere at 100 m/s toward a 0.02-thick
    # static wall 0.8 away; one step of 0.01 (default solver settings, no gravity)
    b = np.zeros(2, abi.BODY_DTYPE)
    b["orientation"][:, 3] = 1.0
    b["linear_damping"] = 0.998
    b["angular_damping"] = 0.995
    b["flags"] = abi.BODY_ACTIVE | abi.BODY_NO_GRAVITY
    b["friction"] = 0.2
    b["position"][0] = (0, 0, -0.8)
    b["motion_type"][0] = abi.MOTION_STATIC
    b["inv_mass"][1] = 1.0
    b["inv_inertia"][1] = (1, 0, 0, 1, 0, 1)
    b["velocity"][1] = (0, 0, -100)
    b["flags"][1] |= abi.BODY_SPECULATIVE
    s = np.zeros(2, abi.SHAPE_DTYPE)
    s["kind"] = (abi.SHAPE_BOX, abi.SHAPE_SPHERE)
    s["body"] = (0, 1)
    s["dims"][0, :3] = (5.0, 5.0, 0.01)
    s["dims"][1, 0] = 0.1
    sc = dict(bodies=b, shapes=s, hull=np.zeros((0, 3), np.float32), triangles=np.zeros(0, abi.TRIANGLE_DTYPE),
              params=dict(gravity=(0.0, 0.0, 0.0)))
    o = O.OracleWorld(sc)
    o.step(0.01)
    assert o.counters()["speculative"] == 1
    assert o.bodies()["position"][1, 2] > -0.8


# ---- the sweep's simplex (Regression/SimplexProjectionTests.cs, the witness-point solver) ---
def _simplex_all_true(vertices, real="f"):
    # every AddVertex call of the reference's helper must report "origin not enclosed"
    for k in range(1, len(vertices) + 1):
        ok, c = O.simplex(vertices[:k], real=real)
        assert ok
    return c


@pytest.mark.parametrize("real", ["f", "d"])
def test_simplex_segment_of_large_vertices_keeps_a_small_gap(real):
    c = _simplex_all_true([(100000, 0.001, 0), (-130000, 0.001, 0)], real)
    np.testing.assert_allclose(c, (0, np.float32(0.001) if real == "f" else 0.001, 0), atol=1e-9)


@pytest.mark.parametrize("real", ["f", "d"])
def test_simplex_triangle_of_large_vertices_keeps_a_small_gap(real):
    off = np.float32(0.001) if real == "f" else 0.001
    c = _simplex_all_true([(100000, 100000, 0.001), (-130000, 100000, 0.001), (100000, -130000, 0.001)], real)
    np.testing.assert_allclose(c, (0, 0, off), atol=1e-9)


@pytest.mark.parametrize("reverse", [False, True])
def test_simplex_segment_beyond_an_end_returns_that_end(reverse):
    near, far = (2, 1, -3), (5, 1, -3)
    c = _simplex_all_true([far, near] if reverse else [near, far])
    np.testing.assert_array_equal(c, near)
    near, far = (0, 2, 3), (4, 2, 3)
    c = _simplex_all_true([far, near] if reverse else [near, far])
    np.testing.assert_array_equal(c, near)


def test_simplex_tiny_edge_keeps_the_second_vertex():
    first, second = (2, 1, 3), (2 + 1e-5, 1, 3)
    np.testing.assert_array_equal(_simplex_all_true([first, second]), np.float32(second))
    np.testing.assert_array_equal(_simplex_all_true([second, first]), np.float32(first))
    np.testing.assert_array_equal(_simplex_all_true([first, first]), first)


def test_simplex_triangle_falls_back_to_an_edge():
    np.testing.assert_allclose(_simplex_all_true([(3, -2, 1), (3, 2, 1), (5, 0, 1)]), (3, 0, 1), atol=1e-6)
    np.testing.assert_allclose(_simplex_all_true([(3, -2, 1), (3, 2, 1), (3, 0, 1)]), (3, 0, 1), atol=1e-6)


@pytest.mark.parametrize("gap, target", [(0.005, 2.0), (0.1, -0.9)])
def test_linear_only_contact_ignores_angular_surface_velocity(gap, target):
    # ContactLifecycleTests.LinearOnlyContact_IgnoresAngularSurfaceVelocity
    # (Behavior/ContactLifecycleTests.cs:71-106): a contact registered with SolveMode.Angular
    # removed (as the speculative branch registers its point) sees neither the spin's surface
    # velocity in its restitution bias nor changes the spin
    from test_oracle_golden import _two_body_scene
    wall = dict(motion_type=abi.MOTION_STATIC, inv_mass=0.0, inv_inertia=np.zeros(6), friction=0.0)
    ball = dict(velocity=(-2, 0, 0), angular_velocity=(0, 0, 10), inv_mass=1.0, inv_inertia=(2.5, 0, 0, 2.5, 0, 2.5),
                friction=0.0, restitution=1.0)
    w = O.OracleWorld(_two_body_scene(wall, ball))
    w.register_contact(0, 1, [-gap, 1, 0], [0, 1, 0], [1, 0, 0], linear_only=True)
    assert w.contacts()[0]["bias"] == pytest.approx(2.0, abs=1e-5)
    w.fn("jor_world_prepare")(w.h, 0.1, 1)
    w.fn("jor_world_iterate")(w.h, 1)
    b = w.bodies()
    assert b["velocity"][1][0] == pytest.approx(target, abs=1e-5)
    np.testing.assert_array_equal(b["angular_velocity"][1], (0, 0, 10))


@pytest.mark.parametrize("speculative", [True, False])
def test_bullet_stops_on_a_triangle_mesh_only_with_speculative_contacts(speculative):
    # the sweep against triangle shapes (NarrowPhase.Sweep on a TriangleShape's support map,
    # World.Detect.cs:168-196): a 0.1 sphere 0.8 above a flat 4 x 4-cell mesh at 100 m/s, one
    # step of 0.01 (1.0 of travel): with the flag it stops on the mesh, without it passes
    tris = scenes.heightfield(cells=4, extent=8.0, amplitude=0.0, base=0.0)
    nt = len(tris)
    b = np.zeros(2, abi.BODY_DTYPE)
    b["orientation"][:, 3] = 1.0
    b["linear_damping"] = 0.998
    b["angular_damping"] = 0.995
    b["flags"] = abi.BODY_ACTIVE | abi.BODY_NO_GRAVITY
    b["friction"] = 0.2
    b["motion_type"][0] = abi.MOTION_STATIC
    b["position"][1] = (0.3, 0.8, 0.3)
    b["inv_mass"][1] = 1.0
    b["inv_inertia"][1] = (1, 0, 0, 1, 0, 1)
    b["velocity"][1] = (0, -100, 0)
    if speculative:
        b["flags"][1] |= abi.BODY_SPECULATIVE
    s = np.zeros(nt + 1, abi.SHAPE_DTYPE)
    s["kind"][:nt] = abi.SHAPE_TRIANGLE
    s["body"][:nt] = 0
    s["data_offset"][:nt] = np.arange(nt)
    s["kind"][nt] = abi.SHAPE_SPHERE
    s["body"][nt] = 1
    s["dims"][nt, 0] = 0.1
    sc = dict(bodies=b, shapes=s, hull=np.zeros((0, 3), np.float32), triangles=tris,
              params=dict(gravity=(0.0, 0.0, 0.0)))
    o = O.OracleWorld(sc)
    o.step(0.01)
    y = o.bodies()["position"][1, 1]
    if speculative:
        assert o.counters()["speculative"] >= 1
        assert y > 0.0
    else:
        assert o.counters()["speculative"] == 0
        assert y < -0.1
