"""Speculative contacts in the oracle (CPU): the sweep and the detect branch that uses it.

Pinned to the reference's own cases: CollisionTests.SweepTest (the sweep's time of impact,
points and normal for a turned sphere and box) and
ContactLifecycleTests.SeparatedContact_UsesOriginalSpeculativeThreshold (the speculative
bias of a separated contact).

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
