"""The servos on the device (AngularServo, LinearServo, LinearAxisServo, TwistServo) and
PointOnLine, through the C ABI.

- One step of servo chains (scenes.servo_chains) from the GPU's state, replayed in the oracle
  in the GPU's order keys and warm-started with the GPU's impulses: velocities within 1e-3,
  impulses within 1e-3 relative.
- The reference's world-level ServoTests (ServoTests.cs) run on the device: a capped servo
  accelerates at its maximum for the elapsed time whatever the step, substep and iteration
  counts; the angular and linear servos track targets given in body 1's frame, also after
  the target changes; a twist servo drives a hinge to its limit and then to a target inside
  it; a linear axis servo reaches a signed position and leaves the perpendicular offset
  alone; an angular servo undoes an initial half turn; a target change wakes a sleeping
  body; the maximum and the twist target are checked.
"""
import numpy as np
import pytest

import oracle_lib as O
from jitterphysics2_gb300 import abi, scenes
from jitterphysics2_gb300.world import world_for_scene

pytestmark = pytest.mark.gpu

SERVOS = (abi.CONSTRAINT_ANGULARSERVO, abi.CONSTRAINT_LINEARSERVO, abi.CONSTRAINT_LINEARAXISSERVO,
          abi.CONSTRAINT_TWISTSERVO, abi.CONSTRAINT_POINTONLINE)
KINDS = ["angular", "twist", "linear", "axis"]


def test_one_step_of_servo_chains_matches_the_oracle():
    sc = scenes.servo_chains(n_chains=16)
    w = world_for_scene(sc)
    for _ in range(40):
        w.step(sc["dt"])
    b0 = w.bodies()
    _, j0 = w.constraints()
    w.step(sc["dt"])
    b1 = w.bodies()
    k1, j1 = w.constraints()
    o = O.OracleWorld(sc, external_order=True)
    o.set_bodies(b0)
    o.set_joint_impulses(j0)
    o.narrowphase()
    o.set_joint_colors(k1)
    o.step(sc["dt"], narrow=False)
    ob = o.bodies()
    dyn = b1["motion_type"] == abi.MOTION_DYNAMIC
    err = np.maximum(np.abs(b1["velocity"][dyn] - ob["velocity"][dyn]).max(axis=1),
                     np.abs(b1["angular_velocity"][dyn] - ob["angular_velocity"][dyn]).max(axis=1))
    jo = o.joint_impulses(len(j1))
    jerr = np.abs(j1 - jo).max(axis=1) / np.maximum(1e-3, np.abs(j1).max(axis=1))
    kinds = np.array([j[0] for j in sc["joints"]])
    for kind in SERVOS:
        assert np.abs(j1[kinds == kind]).max() > 0, kind     # every servo carries an impulse
    assert err.max() < 1e-3, np.sort(err)[-5:]
    assert np.mean(jerr < 1e-3) >= 0.999, np.sort(jerr)[-5:]


def test_servo_chains_reach_their_targets():
    sc = scenes.servo_chains(n_chains=4)
    w = world_for_scene(sc)
    for _ in range(300):
        w.step(sc["dt"])
    assert w.counters()["status"] == 0
    b = w.bodies()
    q = b["orientation"].astype(np.float64)
    for c in range(4):
        a = c * 5
        # link 2 sits at (1, 0.2, 0) from link 1 in link 1's frame
        off = _rotate(_conj(q[a + 1]), b["position"][a + 2] - b["position"][a + 1])
        assert np.abs(off - (1.0, 0.2, 0.0)).max() < 0.01, off
        # link 4's centre is 1.1 along link 3's x axis, and on that line
        x3 = _rotate(q[a + 3], np.array([1.0, 0.0, 0.0]))
        d = b["position"][a + 4] - b["position"][a + 3]
        assert abs(d @ x3 - 1.1) < 0.01
        assert np.linalg.norm(d - (d @ x3) * x3) < 0.01


# ---- the reference's ServoTests on the device ---------------------------------------------

def _conj(q):
    return np.array([-q[0], -q[1], -q[2], q[3]])


def _qmul(a, b):
    ax, ay, az, aw = a
    bx, by, bz, bw = b
    return np.array([aw * bx + ax * bw + ay * bz - az * by, aw * by - ax * bz + ay * bw + az * bx,
                     aw * bz + ax * by - ay * bx + az * bw, aw * bw - ax * bx - ay * by - az * bz])


def _rotate(q, v):
    q = np.asarray(q, np.float64)
    u, s = q[:3], q[3]
    t = 2 * np.cross(u, v)
    return v + s * t + np.cross(u, t)


def _axis_angle(axis, angle):
    a = np.asarray(axis, np.float64)
    a = a / np.linalg.norm(a)
    return tuple(np.append(a * np.sin(angle / 2), np.cos(angle / 2)).astype(np.float32).tolist())


def _scene(n=2, support=abi.MOTION_STATIC, **params):
    """Body 0: the support (the reference's NullBody: static at the origin); bodies 1..: unit
    mass, identity inertia, no damping (ServoTests.CreateBody, ServoTests.cs:58-64)."""
    b = np.zeros(n, abi.BODY_DTYPE)
    b["orientation"][:, 3] = 1.0
    b["flags"] = abi.BODY_ACTIVE | abi.BODY_NO_GRAVITY
    b["linear_damping"] = b["angular_damping"] = 1.0
    b["motion_type"][0] = support
    b["inv_mass"][1:] = 1.0
    b["inv_inertia"][1:] = (1, 0, 0, 1, 0, 1)
    prm = dict(gravity=(0.0, 0.0, 0.0), allow_deactivation=0)
    prm.update(params)
    return dict(bodies=b, shapes=np.zeros(0, abi.SHAPE_DTYPE), hull=np.zeros((0, 3), np.float32),
                triangles=np.zeros(0, abi.TRIANGLE_DTYPE), joints=[], params=prm, dt=0.01)


def _servo_init(kind, maximum):
    """ServoTests.CreateServo (ServoTests.cs:9-37) between the NullBody and a body at the origin."""
    if kind == "angular":
        return abi.CONSTRAINT_ANGULARSERVO, _axis_angle((1, 2, 3), 2.8) + (maximum,)
    if kind == "twist":
        return abi.CONSTRAINT_TWISTSERVO, (1, 0, 0, 1, 0, 0, 1.5, maximum)
    if kind == "linear":
        return abi.CONSTRAINT_LINEARSERVO, (0, 0, 0, 0, 0, 0, 1000, 2000, 3000, maximum)
    return abi.CONSTRAINT_LINEARAXISSERVO, (1, 0, 0, 0, 0, 0, 0, 0, 0, 1000, maximum)


def _speed(w, kind, body=1):
    b = w.bodies()
    return float(np.linalg.norm(b["angular_velocity" if kind in ("angular", "twist") else "velocity"][body]))


@pytest.mark.parametrize("kind", KINDS)
def test_capped_acceleration_uses_elapsed_time(kind):
    # ServoTests.CappedAccelerationUsesElapsedTime (ServoTests.cs:66-90)
    for steps in (30, 120):
        for substeps in (1, 4):
            for iterations in (1, 12):
                sc = _scene(substeps=substeps, solver_iterations=iterations, relax_iterations=0)
                k, init = _servo_init(kind, 2.0)
                sc["joints"] = [(k, 0, 1, init)]
                w = world_for_scene(sc)
                for _ in range(steps):
                    w.step(1.0 / steps)
                assert _speed(w, kind) == pytest.approx(2.0, abs=1e-4), (steps, substeps, iterations)


def test_angular_servo_tracks_targets_in_body1_frame():
    # ServoTests.AngularServoTracksTargetsInBody1Frame (ServoTests.cs:115-138)
    sc = _scene(support=abi.MOTION_KINEMATIC, substeps=4)
    b = sc["bodies"]
    b["inv_mass"][0] = 0.0
    b["inv_inertia"][0] = 0.0
    q_ref = _qmul(_axis_angle((0, 1, 0), 0.7), _axis_angle((1, 0, 0), 0.3))
    b["orientation"][0] = q_ref
    b["orientation"][1] = _axis_angle((0, 0, 1), -0.8)
    before = b["orientation"][1].copy()
    target = _qmul(_axis_angle((1, 0, 0), 0.9), _axis_angle((0, 0, 1), 0.5)).astype(np.float32)
    sc["joints"] = [(abi.CONSTRAINT_ANGULARSERVO, 0, 1, tuple(target) + (20.0,))]
    w = world_for_scene(sc)
    np.testing.assert_array_equal(w.bodies()["orientation"][1], before)
    for change in range(2):
        for _ in range(200):
            w.step(0.01)
        bb = w.bodies()
        expected = _qmul(bb["orientation"][0].astype(np.float64), target)
        assert abs(expected @ bb["orientation"][1]) == pytest.approx(1.0, abs=1e-5)
        target = _qmul(_axis_angle((0, 0, 1), -0.6), _axis_angle((0, 1, 0), 0.4)).astype(np.float32)
        w.set_servo(0, target, 20.0)


def test_linear_servo_tracks_offsets_in_body1_frame():
    # ServoTests.LinearServoTracksOffsetsInBody1Frame (ServoTests.cs:140-163)
    sc = _scene(support=abi.MOTION_KINEMATIC, substeps=4)
    b = sc["bodies"]
    b["inv_mass"][0] = 0.0
    b["inv_inertia"][0] = 0.0
    b["position"][0] = (4, 3, 2)
    b["orientation"][0] = _axis_angle((0, 0, 1), 0.7)
    b["position"][1] = (-1, 2, 3)
    sc["joints"] = [(abi.CONSTRAINT_LINEARSERVO, 0, 1, (4, 3, 2, -1, 2, 3, 0, 0, 0, 100.0))]
    w = world_for_scene(sc)
    np.testing.assert_array_equal(w.bodies()["position"][1], (-1, 2, 3))
    for target in ((0.0, 0.0, 0.0), (1.0, 2.0, -1.0)):
        w.set_servo(0, target, 100.0)
        for _ in range(300):
            w.step(0.01)
        bb = w.bodies()
        expected = bb["position"][0] + _rotate(bb["orientation"][0], np.array(target))
        assert np.linalg.norm(bb["position"][1] - expected) < 0.001


def _x_angle(q):
    return 2.0 * np.arctan2(q[0], q[3])


def test_twist_servo_coexists_with_hinge_limits():
    # ServoTests.TwistServoCoexistsWithHingeLimits (ServoTests.cs:165-180)
    sc = _scene(substeps=4)
    sc["joints"] = [(abi.CONSTRAINT_HINGEANGLE, 0, 1, (1, 0, 0, -0.5, 0.5)),
                    (abi.CONSTRAINT_TWISTSERVO, 0, 1, (1, 0, 0, 1, 0, 0, 0.9, 5.0))]
    w = world_for_scene(sc)
    for _ in range(300):
        w.step(0.01)
    assert _x_angle(w.bodies()["orientation"][1].astype(np.float64)) == pytest.approx(0.5, abs=0.01)
    w.set_servo(1, -0.25, 5.0)
    for _ in range(300):
        w.step(0.01)
    assert _x_angle(w.bodies()["orientation"][1].astype(np.float64)) == pytest.approx(-0.25, abs=0.001)


def test_linear_axis_servo_tracks_signed_position_without_correcting_perpendicular_offset():
    # ServoTests.LinearAxisServoTracksSignedPositionWithoutCorrectingPerpendicularOffset
    # (ServoTests.cs:267-281)
    sc = _scene(substeps=4)
    sc["bodies"]["position"][1] = (3, 4, 5)
    sc["joints"] = [(abi.CONSTRAINT_LINEARAXISSERVO, 0, 1, (1, 0, 0, 0, 0, 0, 3, 4, 5, -1.0, 100.0))]
    w = world_for_scene(sc)
    for _ in range(300):
        w.step(0.01)
    p = w.bodies()["position"][1]
    assert p[0] == pytest.approx(-1.0, abs=0.001)
    assert (p[1], p[2]) == (4.0, 5.0)


def test_angular_servo_corrects_an_initial_half_turn():
    # ServoTests.AngularServoCorrectsAnInitialHalfTurn (ServoTests.cs:406-418)
    sc = _scene(substeps=4)
    sc["bodies"]["orientation"][1] = (0, 1, 0, 0)
    sc["joints"] = [(abi.CONSTRAINT_ANGULARSERVO, 0, 1, (0, 0, 0, 1, 20.0))]
    w = world_for_scene(sc)
    for _ in range(300):
        w.step(0.01)
    assert abs(w.bodies()["orientation"][1][3]) == pytest.approx(1.0, abs=1e-5)


@pytest.mark.parametrize("kind", KINDS)
def test_target_changes_wake_sleeping_bodies(kind):
    # ServoTests.TargetChangesWakeSleepingBodies (ServoTests.cs:233-265); the island is sent
    # to sleep by a short deactivation time instead of World.ForceSleepIsland
    sc = _scene(allow_deactivation=1)
    k, init = _servo_init(kind, 0.0)
    sc["joints"] = [(k, 0, 1, init)]
    w = world_for_scene(sc)
    w.set_body_sleep(1, 0.05)
    for _ in range(20):
        w.step(0.01)
    assert not (w.bodies()["flags"][1] & abi.BODY_ACTIVE)
    new_target = {"angular": _axis_angle((0, 1, 0), 0.8), "twist": 0.8, "linear": (1.0, 0.0, 0.0), "axis": 1.0}[kind]
    w.set_servo(0, new_target, 0.0)
    w.step(0.01)
    assert w.bodies()["flags"][1] & abi.BODY_ACTIVE
    w.set_servo(0, new_target, 2.0)
    w.step(0.01)
    assert _speed(w, kind) > 0


@pytest.mark.parametrize("kind", KINDS)
def test_servo_maximum_is_checked_and_may_be_infinite(kind):
    # ServoTests.MaximumRejectsInvalidValuesAndAllowsInfinity (ServoTests.cs:233-242)
    sc = _scene()
    k, init = _servo_init(kind, 2.0)
    w = world_for_scene(sc)
    target = {"angular": lambda: init[:4], "twist": lambda: init[6], "linear": lambda: init[6:9],
              "axis": lambda: init[9]}[kind]()
    for bad in (-1.0, np.nan, -np.inf):
        bad_init = list(init)
        bad_init[-1] = bad
        with pytest.raises(abi.JitterError) as e:
            w.add_constraint(k, 0, 1, bad_init)
        assert e.value.code == abi.JG_ERR_INVALID_ARG
    j = w.add_constraint(k, 0, 1, init)
    for bad in (-1.0, np.nan, -np.inf):
        with pytest.raises(abi.JitterError):
            w.set_servo(j, target, bad)
    w.set_servo(j, target, np.inf)
    w.step(0.01)
    assert w.counters()["status"] == 0


def test_twist_servo_rejects_targets_outside_its_interval():
    # ServoTests.TwistServoRejectsTargetsOutsideItsAngularInterval (ServoTests.cs:311-331)
    w = world_for_scene(_scene())
    for angle in (-np.pi - 0.01, np.pi + 0.01, np.nan, np.inf, -np.inf):
        with pytest.raises(abi.JitterError):
            w.add_constraint(abi.CONSTRAINT_TWISTSERVO, 0, 1, (1, 0, 0, 1, 0, 0, angle, 1.0))
    j = w.add_constraint(abi.CONSTRAINT_TWISTSERVO, 0, 1, (1, 0, 0, 1, 0, 0, 0.0, 1.0))
    for angle in (-np.pi - 0.01, np.pi + 0.01, np.nan, np.inf, -np.inf):
        with pytest.raises(abi.JitterError):
            w.set_servo(j, angle, 1.0)
    pi32 = float(np.float32(np.pi))
    for angle in (-pi32, pi32):
        w.add_constraint(abi.CONSTRAINT_TWISTSERVO, 0, 1, (1, 0, 0, 1, 0, 0, angle, 1.0))
        w.set_servo(j, -angle, 1.0)


def test_angular_servo_rejects_a_non_unit_target():
    w = world_for_scene(_scene())
    with pytest.raises(abi.JitterError):
        w.add_constraint(abi.CONSTRAINT_ANGULARSERVO, 0, 1, (0, 0, 0.5, 0.5, 1.0))
    j = w.add_constraint(abi.CONSTRAINT_ANGULARSERVO, 0, 1, (0, 0, 0, 0, 1.0))   # the current orientation
    with pytest.raises(abi.JitterError):
        w.set_servo(j, (0, 0, 0, 2), 1.0)


def test_point_on_line_reduces_the_distance_to_its_line():
    # AdditionalConstraintBehaviorTests.PointOnLine_ReducesPerpendicularDistanceToLine
    # (AdditionalConstraintBehaviorTests.cs:55-79): two unit spheres, the line along x through
    # the static one's centre, the other starting 3.6 from it
    sc = _scene(substeps=4)
    b = sc["bodies"]
    b["position"][1] = (0, 3, 2)
    s = np.zeros(2, abi.SHAPE_DTYPE)
    s["kind"] = abi.SHAPE_SPHERE
    s["body"] = (0, 1)
    s["dims"][:, 0] = 1.0
    sc["shapes"] = s
    b["inv_mass"][1] = 1.0 / (4.0 / 3.0 * np.pi)
    sc["joints"] = [(abi.CONSTRAINT_POINTONLINE, 0, 1, (1, 0, 0, 0, 0, 0, 0, 3, 2, -np.inf, np.inf))]
    w = world_for_scene(sc)
    before = np.hypot(3.0, 2.0)
    for _ in range(200):
        w.step(0.01)
    p = w.bodies()["position"][1]
    after = np.hypot(p[1], p[2])
    assert after < before and after < 2.1
    _, imp = w.constraints()
    assert np.linalg.norm(imp[0]) > 0


@pytest.mark.parametrize("init", [
    (0, 0, 0) + (0, 0, 0) + (1, 0, 0) + (0.0, 1.0),        # zero axis
    (1, 0, 0) + (0, 0, 0) + (1, 0, 0) + (np.nan, 1.0),     # NaN limit
    (1, 0, 0) + (np.inf, 0, 0) + (1, 0, 0) + (0.0, 1.0),   # infinite anchor
])
def test_invalid_point_on_line_arguments_raise(init):
    # PointOnLine.Initialize (PointOnLine.cs:92-100): ArgumentCheck.NonZero, Finite, NotNaN
    w = world_for_scene(_scene())
    with pytest.raises(abi.JitterError) as e:
        w.add_constraint(abi.CONSTRAINT_POINTONLINE, 0, 1, init)
    assert e.value.code == abi.JG_ERR_INVALID_ARG


def test_state_round_trip_keeps_servo_and_line_rows():
    """jg_export_state / jg_import_state with every servo kind and PointOnLine: the step after
    an import equals the step after the export, bit for bit."""
    sc = scenes.servo_chains(n_chains=4)
    w = world_for_scene(sc)
    for _ in range(20):
        w.step(sc["dt"])
    blob = w.export_state()
    w.step(sc["dt"])
    a = w.bodies()
    w.import_state(blob)
    w.step(sc["dt"])
    b = w.bodies()
    assert np.array_equal(a["position"], b["position"]) and np.array_equal(a["angular_velocity"], b["angular_velocity"])
