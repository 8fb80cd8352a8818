"""The oracle's ConeLimit and TwistAngle rows pinned to the reference's own
constraint-level tests (AngularCoordinateTests.cs), restated: one Prepare (+ Iterate) of
the joint alone on bodies with unit inverse mass and identity inverse inertia (the
reference's default body), body 0 static where the reference uses its NullBody.

- the Jacobian row of each is the derivative of the angle its getter reports, for either
  body, by central differences (delta 1e-4 and tolerance 0.006 in FP32, 1e-6 and 1e-7 in
  FP64, the reference's values);
- softness acts in angle units on both sides of the former thresholds (the velocity left
  is gamma / (1 + gamma), gamma = softness / dt);
- a tiny cone limit stays distinct from zero, a fixed tilt holds both directions, an
  interior boundary stops only the outward rate, the natural 0 and pi bounds leave motion
  free, and cached impulses keep their units across the former thresholds;
- and from ConstraintSingularityTests.cs, stepped in a world without gravity or damping:
  a twist recovers from a half turn without a huge angular velocity and honours its range
  there, a cone recovers from its endpoint poses into its range, the twist Jacobian matches
  its angle's derivative next to the half turn, and a tiny cone limit corrects a tilt its
  rounded cosine would hide;
- and for the three-row blocks (HingeAngle, a device row, and FixedAngle, restated in the
  oracle as kind 6): their Jacobians are the derivative of the rotation log for both
  bodies, they recover from half turns, and crossing the half turn drops the other branch's
  impulse (for TwistAngle too).
"""
import numpy as np
import pytest

import oracle_lib as O
from jitterphysics2_gb300 import abi
from test_oracle_constraints import _quat_mul

DT = 0.01


def _axis_angle(axis, angle):
    a = np.asarray(axis, np.float64) / np.linalg.norm(axis)
    return np.array([*(a * np.sin(angle / 2)), np.cos(angle / 2)])


def _normalize(q):
    q = np.asarray(q, np.float64)
    return q / np.linalg.norm(q)


def _world(q1, q2, static_first, w2=(0, 0, 0)):
    b = np.zeros(2, abi.BODY_DTYPE)
    b["flags"] = abi.BODY_ACTIVE | abi.BODY_NO_GRAVITY
    b["linear_damping"] = b["angular_damping"] = 1.0
    b["orientation"][0], b["orientation"][1] = q1, q2
    b["inv_mass"] = 1.0
    b["inv_inertia"] = (1, 0, 0, 1, 0, 1)
    if static_first:
        b["motion_type"][0] = abi.MOTION_STATIC
        b["inv_mass"][0] = 0.0
        b["inv_inertia"][0] = 0.0
    b["angular_velocity"][1] = w2
    sc = dict(bodies=b, shapes=np.zeros(0, abi.SHAPE_DTYPE), hull=np.zeros((0, 3), np.float32),
              triangles=np.zeros(0, abi.TRIANGLE_DTYPE))
    return sc


def _set(o, body, q=None, w=None):
    b = o.bodies()
    if q is not None:
        b["orientation"][body] = q
    if w is not None:
        b["angular_velocity"][body] = w
    o.set_bodies(b)


def _perp(axis):
    a = np.asarray(axis, np.float64)
    t = np.cross(a, (1.0, 0.0, 0.0) if abs(a[0]) < 0.9 else (0.0, 1.0, 0.0))
    return t / np.linalg.norm(t)


PREC = {"f": (1e-4, 0.006), "d": (1e-6, 1e-7)}
Q1 = _normalize((1, 2, 3, 4))
Q2 = _normalize((2, -1, 3, 5))
AXIS = np.array([1.0, 3.0, 2.0]) / np.linalg.norm([1.0, 3.0, 2.0])


def _check_jacobian(o, j, jac, perturb_body2, q1, q2, real):
    # orientations go in at the oracle's precision: a 1e-6 turn is below float32's
    delta, tol = PREC[real]
    body = 1 if perturb_body2 else 0
    orig = q2 if perturb_body2 else q1
    for direction in np.eye(3):
        o.set_orientation_d(body, _quat_mul(_axis_angle(direction, delta), orig))
        plus = o.joint_angle(j)
        o.set_orientation_d(body, _quat_mul(_axis_angle(direction, -delta), orig))
        minus = o.joint_angle(j)
        o.set_orientation_d(body, orig)
        expected = float(np.dot(jac, direction)) * (-1 if perturb_body2 else 1)
        assert (plus - minus) / (2 * delta) == pytest.approx(expected, abs=tol)


@pytest.mark.parametrize("real", ["f", "d"])
@pytest.mark.parametrize("perturb_body2", [False, True])
@pytest.mark.parametrize("angle", [0.2, 2.1, 3.13])
def test_twist_jacobian_is_the_derivative_of_its_angle(angle, perturb_body2, real):
    o = O.OracleWorld(_world(Q1, Q2, False), real=real)
    o.set_orientation_d(0, Q1)
    o.set_orientation_d(1, Q2)
    j = o.add_joint(abi.CONSTRAINT_TWISTANGLE, 0, 1, tuple(AXIS) + tuple(AXIS) + (1e-6, -1e-6))
    q2 = _quat_mul(_axis_angle(AXIS, angle), Q2)
    q2 = _quat_mul(_axis_angle(_perp(AXIS), 0.3), q2)
    o.set_orientation_d(1, q2)
    o.joint_solve(j, DT, 0.2, 0.001, iterate=False)
    jac = o.joint_data(j)[0]
    _check_jacobian(o, j, jac, perturb_body2, Q1, q2, real)


@pytest.mark.parametrize("real", ["f", "d"])
@pytest.mark.parametrize("perturb_body2", [False, True])
@pytest.mark.parametrize("angle", [0.2, 0.6, 2.1, 3.13])
def test_cone_jacobian_is_the_derivative_of_its_angle(angle, perturb_body2, real):
    o = O.OracleWorld(_world(Q1, Q2, False), real=real)
    o.set_orientation_d(0, Q1)
    o.set_orientation_d(1, Q2)
    lim = np.radians(30.0)
    j = o.add_joint(abi.CONSTRAINT_CONELIMIT, 0, 1, tuple(AXIS) + tuple(AXIS) + (lim, lim))
    q2 = _quat_mul(_axis_angle(_perp(AXIS), angle), Q2)
    o.set_orientation_d(1, q2)
    o.joint_solve(j, DT, 0.2, 0.001, iterate=False)
    jac = o.joint_data(j)[0]
    _check_jacobian(o, j, jac, perturb_body2, Q1, q2, real)


def _gamma(softness):
    return softness / DT


@pytest.mark.parametrize("degrees", [119.99, 120.01, 179.0])
def test_twist_softness_uses_angle_units(degrees):
    o = O.OracleWorld(_world((0, 0, 0, 1), (0, 0, 0, 1), True))
    j = o.add_joint(abi.CONSTRAINT_TWISTANGLE, 0, 1, (0, 0, 1, 0, 0, 1, 1e-6, -1e-6))
    _set(o, 1, q=_axis_angle((0, 0, 1), np.radians(degrees)), w=(0, 0, 1))
    o.joint_solve(j, DT, 0.0, 0.001)
    g = _gamma(0.001)
    assert o.bodies()["angular_velocity"][1, 2] == pytest.approx(g / (1 + g), abs=1e-5)


@pytest.mark.parametrize("degrees", [29.99, 30.01, 149.99, 150.01])
def test_cone_softness_uses_angle_units(degrees):
    o = O.OracleWorld(_world((0, 0, 0, 1), (0, 0, 0, 1), True))
    j = o.add_joint(abi.CONSTRAINT_CONELIMIT, 0, 1, (0, 0, 1, 0, 0, 1, 0.0, np.radians(10.0)))
    _set(o, 1, q=_axis_angle((1, 0, 0), np.radians(degrees)), w=(1, 0, 0))
    o.joint_solve(j, DT, 0.0, 0.001)
    g = _gamma(0.001)
    assert o.bodies()["angular_velocity"][1, 0] == pytest.approx(g / (1 + g), abs=1e-5)


@pytest.mark.parametrize("lower", [1e-6, 1e-9])
def test_tiny_cone_limits_remain_distinct(lower):
    o = O.OracleWorld(_world((0, 0, 0, 1), (0, 0, 0, 1), True))
    j = o.add_joint(abi.CONSTRAINT_CONELIMIT, 0, 1, (0, 0, 1, 0, 0, 1, lower, 2 * lower))
    _set(o, 1, q=_axis_angle((1, 0, 0), 3 * lower))
    o.joint_solve(j, DT, 0.2, 0.001, iterate=False)
    assert o.joint_data(j)[3] == 1


@pytest.mark.parametrize("softness", [0.0, 0.001])
@pytest.mark.parametrize("direction", [-1, 1])
def test_fixed_cone_tilt_holds_both_directions(direction, softness):
    o = O.OracleWorld(_world((0, 0, 0, 1), (0, 0, 0, 1), True))
    lim = np.radians(30.0)
    j = o.add_joint(abi.CONSTRAINT_CONELIMIT, 0, 1, (0, 0, 1, 0, 0, 1, lim, lim))
    _set(o, 1, q=_axis_angle((1, 0, 0), np.pi / 6), w=(direction, 0, 0))
    o.joint_solve(j, DT, 0.0, softness)
    g = _gamma(softness)
    assert o.joint_data(j)[3] == 3
    assert o.bodies()["angular_velocity"][1, 0] == pytest.approx(direction * g / (1 + g), abs=1e-5)


@pytest.mark.parametrize("softness", [0.0, 0.001])
@pytest.mark.parametrize("outgoing", [False, True])
@pytest.mark.parametrize("upper", [False, True])
def test_interior_cone_boundary_stops_only_the_outward_rate(upper, outgoing, softness):
    o = O.OracleWorld(_world((0, 0, 0, 1), (0, 0, 0, 1), True))
    j = o.add_joint(abi.CONSTRAINT_CONELIMIT, 0, 1, (0, 0, 1, 0, 0, 1, 0.0, np.pi))
    direction = 1 if upper == outgoing else -1
    _set(o, 1, q=_axis_angle((1, 0, 0), 0.5), w=(direction, 0, 0))
    boundary = o.joint_angle(j)
    if upper:
        o.joint_set_limit(j, 0.0, boundary)
    else:
        o.joint_set_limit(j, boundary, np.float32(np.pi))
    o.joint_solve(j, DT, 0.0, softness)
    g = _gamma(softness)
    expected = direction * (g / (1 + g) if outgoing else 1.0)
    assert o.bodies()["angular_velocity"][1, 0] == pytest.approx(expected, abs=1e-5)


@pytest.mark.parametrize("antiparallel", [False, True])
def test_natural_cone_bounds_leave_motion_free(antiparallel):
    o = O.OracleWorld(_world((0, 0, 0, 1), (0, 0, 0, 1), True))
    j = o.add_joint(abi.CONSTRAINT_CONELIMIT, 0, 1, (0, 0, 1, 0, 0, 1, 0.0, np.float32(np.pi)))
    _set(o, 1, q=(1, 0, 0, 0) if antiparallel else (0, 0, 0, 1), w=(1, 2, 3))
    o.joint_solve(j, DT, 0.2, 0.001)
    assert o.joint_data(j)[3] == 0
    np.testing.assert_array_equal(o.bodies()["angular_velocity"][1], (1, 2, 3))


@pytest.mark.parametrize("twist", [False, True])
def test_warm_starts_keep_their_units_across_former_thresholds(twist):
    o = O.OracleWorld(_world((0, 0, 0, 1), (0, 0, 0, 1), True))
    if twist:
        j = o.add_joint(abi.CONSTRAINT_TWISTANGLE, 0, 1, (0, 0, 1, 0, 0, 1, 1e-6, -1e-6))
        axis, before, after, comp = (0, 0, 1), 119.99, 120.01, 2
    else:
        lim = np.radians(30.0)
        j = o.add_joint(abi.CONSTRAINT_CONELIMIT, 0, 1, (0, 0, 1, 0, 0, 1, lim, lim))
        axis, before, after, comp = (1, 0, 0), 29.99, 30.01, 0
    _set(o, 1, q=_axis_angle(axis, np.radians(before)))
    o.joint_solve(j, DT, 0.2, 0.001, iterate=False)
    o.set_joint_impulses([[0.25, 0.0, 0.0]])
    _set(o, 1, q=_axis_angle(axis, np.radians(after)))
    o.joint_solve(j, DT, 0.2, 0.001, iterate=False)
    assert o.joint_data(j)[4] == pytest.approx(0.25)
    assert o.bodies()["angular_velocity"][1, comp] == pytest.approx(0.25, abs=1e-5)


# ---- ConstraintSingularityTests.cs: half turns and cone endpoints, stepped ------------------
# The reference's world for these cases: no gravity, one substep, 8 iterations and no
# relaxation, no damping, no gyroscopic term (ConstraintSingularityTests.cs:74-87).
LOCK_ALL_BUT = {"all": 0, "angular_x": 63 ^ 8, "angular_z": 63 ^ 32}


def _stepped_world(locks):
    sc = _world((0, 0, 0, 1), (0, 0, 0, 1), True)
    b = sc["bodies"]
    b["flags"][1] = abi.BODY_ACTIVE | abi.BODY_NO_GRAVITY | (LOCK_ALL_BUT[locks] << abi.BODY_LOCKS_SHIFT)
    sc["params"] = dict(substeps=1, solver_iterations=8, relax_iterations=0, gravity=(0.0, 0.0, 0.0))
    return sc


def _run_checked(o, steps=100):
    for _ in range(steps):
        o.step(0.01)
        b = o.bodies()
        assert np.linalg.norm(b["angular_velocity"][1]) < 100.0
        assert np.isfinite(b["orientation"][1]).all()


@pytest.mark.parametrize("locks", ["all", "angular_z"])
@pytest.mark.parametrize("softness", [0.0, 0.001])
@pytest.mark.parametrize("sign", [-1, 1])
@pytest.mark.parametrize("offset", [0.0, 1e-5, 0.005])
def test_twist_recovers_from_a_half_turn(offset, sign, softness, locks):
    # Twist_HalfTurnRecoversWithoutHugeAngularVelocity (ConstraintSingularityTests.cs:89-112)
    o = O.OracleWorld(_stepped_world(locks))
    j = o.add_joint(abi.CONSTRAINT_TWISTANGLE, 0, 1, (0, 0, 1, 0, 0, 1, 1e-6, -1e-6))
    o.joint_params(j, 0.2, softness)
    q = (0.0, 0.0, float(sign), 0.0) if offset == 0 else _axis_angle((0, 0, 1), sign * (np.pi - offset))
    _set(o, 1, q=q)
    _run_checked(o)
    assert abs(o.joint_angle(j)) < 0.001


@pytest.mark.parametrize("locks", ["all", "angular_x"])
@pytest.mark.parametrize("softness", [0.0, 0.001])
@pytest.mark.parametrize("antiparallel", [False, True])
@pytest.mark.parametrize("offset", [0.0, 1e-5, 0.002, 0.1])
def test_cone_endpoint_poses_recover_into_the_range(offset, antiparallel, softness, locks):
    # Cone_EndpointPosesRecoverIntoAllowedRange (ConstraintSingularityTests.cs:114-137)
    o = O.OracleWorld(_stepped_world(locks))
    j = o.add_joint(abi.CONSTRAINT_CONELIMIT, 0, 1, (0, 0, 1, 0, 0, 1, np.radians(30.0), np.radians(60.0)))
    o.joint_params(j, 0.2, softness)
    if antiparallel and offset == 0:
        q = (1.0, 0.0, 0.0, 0.0)
    else:
        q = _axis_angle((1, 0, 0), np.pi - offset if antiparallel else offset)
    _set(o, 1, q=q)
    _run_checked(o)
    assert np.pi / 6 - 0.001 <= o.joint_angle(j) <= np.pi / 3 + 0.001


@pytest.mark.parametrize("swing", [0.0, 0.005])
def test_twist_jacobian_near_the_half_turn(swing):
    # Twist_AngleFallbackJacobianMatchesFiniteDifference (ConstraintSingularityTests.cs:139-171)
    o = O.OracleWorld(_world(Q1, Q1, False))
    o.set_orientation_d(0, Q1)
    o.set_orientation_d(1, Q1)
    j = o.add_joint(abi.CONSTRAINT_TWISTANGLE, 0, 1, tuple(AXIS) + tuple(AXIS) + (1e-6, -1e-6))
    q2 = _quat_mul(_axis_angle(AXIS, np.pi - 0.01), Q1)
    q2 = _quat_mul(_axis_angle(_perp(AXIS), swing), q2)
    o.set_orientation_d(1, q2)
    o.joint_solve(j, DT, 0.2, 0.001, iterate=False)
    jac = o.joint_data(j)[0]
    for direction in np.eye(3):
        o.set_orientation_d(0, _quat_mul(_axis_angle(direction, 1e-4), Q1))
        after = o.joint_angle(j)
        o.set_orientation_d(0, _quat_mul(_axis_angle(direction, -1e-4), Q1))
        before = o.joint_angle(j)
        assert (after - before) / 2e-4 == pytest.approx(float(np.dot(jac, direction)), abs=0.004)


@pytest.mark.parametrize("sign", [-1, 1])
def test_twist_half_turn_honours_its_range(sign):
    # Twist_HalfTurnHonorsRangeLimits (ConstraintSingularityTests.cs:173-185)
    o = O.OracleWorld(_stepped_world("angular_z"))
    j = o.add_joint(abi.CONSTRAINT_TWISTANGLE, 0, 1, (0, 0, 1, 0, 0, 1, -np.pi / 6, np.pi / 6))
    o.joint_params(j, 0.2, 0.0)
    _set(o, 1, q=(0.0, 0.0, float(sign), 0.0))
    for _ in range(100):
        o.step(0.01)
    assert abs(o.joint_angle(j)) <= np.pi / 6 + 0.001


def test_tiny_cone_upper_limit_corrects_a_rounded_tilt():
    # Cone_TinyUpperLimitCorrectsTiltDespiteRoundedCosine (ConstraintSingularityTests.cs:187-200)
    o = O.OracleWorld(_world((0, 0, 0, 1), (0, 0, 0, 1), True))
    j = o.add_joint(abi.CONSTRAINT_CONELIMIT, 0, 1, (0, 0, 1, 0, 0, 1, 0.0, 5e-6))
    _set(o, 1, q=_axis_angle((1, 0, 0), 1e-5))
    o.joint_solve(j, DT, 0.2, 0.0)
    assert o.bodies()["angular_velocity"][1, 0] == pytest.approx(-1e-4, abs=1e-6)


def test_twist_created_on_a_pure_swing_starts_at_zero():
    # HistoricalRegressionTests.TwistAngle_Initialize_WithPureSwing_StartsAtZeroTwist
    # (Regression/HistoricalRegressionTests.cs:88-105): body 2 turned a quarter about x, the
    # twist axes y and z of the two bodies: Q0 absorbs the swing, so the twist reads zero
    o = O.OracleWorld(_world((0, 0, 0, 1), _axis_angle((1, 0, 0), np.pi / 2), False))
    j = o.add_joint(abi.CONSTRAINT_TWISTANGLE, 0, 1, (0, 1, 0, 0, 0, 1, 1e-6, -1e-6))
    assert abs(o.joint_angle(j)) < 1e-5


# ---- three-row angular blocks: HingeAngle (device row) and FixedAngle (oracle, kind 6) -------
FIXEDANGLE = 6


def _rotation_log(q):
    q = np.asarray(q, np.float64)
    if q[3] < 0:
        q = -q
    s = np.linalg.norm(q[:3])
    return q[:3] * (np.arctan2(s, q[3]) / s) if s > 0 else np.zeros(3)


@pytest.mark.parametrize("real", ["f", "d"])
@pytest.mark.parametrize("perturb_body2", [False, True])
@pytest.mark.parametrize("hinge", [False, True])
@pytest.mark.parametrize("angle", [0.2, 2.1, 3.13])
def test_rotation_log_jacobian_matches_both_bodies(angle, hinge, perturb_body2, real):
    # AngularCoordinateTests.RotationLogJacobianMatchesBothBodies (AngularCoordinateTests.cs:17-71)
    delta, tol = PREC[real]
    o = O.OracleWorld(_world(Q1, Q2, False), real=real)
    o.set_orientation_d(0, Q1)
    o.set_orientation_d(1, Q2)
    if hinge:
        j = o.add_joint(abi.CONSTRAINT_HINGEANGLE, 0, 1, tuple(AXIS) + (1e-6, -1e-6))
    else:
        j = o.add_joint(FIXEDANGLE, 0, 1, (0, 0, 0))
    q2 = _quat_mul(_axis_angle(np.array([2.0, 1.0, -3.0]), angle), Q2)
    o.set_orientation_d(1, q2)
    o.joint_solve(j, DT, 0.2, 0.001, iterate=False)
    jac, q0, local_axis = o.joint_matrix(j)
    if hinge:
        # the hinge stores its rows' Jacobians as columns; the reference transposes them
        rows = jac.T
        p0 = _orthonormal(local_axis)
        frame = np.stack([p0, np.cross(local_axis, p0), local_axis])
    else:
        rows = jac
    qs = {0: Q1, 1: q2}
    body = 1 if perturb_body2 else 0
    for direction in np.eye(3):
        logs = []
        for sgn in (1, -1):
            qq = dict(qs)
            qq[body] = _quat_mul(_axis_angle(direction, sgn * delta), qs[body])
            rel = _quat_mul(_quat_mul(q0, qq[0] * (-1, -1, -1, 1)), qq[1])
            logs.append(_rotation_log(rel))
        measured = (logs[0] - logs[1]) / (2 * delta)
        measured = frame @ measured if hinge else -2 * measured
        expected = rows @ (direction * (-1 if perturb_body2 else 1))
        assert np.abs(measured - expected).max() < tol


def _orthonormal(v):
    # MathHelper.CreateOrthonormal (MathHelper.cs:204-254) restated for this test: a unit
    # vector orthogonal to v chosen from v's smallest component, as the oracle's helper does
    v = np.asarray(v, np.float64)
    ax = np.abs(v)
    if ax[0] <= ax[1] and ax[0] <= ax[2]:
        r = np.array([0.0, v[2], -v[1]])
    elif ax[1] <= ax[2]:
        r = np.array([-v[2], 0.0, v[0]])
    else:
        r = np.array([v[1], -v[0], 0.0])
    return r / np.linalg.norm(r)


@pytest.mark.parametrize("offset", [0.0, 1e-5])
@pytest.mark.parametrize("softness", [0.0, 0.001])
@pytest.mark.parametrize("pure_twist", [False, True])
@pytest.mark.parametrize("hinge", [False, True])
def test_angular_blocks_recover_from_half_turns(hinge, pure_twist, softness, offset):
    # AngularCoordinateTests.AngularBlocksRecoverFromHalfTurns (AngularCoordinateTests.cs:166-197):
    # no gravity, one substep, default iterations, no damping, no gyroscopic term
    sc = _world((0, 0, 0, 1), (0, 0, 0, 1), True)
    sc["params"] = dict(substeps=1, gravity=(0.0, 0.0, 0.0))
    o = O.OracleWorld(sc)
    if hinge:
        j = o.add_joint(abi.CONSTRAINT_HINGEANGLE, 0, 1, (0, 0, 1, 1e-6, -1e-6))
        o.joint_params(j, 0.2, softness)
        o.joint_limit_params(j, 0.1, softness)
    else:
        j = o.add_joint(FIXEDANGLE, 0, 1, (0, 0, 0))
        o.joint_params(j, 0.2, softness)
    axis = np.array([0.0, 0.0, 1.0]) if pure_twist else np.array([1.0, 2.0, 3.0]) / np.sqrt(14.0)
    q = np.array([*axis, 0.0]) if offset == 0 else _axis_angle(axis, np.pi - offset)
    o.set_orientation_d(1, q)
    for _ in range(200):
        o.step(0.01)
        b = o.bodies()
        assert np.linalg.norm(b["angular_velocity"][1]) < 100.0
        assert np.isfinite(b["orientation"][1]).all()
    assert np.linalg.norm(_rotation_log(o.bodies()["orientation"][1])) < 0.001


@pytest.mark.parametrize("kind", ["hinge", "fixed", "twist"])
def test_crossing_the_half_turn_clears_the_other_branch_impulse(kind):
    # AngularCoordinateTests.CrossingTheHalfTurnClearsThePreviousBranchImpulse
    # (AngularCoordinateTests.cs:199-240)
    o = O.OracleWorld(_world((0, 0, 0, 1), (0, 0, 0, 1), True))
    if kind == "hinge":
        j = o.add_joint(abi.CONSTRAINT_HINGEANGLE, 0, 1, (0, 0, 1, 1e-6, -1e-6))
        cached = [0.0, 0.0, 1.0]
    elif kind == "fixed":
        j = o.add_joint(FIXEDANGLE, 0, 1, (0, 0, 0))
        cached = [0.0, 0.0, 1.0]
    else:
        j = o.add_joint(abi.CONSTRAINT_TWISTANGLE, 0, 1, (0, 0, 1, 0, 0, 1, 1e-6, -1e-6))
        cached = [1.0, 0.0, 0.0]
    o.set_orientation_d(1, _axis_angle((0, 0, 1), np.pi - 0.01))
    o.joint_solve(j, DT, 0.2, 0.001, iterate=False)
    o.set_joint_impulses([cached])
    o.set_orientation_d(1, _axis_angle((0, 0, 1), np.pi + 0.01))
    o.joint_solve(j, DT, 0.2, 0.001, iterate=False)
    np.testing.assert_array_equal(o.joint_impulses(1)[0], 0.0)
    np.testing.assert_array_equal(o.bodies()["angular_velocity"][1], 0.0)


@pytest.mark.parametrize("velocity_sign", [-1, 1])
@pytest.mark.parametrize("pose_sign", [-1, 1])
@pytest.mark.parametrize("hinge", [False, True])
def test_full_ranges_let_a_half_turn_pass(hinge, pose_sign, velocity_sign):
    # AngularCoordinateTests.FullHingeAndTwistRangesAllowCrossingHalfTurns (:346-375)
    o = O.OracleWorld(_world((0, 0, 0, 1), (0, 0, 0, 1), True))
    if hinge:
        j = o.add_joint(abi.CONSTRAINT_HINGEANGLE, 0, 1, (0, 0, 1, -np.pi, np.pi))
        o.joint_limit_params(j, 0.0, 0.001)
    else:
        j = o.add_joint(abi.CONSTRAINT_TWISTANGLE, 0, 1, (0, 0, 1, 0, 0, 1, -np.pi, np.pi))
    _set(o, 1, q=(0, 0, pose_sign, 0), w=(0, 0, velocity_sign))
    o.joint_solve(j, DT, 0.0, 0.001)
    assert o.joint_data(j)[3] == 0
    np.testing.assert_array_equal(o.bodies()["angular_velocity"][1], (0, 0, velocity_sign))


@pytest.mark.parametrize("sign", [-1, 1])
@pytest.mark.parametrize("hinge", [False, True])
def test_partial_ranges_keep_the_half_turn_bound_active(hinge, sign):
    # AngularCoordinateTests.PartialHingeAndTwistRangesKeepTheHalfTurnBoundaryActive (:377-407)
    lo, hi = (0.0, np.pi) if sign == 1 else (-np.pi, 0.0)
    o = O.OracleWorld(_world((0, 0, 0, 1), (0, 0, 0, 1), True))
    if hinge:
        j = o.add_joint(abi.CONSTRAINT_HINGEANGLE, 0, 1, (0, 0, 1, lo, hi))
        o.joint_limit_params(j, 0.0, 0.0)
    else:
        j = o.add_joint(abi.CONSTRAINT_TWISTANGLE, 0, 1, (0, 0, 1, 0, 0, 1, lo, hi))
    _set(o, 1, q=(0, 0, sign, 0), w=(0, 0, sign))
    o.joint_solve(j, DT, 0.0, 0.0)
    assert o.joint_data(j)[3] == (1 if sign == 1 else 2)
    assert np.abs(o.bodies()["angular_velocity"][1]).max() < 1e-5


@pytest.mark.parametrize("nonidentity", [False, True])
@pytest.mark.parametrize("qsign", [-1, 1])
@pytest.mark.parametrize("target_sign", [-1, 1])
@pytest.mark.parametrize("hinge", [False, True])
def test_fixed_half_turn_targets_see_no_bias_from_the_quaternion_sign(hinge, target_sign, qsign, nonidentity):
    # AngularCoordinateTests.FixedHalfTurnTargetsDoNotBiasEquivalentQuaternionRepresentations (:409-442)
    q1, q2 = (Q1, Q2) if nonidentity else (np.array([0, 0, 0, 1.0]), np.array([0, 0, 0, 1.0]))
    axis = AXIS if nonidentity else np.array([0.0, 0.0, 1.0])
    o = O.OracleWorld(_world(q1, q2, False))
    o.set_orientation_d(0, q1)
    o.set_orientation_d(1, q2)
    lim = target_sign * np.pi
    if hinge:
        j = o.add_joint(abi.CONSTRAINT_HINGEANGLE, 0, 1, tuple(axis) + (lim, lim))
    else:
        j = o.add_joint(abi.CONSTRAINT_TWISTANGLE, 0, 1, tuple(axis) + tuple(axis) + (lim, lim))
    local = o.joint_matrix(j)[2]
    o.set_orientation_d(1, _quat_mul(q2, np.array([*(local * qsign), 0.0])))
    if hinge:
        o.joint_solve(j, DT, 0.2, 0.001, iterate=False)
        bias = o.joint_bias(j)[2]
    else:
        o.joint_solve(j, DT, 0.2, 0.001, iterate=False)
        bias = o.joint_bias(j)[0]
    assert abs(bias) < 1e-4


@pytest.mark.parametrize("sign", [-1, 1])
def test_fixed_target_wrapping_handles_large_finite_values(sign):
    # AngularCoordinateTests.FixedAngularTargetWrappingHandlesLargeFiniteValues (:444-453)
    lib = O.load()
    big = float(np.finfo(np.float32).max) * sign
    w = lib.jor_shortest_angle_f(big, float(np.float32(np.pi)))
    assert np.isfinite(w) and -np.pi - 1e-6 <= w <= np.pi + 1e-6
