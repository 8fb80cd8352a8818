"""The servos (AngularServo, LinearServo, LinearAxisServo, TwistServo) in the oracle (CPU).

The reference's constraint-level servo cases (ServoTests.cs), restated with its Solve helper
(one Prepare and 12 Iterates of the servo alone, ServoTests.cs:51-56) on a unit body
(identity inertia, no damping) tied to a static body at the origin (the NullBody):
the warm start under a reduced maximum and a changed step, uncontrolled motion left free,
non-dynamic bodies bitwise unchanged, the angular torque cap on the applied impulse, the
signed twist difference and the shortest angular path, no impulse at zero duration or zero
maximum, and an unlimited servo answering like the fixed constraint it generalises.
"""
import numpy as np
import pytest

import oracle_lib as O
from jitterphysics2_gb300 import abi

KINDS = ["angular", "twist", "linear", "axis"]
F32 = np.float32


def axis_angle(axis, angle):
    """JQuaternion.CreateFromAxisAngle in float32."""
    a = np.asarray(axis, np.float64)
    a = (a / np.linalg.norm(a)).astype(F32)
    h = F32(angle) / F32(2)
    s, c = np.sin(h, dtype=F32), np.cos(h, dtype=F32)
    return (float(a[0] * s), float(a[1] * s), float(a[2] * s), float(c))


def rot_x(angle):
    return axis_angle((1, 0, 0), angle)


def world(n=2, support="static", positions=None, orientations=None):
    """Body 0: the support (static at the origin, or kinematic); bodies 1..: unit bodies."""
    b = np.zeros(n, abi.BODY_DTYPE)
    b["orientation"][:, 3] = 1.0
    b["flags"] = abi.BODY_ACTIVE | abi.BODY_NO_GRAVITY
    b["linear_damping"] = b["angular_damping"] = 1.0
    b["motion_type"][0] = abi.MOTION_STATIC if support == "static" else abi.MOTION_KINEMATIC
    b["inv_mass"][1:] = 1.0
    b["inv_inertia"][1:] = (1, 0, 0, 1, 0, 1)
    if support == "dynamic":
        b["motion_type"][0] = abi.MOTION_DYNAMIC
        b["inv_mass"][0] = 1.0
        b["inv_inertia"][0] = (1, 0, 0, 1, 0, 1)
    for i, p in (positions or {}).items():
        b["position"][i] = p
    for i, q in (orientations or {}).items():
        b["orientation"][i] = q
    sc = dict(bodies=b, shapes=np.zeros(0, abi.SHAPE_DTYPE), hull=np.zeros((0, 3), np.float32),
              triangles=np.zeros(0, abi.TRIANGLE_DTYPE))
    return O.OracleWorld(sc)


def servo_init(kind, maximum, p1=(0, 0, 0), p2=(0, 0, 0)):
    """(constraint kind, init) of ServoTests.CreateServo (ServoTests.cs:9-37)."""
    if kind == "angular":
        return abi.CONSTRAINT_ANGULARSERVO, axis_angle((1, 2, 3), 2.8) + (maximum,)
    if kind == "twist":
        return abi.CONSTRAINT_TWISTSERVO, (1, 0, 0, 1, 0, 0, 1.5, maximum)
    if kind == "linear":
        return abi.CONSTRAINT_LINEARSERVO, tuple(p1) + tuple(p2) + (1000, 2000, 3000, maximum)
    return abi.CONSTRAINT_LINEARAXISSERVO, (1, 0, 0) + tuple(p1) + tuple(p2) + (1000, maximum)


def servo(o, kind, maximum=2.0, b1=0, b2=1):
    k, init = servo_init(kind, maximum)
    return o.add_joint(k, b1, b2, init)


def target_of(kind):
    return {"angular": axis_angle((1, 2, 3), 2.8), "twist": (1.5,), "linear": (1000, 2000, 3000), "axis": (1000,)}[kind]


def speed(o, kind, body=1):
    b = o.bodies()
    v = b["angular_velocity" if kind in ("angular", "twist") else "velocity"][body].astype(np.float64)
    return float(np.linalg.norm(v))


def set_velocity(o, body, v=None, w=None):
    b = o.bodies()
    if v is not None:
        b["velocity"][body] = v
    if w is not None:
        b["angular_velocity"][body] = w
    o.set_bodies(b)


@pytest.mark.parametrize("kind", KINDS)
def test_warm_start_respects_reduced_maximum_and_changed_timestep(kind):
    # ServoTests.WarmStartRespectsReducedMaximumAndChangedTimestep (ServoTests.cs:92-113)
    o = world()
    j = servo(o, kind)
    o.joint_run(j, 0.1)
    for maximum in (0.1, 0.0):
        set_velocity(o, 1, (0, 0, 0), (0, 0, 0))
        o.set_servo(j, target_of(kind), maximum)
        sub = np.float32(0.01) / np.float32(4)
        o.joint_run(j, 0.01, substeps=4, iterations=0)
        assert speed(o, kind) == pytest.approx(maximum * sub, abs=1e-7)
        o.joint_run(j, 0.01, substeps=4, iterations=12, prepare=False)
        assert speed(o, kind) <= maximum * sub + 1e-7


@pytest.mark.parametrize("angular", [False, True])
def test_axis_servo_leaves_uncontrolled_motion_free(angular):
    # ServoTests.AxisServoLeavesUncontrolledMotionFree (ServoTests.cs:182-197)
    o = world()
    set_velocity(o, 1, (0, 2, 3), (0, 4, 5))
    j = servo(o, "twist" if angular else "axis")
    o.joint_run(j, 0.01)
    b = o.bodies()
    v, w = b["velocity"][1], b["angular_velocity"][1]
    assert (v[1], v[2], w[1], w[2]) == (2, 3, 4, 5)
    assert (v[0] if angular else w[0]) == 0
    assert (w[0] if angular else v[0]) > 0


@pytest.mark.parametrize("kind", KINDS)
@pytest.mark.parametrize("support", ["static", "kinematic"])
@pytest.mark.parametrize("reverse", [False, True])
def test_non_dynamic_bodies_remain_bitwise_unchanged(kind, support, reverse):
    # ServoTests.NonDynamicBodiesRemainBitwiseUnchanged (ServoTests.cs:199-215)
    o = world(support=support)
    j = servo(o, kind, b1=1 if reverse else 0, b2=0 if reverse else 1)
    o.joint_run(j, 0.01)
    set_velocity(o, 0, (-0.0, -0.0, -0.0), (-0.0, -0.0, -0.0))
    before = o.bodies()[0].tobytes()
    o.joint_run(j, 0.01)
    assert o.bodies()[0].tobytes() == before


def test_angular_torque_cap_applies_to_physical_impulse_at_large_errors():
    # ServoTests.AngularTorqueCapAppliesToPhysicalImpulseAtLargeErrors (ServoTests.cs:217-231)
    qy, qz = axis_angle((0, 1, 0), 2.8), axis_angle((0, 0, 1), 0.4)
    q = _qmul(qy, qz)
    o = world(orientations={1: q})
    set_velocity(o, 1, w=(20, -30, 40))
    before = o.bodies()["angular_velocity"][1].astype(np.float64)
    j = o.add_joint(abi.CONSTRAINT_ANGULARSERVO, 0, 1, (0, 0, 0, 1, 3.0))
    o.joint_run(j, 0.01)
    after = o.bodies()["angular_velocity"][1].astype(np.float64)
    assert np.linalg.norm(after - before) == pytest.approx(0.03, abs=1e-5)
    jac = o.joint_matrix(j)[0]
    assert np.linalg.norm(jac.T @ o.joint_impulse(j)) == pytest.approx(0.03, abs=1e-6)


def _qmul(a, b):
    ax, ay, az, aw = a
    bx, by, bz, bw = b
    return (aw * bx + ax * bw + ay * bz - az * by, aw * by - ax * bz + ay * bw + az * bx,
            aw * bz + ax * by - ay * bx + az * bw, aw * bw - ax * bx - ay * by - az * bz)


@pytest.mark.parametrize("current,target", [(-179, 179), (179, -179)])
def test_twist_servo_preserves_signed_angle_difference(current, target):
    # ServoTests.TwistServoPreservesSignedAngleDifference (ServoTests.cs:283-296)
    o = world()
    j = o.add_joint(abi.CONSTRAINT_TWISTSERVO, 0, 1, (1, 0, 0, 1, 0, 0, np.radians(target), np.inf))
    b = o.bodies()
    b["orientation"][1] = rot_x(np.radians(current))
    o.set_bodies(b)
    o.joint_run(j, 0.01)
    assert o.bodies()["angular_velocity"][1][0] * np.sign(target - current) > 1


@pytest.mark.parametrize("current,target", [(-179, 179), (179, -179)])
def test_angular_servo_takes_shortest_path_between_orientations(current, target):
    # ServoTests.AngularServoTakesShortestPathBetweenOrientations (ServoTests.cs:297-310)
    o = world(orientations={1: rot_x(np.radians(current))})
    j = o.add_joint(abi.CONSTRAINT_ANGULARSERVO, 0, 1, rot_x(np.radians(target)) + (np.inf,))
    o.joint_run(j, 0.01)
    wx = o.bodies()["angular_velocity"][1][0]
    assert wx * np.sign(current - target) > 0
    assert abs(wx) < 1


@pytest.mark.parametrize("kind", KINDS)
@pytest.mark.parametrize("dt,maximum", [(0.0, np.inf), (0.01, 0.0)])
def test_no_impulse_at_zero_duration_or_zero_maximum(kind, dt, maximum):
    # ServoTests.ZeroDurationWithUnlimitedForceDoesNotApplyImpulse (ServoTests.cs:333-344),
    # ServoTests.ZeroMaximumDoesNotApplyImpulse (ServoTests.cs:346-357)
    o = world()
    j = servo(o, kind, maximum)
    set_velocity(o, 1, (1, 2, 3), (3, 2, 1))
    o.joint_run(j, dt)
    b = o.bodies()
    np.testing.assert_array_equal(b["velocity"][1], (1, 2, 3))
    np.testing.assert_array_equal(b["angular_velocity"][1], (3, 2, 1))


@pytest.mark.parametrize("kind", KINDS)
def test_unlimited_servo_matches_existing_constraint_response(kind):
    # ServoTests.UnlimitedServoMatchesExistingConstraintResponse (ServoTests.cs:359-405): the
    # servo with an unlimited maximum answers as FixedAngle at its target, TwistAngle fixed at
    # its angle, BallSocket from the target to the body's origin, PointOnPlane fixed at its
    # position
    s = world()
    j = servo(s, kind, np.inf)
    if kind == "angular":
        c = world(orientations={1: target_of("angular")})
        k = c.add_joint(abi.CONSTRAINT_FIXEDANGLE, 0, 1, np.zeros(1))
        b = c.bodies()
        b["orientation"][1] = (0, 0, 0, 1)
        c.set_bodies(b)
    elif kind == "twist":
        c = world()
        k = c.add_joint(abi.CONSTRAINT_TWISTANGLE, 0, 1, (1, 0, 0, 1, 0, 0, 1.5, 1.5))
    elif kind == "linear":
        c = world(positions={1: (1000, 2000, 3000)})
        k = c.add_joint(abi.CONSTRAINT_BALLSOCKET, 0, 1, (1000, 2000, 3000))
        b = c.bodies()
        b["position"][1] = (0, 0, 0)
        c.set_bodies(b)
    else:
        c = world()
        k = c.add_joint(abi.CONSTRAINT_POINTONPLANE, 0, 1, (1, 0, 0, 0, 0, 0, 0, 0, 0, 1000, 1000))
    for o in (s, c):
        set_velocity(o, 1, (2, 3, -4), (-3, 1, 2))
    s.joint_run(j, 0.01, substeps=4)
    c.joint_run(k, 0.01, substeps=4)
    bs, bc = s.bodies(), c.bodies()
    assert np.linalg.norm(bs["velocity"][1].astype(np.float64) - bc["velocity"][1]) < 1e-4
    assert np.linalg.norm(bs["angular_velocity"][1].astype(np.float64) - bc["angular_velocity"][1]) < 1e-4


@pytest.mark.parametrize("kind", KINDS)
def test_servo_rows_in_float_follow_double(kind):
    """The FP32 and FP64 oracles agree on a servo pulling a spinning body (a check of the
    restatement's arithmetic, not of the reference)."""
    res = []
    for real in ("f", "d"):
        b = np.zeros(2, abi.BODY_DTYPE)
        b["orientation"][:, 3] = 1.0
        b["orientation"][1] = axis_angle((0.3, 1, -0.2), 0.7)
        b["position"][1] = (0.5, -0.2, 0.3)
        b["flags"] = abi.BODY_ACTIVE | abi.BODY_NO_GRAVITY
        b["linear_damping"] = b["angular_damping"] = 1.0
        b["motion_type"][0] = abi.MOTION_STATIC
        b["inv_mass"][1] = 0.5
        b["inv_inertia"][1] = (1.2, 0.1, 0.0, 0.8, -0.05, 1.5)
        b["velocity"][1] = (0.3, -0.2, 0.1)
        b["angular_velocity"][1] = (0.5, 0.2, -0.4)
        sc = dict(bodies=b, shapes=np.zeros(0, abi.SHAPE_DTYPE), hull=np.zeros((0, 3), np.float32),
                  triangles=np.zeros(0, abi.TRIANGLE_DTYPE), dt=0.01)
        k, init = servo_init(kind, 5.0, (0.1, 0.2, 0.3), (0.4, -0.1, 0.2))
        sc["joints"] = [(k, 0, 1, init)]
        o = O.OracleWorld(sc, real=real)
        for _ in range(20):
            o.step(0.01)
        res.append(o.bodies_d())
    np.testing.assert_allclose(res[0]["velocity"], res[1]["velocity"], atol=2e-4)
    np.testing.assert_allclose(res[0]["angular_velocity"], res[1]["angular_velocity"], atol=2e-4)
