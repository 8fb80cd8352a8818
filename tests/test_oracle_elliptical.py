"""EllipticalConeLimit in the oracle (CPU): the reference's constraint-level cases
(EllipticalConeLimitTests.cs), restated with Prepare (and one Iterate) at TimeStep(0.01).

The initial swing is measured in the bodies' frames; the Jacobian is the unit normal of
the implicit ellipse, on both bodies, with the bias its scaled error; circular ranges answer
as ConeLimit does; the Jacobian stays finite next to the antipode; interior swing and twist
are free, and a dropped warm start applies nothing.
"""
import numpy as np
import pytest

import oracle_lib as O
from jitterphysics2_gb300 import abi

DT = 0.01
RAD = np.pi / 180


def _qn(q):
    q = np.asarray(q, np.float64)
    return q / np.linalg.norm(q)


def _axis_angle(axis, angle):
    a = _qn(axis)
    return np.append(a * np.sin(angle / 2), np.cos(angle / 2))


def _qmul(a, b):
    ax, ay, az, aw = a
    bx, by, bz, bw = b
    return np.array([aw * bx + ax * bw + ay * bz - az * by, aw * by - ax * bz + ay * bw + az * bx,
                     aw * bz + ax * by - ay * bx + az * bw, aw * bw - ax * bx - ay * by - az * bz])


def _rotate(q, v):
    u, s = np.asarray(q[:3], np.float64), float(q[3])
    t = 2 * np.cross(u, v)
    return v + s * t + np.cross(u, t)


def _world(n=2, orientations=None, statics=(0,)):
    b = np.zeros(n, abi.BODY_DTYPE)
    b["orientation"][:, 3] = 1.0
    b["flags"] = abi.BODY_ACTIVE | abi.BODY_NO_GRAVITY
    b["linear_damping"] = b["angular_damping"] = 1.0
    b["inv_mass"] = 1.0
    b["inv_inertia"] = (1, 0, 0, 1, 0, 1)
    for i in statics:
        b["motion_type"][i] = abi.MOTION_STATIC
        b["inv_mass"][i] = 0.0
        b["inv_inertia"][i] = 0.0
    for i, q in (orientations or {}).items():
        b["orientation"][i] = q
    sc = dict(bodies=b, shapes=np.zeros(0, abi.SHAPE_DTYPE), hull=np.zeros((0, 3), np.float32),
              triangles=np.zeros(0, abi.TRIANGLE_DTYPE))
    return O.OracleWorld(sc)


def _cone(o, ax1, ax2, ref, lim1, lim2, b1=0, b2=1):
    return o.add_joint(abi.CONSTRAINT_ELLIPTICALCONELIMIT, b1, b2,
                       tuple(ax1) + tuple(ax2) + tuple(ref) + tuple(np.multiply(lim1, RAD)) + tuple(np.multiply(lim2, RAD)))


def _ellipse(o, j, a, b):
    """EllipticalConeLimitTests.EllipseValue (:273-285)."""
    x, y = o.elliptical_swing(j)
    return np.hypot(x / (a * RAD), y / (b * RAD))


def _set_q(o, body, q):
    b = o.bodies()
    b["orientation"][body] = q
    o.set_bodies(b)


def _set_w(o, body, w):
    b = o.bodies()
    b["angular_velocity"][body] = w
    o.set_bodies(b)


@pytest.mark.parametrize("limits", [(0, 60, 0, 25), (15, 60, 5, 25), (60, 60, 25, 25), (100, 160, 30, 120)])
def test_initial_swing_is_measured_in_the_bodies_frames(limits):
    # EllipticalConeLimitTests.InitializationStoresWorldFrameOnCorrespondingBodies (:15-42):
    # body 2's axis starts 45 degrees from body 1's, along the reference
    q1, q2 = _qn((1, 2, 3, 4)), _qn((2, -1, 3, 5))
    o = _world(3, orientations={1: q1, 2: q2}, statics=())
    axis = _qn((1, 3, 2))
    ref = _qn(np.cross(axis, (1.0, 0.0, 0.0)))
    target = _qn(axis + ref)
    j = _cone(o, axis, target, ref + 2 * axis, limits[:2], limits[2:], b1=1, b2=2)
    x, y = o.elliptical_swing(j)
    assert x / RAD == pytest.approx(45, abs=1e-4)
    assert y / RAD == pytest.approx(0, abs=1e-4)
    # rotating body 1 carries its reference along and leaves body 2's axis where it was
    _set_q(o, 1, _qmul(_axis_angle((0, 1, 0), 0.7), q1))
    x2, _ = o.elliptical_swing(j)
    assert abs(x2 / RAD - 45) > 1


@pytest.mark.parametrize("angle", [0.2, 0.8, 2.8, 3.13])
@pytest.mark.parametrize("perturb_body2", [False, True])
def test_jacobian_matches_the_implicit_ellipse_derivative_on_both_bodies(angle, perturb_body2):
    # EllipticalConeLimitTests.JacobianMatchesImplicitEllipseDerivativeOnBothBodies (:84-126),
    # single-precision tolerances; the numerical derivative of the ellipse value is taken in
    # the double-precision oracle (the reference's Jitter2.Double leg, delta 1e-6)
    q1, q2 = _qn((1, 2, 3, 4)), _qn((2, -1, 3, 5))
    axis = _qn((1, 3, 2))
    ref = _qn(np.cross(axis, (1.0, 0.0, 0.0)))
    direction = _qn(ref + np.cross(axis, ref) * 0.6)
    turned = _qmul(_axis_angle(np.cross(axis, direction), angle), q2)
    worlds = []
    for real in ("f", "d"):
        b = np.zeros(3, abi.BODY_DTYPE)
        b["orientation"][:, 3] = 1.0
        b["flags"] = abi.BODY_ACTIVE | abi.BODY_NO_GRAVITY
        b["linear_damping"] = b["angular_damping"] = 1.0
        b["inv_mass"] = 1.0
        b["inv_inertia"] = (1, 0, 0, 1, 0, 1)
        b["orientation"][1], b["orientation"][2] = q1, q2
        sc = dict(bodies=b, shapes=np.zeros(0, abi.SHAPE_DTYPE), hull=np.zeros((0, 3), np.float32),
                  triangles=np.zeros(0, abi.TRIANGLE_DTYPE))
        o = O.OracleWorld(sc, real=real)
        j = _cone(o, axis, axis, ref, (60, 60), (25, 25), b1=1, b2=2)
        worlds.append((o, j))
    (o, j), (od, jd) = worlds
    _set_q(o, 2, turned)
    o.joint_run(j, DT, iterations=0)
    jac = o.joint_data(j)[0]
    bias = o.joint_bias(j)[0]
    body = 2 if perturb_body2 else 1
    q_turned = o.bodies()["orientation"]
    od_b = od.bodies()
    od_b["orientation"] = q_turned
    od.set_bodies(od_b)
    original = q_turned[body].astype(np.float64)
    delta = 1e-6
    num = np.zeros(3)
    for c, d in enumerate(np.eye(3)):
        for sign in (1, -1):
            qq = od.bodies_d()["orientation"].copy()
            qq[body] = _qmul(_axis_angle(d, sign * delta), original)
            od.fn("jor_world_set_orientation_d")(od.h, body, np.ascontiguousarray(qq[body], np.float64).ctypes.data)
            value = _ellipse(od, jd, 60, 25) - 1
            num[c] += sign * value
        od.fn("jor_world_set_orientation_d")(od.h, body, np.ascontiguousarray(original, np.float64).ctypes.data)
    num /= 2 * delta
    expected = jac * (-1 if perturb_body2 else 1)
    assert np.linalg.norm(num / np.linalg.norm(num) - expected) < 0.006
    error = (_ellipse(od, jd, 60, 25) - 1) / np.linalg.norm(num)
    assert bias == pytest.approx(error * 0.2 / DT, abs=max(0.002, abs(error) * 0.02))
    local2 = _rotate(q2 * np.array([-1, -1, -1, 1]), axis)      # body 2's cone axis, local
    axis2 = _rotate(q_turned[2].astype(np.float64), local2)
    assert abs(jac @ axis2) < 1e-5


@pytest.mark.parametrize("angle", [0.1, 0.7, 1.7])
def test_circular_ranges_match_cone_limit(angle):
    # EllipticalConeLimitTests.CircularRangesMatchConeLimit (:186-206)
    q = _axis_angle((1, 2, 0), angle)
    o = _world(3)
    ce = _cone(o, (0, 0, 1), (0, 0, 1), (1, 0, 0), (20, 60), (20, 60), b2=1)
    cc = o.add_joint(abi.CONSTRAINT_CONELIMIT, 0, 2, (0, 0, 1, 0, 0, 1, 20 * RAD, 60 * RAD))
    for body in (1, 2):
        _set_q(o, body, q)
        _set_w(o, body, (1, -2, 3))
    for j in (ce, cc):
        o.joint_run(j, DT, iterations=1)
    w = o.bodies()["angular_velocity"].astype(np.float64)
    assert np.linalg.norm(w[1] - w[2]) < 1e-5
    assert o.joint_impulse(ce)[0] == pytest.approx(o.joint_impulse(cc)[0], abs=1e-5)


def test_the_jacobian_stays_finite_next_to_the_antipode():
    # EllipticalConeLimitTests.NearAntipodeJacobianNormalizationDoesNotOverflow (:208-218)
    o = _world()
    j = _cone(o, (0, 0, 1), (0, 0, 1), (1, 0, 0), (0, 60), (0, 25))
    _set_q(o, 1, _qn((0.6, 0.8, 0.0, 1e-20)))
    o.joint_run(j, DT, iterations=0)
    jac, _, eff, _, _ = o.joint_data(j)
    assert np.linalg.norm(jac) == pytest.approx(1.0, abs=1e-5)
    assert np.isfinite(o.joint_bias(j)[0])
    assert eff > 0


def test_interior_swing_and_twist_are_free_and_a_dropped_warm_start_applies_nothing():
    # EllipticalConeLimitTests.InteriorSwingAndTwistAreUnconstrainedAndWarmStartCanBeReset
    # (:220-243), without the SetLimits part
    o = _world()
    j = _cone(o, (0, 0, 1), (0, 0, 1), (1, 0, 0), (0, 60), (0, 25))
    _set_q(o, 1, _axis_angle((0, 1, 0), 1.3))
    o.joint_params(j, 0.2, 0.0)
    o.joint_run(j, DT, iterations=1)
    assert o.joint_impulse(j)[0] != 0
    o.set_joint_impulses([[0.0, 0.0, 0.0]])
    _set_w(o, 1, (0, 0, 0))
    o.joint_run(j, DT, iterations=0)
    np.testing.assert_array_equal(o.bodies()["angular_velocity"][1], (0, 0, 0))
    q = _axis_angle((0, 1, 0), 0.3)
    _set_q(o, 1, q)
    w = (_rotate(o.bodies()["orientation"][1].astype(np.float64), np.array([0.0, 0.0, 1.0])) * 2).astype(np.float32)
    _set_w(o, 1, w)
    o.set_joint_impulses([[2.0, 0.0, 0.0]])
    o.joint_run(j, DT, iterations=1)
    np.testing.assert_array_equal(o.bodies()["angular_velocity"][1], w)
    assert o.joint_impulse(j)[0] == 0
