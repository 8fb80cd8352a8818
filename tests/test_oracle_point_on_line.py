"""PointOnLine in the oracle (CPU): the reference's constraint-level cases, restated with one
Prepare and one Iterate at TimeStep(1/100) (CoupledLimitTests.cs:12-153,
ConstraintMassRegressionTests.cs:14-31).

A clamped limit leaves inward motion along the line alone, with or without a warm start;
the block solve satisfies the active rows and does not add energy; a singular coupled block
still leaves inward motion free; a changed limit discards a warm start of the wrong sign;
two moving bodies keep their free inward motion; an inactive limit leaves tiny but
responsive rows working.
"""
import numpy as np
import pytest

import oracle_lib as O
from jitterphysics2_gb300 import abi

TOL = 2e-5   # CoupledLimitTests.cs:9, single precision
DT = 0.01


def _world(n=2, inv_inertia=(1, 0, 0, 1, 0, 1), inv_mass=1.0):
    """Body 0: static at the origin (the NullBody); bodies 1..: dynamic at the origin."""
    b = np.zeros(n, abi.BODY_DTYPE)
    b["orientation"][:, 3] = 1.0
    b["flags"] = abi.BODY_ACTIVE | abi.BODY_NO_GRAVITY
    b["linear_damping"] = b["angular_damping"] = 1.0
    b["motion_type"][0] = abi.MOTION_STATIC
    b["inv_mass"][1:] = inv_mass
    b["inv_inertia"][1:] = inv_inertia
    sc = dict(bodies=b, shapes=np.zeros(0, abi.SHAPE_DTYPE), hull=np.zeros((0, 3), np.float32),
              triangles=np.zeros(0, abi.TRIANGLE_DTYPE))
    return O.OracleWorld(sc)


def _line(o, axis, a1, a2, lo, hi, bias=0.0, softness=0.0, b1=0, b2=1):
    j = o.add_joint(abi.CONSTRAINT_POINTONLINE, b1, b2, tuple(axis) + tuple(a1) + tuple(a2) + (lo, hi))
    o.joint_params(j, bias, softness)
    o.joint_limit_params(j, bias, softness)
    return j


def _set(o, body, v=None, w=None):
    b = o.bodies()
    if v is not None:
        b["velocity"][body] = v
    if w is not None:
        b["angular_velocity"][body] = w
    o.set_bodies(b)


def _limit(upper):
    return (-1.0, 0.0) if upper else (0.0, 1.0)


@pytest.mark.parametrize("upper", [False, True])
@pytest.mark.parametrize("warm", [False, True])
@pytest.mark.parametrize("softness", [0.0, 1e-5])
def test_inward_motion_is_unaffected_by_a_clamped_limit(upper, warm, softness):
    # CoupledLimitTests.PointOnLine_InwardMotionIsUnaffectedByClampedLimit (:12-34)
    o = _world()
    j = _line(o, (0, 0, 1), (1, 1, 1), (1, 1, 1), *_limit(upper), softness=softness)
    d = -1.0 if upper else 1.0
    _set(o, 1, v=(0, 0, d))
    if warm:
        o.set_joint_impulses([[0.2, -0.3, d * 0.4]])
    o.joint_run(j, DT, iterations=1)
    assert o.joint_impulse(j)[2] == 0
    b = o.bodies()
    assert np.abs(b["velocity"][1] - (0, 0, d)).max() < TOL
    assert np.abs(b["angular_velocity"][1]).max() < TOL


@pytest.mark.parametrize("upper", [False, True])
@pytest.mark.parametrize("inward", [False, True])
@pytest.mark.parametrize("softness", [0.0, 1e-5])
def test_block_solve_satisfies_active_rows_and_dissipates_energy(upper, inward, softness):
    # CoupledLimitTests.PointOnLine_BlockSolveSatisfiesActiveRowsAndDissipatesEnergy (:36-76)
    inv_i = np.array([[2, 0.3, -0.4], [0.3, 1, 0.2], [-0.4, 0.2, 3]])
    inertia = np.linalg.inv(inv_i)
    o = _world(inv_inertia=(2, 0.3, -0.4, 1, 0.2, 3))
    anchor = np.array([1.0, 1.0, 1.0])
    j = _line(o, (0, 0, 1), anchor, anchor, *_limit(upper), softness=softness)
    v0 = np.array([0.5, -0.25, (-5 if upper else 5) * (1 if inward else -1)])
    w0 = np.array([0.1, 0.2, -0.1])
    _set(o, 1, v=v0, w=w0)
    e0 = v0 @ v0 + w0 @ inertia @ w0
    o.joint_run(j, DT, iterations=1)
    b = o.bodies()
    v, w = b["velocity"][1].astype(np.float64), b["angular_velocity"][1].astype(np.float64)
    imp = o.joint_impulse(j)
    pv = v + np.cross(w, anchor)
    rx = pv[1] + 100 * softness * imp[0]
    ry = -pv[0] + 100 * softness * imp[1]
    if inward:
        assert imp[2] == 0
    else:
        assert imp[2] * (-1 if upper else 1) > 0
        assert abs(pv[2] + 100 * softness * imp[2]) < TOL
    assert abs(rx) < TOL and abs(ry) < TOL
    assert v @ v + w @ inertia @ w <= e0 + TOL


@pytest.mark.parametrize("upper", [False, True])
def test_a_singular_coupled_block_still_leaves_inward_motion_free(upper):
    # CoupledLimitTests.PointOnLine_SingularCoupledBlockStillLeavesInwardMotionFree (:78-97)
    o = _world(inv_inertia=(1, 0, 0, 1, 0, 0), inv_mass=0.0)
    j = _line(o, (0, 0, 1), (1, 1, 1), (1, 1, 1), *_limit(upper))
    d = -1.0 if upper else 1.0
    _set(o, 1, v=(0, 0, d))
    o.joint_run(j, DT, iterations=1)
    b = o.bodies()
    assert o.joint_impulse(j)[2] == 0
    assert np.abs(b["angular_velocity"][1]).max() < TOL
    np.testing.assert_array_equal(b["velocity"][1], (0, 0, d))


@pytest.mark.parametrize("upper", [False, True])
@pytest.mark.parametrize("inactive", [False, True])
def test_a_changed_limit_discards_an_inadmissible_warm_start(upper, inactive):
    # CoupledLimitTests.PointOnLine_ChangedLimitDiscardsInadmissibleWarmStart (:99-121)
    o = _world()
    j = _line(o, (0, 0, 1), (1, 1, 1), (1, 1, 1), 1e-6, -1e-6)
    o.set_joint_impulses([[0.0, 0.0, 1.0 if upper else -1.0]])
    lo, hi = (-np.inf, np.inf) if inactive else _limit(upper)
    o.joint_set_limit(j, lo, hi)
    d = -1.0 if upper else 1.0
    _set(o, 1, v=(0, 0, d))
    o.joint_run(j, DT, iterations=0)
    b = o.bodies()
    assert o.joint_impulse(j)[2] == 0
    np.testing.assert_array_equal(b["velocity"][1], (0, 0, d))
    np.testing.assert_array_equal(b["angular_velocity"][1], (0, 0, 0))
    o.joint_run(j, DT, iterations=1, prepare=False)
    b = o.bodies()
    assert np.abs(b["velocity"][1] - (0, 0, d)).max() < TOL
    assert np.abs(b["angular_velocity"][1]).max() < TOL


def _qnorm(q):
    q = np.asarray(q, np.float64)
    return tuple((q / np.linalg.norm(q)).astype(np.float32).tolist())


@pytest.mark.parametrize("upper", [False, True])
def test_two_moving_bodies_retain_free_inward_motion(upper):
    # CoupledLimitTests.PointOnLine_TwoMovingBodiesRetainFreeInwardMotion (:123-153): the limit
    # starts or ends at the anchors' distance along the line
    b = np.zeros(3, abi.BODY_DTYPE)
    b["orientation"][:, 3] = 1.0
    b["flags"] = abi.BODY_ACTIVE | abi.BODY_NO_GRAVITY
    b["linear_damping"] = b["angular_damping"] = 1.0
    b["motion_type"][0] = abi.MOTION_STATIC
    b["inv_mass"][1:] = 1.0
    b["inv_inertia"][1:] = (1, 0, 0, 1, 0, 1)
    b["orientation"][1] = _qnorm((1, 2, 3, 4))
    b["position"][2] = (1, -2, 0.5)
    b["orientation"][2] = (0.0, float(np.sin(0.15)), 0.0, float(np.cos(0.15)))
    sc = dict(bodies=b, shapes=np.zeros(0, abi.SHAPE_DTYPE), hull=np.zeros((0, 3), np.float32),
              triangles=np.zeros(0, abi.TRIANGLE_DTYPE))
    o = O.OracleWorld(sc)
    axis = np.array([1.0, 2.0, 3.0]) / np.sqrt(14.0)
    anchor = (0.2, 0.4, 0.3)
    j = _line(o, axis, anchor, anchor, *_limit(upper), b1=1, b2=2)
    dist = o.line_distance(j)
    o.joint_set_limit(j, dist - 1 if upper else dist, dist if upper else dist + 1)
    v1 = axis * 0.3
    v2 = v1 + axis * (-1 if upper else 1)
    _set(o, 1, v=v1)
    _set(o, 2, v=v2)
    o.joint_run(j, DT, iterations=1)
    assert o.joint_data(j)[3] == (1 if upper else 2)   # the clamp state
    bb = o.bodies()
    assert np.abs(bb["velocity"][1] - v1).max() < TOL
    assert np.abs(bb["velocity"][2] - v2).max() < TOL
    assert np.abs(bb["angular_velocity"][1:3]).max() < TOL


@pytest.mark.parametrize("inv_mass", [1e-7, 1e-13])
def test_an_inactive_limit_preserves_small_responsive_rows(inv_mass):
    # ConstraintMassRegressionTests.PointOnLine_InactiveLimitPreservesSmallResponsiveRows
    # (:14-31), the unlocked cases
    o = _world(inv_inertia=(0, 0, 0, 0, 0, 0), inv_mass=inv_mass)
    j = _line(o, (0, 0, 1), (0, 0, 0), (0, 0, 0), -np.inf, np.inf)
    _set(o, 1, v=(1, 0, 2))
    o.joint_run(j, DT, iterations=1)
    assert np.abs(o.bodies()["velocity"][1] - (0, 0, 2)).max() < 1e-5
