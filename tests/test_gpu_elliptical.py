"""EllipticalConeLimit on the device, through the C ABI.

- Thirty steps of pendulums held by a BallSocket and an EllipticalConeLimit, each replayed
  in the oracle from the GPU's state, in the GPU's order keys with the GPU's impulses:
  velocities within 1e-3, impulses within 1e-3 relative.
- The reference's world-level case (EllipticalConeLimitTests.SimulationRecoversIntoAllowedRegion,
  EllipticalConeLimitTests.cs:128-168): from poses outside the maximum, inside a band's
  inner ellipse, at and next to the antipode, the body comes back into the allowed region
  (or onto a fixed ellipse) within 400 steps, with finite orientations and bounded spin.
- The reference's argument checks (EllipticalConeLimitTests.cs:44-82) and the Bias /
  Softness setter.
"""
import numpy as np
import pytest

import oracle_lib as O
from jitterphysics2_gb300 import abi
from jitterphysics2_gb300.world import world_for_scene

pytestmark = pytest.mark.gpu
RAD = np.pi / 180


def _scene(n=2, **params):
    b = np.zeros(n, abi.BODY_DTYPE)
    b["orientation"][:, 3] = 1.0
    b["flags"] = abi.BODY_ACTIVE | abi.BODY_NO_GRAVITY
    b["linear_damping"] = b["angular_damping"] = 1.0
    b["motion_type"][0] = abi.MOTION_STATIC
    b["inv_mass"][1:] = 1.0
    b["inv_inertia"][1:] = (1, 0, 0, 1, 0, 1)
    prm = dict(gravity=(0.0, 0.0, 0.0), allow_deactivation=0)
    prm.update(params)
    return dict(bodies=b, shapes=np.zeros(0, abi.SHAPE_DTYPE), hull=np.zeros((0, 3), np.float32),
                triangles=np.zeros(0, abi.TRIANGLE_DTYPE), joints=[], params=prm, dt=0.01)


def _cone_init(lim1=(0, 60), lim2=(0, 25)):
    """EllipticalConeLimitTests.CreateCone (:245-250): axis z on both bodies, reference x."""
    return (0, 0, 1, 0, 0, 1, 1, 0, 0) + tuple(np.multiply(lim1, RAD)) + tuple(np.multiply(lim2, RAD))


def _ellipse(q, a, b):
    """EllipseValue of body 1's swing (GetSwing, EllipticalConeLimit.cs:206-221) against
    semiaxes a, b (degrees), for the cone of _cone_init on a body created unrotated."""
    q = np.asarray(q, np.float64)
    u, s = q[:3], q[3]
    z = np.array([0.0, 0.0, 1.0])
    t = 2 * np.cross(u, z)
    target = z + s * t + np.cross(u, t)
    x, y = target[0], target[1]
    sine = np.hypot(x, y)
    angle = np.arctan2(sine, target[2])
    factor = angle / sine if sine > 0 else 0.0
    along = x * factor if sine > 0 else angle
    return np.hypot(along / (a * RAD), y * factor / (b * RAD))


def pendulums(n=16, seed=12355):
    """Boxes hanging from static anchors (no shapes) by a BallSocket at their top, each held
    in an elliptical cone (60 x 25 degrees, a 20 x 10 degree inner band) about the vertical,
    set swinging by random angular velocities: the outer and inner limits both engage.
    The pendulums are 4 apart: no contacts."""
    rng = np.random.Generator(np.random.PCG64(seed))
    b = np.zeros(2 * n, abi.BODY_DTYPE)
    b["orientation"][:, 3] = 1.0
    b["flags"] = abi.BODY_ACTIVE
    b["linear_damping"], b["angular_damping"] = 0.998, 0.995
    s = np.zeros(n, abi.SHAPE_DTYPE)
    joints = []
    for i in range(n):
        a, k = 2 * i, 2 * i + 1
        base = np.array([4.0 * i, 10.0, 0.0])
        b["position"][a] = base
        b["motion_type"][a] = abi.MOTION_STATIC
        b["position"][k] = base - (0.0, 0.55, 0.0)
        b["motion_type"][k] = abi.MOTION_DYNAMIC
        b["inv_mass"][k] = 1.0 / (0.2 * 1.0 * 0.2)
        b["inv_inertia"][k] = (30.0, 0.0, 0.0, 300.0, 0.0, 30.0)
        b["angular_velocity"][k] = rng.normal(0.0, 3.0, 3)
        s["kind"][i] = abi.SHAPE_BOX
        s["body"][i] = k
        s["dims"][i, :3] = (0.1, 0.5, 0.1)
        joints.append((abi.CONSTRAINT_BALLSOCKET, a, k, tuple(base - (0.0, 0.05, 0.0))))
        joints.append((abi.CONSTRAINT_ELLIPTICALCONELIMIT, a, k,
                       (0, -1, 0, 0, -1, 0, 1, 0, 0, 20 * RAD, 60 * RAD, 10 * RAD, 25 * RAD)))
    return dict(bodies=b, shapes=s, hull=np.zeros((0, 3), np.float32), triangles=np.zeros(0, abi.TRIANGLE_DTYPE),
                joints=joints, params=dict(substeps=4, solver_iterations=8, relax_iterations=4), dt=0.01)


def test_elliptical_pendulums_step_with_the_oracle():
    """Every step of 30, replayed in the oracle from the GPU's state and impulses in the GPU's
    order keys; the oracle keeps the cones' own state between steps (the last clamp and
    Jacobian, which decide whether a warm start survives), as the device does."""
    sc = pendulums()
    w = world_for_scene(sc)
    o = O.OracleWorld(sc, external_order=True)
    kinds = np.array([j[0] for j in sc["joints"]])
    worst, engaged = 0.0, 0
    for _ in range(30):
        b0 = w.bodies()
        _, j0 = w.constraints()
        w.step(sc["dt"])
        b1 = w.bodies()
        k1, j1 = w.constraints()
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
        worst = max(worst, float(err.max()))
        assert np.mean(jerr < 1e-3) >= 0.999, np.sort(jerr)[-5:]
        engaged += np.count_nonzero(j1[kinds == abi.CONSTRAINT_ELLIPTICALCONELIMIT][:, 0])
    assert engaged >= 30
    assert worst < 1e-3, worst


CASES = [(0.0, 0.6, "Maximum"), (0.15, 0.6, "Band"), (1.8, 0.6, "Maximum"), (1.8, 0.6, "Band"),
         (0.0, 0.6, "Fixed"), (1.8, 0.6, "Fixed"), (np.pi, 0.0, "Band"), (3.14158, 0.6, "Band")]


@pytest.mark.parametrize("angle,azimuth,kind", CASES)
def test_simulation_recovers_into_the_allowed_region(angle, azimuth, kind):
    # EllipticalConeLimitTests.SimulationRecoversIntoAllowedRegion (:128-168), softness 0,
    # the body's angular damping 0.01 and no gyroscopic term, one substep, (8, 0) iterations
    lim = {"Maximum": ((0, 60), (0, 25)), "Band": ((20, 60), (10, 25)), "Fixed": ((60, 60), (25, 25))}[kind]
    sc = _scene(substeps=1, solver_iterations=8, relax_iterations=0)
    sc["bodies"]["angular_damping"][1] = 0.99
    sc["joints"] = [(abi.CONSTRAINT_ELLIPTICALCONELIMIT, 0, 1, _cone_init(*lim))]
    w = world_for_scene(sc)
    w.set_constraint_params(0, softness=0.0)
    axis = np.array([-np.sin(azimuth), np.cos(azimuth), 0.0])
    if angle == np.pi:
        q = np.append(axis, 0.0)
    else:
        q = np.append(axis * np.sin(angle / 2), np.cos(angle / 2))
    w.set_body(1, "orientation", q.astype(np.float32))
    for _ in range(400):
        w.step(0.01)
        b = w.bodies()
        assert np.isfinite(np.sum(b["orientation"][1].astype(np.float64) ** 2))
        assert np.linalg.norm(b["angular_velocity"][1]) < 100
    q1 = w.bodies()["orientation"][1]
    assert _ellipse(q1, 60, 25) <= 1.003
    if kind == "Band":
        assert _ellipse(q1, 20, 10) >= 0.997
    if kind == "Fixed":
        assert _ellipse(q1, 60, 25) == pytest.approx(1.0, abs=0.003)


@pytest.mark.parametrize("lim", [(-1, 60, 5, 25), (61, 60, 5, 25), (0, 0, 0, 25), (0, 180, 0, 25), (0, 60, 5, 25),
                                 (15, 60, 0, 25), (np.nan, 60, 5, 25), (15, np.inf, 5, 25)])
def test_invalid_limits_are_rejected(lim):
    # EllipticalConeLimitTests.InvalidLimitsLeaveExistingConfigurationUnchanged (:44-65)
    w = world_for_scene(_scene())
    with pytest.raises(abi.JitterError) as e:
        w.add_constraint(abi.CONSTRAINT_ELLIPTICALCONELIMIT, 0, 1, _cone_init(lim[:2], lim[2:]))
    assert e.value.code == abi.JG_ERR_INVALID_ARG


def test_invalid_directions_are_rejected():
    # EllipticalConeLimitTests.InvalidDirectionsAreRejectedBeforeChangingTheFrame (:67-82)
    w = world_for_scene(_scene())
    lim = (0.0, 45 * RAD, 0.0, 45 * RAD)
    for bad in ((0, 0, 0), (np.nan, 0, 0)):
        for init in (bad + (0, 0, 1) + (1, 0, 0), (0, 0, 1) + bad + (1, 0, 0), (0, 0, 1) + (0, 0, 1) + bad):
            with pytest.raises(abi.JitterError):
                w.add_constraint(abi.CONSTRAINT_ELLIPTICALCONELIMIT, 0, 1, init + lim)
    with pytest.raises(abi.JitterError):   # a reference along the axis
        w.add_constraint(abi.CONSTRAINT_ELLIPTICALCONELIMIT, 0, 1, (1, 0, 0, 1, 0, 0, 1, 0, 0) + lim)
    w.add_constraint(abi.CONSTRAINT_ELLIPTICALCONELIMIT, 0, 1, _cone_init())


def test_constraint_params_are_checked():
    sc = _scene()
    sc["joints"] = [(abi.CONSTRAINT_ELLIPTICALCONELIMIT, 0, 1, _cone_init()),
                    (abi.CONSTRAINT_HINGEANGLE, 0, 1, (0, 0, 1, -1.0, 1.0)),
                    (abi.CONSTRAINT_ANGULARMOTOR, 0, 1, (0, 0, 1, 0, 0, 1, 1.0, 1.0))]
    w = world_for_scene(sc)
    w.set_constraint_params(0, bias=0.3, softness=0.0)
    w.set_constraint_params(1, limit_bias=0.05, limit_softness=0.0)
    for bad in (dict(bias=-1.0), dict(softness=-0.1), dict(limit_bias=0.1)):
        with pytest.raises(abi.JitterError):
            w.set_constraint_params(0, **bad)
    with pytest.raises(abi.JitterError):
        w.set_constraint_params(2, softness=0.0)   # a motor has no softness
    w.step(0.01)
    assert w.counters()["status"] == 0
