"""Body state through host buffers (jg_upload_bodies, jg_download_bodies, jg_step_host).

The host-buffer step must give bit-identical state to an upload, a device-resident step
and a download; an invalid body must be rejected with the reference's error (non-finite
state: JG_ERR_NONFINITE; bad motion type or world: JG_ERR_INVALID_ARG) and leave the
world's state as it was.
"""
import numpy as np
import pytest

from jitterphysics2_gb300 import abi, scenes
from jitterphysics2_gb300.world import world_for_scene

pytestmark = pytest.mark.gpu


def _settled(steps=30):
    sc = scenes.mixed_pile(n=600, box=(10.0, 20.0, 10.0), seed=424)
    w = world_for_scene(sc)
    for _ in range(steps):
        w.step(sc["dt"])
    return sc, w


def test_step_host_matches_device_step_bitwise():
    sc, a = _settled()
    state = a.export_state()
    b = world_for_scene(sc)
    b.import_state(state)
    host = np.ascontiguousarray(a.bodies())
    for _ in range(3):
        a.step_host(sc["dt"], host)
        b.step(sc["dt"])
    ref = b.bodies()
    for f in ("position", "orientation", "velocity", "angular_velocity", "delta_velocity",
              "delta_angular_velocity", "inv_inertia", "inv_mass", "friction", "motion_type", "world"):
        assert np.array_equal(host[f], ref[f]), f
    assert np.all(host["force"] == 0) and np.all(host["torque"] == 0)
    assert a.counters()["contacts"] == b.counters()["contacts"]


def test_download_keeps_uploaded_settings():
    sc, w = _settled(steps=2)
    up = np.ascontiguousarray(w.bodies())
    up["friction"] = np.linspace(0.1, 0.9, len(up)).astype(np.float32)
    up["linear_damping"] = 0.97
    w.set_bodies(up)
    w.step(sc["dt"])
    down = w.bodies()
    assert np.array_equal(down["friction"], up["friction"])
    assert np.all(down["linear_damping"] == np.float32(0.97))
    assert not np.array_equal(down["position"], up["position"])


@pytest.mark.parametrize("field,value,code", [
    ("position", np.nan, abi.JG_ERR_NONFINITE),
    ("angular_velocity", np.inf, abi.JG_ERR_NONFINITE),
    ("motion_type", 7, abi.JG_ERR_INVALID_ARG),
    ("world", 3, abi.JG_ERR_INVALID_ARG),
])
def test_invalid_body_is_rejected_and_state_kept(field, value, code):
    sc, w = _settled(steps=2)
    before = w.bodies()
    bad = before.copy()
    if bad[field].ndim > 1:
        bad[field][17, 1] = value
    else:
        bad[field][17] = value
    with pytest.raises(abi.JitterError) as e:
        w.set_bodies(bad)
    assert e.value.code == code
    with pytest.raises(abi.JitterError) as e:
        w.step_host(sc["dt"], bad)
    assert e.value.code == code
    after = w.bodies()
    for f in ("position", "orientation", "velocity", "angular_velocity", "motion_type"):
        assert np.array_equal(after[f], before[f]), f
    w.step(sc["dt"])
    assert w.counters()["status"] == 0


def test_first_invalid_body_decides_the_error():
    sc, w = _settled(steps=1)
    bad = w.bodies().copy()
    bad["motion_type"][5] = -1         # invalid argument at body 5
    bad["velocity"][40, 0] = np.nan    # non-finite at body 40
    with pytest.raises(abi.JitterError) as e:
        w.set_bodies(bad)
    assert e.value.code == abi.JG_ERR_INVALID_ARG
    bad["velocity"][2, 2] = np.inf     # non-finite at body 2 comes first now
    with pytest.raises(abi.JitterError) as e:
        w.set_bodies(bad)
    assert e.value.code == abi.JG_ERR_NONFINITE


@pytest.mark.parametrize("cells", [-1.0, float("nan"), float("inf"), 65.0])
def test_invalid_cell_density_is_rejected(cells):
    from jitterphysics2_gb300.world import World
    with pytest.raises(abi.JitterError) as e:
        World(max_bodies=16, sched_cells_per_sm=cells)
    assert e.value.code == abi.JG_ERR_INVALID_ARG
    w = World(max_bodies=16, sched_cells_per_sm=3.0)   # a valid density; 0 means the default
    w.close()
