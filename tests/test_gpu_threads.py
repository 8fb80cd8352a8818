"""Worlds are independent: each keeps its own scratch and launch shapes, so two worlds
stepped by two host threads at once (one host thread per world, the reference's single
owner per World, docfx/docs/documentation/world.md:75-97) give the bits each gives alone.
Also the World property setters (jg_set_params) and the checkpoint import's validation."""
import threading

import numpy as np
import pytest

from jitterphysics2_gb300 import abi, scenes
from jitterphysics2_gb300.abi import JitterError
from jitterphysics2_gb300.world import world_for_scene

pytestmark = pytest.mark.gpu

STEPS = 60


def _run(sc, kw, steps, out, key):
    w = world_for_scene(sc, **kw)
    for _ in range(steps):
        w.step(sc["dt"])
    out[key] = (w.bodies(), w.counters())
    w.close()


def test_two_worlds_on_two_threads_match_their_runs_alone():
    sa = scenes.mixed_pile(n=300, box=(15.0, 6.0, 15.0), y0=0.0, cells=8, seed=31, lattice=2.5)
    sb = scenes.mixed_pile(n=600, box=(20.0, 8.0, 20.0), y0=0.0, cells=8, seed=32, lattice=2.5)
    ka = dict(solver_ctas_per_sm=1, max_arbiters=4096)
    kb = dict(solver_ctas_per_sm=2, max_arbiters=20000, partitioned_solve=0)
    alone = {}
    _run(sa, ka, STEPS, alone, "a")
    _run(sb, kb, STEPS, alone, "b")
    together = {}
    ta = threading.Thread(target=_run, args=(sa, ka, STEPS, together, "a"))
    tb = threading.Thread(target=_run, args=(sb, kb, STEPS, together, "b"))
    ta.start(); tb.start(); ta.join(); tb.join()
    for k in ("a", "b"):
        b0, c0 = alone[k]
        b1, c1 = together[k]
        assert c0["status"] == 0 and c1["status"] == 0
        assert c0["contacts"] > 50
        assert np.array_equal(b0["position"], b1["position"]), k
        assert np.array_equal(b0["velocity"], b1["velocity"]), k


def test_set_params_changes_the_solver_settings():
    sc = scenes.box_grid(n_side=3)
    w = world_for_scene(sc)
    p = abi.WorldParams()
    abi.check(w._lib.jg_get_params(w.handle, abi.ctypes.byref(p)), "jg_get_params")
    assert p.substeps == sc["params"]["substeps"]
    p.substeps, p.solver_iterations = 2, 3
    abi.check(w._lib.jg_set_params(w.handle, abi.ctypes.byref(p)), "jg_set_params")
    q = abi.WorldParams()
    w._lib.jg_get_params(w.handle, abi.ctypes.byref(q))
    assert (q.substeps, q.solver_iterations) == (2, 3)
    w.step(sc["dt"])
    # the reference's ArgumentOutOfRangeException cases and a capacity change are refused
    for field, value in (("substeps", 0), ("solver_iterations", 0), ("relax_iterations", -1),
                         ("max_bodies", q.max_bodies + 1)):
        bad = abi.WorldParams()
        w._lib.jg_get_params(w.handle, abi.ctypes.byref(bad))
        setattr(bad, field, value)
        assert w._lib.jg_set_params(w.handle, abi.ctypes.byref(bad)) == abi.JG_ERR_INVALID_ARG, field
    w.close()


def test_import_rejects_a_corrupted_state_and_keeps_the_world():
    sc = scenes.mixed_pile(n=200, box=(12.0, 4.0, 12.0), y0=0.0, cells=8, seed=3, lattice=2.5)
    w = world_for_scene(sc)
    for _ in range(30):
        w.step(sc["dt"])
    blob = w.export_state()
    before = w.bodies()
    for bad in (blob[:-1], blob[:10]):
        with pytest.raises(JitterError):
            w.import_state(bad)
    # an arbiter naming a body outside the world
    nb = len(before)
    narb = int(np.frombuffer(blob[12:16].tobytes(), np.int32)[0])
    assert narb > 0
    off = 24 + abi.BODY_DTYPE.itemsize * nb + 8 * narb  # first arbiter's body pair
    corrupt = blob.copy()
    corrupt[off:off + 4] = np.frombuffer(np.int32(nb + 7).tobytes(), np.uint8)
    with pytest.raises(JitterError):
        w.import_state(corrupt)
    assert np.array_equal(w.bodies()["position"], before["position"])
    w.import_state(blob)
    w.step(sc["dt"])
    assert w.counters()["status"] == 0
