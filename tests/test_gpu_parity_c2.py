"""GPU parity on the 20k-body mixed pile (60 x 120 x 60 over a ground box and a 64 x 64-cell
heightfield, seed 12346), the narrowphase workload's own configuration, through the C ABI.

After the pile has formed on the device, one step from identical state is compared with
the oracle: the contact cache the narrowphase registers (every colliding pair, its slots,
normal and point within 1e-4 for at least 99.9 % of contacts) and the post-solve
velocities with the oracle replaying the GPU's solve order (within 1e-3 for at least
99.9 % of bodies).
"""
import numpy as np
import pytest

import oracle_lib as O
from jitterphysics2_gb300 import scenes
from jitterphysics2_gb300.world import world_for_scene
from test_gpu_parity import _one_step_velocity_errors, compare_contact_caches

pytestmark = pytest.mark.gpu

SETTLE = 300


@pytest.fixture(scope="module")
def settled_c2():
    sc = scenes.mixed_pile(n=20000, box=(60.0, 120.0, 60.0), seed=12346)
    w = world_for_scene(sc)
    for _ in range(SETTLE):
        w.step(sc["dt"])
    assert w.counters()["status"] == 0
    return sc, w


def test_c2_narrowphase_matches_oracle(settled_c2):
    sc, w = settled_c2
    sc2 = dict(sc)
    sc2["bodies"] = w.bodies()
    g = world_for_scene(sc2)
    g.step(sc["dt"])
    gc = g.contacts()
    g.close()
    o = O.OracleWorld(sc2)
    o.narrowphase()
    oc = o.contacts()
    assert len(gc) > 10000, len(gc)
    stats = compare_contact_caches(gc, oc)
    print("20k pile narrowphase:", stats)
    assert stats["common_keys"] >= 0.999 * stats["keys"], stats
    assert stats["slot_mismatch"] <= 0.001 * stats["common_keys"], stats
    assert stats["normal_ok"] >= 0.999 and stats["point_ok"] >= 0.999, stats


def test_c2_one_step_velocities_match_oracle(settled_c2):
    sc, w = settled_c2
    err = _one_step_velocity_errors(sc, w)
    print("20k pile one-step velocity error: max %.3g, within 1e-3 %.5f" % (err.max(), np.mean(err < 1e-3)))
    assert np.mean(err < 1e-3) >= 0.999, (np.mean(err < 1e-3), np.sort(err)[-5:])


def test_c2_one_step_velocities_with_more_tasks_than_blocks(settled_c2):
    # a dense partition (9 cells per grid and SM, down to the floor of three arbiter widths)
    # on one task CTA per SM: each block runs several tasks per grid phase, and the result
    # still replays in the oracle's order
    sc, w = settled_c2
    w2 = world_for_scene(sc, sched_cells_per_sm=9.0, solver_ctas_per_sm=1)
    w2.import_state(w.export_state())
    w2.step(sc["dt"])
    c = w2.counters()
    assert c["status"] == 0 and c["solver_tasks"] > 152 and c["task_arbiters"] == c["arbiters"], c
    err = _one_step_velocity_errors(sc, w2)
    print("20k pile, dense partition: max %.3g, within 1e-3 %.5f" % (err.max(), np.mean(err < 1e-3)))
    assert np.mean(err < 1e-3) >= 0.999, (np.mean(err < 1e-3), np.sort(err)[-5:])
