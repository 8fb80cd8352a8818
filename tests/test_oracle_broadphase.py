"""The oracle's grid pair finder against its sort-and-sweep: both evaluate the
reference's pair contract (non-disjoint world AABBs, different bodies of one world, one
active, one dynamic; DynamicTree.cs:266-286, World.cs:447-455) and must agree exactly."""
import numpy as np
import pytest

import oracle_lib as O
from jitterphysics2_gb300 import scenes


@pytest.mark.parametrize("make", [
    lambda: scenes.mixed_pile(n=600, box=(10.0, 6.0, 10.0), y0=-3.0, cells=8, seed=3),   # overlaps, heightfield
    lambda: scenes.box_grid(n_side=5, spacing=1.0),                                       # touching AABBs
    lambda: scenes.batched_worlds(n_worlds=20, lo=8, hi=60, seed=1),                      # worlds on top of each other
    lambda: scenes.free_cluster(n=200, spacing=1.0),                                      # dense, no static body
])
def test_grid_pairs_equal_sweep_pairs(make):
    o = O.OracleWorld(make())
    grid = o.pairs()
    sweep = o.pairs(sweep=True)
    assert np.array_equal(grid, sweep), (len(grid), len(sweep))
