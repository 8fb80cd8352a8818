"""The cell neighbourhood behind the partitioned solve's phase hand-off (CPU).

The schedule places a body in cell floor((x - x0) / h + g / 3) of grid g (clamped to the
grid), per axis, in float32 as the device computes it.  A task of grid g waits for the tasks
of the two grids before it whose cells may hold one of its bodies: cells ix - 1 .. ix of a
grid with a smaller offset and ix .. ix + 1 of one with a larger offset.  Every body's cell
in any other grid must therefore lie in that window, at the edges of the grid as well.
"""
import numpy as np


def cell_of(x, x0, h, g, ncx):
    off = np.float32(0.0) if g == 0 else (np.float32(1.0 / 3.0) if g == 1 else np.float32(2.0 / 3.0))
    u = (np.float32(x) - np.float32(x0)) / np.float32(h) + off
    return np.clip(np.floor(u).astype(np.int64), 0, ncx - 1)


def test_other_grid_cells_lie_in_the_dependency_window():
    rng = np.random.Generator(np.random.PCG64(7))
    for trial in range(200):
        h = np.float32(rng.uniform(0.2, 12.0))
        x0 = np.float32(rng.uniform(-100, 100))
        ncx = int(rng.integers(1, 40))
        # positions across the grid, past both edges, and right on cell boundaries
        xs = np.concatenate([
            rng.uniform(x0 - 2 * h, x0 + (ncx + 2) * h, 4000),
            x0 + h * (np.arange(-2, ncx + 3) + rng.choice([0.0, 1 / 3, 2 / 3], ncx + 5)),
        ]).astype(np.float32)
        for g in range(3):
            cg = cell_of(xs, x0, h, g, ncx)
            for gp in range(3):
                if gp == g:
                    continue
                d0 = 0 if gp > g else -1
                lo = np.clip(cg + d0, 0, ncx - 1)
                hi = np.clip(cg + d0 + 1, 0, ncx - 1)
                c = cell_of(xs, x0, h, gp, ncx)
                bad = (c < lo) | (c > hi)
                assert not bad.any(), (trial, g, gp, xs[bad][:3], cg[bad][:3], c[bad][:3])


def test_each_grid_phase_has_both_earlier_phases_as_dependencies():
    # the hand-off waits on grids g - 1 and g - 2 (mod 3): the union over both offsets of a
    # grid-g cell's window covers every other grid, so no earlier access to a body is missed
    for g in range(3):
        earlier = {(g - 1) % 3, (g - 2) % 3}
        assert earlier == set(range(3)) - {g}
