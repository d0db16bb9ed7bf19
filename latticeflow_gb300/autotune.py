"""Autotuner for the solve knobs: tile shape, local sweeps, launches per relabel.

The knobs trade tile occupancy (tile rows), work per tile visit (local
push/relabel sweeps) and global-relabel frequency (push/relabel passes
between two global relabels).  Their best values depend on the kernel and the
lattice sizes, so they are measured: every candidate is timed on the actual
problem (device time of complete solves: one untimed solve, then the median
of ``repeats`` timed ones, so that a lucky single run does not win), the fastest is
applied and remembered per key (kernel set and size class) in memory and,
when ``cache_path`` is given, in a JSON file.  Results do not depend on the
knobs (the cut sets are canonical), only the time does.
"""
import itertools
import json
import math
import os

DEFAULT_GRID = {
    "pr_kernel": (0, 3),
    "tile_rows": (4, 8, 16, 32),
    "local_sweeps": (1, 2, 4),
    "launches_per_relabel": (4, 8, 16),
}

# 3-d lattices: tiles of 4 planes x 2, 4 or 8 rows x 32 (the staged 3-d pass
# takes 2 and 4 rows for 18 and 26 directions, every height for 6), the
# staged pass (0) or the generic one (1)
VOLUME_GRID = {
    "pr_kernel": (0, 1),
    "tile_rows": (2, 4, 8),
    "local_sweeps": (1, 2, 4),
    "launches_per_relabel": (4, 8, 16),
}

_memory = {}


def size_class(n_nodes):
    """log2 bucket of the node count."""
    return int(math.floor(math.log2(max(1, n_nodes))))


def problem_key(kernels, n_nodes):
    return "%s|%d" % ("+".join(sorted(set(kernels))), size_class(n_nodes))


def _load(cache_path):
    if cache_path and os.path.exists(cache_path):
        with open(cache_path) as f:
            return json.load(f)
    return {}


def _store(cache_path, table):
    if not cache_path:
        return
    d = os.path.dirname(cache_path)
    if d:
        os.makedirs(d, exist_ok=True)
    tmp = cache_path + ".tmp"
    with open(tmp, "w") as f:
        json.dump(table, f, indent=1, sort_keys=True)
    os.replace(tmp, cache_path)


def tune(solver, key, grid=None, repeats=3, cache_path=None, force=False):
    """Choose and apply the fastest knob setting for ``solver``.

    ``solver`` is a ``LatticeFlow`` or ``LatticeBatch`` that is already
    filled; it must offer ``setParam``, ``run`` and ``runTime``.  Returns
    (setting, seconds, table of all timings).
    """
    table = dict(_memory)
    table.update(_load(cache_path))
    if not force and key in table:
        best = table[key]["setting"]
        for k, v in best.items():
            solver.setParam(k, v)
        return best, table[key]["seconds"], None
    grid = grid or DEFAULT_GRID
    names = sorted(grid)
    timings = []
    best, best_t = None, float("inf")
    for values in itertools.product(*[grid[n] for n in names]):
        setting = dict(zip(names, values))
        for k, v in setting.items():
            solver.setParam(k, v)
        _timed(solver)  # first solve of a setting: kernel variants load, caches fill
        ts = sorted(_timed(solver) for _ in range(max(1, repeats)))
        t = ts[len(ts) // 2]
        timings.append((setting, t))
        if t < best_t:
            best, best_t = setting, t
    for k, v in best.items():
        solver.setParam(k, v)
    entry = {"setting": best, "seconds": best_t}
    _memory[key] = entry
    if cache_path:
        disk = _load(cache_path)
        disk[key] = entry
        _store(cache_path, disk)
    return best, best_t, timings


def _timed(solver):
    solver.run()
    return solver.runTime()
