"""Parametric flow and single-lambda TV on the GPU, against the oracle.

What is exact, and checked exactly, for TV: the level-set partition (every
node's level set, the sets numbered in the reference's order), every level
set's sum of final 2x-scaled values r, and so how many of its nodes hold
each of its (at most two, adjacent) values and how many are on (r < 0).
What is not: which nodes of a level set hold the upper value -- the
reference hands the rounding remainder inside a final level set to nodes in
the order of its pushes, so any other push order (here: parallel) gives
other nodes the +1.  Per node, r is therefore within R_TOL = 1 raw unit, and
the double outputs of the TV solver within OUT_RTOL relative (1 raw unit is
2^-41 of the function range).  For the level-set solver on small integer
energies (check_level_sums) the same remainder can also decide whether two
neighbouring sets one unit apart are separated; there the exact bar is the
sum over every level set.
"""
import glob
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden")
R_TOL = 1
OUT_RTOL = 1e-9


def _close_out(a, b):
    scale = max(1.0, float(np.abs(b).max()))
    return float(np.abs(a - b).max()) <= OUT_RTOL * scale


def check_level_sums(r, sets, r_ref, sets_ref):
    """For integer energies whose neighbouring level sets differ by one raw
    unit, which of them the reference finally separates depends on its push
    order (a final range spread over two units splits once more); what is
    exact is the sum of r over every level set of the GPU solve, equal to the
    reference's sum over the same nodes.  Within a set of either solver the
    values differ by at most one unit, and per node by at most one unit."""
    r, sets = np.asarray(r).reshape(-1), np.asarray(sets).reshape(-1)
    r_ref, sets_ref = np.asarray(r_ref).reshape(-1), np.asarray(sets_ref).reshape(-1)
    assert sets.min() == 0
    for ids, vals in ((sets, r), (sets_ref, r_ref)):
        n = int(ids.max()) + 1
        lo = np.full(n, np.iinfo(np.int64).max)
        hi = np.full(n, np.iinfo(np.int64).min)
        np.minimum.at(lo, ids, vals)
        np.maximum.at(hi, ids, vals)
        assert int((hi - lo).max()) <= 1
    n = int(sets.max()) + 1
    a = np.zeros(n, dtype=object)
    b = np.zeros(n, dtype=object)
    for k, x, y in zip(sets.tolist(), r.tolist(), r_ref.tolist()):
        a[k] += x
        b[k] += y
    assert all(int(x) == int(y) for x, y in zip(a, b))
    assert int(np.abs(r - r_ref).max()) <= R_TOL


def check_level_sets(r, sets, r_ref, sets_ref):
    """Exact partition and per-set sums; within a set the values are v or
    v + 1 on both sides with the same counts; per node within one unit."""
    r, sets = np.asarray(r).reshape(-1), np.asarray(sets).reshape(-1)
    r_ref, sets_ref = np.asarray(r_ref).reshape(-1), np.asarray(sets_ref).reshape(-1)
    assert np.array_equal(sets, sets_ref)
    n_sets = int(sets_ref.max()) + 1
    assert sets_ref.min() == 0 and np.all(np.bincount(sets_ref, minlength=n_sets) > 0)
    order = np.argsort(sets_ref, kind="stable")
    bounds = np.searchsorted(sets_ref[order], np.arange(n_sets + 1))
    for k in range(n_sets):
        idx = order[bounds[k]:bounds[k + 1]]
        a, b = r[idx], r_ref[idx]
        assert int(a.sum()) == int(b.sum()), k
        assert int(a.max() - a.min()) <= 1 and int(b.max() - b.min()) <= 1, k
        assert int(a.min()) == int(b.min()) or int(a.max()) == int(b.max()), k
        assert np.array_equal(np.sort(a), np.sort(b)), k
        assert int((a < 0).sum()) == int((b < 0).sum()), k
    assert int(np.abs(r - r_ref).max()) <= R_TOL


@pytest.mark.parametrize("path", sorted(glob.glob(os.path.join(GOLD, "tv_*.npz"))),
                         ids=lambda p: os.path.basename(p))
def test_tv_golden(native, gpu, oracle_port, path):
    import latticeflow_gb300 as lf
    z = np.load(path)
    kernel = str(z["kernel"])
    out, lv, sets = lf.calculate2dTV(z["f"], float(z["lam"]), kernel=kernel, return_levels=True,
                                     return_sets=True)
    _, r, _, sets_ref = oracle_port.port_tv_single(kernel, z["f"], float(z["lam"]), return_sets=True)
    dr = int(np.abs(lv - r).max())
    print(os.path.basename(path), "max |dr| =", dr, "max |dout| =", float(np.abs(out - z["out"]).max()))
    check_level_sets(lv, sets, r, sets_ref)
    assert _close_out(out, z["out"])


@pytest.mark.parametrize("lam", [0.002, 0.3, 5.0, 100.0])
def test_tv_image_vs_oracle(native, gpu, oracle_port, lam):
    import latticeflow_gb300 as lf
    from latticeflow_gb300 import workloads as W
    f = W.tv_image(1, n=96, polygons=6)
    out, lv, sets = lf.calculate2dTV(f, lam, return_levels=True, return_sets=True)
    ref, r, _, sets_ref = oracle_port.port_tv_single("Full2d_4", f, lam, return_sets=True)
    dr = int(np.abs(lv - r).max())
    print("lam", lam, "max |dr| =", dr, "levels", len(np.unique(r)))
    check_level_sets(lv, sets, r, sets_ref)
    assert _close_out(out, ref)


def test_tv_ragged_and_tiny(native, gpu, oracle_port):
    import latticeflow_gb300 as lf
    rng = np.random.default_rng(4)
    for shape in [(1, 1), (1, 7), (5, 1), (33, 65), (70, 3)]:
        f = rng.random(shape)
        out, lv, sets = lf.calculate2dTV(f, 20.0, return_levels=True, return_sets=True)
        ref, r, _, sets_ref = oracle_port.port_tv_single("Full2d_4", f, 20.0, return_sets=True)
        check_level_sets(lv, sets, r, sets_ref)
        assert _close_out(out, ref), shape


@pytest.mark.parametrize("kernel,dims", [("Full2d_4", (40, 37)), ("Full2d_8", (31, 29)),
                                         ("Full3d_6", (9, 10, 33)), ("Full1d_4", (300,)),
                                         ("Full1d_14", (129,))])
def test_level_reductions_vs_oracle(native, gpu, oracle_port, kernel, dims):
    """LatticeLevelReductions through the generic interface (pf_policies.hpp:31-46)."""
    import latticeflow_gb300 as lf
    O = oracle_port
    rng = np.random.default_rng(11)
    offs, _ = O.lattice_offsets(kernel)
    N, Kp = int(np.prod(dims)), len(offs) // 2
    u = rng.integers(0, 1000, size=(N, 2)).astype(np.int64)
    w = rng.integers(0, 300, size=(N, Kp)).astype(np.int64)
    b = np.zeros((N, Kp, 4), np.int64)
    b[:, :, 1] = w
    b[:, :, 2] = w
    r_ref, cut_ref, _, sets_ref = O.port_pf(kernel, dims, u, b, return_sets=True)
    L = lf.LatticeFlow(kernel, "LatticeLevelReductions", dims)
    L.addEnergyPotentials(u, b)
    L.run()
    r = L.levels()
    dr = int(np.abs(r - r_ref).max())
    print(kernel, "max |dr| =", dr, "levels", len(np.unique(r_ref)))
    check_level_sums(r, L.levelSets(), r_ref, sets_ref)
    assert int(r.sum()) == int(r_ref.sum())      # total is exact
    # getCut = (r < 0): equal wherever a level set lies on one side of 0
    # (per set, the number of on nodes is equal; see check_level_sets)
    assert np.array_equal(L.getCut(), (r < 0).astype(L.getCut().dtype))


@pytest.mark.parametrize("kernel,dims", [("Full2d_4", (70, 66)), ("Full2d_8", (45, 52))])
@pytest.mark.parametrize("pr_kernel,device_loops,tile_rows", [(0, 1, 8), (0, 1, 16), (0, 0, 32),
                                                              (1, 1, 16), (1, 0, 32), (0, 0, 4)])
def test_level_reductions_pass_variants(native, gpu, oracle_port, kernel, dims, pr_kernel,
                                        device_loops, tile_rows):
    """Section solves through the TMA-staged 64-bit pass with section masks
    (pr_kernel 0; one launch per pass or device-side loops) and the generic
    tile pass (1): levels within one raw unit of the oracle, totals exact."""
    import latticeflow_gb300 as lf
    O = oracle_port
    rng = np.random.default_rng(23)
    offs, _ = O.lattice_offsets(kernel)
    N, Kp = int(np.prod(dims)), len(offs) // 2
    u = rng.integers(0, 5000, size=(N, 2)).astype(np.int64)
    w = rng.integers(0, 900, size=(N, Kp)).astype(np.int64)
    b = np.zeros((N, Kp, 4), np.int64)
    b[:, :, 1] = w
    b[:, :, 2] = w
    r_ref, cut_ref, _, sets_ref = O.port_pf(kernel, dims, u, b, return_sets=True)
    L = lf.LatticeFlow(kernel, "LatticeLevelReductions", dims)
    L.setParam("pr_kernel", pr_kernel)
    L.setParam("device_loops", device_loops)
    L.setParam("tile_rows", tile_rows)
    L.addEnergyPotentials(u, b)
    L.run()
    r = L.levels()
    check_level_sums(r, L.levelSets(), r_ref, sets_ref)
    assert int(r.sum()) == int(r_ref.sum())
