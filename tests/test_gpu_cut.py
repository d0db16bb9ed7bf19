"""GPU parity of the binary cut through the C ABI.

Bar: bit-exact.  The flow value / minimum energy equals the reference's, the
minimal on-set equals the reference BK labelling (golden fixtures) and the
restated solver's minimal set, the maximal on-set equals the restated
solver's maximal set.  Full-size problems are checked through
size-independent properties (energy of both sets equals the reported
minimum, minimal set inside maximal set).
"""
import glob
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden")


def solve(kernel, dims, unary, binary, solver="LatticeEnergyMinimizer", tuning=None):
    import latticeflow_gb300 as lf
    L = lf.LatticeFlow(kernel, solver, dims)
    if tuning:
        L.setTuning(**tuning)
    L.addEnergyPotentials(unary, binary)
    L.run()
    return L


@pytest.mark.parametrize("path", sorted(glob.glob(os.path.join(GOLD, "cut_*.npz"))),
                         ids=lambda p: os.path.basename(p))
def test_golden_cut(native, gpu, oracle_port, path):
    z = np.load(path)
    kernel = str(z["kernel"])
    dims = tuple(int(v) for v in z["dims"])
    L = solve(kernel, dims, z["unary"], z["binary"])
    flow, energy = L.flow()
    assert energy == int(z["energy"])
    cmin = L.getCut()
    assert np.array_equal(cmin, z["bk_cut"])
    _, _, cmax, _, _ = oracle_port.port_canonical(kernel, dims, z["unary"], z["binary"])
    assert np.array_equal(L.getCutMax(), cmax)


CASES = [
    ("Full2d_4", (64, 64)), ("Full2d_4", (1, 100)), ("Full2d_4", (100, 1)), ("Full2d_4", (33, 65)),
    ("Full2d_8", (70, 45)), ("Full2d_12", (40, 41)), ("Star2d_16", (37, 50)), ("Full2d_24", (30, 30)),
    ("Full2d_48", (25, 26)), ("Full3d_6", (10, 12, 40)), ("Full3d_18", (9, 9, 33)),
    ("Full3d_26", (12, 10, 35)), ("Full3d_32", (8, 9, 34)),
    ("Full1d_2", (300,)), ("Full1d_4", (77,)), ("Full1d_6", (1,)), ("Full1d_8", (150,)),
    ("Full1d_10", (33,)), ("Full1d_12", (64,)), ("Full1d_14", (201,)),
]


@pytest.mark.parametrize("kernel,dims", CASES, ids=lambda v: str(v))
@pytest.mark.parametrize("seed", [0, 1])
def test_random_vs_oracle(native, gpu, oracle_port, kernel, dims, seed):
    O = oracle_port
    rng = np.random.default_rng(seed + 17)
    offs, _ = O.lattice_offsets(kernel)
    N, Kp = int(np.prod(dims)), len(offs) // 2
    u = rng.integers(0, 100, size=(N, 2)).astype(np.int64)
    w = rng.integers(0, 60, size=(N, Kp)).astype(np.int64)
    b = np.zeros((N, Kp, 4), np.int64)
    b[:, :, 1] = w
    b[:, :, 2] = w
    E, cmin, cmax, _, _ = O.port_canonical(kernel, dims, u, b)
    L = solve(kernel, dims, u, b)
    assert L.flow()[1] == E
    assert np.array_equal(L.getCut(), cmin)
    assert np.array_equal(L.getCutMax(), cmax)


def test_plain_cut_config_full_size(native, gpu, oracle_port):
    from latticeflow_gb300 import workloads as W
    p = W.plain_cut(0)
    u, b = p.energies()
    E, cmin, cmax, _, _ = oracle_port.port_canonical(p.kernel, p.dims, u, b)
    L = solve(p.kernel, p.dims, u, b)
    assert L.flow()[1] == E
    assert np.array_equal(L.getCut(), cmin) and np.array_equal(L.getCutMax(), cmax)


def test_capacity_form_equals_energy_form(native, gpu):
    import latticeflow_gb300 as lf
    from latticeflow_gb300 import workloads as W
    p = W.plain_cut(4, (90, 77), "Full2d_8")
    u, b = p.energies()
    L1 = solve(p.kernel, p.dims, u, b)
    L2 = lf.LatticeFlow(p.kernel, "GPUPushRelabel", p.dims)
    L2.addCapacities(p.source, p.sink, p.edge)
    L2.run()
    assert L1.flow() == L2.flow()
    assert np.array_equal(L1.getCut(), L2.getCut())


def test_large_cut_scaled_vs_oracle(native, gpu, oracle_port):
    from latticeflow_gb300 import workloads as W
    p = W.large_cut(0, n=384)
    u, b = p.energies()
    E, cmin, cmax, _, _ = oracle_port.port_canonical(p.kernel, p.dims, u, b)
    L = solve(p.kernel, p.dims, u, b)
    assert L.flow()[1] == E
    assert np.array_equal(L.getCut(), cmin) and np.array_equal(L.getCutMax(), cmax)


def test_large_cut_full_size_properties(native, gpu, oracle_port):
    import latticeflow_gb300 as lf
    from latticeflow_gb300 import workloads as W
    p = W.large_cut(0)
    L = lf.LatticeFlow(p.kernel, "LatticeEnergyMinimizer", p.dims)
    L.addCapacities(p.source, p.sink, p.edge)
    L.run()
    flow, energy = L.flow()
    cmin, cmax = L.getCut(), L.getCutMax()
    assert np.all(cmin <= cmax)
    u, b = p.energies()
    assert oracle_port.energy(p.kernel, p.dims, u, b, cmin) == energy
    assert oracle_port.energy(p.kernel, p.dims, u, b, cmax) == energy


def test_int64_capacities(native, gpu, oracle_port):
    O = oracle_port
    rng = np.random.default_rng(3)
    dims = (40, 50)
    N = 2000
    u = rng.integers(0, 3 * 10 ** 9, size=(N, 2)).astype(np.int64)
    w = rng.integers(0, 2 * 10 ** 9, size=(N, 2)).astype(np.int64)
    b = np.zeros((N, 2, 4), np.int64)
    b[:, :, 1] = w
    b[:, :, 2] = w
    E, cmin, cmax, _, _ = O.port_canonical("Full2d_4", dims, u, b)
    L = solve("Full2d_4", dims, u, b)
    assert L.flow()[1] == E
    assert np.array_equal(L.getCut(), cmin) and np.array_equal(L.getCutMax(), cmax)


def test_general_submodular_tables(native, gpu, oracle_port):
    z = np.load(os.path.join(GOLD, "cut_f4_general.npz"))
    dims = tuple(int(v) for v in z["dims"])
    L = solve("Full2d_4", dims, z["unary"], z["binary"])
    assert L.flow()[1] == int(z["energy"])
    assert np.array_equal(L.getCut(), z["bk_cut"])


def test_accumulating_fill(native, gpu, oracle_port):
    import latticeflow_gb300 as lf
    from latticeflow_gb300 import workloads as W
    p = W.plain_cut(6, (48, 52))
    u, b = p.energies()
    L = lf.LatticeFlow(p.kernel, "LatticeEnergyMinimizer", p.dims)
    L.addEnergyPotentials(u, b)
    L.addEnergyPotentials(u, b)
    L.run()
    E, cmin, _, _, _ = oracle_port.port_canonical(p.kernel, p.dims, 2 * u, 2 * b)
    assert L.flow()[1] == E and np.array_equal(L.getCut(), cmin)


def test_errors(native, gpu):
    import latticeflow_gb300 as lf
    L = lf.LatticeFlow("Full2d_4", "LatticeEnergyMinimizer", (4, 4))
    with pytest.raises(lf.LatticeFlowError):
        L.getCut()
    u = np.zeros((16, 2), np.int64)
    b = np.zeros((16, 2, 4), np.int64)
    b[:, :, 0] = 10   # E00 + E11 > E01 + E10: not submodular
    with pytest.raises(OverflowError):
        L.addEnergyPotentials(u, b)


def test_repeat_run_is_stable(native, gpu):
    from latticeflow_gb300 import workloads as W
    p = W.plain_cut(2, (128, 96), "Full2d_8")
    u, b = p.energies()
    L = solve(p.kernel, p.dims, u, b)
    c1, f1 = L.getCut(), L.flow()
    L.run()
    assert L.flow() == f1 and np.array_equal(L.getCut(), c1)


@pytest.mark.parametrize("tuning", [dict(tile_rows=8), dict(local_sweeps=4), dict(launches_per_relabel=1),
                                    dict(tile_rows=16, local_sweeps=200, launches_per_relabel=50)])
def test_tuning_does_not_change_result(native, gpu, oracle_port, tuning):
    from latticeflow_gb300 import workloads as W
    p = W.plain_cut(8, (100, 120), "Full2d_8")
    u, b = p.energies()
    E, cmin, cmax, _, _ = oracle_port.port_canonical(p.kernel, p.dims, u, b)
    L = solve(p.kernel, p.dims, u, b, tuning=tuning)
    assert L.flow()[1] == E
    assert np.array_equal(L.getCut(), cmin) and np.array_equal(L.getCutMax(), cmax)


def test_pinned_host_arrays_read_in_place(native, gpu):
    """Pinned host energies / capacities are read by the fill kernels in
    place; the result equals the copied (pageable) path bit for bit."""
    import ctypes
    torch = pytest.importorskip("torch")
    import latticeflow_gb300 as lf
    from latticeflow_gb300 import _native as N
    from latticeflow_gb300 import workloads as W
    p = W.plain_cut(21, (150, 170), "Full2d_8")
    u, b = p.energies()
    pu = torch.from_numpy(u).pin_memory()
    pb = torch.from_numpy(b).pin_memory()
    a = lf.LatticeFlow(p.kernel, "LatticeEnergyMinimizer", p.dims)
    N.check(N.lib().lf_add_energy_potentials(a._h, ctypes.c_void_p(pu.data_ptr()),
                                             ctypes.c_void_p(pb.data_ptr())))
    a.run()
    c = lf.LatticeFlow(p.kernel, "LatticeEnergyMinimizer", p.dims)
    N.check(N.lib().lf_add_energy_potentials(c._h, u.ctypes.data_as(ctypes.c_void_p),
                                             b.ctypes.data_as(ctypes.c_void_p)))
    c.run()
    assert a.flow() == c.flow()
    assert np.array_equal(a.getCut(), c.getCut()) and np.array_equal(a.getCutMax(), c.getCutMax())
    # the same pinned arrays staged into device memory by the copy engine
    s = lf.LatticeFlow(p.kernel, "LatticeEnergyMinimizer", p.dims)
    s.setParam("host_stage", 1)
    for _ in range(2):
        s.clear()
        N.check(N.lib().lf_add_energy_potentials(s._h, ctypes.c_void_p(pu.data_ptr()),
                                                 ctypes.c_void_p(pb.data_ptr())))
        s.run()
        assert s.flow() == c.flow()
        assert np.array_equal(s.getCut(), c.getCut()) and np.array_equal(s.getCutMax(), c.getCutMax())
    # capacities
    ps = torch.from_numpy(p.source).pin_memory()
    pk = torch.from_numpy(p.sink).pin_memory()
    pe = torch.from_numpy(np.ascontiguousarray(p.edge)).pin_memory()
    d = lf.LatticeFlow(p.kernel, "LatticeEnergyMinimizer", p.dims)
    N.check(N.lib().lf_add_capacities(d._h, ctypes.c_void_p(ps.data_ptr()), ctypes.c_void_p(pk.data_ptr()),
                                      ctypes.c_void_p(pe.data_ptr())))
    d.run()
    e = lf.LatticeFlow(p.kernel, "LatticeEnergyMinimizer", p.dims)
    e.addCapacities(p.source, p.sink, p.edge)
    e.run()
    assert d.flow() == e.flow() and np.array_equal(d.getCut(), e.getCut())


@pytest.mark.parametrize("pr_kernel,bfs_kernel,device_loops", [(0, 0, 1), (0, 0, 0), (1, 1, 1), (2, 0, 1),
                                                                (1, 0, 1), (0, 1, 1), (3, 0, 0),
                                                                (3, 1, 0)])
@pytest.mark.parametrize("kernel,dims,tile_rows", [
    ("Full2d_8", (200, 230), 8), ("Full2d_8", (256, 160), 16), ("Full2d_8", (97, 300), 32),
    ("Full2d_4", (210, 190), 16), ("Full2d_4", (64, 500), 32), ("Full2d_8", (150, 170), 4),
    ("Full2d_4", (130, 99), 4)], ids=lambda v: str(v))
def test_push_relabel_kernels_agree(native, gpu, oracle_port, pr_kernel, bfs_kernel, device_loops,
                                    kernel, dims, tile_rows):
    """The TMA-staged 2-d passes (pr_kernel 0, 2, 3; bfs_kernel 0), in
    device-side loops (device_loops 1) or launched one by one (0), and the
    generic tile passes (1) give the reference's exact answer at every tile
    height."""
    import latticeflow_gb300 as lf
    from latticeflow_gb300 import workloads as W
    p = W.plain_cut(30 + tile_rows, dims, kernel)
    u, b = p.energies()
    E, cmin, cmax, _, _ = oracle_port.port_canonical(p.kernel, p.dims, u, b)
    L = lf.LatticeFlow(p.kernel, "LatticeEnergyMinimizer", p.dims)
    L.setParam("pr_kernel", pr_kernel)
    L.setParam("bfs_kernel", bfs_kernel)
    L.setParam("device_loops", device_loops)
    L.setTuning(tile_rows=tile_rows, local_sweeps=3, launches_per_relabel=4)
    L.addEnergyPotentials(u, b)
    L.run()
    assert L.layout()[0] == (1, tile_rows, 32)
    assert L.flow()[1] == E
    assert np.array_equal(L.getCut(), cmin) and np.array_equal(L.getCutMax(), cmax)


def _random_3d(kernel, dims, seed, O):
    rng = np.random.default_rng(seed)
    offs, _ = O.lattice_offsets(kernel)
    N, Kp = int(np.prod(dims)), len(offs) // 2
    u = rng.integers(0, 120, size=(N, 2)).astype(np.int64)
    w = rng.integers(0, 40, size=(N, Kp)).astype(np.int64)
    b = np.zeros((N, Kp, 4), np.int64)
    b[:, :, 1] = w
    b[:, :, 2] = w + rng.integers(0, 3, size=(N, Kp))
    return u, b


@pytest.mark.parametrize("pr_kernel,bfs_kernel", [(0, 0), (1, 1), (0, 1), (1, 0)])
@pytest.mark.parametrize("kernel,dims,tile_rows", [
    ("Full3d_26", (12, 18, 70), 2), ("Full3d_26", (9, 20, 40), 4), ("Full3d_18", (13, 10, 45), 2),
    ("Full3d_18", (8, 16, 33), 4), ("Full3d_6", (10, 24, 50), 8), ("Full3d_6", (7, 9, 64), 2),
    ("Full3d_26", (5, 3, 31), 2)], ids=lambda v: str(v))
def test_tma_pass_3d(native, gpu, oracle_port, pr_kernel, bfs_kernel, kernel, dims, tile_rows):
    """The TMA-staged 3-d passes (pr_kernel / bfs_kernel 0: 4 x rows x 32
    tiles; push/relabel with the residual planes as one 4-d box, BFS with
    heights and masks as 3-d boxes) and the generic passes (1), in every
    combination, give the reference's exact answer."""
    import latticeflow_gb300 as lf
    u, b = _random_3d(kernel, dims, 40 + tile_rows, oracle_port)
    E, cmin, cmax, _, _ = oracle_port.port_canonical(kernel, dims, u, b)
    L = lf.LatticeFlow(kernel, "LatticeEnergyMinimizer", dims)
    L.setParam("pr_kernel", pr_kernel)
    L.setParam("bfs_kernel", bfs_kernel)
    L.setTuning(tile_rows=tile_rows, local_sweeps=3, launches_per_relabel=4)
    for _ in range(2):
        L.clear()
        L.addEnergyPotentials(u, b)
        L.run()
        assert L.layout()[0] == (4, tile_rows, 32)
        assert L.flow()[1] == E
        assert np.array_equal(L.getCut(), cmin) and np.array_equal(L.getCutMax(), cmax)


def test_tma_bfs_3d_int64(native, gpu, oracle_port):
    """Capacities beyond 32 bits on a 3-d lattice: 64-bit working arrays, the
    generic push/relabel pass and the staged 3-d BFS (it reads only masks and
    heights) give the reference's exact answer."""
    import latticeflow_gb300 as lf
    rng = np.random.default_rng(9)
    kernel, dims = "Full3d_26", (8, 12, 40)
    offs, _ = oracle_port.lattice_offsets(kernel)
    N, Kp = int(np.prod(dims)), len(offs) // 2
    u = rng.integers(0, 3 * 10 ** 9, size=(N, 2)).astype(np.int64)
    w = rng.integers(0, 10 ** 9, size=(N, Kp)).astype(np.int64)
    b = np.zeros((N, Kp, 4), np.int64)
    b[:, :, 1] = w
    b[:, :, 2] = w
    E, cmin, cmax, _, _ = oracle_port.port_canonical(kernel, dims, u, b)
    L = lf.LatticeFlow(kernel, "LatticeEnergyMinimizer", dims)
    L.setTuning(tile_rows=2, local_sweeps=2, launches_per_relabel=8)
    L.addEnergyPotentials(u, b)
    L.run()
    assert L.layout()[2] == 8
    assert L.flow()[1] == E
    assert np.array_equal(L.getCut(), cmin) and np.array_equal(L.getCutMax(), cmax)


@pytest.mark.parametrize("tile_rows", [2, 4])
def test_tma_pass_3d_volume(native, gpu, oracle_port, tile_rows):
    """A 96^3 Full3d_26 volume (the volume workload's generator) through the
    staged 3-d pass: the reference's energy and both cut sets."""
    import latticeflow_gb300 as lf
    from latticeflow_gb300 import workloads as W
    p = W.volume_cut(2, n=96)
    u, b = p.energies()
    E, cmin, cmax, _, _ = oracle_port.port_canonical(p.kernel, p.dims, u, b)
    L = lf.LatticeFlow(p.kernel, "LatticeEnergyMinimizer", p.dims)
    L.setTuning(tile_rows=tile_rows, local_sweeps=2, launches_per_relabel=8)
    L.addEnergyPotentials(u, b)
    L.run()
    assert L.flow()[1] == E
    assert np.array_equal(L.getCut(), cmin) and np.array_equal(L.getCutMax(), cmax)


@pytest.mark.parametrize("pr_kernel", [0, 2])
def test_tma_pass_large_cut_scaled(native, gpu, oracle_port, pr_kernel):
    import latticeflow_gb300 as lf
    from latticeflow_gb300 import workloads as W
    p = W.large_cut(1, n=512)
    u, b = p.energies()
    E, cmin, cmax, _, _ = oracle_port.port_canonical(p.kernel, p.dims, u, b)
    L = lf.LatticeFlow(p.kernel, "LatticeEnergyMinimizer", p.dims)
    L.setParam("pr_kernel", pr_kernel)
    L.addEnergyPotentials(u, b)
    L.run()
    assert L.flow()[1] == E
    assert np.array_equal(L.getCut(), cmin) and np.array_equal(L.getCutMax(), cmax)


def test_tma_pass_full_size_all_variants(native, gpu, oracle_port):
    """2048x2048 Full2d_8 at full size through every push/relabel variant and
    tile height: the same flow value, both cut sets identical, each set's
    energy equal to the reported minimum (a pass that loses flow at a tile
    edge shows up here as a larger flow than the cut's energy)."""
    import latticeflow_gb300 as lf
    from latticeflow_gb300 import workloads as W
    p = W.large_cut(0)
    u, b = p.energies()
    ref = None
    for prk, rows, dl in ((1, 16, 0), (0, 16, 1), (0, 16, 0), (2, 16, 1), (0, 8, 1), (2, 8, 0),
                          (0, 32, 1), (2, 32, 0), (0, 4, 0), (2, 4, 0), (3, 4, 0), (3, 8, 0)):
        L = lf.LatticeFlow(p.kernel, "LatticeEnergyMinimizer", p.dims)
        L.setParam("pr_kernel", prk)
        L.setParam("bfs_kernel", 1 if ref is None else 0)  # the reference run: generic passes
        L.setParam("device_loops", dl)
        L.setTuning(tile_rows=rows, local_sweeps=2, launches_per_relabel=8)
        for _ in range(2):
            L.clear()
            L.addEnergyPotentials(u, b)
            L.run()
            flow, energy = L.flow()
            cmin, cmax = L.getCut(), L.getCutMax()
            if ref is None:
                assert flow == energy
                assert oracle_port.energy(p.kernel, p.dims, u, b, cmin) == energy
                assert oracle_port.energy(p.kernel, p.dims, u, b, cmax) == energy
                ref = (flow, energy, cmin.copy(), cmax.copy())
            assert (flow, energy) == ref[:2], (prk, rows)
            assert np.array_equal(cmin, ref[2]) and np.array_equal(cmax, ref[3]), (prk, rows)
        del L


@pytest.mark.gpu
@pytest.mark.parametrize("kernel,dims", [("Full2d_4", (70, 45)), ("Full2d_8", (44, 90)),
                                         ("Star2d_16", (37, 50)), ("Full2d_12", (40, 41)),
                                         ("Full3d_26", (9, 10, 37))])
def test_fill_forms_agree(native, gpu, oracle_port, kernel, dims):
    """The three forms of the energy fill for device arrays (fill_kernel 0:
    one lane per filling edge where K/2 divides a warp, else one thread per
    node; 1: one thread per node; 2: scattered with atomics), with 16-byte
    aligned and unaligned arrays, give the oracle's minimum energy and cut
    sets.  The pairwise tables are general submodular ones: B - A and C - D
    take both signs, so every branch of the decomposition runs."""
    import ctypes
    torch = pytest.importorskip("torch")
    import latticeflow_gb300 as lf
    from latticeflow_gb300 import _native as N
    rng = np.random.default_rng(5)
    n = int(np.prod(dims))
    kp = len(oracle_port.lattice_offsets(kernel)[0]) // 2
    u = rng.integers(-60, 61, size=(n, 2)).astype(np.int64)
    A = rng.integers(-40, 41, size=(n, kp))
    D = rng.integers(-40, 41, size=(n, kp))
    x = rng.integers(-30, 61, size=(n, kp))
    y = np.maximum(rng.integers(-30, 61, size=(n, kp)), -x)   # x + y >= 0: submodular
    b = np.stack([A, A + x, D + y, D], axis=2).astype(np.int64)
    E, cmin, cmax, _, _ = oracle_port.port_canonical(kernel, dims, u, b)
    for form in (0, 1, 2):
        for off in (0, 1):
            ub = torch.zeros(u.size + 2, dtype=torch.int64, device="cuda")
            bb = torch.zeros(b.size + 2, dtype=torch.int64, device="cuda")
            uu = ub[off:off + u.size]
            bv = bb[off:off + b.size]
            uu.copy_(torch.from_numpy(u.reshape(-1)))
            bv.copy_(torch.from_numpy(b.reshape(-1)))
            torch.cuda.synchronize()
            L = lf.LatticeFlow(kernel, "LatticeEnergyMinimizer", dims)
            L.setParam("fill_kernel", form)
            N.check(N.lib().lf_add_energy_potentials_device(L._h, ctypes.c_void_p(uu.data_ptr()),
                                                            ctypes.c_void_p(bv.data_ptr())))
            L.run()
            assert L.flow()[1] == E, (form, off)
            assert np.array_equal(L.getCut(), cmin) and np.array_equal(L.getCutMax(), cmax), (form, off)


@pytest.mark.gpu
def test_unaligned_energy_arrays(native, gpu, oracle_port):
    """Device energy arrays that are 8- but not 16-byte aligned take the
    scalar fill (aligned ones the 16-byte vector fill); both give the
    oracle's answer."""
    import ctypes
    torch = pytest.importorskip("torch")
    import latticeflow_gb300 as lf
    from latticeflow_gb300 import _native as N
    from latticeflow_gb300 import workloads as W
    p = W.plain_cut(44, (90, 110), "Full2d_8")
    u, b = p.energies()
    E, cmin, cmax, _, _ = oracle_port.port_canonical(p.kernel, p.dims, u, b)
    for off in (0, 1):
        ub = torch.zeros(u.size + 2, dtype=torch.int64, device="cuda")
        bb = torch.zeros(b.size + 2, dtype=torch.int64, device="cuda")
        uu = ub[off:off + u.size]
        bv = bb[off:off + b.size]
        uu.copy_(torch.from_numpy(u.reshape(-1)))
        bv.copy_(torch.from_numpy(b.reshape(-1)))
        assert (uu.data_ptr() % 16 == 0) == (off == 0) and (bv.data_ptr() % 16 == 0) == (off == 0)
        torch.cuda.synchronize()
        L = lf.LatticeFlow(p.kernel, "LatticeEnergyMinimizer", p.dims)
        N.check(N.lib().lf_add_energy_potentials_device(L._h, ctypes.c_void_p(uu.data_ptr()),
                                                        ctypes.c_void_p(bv.data_ptr())))
        L.run()
        assert L.flow()[1] == E
        assert np.array_equal(L.getCut(), cmin) and np.array_equal(L.getCutMax(), cmax)
