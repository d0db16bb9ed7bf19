"""The oracle itself: pinned against the reference's own outputs.

The restated solver must reproduce, bit for bit, the labelling of the
reference push-relabel and the minimal set of the bundled BK solver stored
in tests/golden (generated from the compiled reference), and the TV
single-lambda outputs.  Where the compiled reference is present it is also
compared directly on fresh random inputs.
"""
import glob
import os

import numpy as np
import pytest

from oracle import kernels as K

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def test_kernel_generator_names_and_sizes():
    specs = K.generate()
    assert specs["Full2d_4"].size == 4 and specs["Full2d_8"].size == 8
    assert specs["Star2d_16"].size == 16 and specs["Full2d_48"].size == 48
    assert specs["Full3d_6"].size == 6 and specs["Full3d_18"].size == 18
    assert specs["Full3d_32"].size == 32
    # sqrt(3)**2 < 3 in double: no 26-connected Full kernel; Star3d_26 is the 3x3x3 set
    assert "Full3d_26" in specs and specs["Full3d_26"].alias_of == "Star3d_26"
    assert specs["Star2d_4"].alias_of == "Full2d_4"


def test_kernel_generator_optional_dimensions():
    """The reference's opt-in builds: --1d gives Full1d_2 .. Full1d_14 (integer
    radii 1-7, Full only), --4d gives Full4d_8 with Star4d_8 as its alias;
    the default set is unchanged by them."""
    default = K.generate()
    specs = K.generate(optional=True)
    extra = [n for n in specs if n not in default]
    assert extra == ["Full1d_%d" % (2 * r) for r in range(1, 8)] + ["Full4d_8", "Star4d_8"]
    assert [n for n in specs if n in default] == list(default)
    assert specs["Full1d_6"].offsets == [(-3,), (-2,), (-1,), (1,), (2,), (3,)]
    assert specs["Star4d_8"].alias_of == "Full4d_8" and specs["Full4d_8"].size == 8


def test_reference_driver_instantiates_every_distinct_kernel():
    """oracle/ref_driver.cpp instantiates the reference solvers for exactly
    the distinct (non-alias) kernels the generator gives, default and opt-in,
    and maps every alias name onto its base."""
    import re
    src = open(os.path.join(os.path.dirname(GOLD), "..", "oracle", "ref_driver.cpp")).read()
    listed = re.findall(r"X\((\d), (\w+)\)", src)
    specs = K.generate(optional=True)
    base = {n: s for n, s in specs.items() if not s.alias_of and n != "Full3d_26"}
    assert sorted(n for _, n in listed) == sorted(base)
    for nd, n in listed:
        assert int(nd) == base[n].dim, n
    for n, s in specs.items():
        if s.alias_of:
            assert 'k == "%s") k = "%s"' % (n, s.alias_of) in src, n


def test_kernel_lattice_order_reverse_pairs():
    for name, s in K.generate(optional=True).items():
        offs, w = s.lattice_order()
        k = len(offs)
        for i in range(k // 2):
            assert tuple(-v for v in offs[i]) == offs[i + k // 2]
            assert offs[i] > tuple([0] * s.dim)
        assert offs[:k // 2] == sorted(offs[:k // 2])


def test_geocut_weights_full2d():
    s = K.generate()
    _, w4 = s["Full2d_4"].lattice_order()
    assert np.allclose(w4, np.pi / 4)
    offs8, w8 = s["Full2d_8"].lattice_order()
    for o, w in zip(offs8, w8):
        expect = np.pi / 8 if 0 in o else np.pi / (8 * np.sqrt(2))
        assert abs(w - expect) < 1e-15


@pytest.mark.parametrize("path", sorted(glob.glob(os.path.join(GOLD, "cut_*.npz"))),
                         ids=lambda p: os.path.basename(p))
def test_port_matches_reference_golden_cut(oracle_port, path):
    O = oracle_port
    z = np.load(path)
    kernel = str(z["kernel"])
    dims = tuple(int(v) for v in z["dims"])
    E, cmin, cmax, cpr, _ = O.port_canonical(kernel, dims, z["unary"], z["binary"])
    assert np.array_equal(cpr, z["pr_cut"])      # reference push-relabel labelling
    assert np.array_equal(cmin, z["bk_cut"])     # bundled BK labelling = minimal on-set
    assert E == int(z["energy"])
    assert O.energy(kernel, dims, z["unary"], z["binary"], cmax) == E
    assert np.all(cmin <= cmax)


@pytest.mark.parametrize("path", sorted(glob.glob(os.path.join(GOLD, "tv_*.npz"))),
                         ids=lambda p: os.path.basename(p))
def test_port_matches_reference_golden_tv(oracle_port, path):
    O = oracle_port
    z = np.load(path)
    out, r, _ = O.port_tv_single(str(z["kernel"]), z["f"], float(z["lam"]))
    assert np.array_equal(out, z["out"])


def test_port_against_compiled_reference_random(oracle_port):
    O = oracle_port
    if not O.ref_available():
        pytest.skip("compiled reference not present")
    rng = np.random.default_rng(99)
    for kernel, dims in [("Full2d_4", (30, 31)), ("Full2d_8", (25, 27)), ("Full3d_26", (6, 6, 7))]:
        offs, _ = O.lattice_offsets(kernel)
        N, Kp = int(np.prod(dims)), len(offs) // 2
        u = rng.integers(0, 80, size=(N, 2)).astype(np.int64)
        w = rng.integers(0, 50, size=(N, Kp)).astype(np.int64)
        b = np.zeros((N, Kp, 4), np.int64)
        b[:, :, 1] = w
        b[:, :, 2] = w
        pr, _ = O.ref_solve("LatticeEnergyMinimizer", kernel, dims, u, b)
        bk, _ = O.ref_solve("BKGCEnergyMinimizer", kernel, dims, u, b)
        E, cmin, cmax, cpr, _ = O.port_canonical(kernel, dims, u, b)
        assert np.array_equal(cpr, pr) and np.array_equal(cmin, bk)
        assert O.energy(kernel, dims, u, b, pr) == E


def test_port_against_compiled_reference_general_tables(oracle_port):
    """General submodular pairwise tables (E01 - E00 and E10 - E11 of both
    signs, so every branch of the reparametrisation runs,
    network_flow_node.hpp:420-485), on the kernels and sizes of the GPU
    fill-form test: the port's labellings and energy equal the compiled
    reference's PR and BK solvers."""
    O = oracle_port
    if not O.ref_available():
        pytest.skip("compiled reference not present")
    for kernel, dims in [("Full2d_4", (70, 45)), ("Full2d_8", (44, 90)), ("Star2d_16", (37, 50)),
                         ("Full2d_12", (40, 41)), ("Full3d_26", (9, 10, 37))]:
        rng = np.random.default_rng(5)
        n = int(np.prod(dims))
        kp = len(O.lattice_offsets(kernel)[0]) // 2
        u = rng.integers(-60, 61, size=(n, 2)).astype(np.int64)
        A = rng.integers(-40, 41, size=(n, kp))
        D = rng.integers(-40, 41, size=(n, kp))
        x = rng.integers(-30, 61, size=(n, kp))
        y = np.maximum(rng.integers(-30, 61, size=(n, kp)), -x)
        b = np.stack([A, A + x, D + y, D], axis=2).astype(np.int64)
        pr, _ = O.ref_solve("LatticeEnergyMinimizer", kernel, dims, u, b)
        bk, _ = O.ref_solve("BKGCEnergyMinimizer", kernel, dims, u, b)
        E, cmin, cmax, cpr, _ = O.port_canonical(kernel, dims, u, b)
        assert np.array_equal(cpr, pr) and np.array_equal(cmin, bk), kernel
        assert O.energy(kernel, dims, u, b, pr) == E, kernel
        assert O.energy(kernel, dims, u, b, cmax) == E, kernel


@pytest.mark.parametrize("kernel,dims", [
    ("Full2d_4", (33, 65)), ("Full2d_8", (30, 31)), ("Full2d_12", (20, 21)), ("Star2d_16", (19, 25)),
    ("Full2d_20", (17, 19)), ("Full2d_24", (18, 18)), ("Star2d_24", (17, 18)), ("Full2d_28", (16, 17)),
    ("Star2d_32", (16, 18)), ("Full2d_36", (15, 17)), ("Full2d_48", (15, 16)), ("Full3d_6", (6, 7, 20)),
    ("Full3d_18", (5, 6, 19)), ("Full3d_26", (6, 6, 17)), ("Full3d_32", (5, 6, 18))])
def test_port_against_compiled_reference_every_kernel(oracle_port, kernel, dims):
    """Every distinct kernel of the reference's default build, general
    submodular tables: the port's labellings and energy equal the compiled
    reference's PR and BK solvers."""
    O = oracle_port
    if not O.ref_available():
        pytest.skip("compiled reference not present")
    rng = np.random.default_rng(11)
    n = int(np.prod(dims))
    kp = len(O.lattice_offsets(kernel)[0]) // 2
    u = rng.integers(-60, 61, size=(n, 2)).astype(np.int64)
    A = rng.integers(-40, 41, size=(n, kp))
    D = rng.integers(-40, 41, size=(n, kp))
    x = rng.integers(-30, 61, size=(n, kp))
    y = np.maximum(rng.integers(-30, 61, size=(n, kp)), -x)
    b = np.stack([A, A + x, D + y, D], axis=2).astype(np.int64)
    pr, _ = O.ref_solve("LatticeEnergyMinimizer", kernel, dims, u, b)
    bk, _ = O.ref_solve("BKGCEnergyMinimizer", kernel, dims, u, b)
    E, cmin, cmax, cpr, _ = O.port_canonical(kernel, dims, u, b)
    assert np.array_equal(cpr, pr) and np.array_equal(cmin, bk)
    assert O.energy(kernel, dims, u, b, pr) == E == O.energy(kernel, dims, u, b, cmax)


@pytest.mark.parametrize("kernel,dims", [
    ("Full1d_2", (500,)), ("Full1d_4", (400,)), ("Full1d_6", (300,)), ("Full1d_8", (300,)),
    ("Full1d_10", (250,)), ("Full1d_12", (250,)), ("Full1d_14", (200,)),
    ("Full4d_8", (5, 6, 7, 8)), ("Star4d_8", (4, 5, 6, 7))])
def test_port_against_compiled_reference_optional_kernels(oracle_port, kernel, dims):
    """The kernels of the reference's opt-in 1-d and 4-d builds: offset
    tables equal the compiled reference's edgeDeltas(), and the port's
    labellings and energy equal its PR and BK solvers on general tables."""
    O = oracle_port
    if not O.ref_available():
        pytest.skip("compiled reference not present")
    rng = np.random.default_rng(13)
    n = int(np.prod(dims))
    offs = O.lattice_offsets(kernel)[0]
    kp = len(offs) // 2
    assert np.array_equal(O.ref_filling_deltas(kernel, dims), offs[:kp])
    u = rng.integers(-60, 61, size=(n, 2)).astype(np.int64)
    A = rng.integers(-40, 41, size=(n, kp))
    D = rng.integers(-40, 41, size=(n, kp))
    x = rng.integers(-30, 61, size=(n, kp))
    y = np.maximum(rng.integers(-30, 61, size=(n, kp)), -x)
    b = np.stack([A, A + x, D + y, D], axis=2).astype(np.int64)
    pr, _ = O.ref_solve("LatticeEnergyMinimizer", kernel, dims, u, b)
    bk, _ = O.ref_solve("BKGCEnergyMinimizer", kernel, dims, u, b)
    E, cmin, cmax, cpr, _ = O.port_canonical(kernel, dims, u, b)
    assert np.array_equal(cpr, pr) and np.array_equal(cmin, bk)
    assert O.energy(kernel, dims, u, b, pr) == E == O.energy(kernel, dims, u, b, cmax)


def test_port_tv_against_compiled_reference(oracle_port):
    O = oracle_port
    if not O.ref_available():
        pytest.skip("compiled reference not present")
    f = np.random.default_rng(5).random((27, 23))
    for lam in (0.01, 3.0, 40.0):
        ro, _ = O.ref_tv_single("Full2d_4", f, lam)
        po, _, _ = O.port_tv_single("Full2d_4", f, lam)
        assert np.array_equal(ro, po)


@pytest.mark.parametrize("path", sorted(glob.glob(os.path.join(GOLD, "path_*.npz"))),
                         ids=lambda p: os.path.basename(p))
def test_port_matches_reference_golden_path(oracle_port, path):
    """The restated regularisation-path tracker reproduces the compiled
    reference's calculate2dTV(nx, ny, f, lambdas) output bit for bit."""
    O = oracle_port
    z = np.load(path)
    out, _, _ = O.port_tv_path(str(z["kernel"]), z["f"], z["lams"])
    assert np.array_equal(out, z["out"])


def test_port_path_against_compiled_reference(oracle_port):
    O = oracle_port
    if not O.ref_available():
        pytest.skip("compiled reference not present")
    from latticeflow_gb300 import workloads as W
    rng = np.random.default_rng(31)
    cases = [("Full2d_4", W.tv_image(3, n=56, polygons=6), [1e-3 * 1000 ** (i / 9) for i in range(10)]),
             ("Full2d_8", rng.random((30, 26)), [0.02, 0.4, 0.0, 1.5]),
             ("Star2d_16", W.tv_image(4, n=28, polygons=4), [0.05, 0.5])]
    for kernel, f, lams in cases:
        ro, _ = O.ref_tv_path(kernel, f, np.array(lams))
        po, _, _ = O.port_tv_path(kernel, f, np.array(lams))
        assert np.array_equal(ro, po), kernel


def test_oracle_detects_planted_error(oracle_port):
    """A wrong labelling planted in the oracle's output is caught by the energy check."""
    O = oracle_port
    z = np.load(os.path.join(GOLD, "cut_f4_rand.npz"))
    dims = tuple(int(v) for v in z["dims"])
    E, cmin, _, _, _ = O.port_canonical("Full2d_4", dims, z["unary"], z["binary"])
    bad = cmin.copy().reshape(-1)
    bad[np.argmax(bad == 0)] ^= 1
    assert O.energy("Full2d_4", dims, z["unary"], z["binary"], bad) != E or not np.array_equal(bad, cmin.reshape(-1))
