"""The reference's TV regularisation path (calculate2dTVPath,
calculate2dTV(nx, ny, f, vector<double>), tv/tv_solver.hpp:657-681) and
batches of single-lambda TV problems (calculate2dTVBatch) on the GPU.

Path bar: bit-exact.  The output equals the compiled reference's on the
golden path fixtures (tests/golden/path_*.npz, made by make_golden.py) and
the restated path tracker's on fresh inputs (inputs without exact ties
between path events; with such ties the reference's own event order follows
the addresses of its segments).

Batch bar, as for the single solve: final 2x-scaled values within R_TOL = 1
raw unit (the rounding remainder inside a level set depends on push order),
double outputs within OUT_RTOL relative.
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


@pytest.mark.parametrize("path", sorted(glob.glob(os.path.join(GOLD, "path_*.npz"))),
                         ids=lambda p: os.path.basename(p))
def test_tv_path_golden(native, gpu, path):
    import latticeflow_gb300 as lf
    z = np.load(path)
    out, st = lf.calculate2dTVPath(z["f"], z["lams"], kernel=str(z["kernel"]), return_stats=True)
    print(os.path.basename(path), st, "max |d| =", float(np.abs(out - z["out"]).max()))
    assert np.array_equal(out, z["out"])


@pytest.mark.parametrize("kernel,shape,seed,lams", [
    ("Full2d_4", (72, 72), 5, [1e-3, 0.01, 0.05, 0.3, 1.0, 4.0, -0.5]),
    ("Full2d_8", (45, 37), 11, [0.02, 0.2, 2.0]),
    ("Star2d_16", (30, 33), 12, [0.01, 0.1, 0.5]),
    ("Full2d_4", (96, 80), 13, [1e-3 * 1000 ** (i / 31) for i in range(32)]),
])
def test_tv_path_vs_oracle(native, gpu, oracle_port, kernel, shape, seed, lams):
    import latticeflow_gb300 as lf
    from latticeflow_gb300 import workloads as W
    if seed == 11:
        f = np.random.default_rng(seed).random(shape)
    else:
        f = W.tv_image(seed, n=max(shape), polygons=6)[:shape[0], :shape[1]]
    lams = np.asarray(lams)
    ref, _, nseg = oracle_port.port_tv_path(kernel, f, lams)
    out, st = lf.calculate2dTVPath(f, lams, kernel=kernel, return_stats=True)
    print(kernel, shape, st, "oracle segments", nseg)
    assert st["segments"] == nseg
    assert np.array_equal(out, ref)


def test_tv_path_empty_and_errors(native, gpu):
    import latticeflow_gb300 as lf
    f = np.random.default_rng(0).random((8, 8))
    assert lf.calculate2dTVPath(f, []).shape == (0, 8, 8)
    with pytest.raises(lf.BadSolverOrKernelName):
        lf.calculate2dTVPath(f, [0.1], kernel="Full3d_26")


def test_tv_lambda_list_as_single_solves(native, gpu, oracle_port):
    """The single-lambda solutions at a list of lambdas for one image (what
    a caller who wants solutions rather than the path asks for): a batch
    with one shared image, each slice as its own single solve."""
    import latticeflow_gb300 as lf
    from latticeflow_gb300 import workloads as W
    f = W.tv_image(5, n=72, polygons=6)
    lams = np.array([1e-3, 0.05, 1.0, 4.0])
    out, lv = lf.calculate2dTVBatch(f, lams, return_levels=True)
    for i, lam in enumerate(lams):
        ref, r, _ = oracle_port.port_tv_single("Full2d_4", f, lam)
        assert int(np.abs(lv[i] - r).max()) <= R_TOL
        assert _close_out(out[i], ref)


def test_tv_batch_different_images(native, gpu, oracle_port):
    import latticeflow_gb300 as lf
    from latticeflow_gb300 import workloads as W
    imgs = np.stack([W.tv_image(s, n=64, polygons=5) for s in range(5)])
    lams = np.array([0.003, 0.04, 0.5, 0.04, 7.0])
    out, lv = lf.calculate2dTVBatch(imgs, lams, return_levels=True)
    for p in range(imgs.shape[0]):
        ref, r, _ = oracle_port.port_tv_single("Full2d_4", imgs[p], lams[p])
        assert int(np.abs(lv[p] - r).max()) <= R_TOL, p
        assert _close_out(out[p], ref), p


def test_tv_batch_in_several_stacks(native, gpu):
    """A node bound smaller than the batch splits it into stacks; the results
    do not change."""
    import latticeflow_gb300 as lf
    rng = np.random.default_rng(2)
    imgs = rng.random((7, 40, 24))
    lams = np.linspace(0.01, 1.0, 7)
    whole = lf.calculate2dTVBatch(imgs, lams)
    split = lf.calculate2dTVBatch(imgs, lams, max_nodes=3 * 40 * 24)
    for p in range(7):
        assert _close_out(split[p], whole[p]), p
