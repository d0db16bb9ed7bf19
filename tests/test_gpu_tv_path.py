"""TV at many lambdas (calculate2dTVPath) and batches of TV problems of one
shape (calculate2dTVBatch) on the GPU: every slice against the oracle's
single-lambda solve of the same image and lambda.

Tolerances as for the single solve: final 2x-scaled values within R_TOL = 1
raw unit (the rounding remainder inside a level set depends on push order),
double outputs within OUT_RTOL relative.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
R_TOL = 1
OUT_RTOL = 1e-9


def _close_out(a, b):
    scale = max(1.0, float(np.abs(b).max()))
    return float(np.abs(a - b).max()) <= OUT_RTOL * scale


def test_tv_path_slices_equal_single_solves(native, gpu, oracle_port):
    import latticeflow_gb300 as lf
    from latticeflow_gb300 import workloads as W
    f = W.tv_image(5, n=72, polygons=6)
    lams = np.array([1e-3, 0.01, 0.05, 0.3, 1.0, 4.0, -0.5])
    P = lf.calculate2dTVPath(f, lams)
    assert P.shape == (lams.size, 72, 72)
    for i, lam in enumerate(lams):
        ref, r, _ = oracle_port.port_tv_single("Full2d_4", f, max(lam, 0.0))
        single, lv = lf.calculate2dTV(f, max(lam, 0.0), return_levels=True)
        assert int(np.abs(lv - r).max()) <= R_TOL
        print("lam", lam, "max |path - oracle|", float(np.abs(P[i] - ref).max()))
        assert _close_out(P[i], ref)
        assert _close_out(P[i], single)


def test_tv_path_kernels_and_ragged_shape(native, gpu, oracle_port):
    import latticeflow_gb300 as lf
    rng = np.random.default_rng(11)
    f = rng.random((45, 37))
    lams = np.array([0.02, 0.2, 2.0])
    for kernel in ("Full2d_4", "Full2d_8"):
        P = lf.calculate2dTVPath(f, lams, kernel=kernel)
        for i, lam in enumerate(lams):
            ref, _, _ = oracle_port.port_tv_single(kernel, f, lam)
            assert _close_out(P[i], ref), (kernel, lam)


def test_tv_path_empty_and_errors(native, gpu):
    import latticeflow_gb300 as lf
    f = np.random.default_rng(0).random((8, 8))
    assert lf.calculate2dTVPath(f, []).shape == (0, 8, 8)
    with pytest.raises(lf.BadSolverOrKernelName):
        lf.calculate2dTVPath(f, [0.1], kernel="Full3d_26")


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
