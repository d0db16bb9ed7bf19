"""Failure detection without a GPU fault: a solve that hits its epoch cap
ends with LF_ERR_NO_CONVERGENCE on the host, leaves no result behind, and the
same handle solves correctly afterwards."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_epoch_cap_reports_and_handle_recovers(native, gpu):
    import latticeflow_gb300 as lf
    from latticeflow_gb300 import workloads as W
    p = W.plain_cut(3, (192, 160), "Full2d_8")
    ref = lf.LatticeFlow(p.kernel, "LatticeEnergyMinimizer", p.dims)
    ref.addCapacities(p.source, p.sink, p.edge)
    ref.run()
    L = lf.LatticeFlow(p.kernel, "LatticeEnergyMinimizer", p.dims)
    L.addCapacities(p.source, p.sink, p.edge)
    L.setParam("max_epochs", 1)
    with pytest.raises(lf.LatticeFlowError) as e:
        L.run()
    assert e.value.code == 4                   # LF_ERR_NO_CONVERGENCE
    with pytest.raises(lf.LatticeFlowError):  # no cut from a failed solve
        L.getCut()
    L.setParam("max_epochs", 0)
    L.run()
    assert L.flow() == ref.flow()
    assert np.array_equal(L.getCut(), ref.getCut())
    assert np.array_equal(L.getCutMax(), ref.getCutMax())


def test_epoch_cap_in_a_batch(native, gpu):
    import latticeflow_gb300 as lf
    from latticeflow_gb300 import workloads as W
    probs = [W.plain_cut(10 + i, (96 + 8 * i, 80), "Full2d_4") for i in range(3)]
    B = lf.LatticeBatch()
    for p in probs:
        B.add(p.kernel, p.dims)
    for i, p in enumerate(probs):
        B.addCapacities(i, p.source, p.sink, p.edge)
    B.setParam("max_epochs", 1)
    with pytest.raises(lf.LatticeFlowError) as e:
        B.run()
    assert e.value.code == 4
    B.setParam("max_epochs", 0)
    B.run()
    for i, p in enumerate(probs):
        L = lf.LatticeFlow(p.kernel, "LatticeEnergyMinimizer", p.dims)
        L.addCapacities(p.source, p.sink, p.edge)
        L.run()
        assert B.flow(i) == L.flow() and np.array_equal(B.getCut(i), L.getCut())


# ------------------------------------------------------------------ serving
# Failures of the request server, made on the host: a wait that runs out, a
# request cancelled while queued, an engine allocation that fails.


def test_server_wait_timeout_then_result(native, gpu):
    import latticeflow_gb300 as lf
    from latticeflow_gb300 import workloads as W
    f = W.tv_image(7, n=1024, polygons=12)
    S = lf.LatticeServer(workers=1)
    try:
        t = S.submit_tv(f, 0.01)
        with pytest.raises(lf.LatticeFlowError) as e:
            S.wait(t, timeout=1e-4)      # a 1024^2 solve takes far longer
        assert e.value.code == 8        # LF_ERR_STATE: not finished within the timeout
        S.wait(t)
        out, _ = S.result(t)
        assert np.allclose(out, lf.calculate2dTV(f, 0.01), rtol=0, atol=1e-9)
    finally:
        S.close()


def test_server_cancel_queued_request(native, gpu):
    import latticeflow_gb300 as lf
    from latticeflow_gb300 import workloads as W
    big = W.tv_image(8, n=1024, polygons=12)
    small = W.tv_image(9, n=64, polygons=4)
    S = lf.LatticeServer(workers=1, max_group=1)
    try:
        t1 = S.submit_tv(big, 0.01)     # occupies the only worker
        t2 = S.submit_tv(small, 0.1)    # waits in the queue behind it
        S.cancel(t2)
        with pytest.raises(lf.LatticeFlowError) as e:
            S.wait(t2)
        assert e.value.code == 8 and "cancelled" in str(e.value)
        S.wait(t1)
        with pytest.raises(lf.LatticeFlowError):
            S.cancel(t1)                # finished: nothing to cancel
        t3 = S.submit_tv(small, 0.1)    # the server carries on
        S.wait(t3)
        out, _ = S.result(t3)
        assert np.allclose(out, lf.calculate2dTV(small, 0.1), rtol=0, atol=1e-9)
    finally:
        S.close()


def test_server_injected_allocation_failure(native, gpu):
    import latticeflow_gb300 as lf
    from latticeflow_gb300 import workloads as W
    p = W.plain_cut(12, (120, 96), "Full2d_8")
    ref = lf.LatticeFlow(p.kernel, "LatticeEnergyMinimizer", p.dims)
    ref.addCapacities(p.source, p.sink, p.edge)
    ref.run()
    S = lf.LatticeServer(workers=2)
    try:
        S.inject_alloc_failures(1)
        t = S.submit_cut(p.kernel, p.dims, p.source, p.sink, p.edge)
        with pytest.raises(lf.LatticeFlowError) as e:
            S.wait(t)
        assert e.value.code == 5        # LF_ERR_OOM
        S.release(t)
        t = S.submit_cut(p.kernel, p.dims, p.source, p.sink, p.edge)
        S.wait(t)
        cut, fe = S.result(t)
        assert fe == ref.flow() and np.array_equal(cut, ref.getCut())
    finally:
        S.close()
