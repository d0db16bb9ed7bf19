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
