"""Request server: every result is the same alone and in the mix.

TV results are compared with the same request solved alone (calculate2dTV)
and with the oracle within the TV tolerance (1 raw unit, outputs 1e-9
relative); cut results must be identical to a plain solve."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _tv_close(a, b):
    return float(np.abs(a - b).max()) <= 1e-9 * max(1.0, float(np.abs(b).max()))


def test_server_mix_equals_alone(native, gpu, oracle_port):
    import latticeflow_gb300 as lf
    from latticeflow_gb300 import workloads as W
    rng = np.random.default_rng(7)
    tv_reqs = []
    for i, (n, lam) in enumerate([(64, 0.01), (96, 5.0), (128, 40.0), (48, 0.3), (160, 2.0), (64, 80.0)]):
        tv_reqs.append((W.tv_image(20 + i, n=n, polygons=5), lam))
    cut_reqs = [W.plain_cut(40 + i, (int(rng.integers(30, 200)), int(rng.integers(30, 200))),
                            "Full2d_4" if i % 2 else "Full2d_8") for i in range(6)]
    S = lf.LatticeServer(workers=4)
    tickets = []
    for k in range(max(len(tv_reqs), len(cut_reqs))):
        if k < len(tv_reqs):
            tickets.append(("tv", k, S.submit_tv(*tv_reqs[k])))
        if k < len(cut_reqs):
            p = cut_reqs[k]
            tickets.append(("cut", k, S.submit_cut(p.kernel, p.dims, p.source, p.sink, p.edge)))
    for kind, k, t in tickets:
        lat = S.wait(t)
        assert lat >= 0
        if kind == "tv":
            f, lam = tv_reqs[k]
            out, lv = S.result(t)
            alone, lv_alone = lf.calculate2dTV(f, lam, return_levels=True)
            ref, r, _ = oracle_port.port_tv_single("Full2d_4", f, lam)
            assert int(np.abs(lv - lv_alone).max()) <= 1 and _tv_close(out, alone)
            assert int(np.abs(lv - r).max()) <= 1 and _tv_close(out, ref)
        else:
            p = cut_reqs[k]
            cut, fe = S.result(t)
            L = lf.LatticeFlow(p.kernel, "LatticeEnergyMinimizer", p.dims)
            L.addCapacities(p.source, p.sink, p.edge)
            L.run()
            assert fe == L.flow() and np.array_equal(cut, L.getCut())
        S.release(t)
    st = S.stats()
    assert st["completed"] == len(tickets)
    assert st["max_in_flight"] >= 2          # requests overlapped on the device
    S.close()


def test_server_budget_admission(native, gpu):
    """A budget smaller than any request: each still runs, one at a time."""
    import latticeflow_gb300 as lf
    from latticeflow_gb300 import workloads as W
    S = lf.LatticeServer(workers=3, hbm_budget_bytes=1)
    ts = [S.submit_tv(W.tv_image(60 + i, n=64, polygons=3), 10.0) for i in range(5)]
    for t in ts:
        S.wait(t)
    st = S.stats()
    assert st["completed"] == 5 and st["max_in_flight"] == 1
    with pytest.raises(lf.BadSolverOrKernelName):
        S.submit_tv(np.zeros((4, 4)), 1.0, kernel="Full2d_12")   # no geocut weights
    S.close()


def test_server_groups_same_shape_tv(native, gpu, oracle_port):
    """Same-shape TV requests queued behind a running one are solved as one
    stacked problem; each result still equals its own solve."""
    import latticeflow_gb300 as lf
    from latticeflow_gb300 import workloads as W
    S = lf.LatticeServer(workers=1, max_group=4)
    first = S.submit_tv(W.tv_image(90, n=256, polygons=8), 0.05)
    reqs = [(W.tv_image(91 + i, n=64, polygons=4), lam)
            for i, lam in enumerate([0.01, 0.2, 3.0, 0.05, 9.0, 0.7])]
    ts = [S.submit_tv(f, lam) for f, lam in reqs]
    S.wait(first)
    for (f, lam), t in zip(reqs, ts):
        S.wait(t)
        out, lv = S.result(t)
        ref, r, _ = oracle_port.port_tv_single("Full2d_4", f, lam)
        assert int(np.abs(lv - r).max()) <= 1 and _tv_close(out, ref)
    st = S.stats()
    assert st["completed"] == 7
    assert st["groups"] >= 1 and st["grouped_requests"] >= 2
    S.close()
