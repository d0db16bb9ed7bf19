"""Batched solves: every lattice of a batch gets exactly the result of its own
plain solve and of the oracle (energy, minimal and maximal on-sets)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_batch_mixed_kernels_vs_oracle(native, gpu, oracle_port):
    import latticeflow_gb300 as lf
    from latticeflow_gb300 import workloads as W
    rng = np.random.default_rng(0)
    probs = []
    for i in range(24):
        shape = (int(rng.integers(20, 150)), int(rng.integers(20, 150)))
        kernel = "Full2d_4" if i % 2 == 0 else "Full2d_8"
        probs.append(W.plain_cut(500 + i, shape, kernel))
    B = lf.LatticeBatch()
    for p in probs:
        B.add(p.kernel, p.dims)
    for i, p in enumerate(probs):
        if i % 3 == 0:
            B.addEnergyPotentials(i, *p.energies())
        else:
            B.addCapacities(i, p.source, p.sink, p.edge)
    B.run()
    for i, p in enumerate(probs):
        u, b = p.energies()
        E, cmin, cmax, _, _ = oracle_port.port_canonical(p.kernel, p.dims, u, b)
        assert B.flow(i)[1] == E, i
        assert np.array_equal(B.getCut(i), cmin), i
        assert np.array_equal(B.getCutMax(i), cmax), i


def test_batch_equals_plain_and_reruns(native, gpu):
    import latticeflow_gb300 as lf
    from latticeflow_gb300 import workloads as W
    shapes = W.batch_shapes(16, seed=3, lo=32, hi=300)
    probs = [W.plain_cut(900 + i, s, "Full2d_4" if i % 2 else "Full2d_8") for i, s in enumerate(shapes)]
    B = lf.LatticeBatch()
    for p in probs:
        B.add(p.kernel, p.dims)
    for i, p in enumerate(probs):
        B.addCapacities(i, p.source, p.sink, p.edge)
    B.run()
    first = [(B.flow(i), B.getCut(i).copy()) for i in range(len(probs))]
    for i, p in enumerate(probs):
        L = lf.LatticeFlow(p.kernel, "LatticeEnergyMinimizer", p.dims)
        L.addCapacities(p.source, p.sink, p.edge)
        L.run()
        assert L.flow() == first[i][0]
        assert np.array_equal(L.getCut(), first[i][1])
    # clear + refill + rerun gives the same answers
    B.clear()
    for i, p in enumerate(probs):
        B.addCapacities(i, p.source, p.sink, p.edge)
    B.run()
    for i in range(len(probs)):
        assert B.flow(i) == first[i][0] and np.array_equal(B.getCut(i), first[i][1])


def test_batch_3d_and_errors(native, gpu, oracle_port):
    import latticeflow_gb300 as lf
    rng = np.random.default_rng(5)
    B = lf.LatticeBatch()
    dims = [(6, 7, 40), (9, 5, 33), (4, 4, 4)]
    data = []
    for d in dims:
        B.add("Full3d_26", d)
    for i, d in enumerate(dims):
        N = int(np.prod(d))
        u = rng.integers(0, 100, size=(N, 2)).astype(np.int64)
        w = rng.integers(0, 50, size=(N, 13)).astype(np.int64)
        b = np.zeros((N, 13, 4), np.int64)
        b[:, :, 1] = w
        b[:, :, 2] = w
        B.addEnergyPotentials(i, u, b)
        data.append((u, b))
    B.run()
    for i, d in enumerate(dims):
        E, cmin, cmax, _, _ = oracle_port.port_canonical("Full3d_26", d, *data[i])
        assert B.flow(i)[1] == E
        assert np.array_equal(B.getCut(i), cmin) and np.array_equal(B.getCutMax(i), cmax)
    with pytest.raises(lf.LatticeFlowError):
        B.add("Full3d_6", (4, 4, 4))   # lattices are added before the first fill
    B2 = lf.LatticeBatch()
    B2.add("Full2d_4", (8, 8))
    B2.add("Full2d_8", (8, 8))
    with pytest.raises(ValueError):
        B2.add("Star2d_16", (8, 8))    # at most two kernel sizes


@pytest.mark.parametrize("pr_kernel,bfs_kernel,device_loops", [(0, 0, 1), (0, 0, 0), (1, 1, 0), (2, 0, 1)])
@pytest.mark.parametrize("tile_rows", [4, 8, 16, 32])
def test_batch_pass_variants(native, gpu, oracle_port, pr_kernel, bfs_kernel, device_loops, tile_rows):
    """A pool of mixed 4- and 8-connected lattices through the TMA-staged pool
    passes (device-side loops or one launch per pass) and the generic tile
    passes: every lattice gets the oracle's energy and both cut sets."""
    import latticeflow_gb300 as lf
    from latticeflow_gb300 import workloads as W
    shapes = W.batch_shapes(20, seed=7 + tile_rows, lo=24, hi=260)
    probs = [W.plain_cut(1200 + i, s, "Full2d_8" if i % 3 else "Full2d_4") for i, s in enumerate(shapes)]
    B = lf.LatticeBatch()
    for p in probs:
        B.add(p.kernel, p.dims)
    B.setParam("pr_kernel", pr_kernel)
    B.setParam("bfs_kernel", bfs_kernel)
    B.setParam("device_loops", device_loops)
    B.setParam("tile_rows", tile_rows)
    B.setParam("local_sweeps", 2)
    B.setParam("launches_per_relabel", 4)
    for i, p in enumerate(probs):
        B.addCapacities(i, p.source, p.sink, p.edge)
    for rep in range(2):
        B.run()
        for i, p in enumerate(probs):
            u, b = p.energies()
            E, cmin, cmax, _, _ = oracle_port.port_canonical(p.kernel, p.dims, u, b)
            assert B.flow(i)[1] == E, (rep, i)
            assert np.array_equal(B.getCut(i), cmin), (rep, i)
            assert np.array_equal(B.getCutMax(i), cmax), (rep, i)


def test_batch_packed_fill_and_results(native, gpu, oracle_port):
    """The packed calls (one fill for every lattice, every cut in one array)
    give the per-lattice calls' results and the oracle's."""
    import latticeflow_gb300 as lf
    from latticeflow_gb300 import workloads as W
    shapes = W.batch_shapes(20, seed=8, lo=20, hi=160)
    probs = [W.plain_cut(700 + i, s, "Full2d_4" if i % 2 else "Full2d_8") for i, s in enumerate(shapes)]
    B = lf.LatticeBatch()
    for p in probs:
        B.add(p.kernel, p.dims)
    B.addCapacitiesPacked(np.concatenate([p.source for p in probs]),
                          np.concatenate([p.sink for p in probs]),
                          np.concatenate([p.edge.reshape(-1) for p in probs]))
    B.run()
    cuts = B.getCutsPacked()
    cuts_max = B.getCutsPacked(maximal=True)
    flows, energies = B.flows()
    off = 0
    for i, p in enumerate(probs):
        u, b = p.energies()
        E, cmin, cmax, _, _ = oracle_port.port_canonical(p.kernel, p.dims, u, b)
        assert energies[i] == E and B.flow(i) == (flows[i], energies[i])
        assert np.array_equal(cuts[off:off + p.n].reshape(p.dims), cmin)
        assert np.array_equal(cuts_max[off:off + p.n].reshape(p.dims), cmax)
        assert np.array_equal(B.getCut(i), cmin)
        off += p.n
    with pytest.raises(ValueError):
        B.addCapacitiesPacked(np.zeros(3, dtype=np.int32))
    # pinned host arrays are read in place by the fill kernels: same results
    import torch

    def pinned(a):
        return torch.from_numpy(np.ascontiguousarray(a)).pin_memory().numpy()
    B.clear()
    B.addCapacitiesPacked(pinned(np.concatenate([p.source for p in probs])),
                          pinned(np.concatenate([p.sink for p in probs])),
                          pinned(np.concatenate([p.edge.reshape(-1) for p in probs])))
    B.run()
    assert np.array_equal(B.getCutsPacked(out=pinned(np.zeros(cuts.size, np.int32))), cuts)
    assert np.array_equal(B.flows()[1], energies)
    # the same pinned arrays moved into the batch's kept staging buffer by the
    # copy engine first (twice: the buffer is reused)
    B.setParam("host_stage", 1)
    for _ in range(2):
        B.clear()
        B.addCapacitiesPacked(pinned(np.concatenate([p.source for p in probs])),
                              pinned(np.concatenate([p.sink for p in probs])),
                              pinned(np.concatenate([p.edge.reshape(-1) for p in probs])))
        B.run()
        assert np.array_equal(B.getCutsPacked(), cuts)
        assert np.array_equal(B.getCutsPacked(maximal=True), cuts_max)
        assert np.array_equal(B.flows()[1], energies)
