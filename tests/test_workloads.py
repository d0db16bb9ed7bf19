import numpy as np

from latticeflow_gb300 import workloads as W


def test_plain_cut_shapes_and_determinism():
    a = W.plain_cut(3)
    b = W.plain_cut(3)
    assert a.dims == (256, 256) and a.edge.shape == (65536, 2)
    assert np.array_equal(a.source, b.source) and np.array_equal(a.edge, b.edge)
    assert a.source.min() >= 0 and a.sink.min() >= 0 and a.edge.min() >= 0
    # no node is both source and sink connected
    assert not np.any((a.source > 0) & (a.sink > 0))
    u, bb = a.energies()
    assert u.shape == (65536, 2) and bb.shape == (65536, 2, 4)


def test_edges_leaving_lattice_are_zero():
    p = W.plain_cut(1, (17, 23), "Full2d_8")
    e = p.edge.reshape(17, 23, 4)
    offs = W.positive_offsets("Full2d_8")
    for k, (dx, dy) in enumerate(offs):
        if dx > 0:
            assert np.all(e[17 - dx:, :, k] == 0)
        if dy > 0:
            assert np.all(e[:, 23 - dy:, k] == 0)
        if dy < 0:
            assert np.all(e[:, :-dy, k] == 0)


def test_batch_shapes():
    s = W.batch_shapes(512)
    a = np.asarray(s)
    assert a.shape == (512, 2) and a.min() >= 64 and a.max() <= 1024


def test_tv_image():
    f = W.tv_image(0, n=128, polygons=5)
    assert f.shape == (128, 128) and f.dtype == np.float64
    assert np.array_equal(f, f.astype(np.float32).astype(np.float64))
