"""The Python surface of pylatticeflow.pyx:80-302 on the GPU: addEnergy with
float energies (scaled by 1 / numerical_precision and rounded to int64, as
pylatticeflow.pyx:157-162 does), flat and lattice-shaped arrays, and its
shape errors.  Results against the oracle on the same rounded energies:
minimum energy and both canonical cut sets, bit-exact.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _float_problem(kernel, dims, seed, O):
    rng = np.random.default_rng(seed)
    offs, _ = O.lattice_offsets(kernel)
    N, Kp = int(np.prod(dims)), len(offs) // 2
    u = rng.uniform(-0.5, 1.5, size=(N, 2))
    w = rng.uniform(0.1, 0.9, size=(N, Kp))
    b = np.zeros((N, Kp, 4))
    b[:, :, 1] = w + rng.uniform(0, 0.1, size=(N, Kp))
    b[:, :, 2] = w
    b[:, :, 0] = rng.uniform(0, 0.05, size=(N, Kp))
    b[:, :, 3] = rng.uniform(0, 0.05, size=(N, Kp))  # E00 + E11 <= E01 + E10 holds
    return u, b


@pytest.mark.parametrize("kernel,dims,precision,shaped", [
    ("Full2d_4", (37, 41), 1e-6, False),
    ("Full2d_8", (30, 29), 1e-3, True),
    ("Full3d_6", (7, 9, 11), 1e-4, True),
])
def test_add_energy_floats_vs_oracle(native, gpu, oracle_port, kernel, dims, precision, shaped):
    import latticeflow_gb300 as lf
    O = oracle_port
    u, b = _float_problem(kernel, dims, 3, O)
    L = lf.LatticeFlow(kernel, "LatticeEnergyMinimizer", dims, numerical_precision=precision)
    if shaped:
        L.addEnergy(u.reshape(dims + (2,)), b.reshape(dims + b.shape[1:]))
    else:
        L.addEnergy(u, b)
    L.run()
    nf = 1.0 / precision
    ui = np.round(nf * u).astype(np.int64)
    bi = np.round(nf * b).astype(np.int64)
    E, cmin, cmax, _, _ = O.port_canonical(kernel, dims, ui, bi)
    assert L.flow()[1] == E
    assert np.array_equal(L.getCut(), cmin)
    assert np.array_equal(L.getCutMax(), cmax)


def test_add_energy_accumulates(native, gpu, oracle_port):
    """Two addEnergy calls add up (the reference's filler accumulates)."""
    import latticeflow_gb300 as lf
    O = oracle_port
    dims = (25, 22)
    u1, b1 = _float_problem("Full2d_4", dims, 5, O)
    u2, b2 = _float_problem("Full2d_4", dims, 6, O)
    L = lf.LatticeFlow("Full2d_4", "LatticeEnergyMinimizer", dims, numerical_precision=1e-3)
    L.addEnergy(u1, b1)
    L.addEnergy(u2, b2)
    L.run()
    ui = np.round(1e3 * u1).astype(np.int64) + np.round(1e3 * u2).astype(np.int64)
    bi = np.round(1e3 * b1).astype(np.int64) + np.round(1e3 * b2).astype(np.int64)
    E, cmin, _, _, _ = O.port_canonical("Full2d_4", dims, ui, bi)
    assert L.flow()[1] == E and np.array_equal(L.getCut(), cmin)


def test_add_energy_shape_errors(native, gpu):
    import latticeflow_gb300 as lf
    L = lf.LatticeFlow("Full2d_4", "LatticeEnergyMinimizer", (6, 5))
    ok_u, ok_b = np.zeros((30, 2)), np.zeros((30, 2, 4))
    with pytest.raises(ValueError, match="# unary_array_nodes"):
        L.addEnergy(np.zeros((29, 2)), ok_b)
    with pytest.raises(ValueError, match="2 required"):
        L.addEnergy(np.zeros((30, 3)), ok_b)
    with pytest.raises(ValueError, match="dimension 1 = 5"):
        L.addEnergy(np.zeros((6, 4, 2)), ok_b)
    with pytest.raises(ValueError, match="wrong number of edges"):
        L.addEnergy(ok_u, np.zeros((30, 3, 4)))
    with pytest.raises(ValueError, match="pairwise energy terms"):
        L.addEnergy(ok_u, np.zeros((30, 2, 3)))
    with pytest.raises(ValueError, match="wrong number of dimensions"):
        L.addEnergy(ok_u, np.zeros((30, 8)))
    L.addEnergy(ok_u, ok_b)  # the valid call still works after the errors
    L.run()
    assert L.flow()[1] == 0
