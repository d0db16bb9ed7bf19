"""Generates the golden fixtures in tests/golden/ from the compiled reference.

Run where the reference sources are available (they are not on GPU hosts):

    python tests/golden/make_golden.py

Each cut case stores the integer energies (interface layout), the reference
push-relabel labelling (LatticeEnergyMinimizer), the bundled BK labelling
(BKGCEnergyMinimizer) and the minimum energy.  Each TV case stores the input
image and calculate2dTV<Kernel, int64>'s output for one lambda; each path
case the image, a list of lambdas and calculate2dTV's regularisation-path
output (tv_solver.hpp:657-681).  The inputs are seeded, so the script is
deterministic.
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))

CUT_CASES = [
    # name, kernel, dims, generator, seed
    ("f4_rand", "Full2d_4", (23, 29), "random", 1),
    ("f4_zero", "Full2d_4", (8, 8), "zero", 0),
    ("f4_line", "Full2d_4", (1, 57), "random", 2),
    ("f8_rand", "Full2d_8", (31, 22), "random", 3),
    ("f8_seg", "Full2d_8", (40, 36), "segment", 4),
    ("s16_rand", "Star2d_16", (17, 19), "random", 5),
    ("f12_rand", "Full2d_12", (15, 18), "random", 6),
    ("f3d6_rand", "Full3d_6", (7, 9, 8), "random", 7),
    ("f3d26_rand", "Full3d_26", (6, 7, 9), "random", 8),
    ("f3d26_seg", "Full3d_26", (9, 8, 10), "segment", 9),
    ("f4_general", "Full2d_4", (12, 13), "general", 10),
]

TV_CASES = [
    ("tv_f4_a", "Full2d_4", (2, 2), 0.3, 11),
    ("tv_f4_b", "Full2d_4", (16, 16), 0.02, 12),
    ("tv_f4_c", "Full2d_4", (21, 18), 0.5, 13),
    ("tv_f8_a", "Full2d_8", (14, 17), 0.1, 14),
    ("tv_s16_a", "Star2d_16", (12, 12), 0.2, 15),
    ("tv_f4_d", "Full2d_4", (20, 24), 8.0, 16),
    ("tv_f4_e", "Full2d_4", (32, 32), 60.0, 17),
    ("tv_f8_b", "Full2d_8", (24, 20), 30.0, 18),
    ("tv_s16_b", "Star2d_16", (16, 18), 20.0, 19),
]


PATH_CASES = [
    # name, kernel, image, lambdas (calculate2dTV(nx, ny, f, vector<double>))
    ("f4_poly48", "Full2d_4", ("poly", 48, 6, 21), ("geom", 16)),
    ("f8_poly40", "Full2d_8", ("poly", 40, 5, 22), ("geom", 12)),
    ("s16_rand", "Star2d_16", ("rand", (24, 20), 23), ("list", [0.01, 0.05, 0.2, 1.0])),
    ("f4_rand_unsorted", "Full2d_4", ("rand", (33, 30), 24), ("list", [0.3, -0.5, 0.01, 2.0, 0.07])),
    ("f4_line", "Full2d_4", ("rand", (1, 40), 25), ("list", [0.1, 1.0])),
    ("f4_poly64", "Full2d_4", ("poly", 64, 8, 26), ("geom", 64)),
    # regions above the GPU's one-block probe bound (2,048 nodes): probes on
    # the lattice-wide solver
    ("f4_poly128", "Full2d_4", ("poly", 128, 12, 27), ("geom", 24)),
]


def path_inputs(image, lams):
    from latticeflow_gb300 import workloads as W
    if image[0] == "poly":
        f = W.tv_image(image[3], n=image[1], polygons=image[2])
    else:
        f = np.random.default_rng(image[2]).random(image[1])
    if lams[0] == "geom":
        lv = np.array([1e-3 * 1000.0 ** (i / (lams[1] - 1)) for i in range(lams[1])])
    else:
        lv = np.array(lams[1], dtype=np.float64)
    return f, lv


def make_energies(kernel, dims, gen, seed):
    rng = np.random.default_rng(seed)
    offs, _ = O.lattice_offsets(kernel)
    N = int(np.prod(dims))
    Kp = len(offs) // 2
    if gen == "zero":
        return np.zeros((N, 2), np.int64), np.zeros((N, Kp, 4), np.int64)
    if gen == "random":
        u = rng.integers(0, 100, size=(N, 2)).astype(np.int64)
        w = rng.integers(0, 60, size=(N, Kp)).astype(np.int64)
    elif gen == "segment":
        y = rng.normal(0, 0.3, size=dims) + (rng.random(dims) > 0.5)
        y = y.reshape(-1)
        u = np.stack([np.round(100 * np.maximum(0, y - 0.5)),
                      np.round(100 * np.maximum(0, 0.5 - y))], axis=1).astype(np.int64)
        w = rng.integers(1, 40, size=(N, Kp)).astype(np.int64)
    elif gen == "general":
        # general submodular tables: E00 + E11 <= E01 + E10, some negatives
        u = rng.integers(-50, 100, size=(N, 2)).astype(np.int64)
        b = rng.integers(-20, 40, size=(N, Kp, 4)).astype(np.int64)
        s = b[:, :, 0] + b[:, :, 3] - b[:, :, 1] - b[:, :, 2]
        b[:, :, 1] += np.maximum(s, 0)
        return u, b
    b = np.zeros((N, Kp, 4), np.int64)
    b[:, :, 1] = w
    b[:, :, 2] = w
    return u, b


def main():
    if not O.ref_available() and not O.build_ref():
        raise SystemExit("compiled reference not available")
    # optional names of fixtures to (re)make, e.g. "path_f4_poly128"; all by default
    only = set(sys.argv[1:])

    def wanted(kind, name):
        return not only or "%s_%s" % (kind, name) in only

    for name, kernel, dims, gen, seed in CUT_CASES:
        if not wanted("cut", name):
            continue
        u, b = make_energies(kernel, dims, gen, seed)
        pr, _ = O.ref_solve("LatticeEnergyMinimizer", kernel, dims, u, b)
        bk, _ = O.ref_solve("BKGCEnergyMinimizer", kernel, dims, u, b)
        e = O.energy(kernel, dims, u, b, bk)
        assert e == O.energy(kernel, dims, u, b, pr)
        np.savez_compressed(os.path.join(OUT, "cut_%s.npz" % name), kernel=kernel,
                            dims=np.asarray(dims), unary=u, binary=b, pr_cut=pr.astype(np.int8),
                            bk_cut=bk.astype(np.int8), energy=np.int64(e))
        print(name, e, int(bk.sum()), int(pr.sum()))
    for name, kernel, dims, lam, seed in TV_CASES:
        if not wanted("tv", name):
            continue
        f = np.random.default_rng(seed).random(dims)
        out, _ = O.ref_tv_single(kernel, f, lam)
        np.savez_compressed(os.path.join(OUT, "tv_%s.npz" % name), kernel=kernel, f=f,
                            lam=np.float64(lam), out=out)
        print(name, float(out.min()), float(out.max()), len(np.unique(out)))
    for name, kernel, image, lams in PATH_CASES:
        if not wanted("path", name):
            continue
        f, lv = path_inputs(image, lams)
        out, _ = O.ref_tv_path(kernel, f, lv)
        again, _ = O.ref_tv_path(kernel, f, lv)
        assert np.array_equal(out, again), name  # no event ties: the reference is repeatable
        np.savez_compressed(os.path.join(OUT, "path_%s.npz" % name), kernel=kernel, f=f,
                            lams=lv, out=out)
        print(name, out.shape, float(out.min()), float(out.max()))


if __name__ == "__main__":
    main()
