"""Seeded synthetic workloads with the shapes of the benchmark configurations.

The reference publishes no dataset; these generators stand in for it
(numpy ``default_rng(seed)``, float64 generation, integer capacities by
``round``).  Convention: "on" = source side; a node pays ``source`` (E0)
when off and ``sink`` (E1) when on; a symmetric edge of capacity w is the
pairwise table (E00, E01, E10, E11) = (0, w, w, 0).

* ``plain_cut``   256x256 Full2d_4: two random ellipses (1) on 0 + N(0, 0.3^2);
                  source = round(100 max(0, y - 0.5)), sink = round(100 max(0, 0.5 - y)),
                  w = round(50 exp(-dy^2 / (2 0.1^2))) + 1.
* ``large_cut``   2048x2048 Full2d_8: 20 ellipses at U[0,1] intensities + N(0, 0.2^2);
                  t = round(100 (-log p_fg + log p_bg)) with Gaussian models at
                  0.7 (fg) and 0.3 (bg), sigma 0.15; t > 0 -> sink = t, else source = -t;
                  w = round(100 exp(-dy^2 / (2 0.05^2)) / |offset|) + 1.
* ``volume_cut``  256^3 Full3d_26: sum of 50 Gaussian blobs thresholded at 0.5
                  + N(0, 0.25^2); terminals as plain_cut, w = round(50 exp(-dy^2 /
                  (2 0.1^2)) / |offset|) + 1.
* ``batch``       512 lattices, sides exp(U[ln 64, ln 1024]) per axis, even index
                  Full2d_4, odd Full2d_8, plain_cut terminals/edges, seed = base + i.
* ``tv_image``    1024x1024: 30 random polygons with U[0,1] values + N(0, 0.1^2),
                  cast to float32 and back to float64.
"""
import math

import numpy as np


def positive_offsets(kernel):
    """Filling-edge offsets in lattice order (positive half, ascending)."""
    full = {
        "Full2d_4": [(0, 1), (1, 0)],
        "Full2d_8": [(0, 1), (1, -1), (1, 0), (1, 1)],
        "Full3d_6": [(0, 0, 1), (0, 1, 0), (1, 0, 0)],
    }
    if kernel in full:
        return np.asarray(full[kernel], dtype=np.int64)
    if kernel in ("Full3d_26", "Star3d_26"):
        offs = [o for o in np.ndindex(3, 3, 3)]
        offs = [tuple(v - 1 for v in o) for o in offs]
        pos = sorted(o for o in offs if o > (0, 0, 0))
        return np.asarray(pos, dtype=np.int64)
    raise ValueError("no built-in offsets for " + kernel)


class CutProblem(object):
    """A lattice cut in capacity form (int32) with an energy view."""

    def __init__(self, kernel, dims, source, sink, edge):
        self.kernel = kernel
        self.dims = tuple(int(d) for d in dims)
        self.source = source.astype(np.int32, copy=False).reshape(-1)
        self.sink = sink.astype(np.int32, copy=False).reshape(-1)
        self.edge = edge.astype(np.int32, copy=False).reshape(self.source.size, -1)

    @property
    def n(self):
        return self.source.size

    def energies(self):
        """(unary int64[N,2], binary int64[N,K/2,4]) in the interface layout."""
        u = np.stack([self.source, self.sink], axis=1).astype(np.int64)
        b = np.zeros((self.n, self.edge.shape[1], 4), dtype=np.int64)
        b[:, :, 1] = self.edge
        b[:, :, 2] = self.edge
        return u, b


def _edge_caps(img, offs, fn):
    """Capacity of each filling edge: fn(|dy|^2, |offset|); 0 where the edge leaves."""
    dims = img.shape
    out = np.zeros(dims + (len(offs),), dtype=np.int64)
    for e, d in enumerate(offs):
        src = []
        dst = []
        for ax, dv in enumerate(d):
            n = dims[ax]
            if dv >= 0:
                src.append(slice(0, n - dv))
                dst.append(slice(dv, n))
            else:
                src.append(slice(-dv, n))
                dst.append(slice(0, n + dv))
        dy = img[tuple(src)] - img[tuple(dst)]
        dist = math.sqrt(float(np.sum(np.asarray(d) ** 2)))
        out[tuple(src) + (e,)] = fn(dy * dy, dist)
    return out


def _ellipses(rng, n, count, values):
    img = np.zeros((n, n))
    yy, xx = np.mgrid[0:n, 0:n].astype(np.float64)
    for i in range(count):
        cx, cy = rng.uniform(0.2, 0.8, size=2) * n
        ax, ay = rng.uniform(0.08, 0.3, size=2) * n
        th = rng.uniform(0, math.pi)
        c, s = math.cos(th), math.sin(th)
        u = ((xx - cx) * c + (yy - cy) * s) / ax
        v = (-(xx - cx) * s + (yy - cy) * c) / ay
        img[u * u + v * v <= 1.0] = values[i]
    return img


def plain_cut(seed=0, shape=(256, 256), kernel="Full2d_4"):
    rng = np.random.default_rng(seed)
    nx, ny = shape
    n = max(nx, ny)
    img = _ellipses(rng, n, 2, [1.0, 1.0])[:nx, :ny]
    y = img + rng.normal(0, 0.3, size=img.shape)
    source = np.round(100 * np.maximum(0, y - 0.5))
    sink = np.round(100 * np.maximum(0, 0.5 - y))
    offs = positive_offsets(kernel)
    edge = _edge_caps(y, offs, lambda d2, dist: np.round(50 * np.exp(-d2 / (2 * 0.1 ** 2))) + 1)
    return CutProblem(kernel, shape, source, sink, edge)


def large_cut(seed=0, n=2048, kernel="Full2d_8", sigma=0.15):
    rng = np.random.default_rng(seed)
    img = _ellipses(rng, n, 20, rng.uniform(0, 1, size=20))
    y = img + rng.normal(0, 0.2, size=img.shape)
    t = np.round(100 * (((y - 0.7) ** 2 - (y - 0.3) ** 2) / (2 * sigma ** 2)))
    sink = np.maximum(t, 0)
    source = np.maximum(-t, 0)
    offs = positive_offsets(kernel)
    edge = _edge_caps(y, offs, lambda d2, dist: np.round(100 * np.exp(-d2 / (2 * 0.05 ** 2)) / dist) + 1)
    return CutProblem(kernel, (n, n), source, sink, edge)


def volume_cut(seed=0, n=256, kernel="Full3d_26", blobs=50):
    rng = np.random.default_rng(seed)
    ax = np.arange(n, dtype=np.float64)
    vol = np.zeros((n, n, n))
    for _ in range(blobs):
        c = rng.uniform(0, n, size=3)
        s = rng.uniform(0.03, 0.08) * n
        gx = np.exp(-(ax - c[0]) ** 2 / (2 * s * s))
        gy = np.exp(-(ax - c[1]) ** 2 / (2 * s * s))
        gz = np.exp(-(ax - c[2]) ** 2 / (2 * s * s))
        vol += gx[:, None, None] * gy[None, :, None] * gz[None, None, :]
    y = (vol > 0.5).astype(np.float64) + rng.normal(0, 0.25, size=vol.shape)
    source = np.round(100 * np.maximum(0, y - 0.5))
    sink = np.round(100 * np.maximum(0, 0.5 - y))
    offs = positive_offsets(kernel)
    edge = _edge_caps(y, offs, lambda d2, dist: np.round(50 * np.exp(-d2 / (2 * 0.1 ** 2)) / dist) + 1)
    return CutProblem(kernel, (n, n, n), source, sink, edge)


def batch_shapes(count=512, seed=0, lo=64, hi=1024):
    rng = np.random.default_rng(seed)
    sides = np.round(np.exp(rng.uniform(math.log(lo), math.log(hi), size=(count, 2)))).astype(int)
    return [(int(a), int(b)) for a, b in sides]


def batch(count=512, seed=0, base_seed=1000):
    shapes = batch_shapes(count, seed)
    out = []
    for i, s in enumerate(shapes):
        kernel = "Full2d_4" if i % 2 == 0 else "Full2d_8"
        out.append(plain_cut(base_seed + i, s, kernel))
    return out


def _polygon_mask(n, verts):
    """Even-odd rule rasterisation of one polygon on an n x n grid (pixel centres)."""
    xs, ys = verts[:, 0], verts[:, 1]
    x0, x1 = int(max(0, math.floor(xs.min()))), int(min(n, math.ceil(xs.max()) + 1))
    y0, y1 = int(max(0, math.floor(ys.min()))), int(min(n, math.ceil(ys.max()) + 1))
    mask = np.zeros((n, n), dtype=bool)
    if x1 <= x0 or y1 <= y0:
        return mask
    py, px = np.mgrid[y0:y1, x0:x1].astype(np.float64)
    inside = np.zeros(px.shape, dtype=bool)
    m = len(verts)
    for i in range(m):
        xa, ya = verts[i]
        xb, yb = verts[(i + 1) % m]
        cond = (ya > py) != (yb > py)
        with np.errstate(divide="ignore", invalid="ignore"):
            xint = xa + (py - ya) * (xb - xa) / (yb - ya)
        inside ^= cond & (px < xint)
    mask[y0:y1, x0:x1] = inside
    return mask


def tv_image(seed=0, n=1024, polygons=30, noise=0.1):
    rng = np.random.default_rng(seed)
    img = np.zeros((n, n))
    for _ in range(polygons):
        c = rng.uniform(0, n, size=2)
        k = int(rng.integers(3, 9))
        ang = np.sort(rng.uniform(0, 2 * math.pi, size=k))
        rad = rng.uniform(0.05, 0.25, size=k) * n
        verts = np.stack([c[0] + rad * np.cos(ang), c[1] + rad * np.sin(ang)], axis=1)
        img[_polygon_mask(n, verts)] = rng.uniform(0, 1)
    f = img + rng.normal(0, noise, size=img.shape)
    return f.astype(np.float32).astype(np.float64)
