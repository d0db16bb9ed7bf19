"""Oracle-side restatement of latticeflow's kernel (neighbourhood) generator.

TEST INFRASTRUCTURE ONLY: this module is an oracle.  It is used by tests,
by the oracle's own build step (to emit the kernel header that the compiled
reference needs) and never by the product path.

It restates, in new code, the rules of the reference generator
``install/code_setup.py``:

* ``Full`` kernels (code_setup.py:200-222): every integer offset x with
  ``0 < sum(x_i^2) <= radius**2`` (radius a float, so sqrt(3)**2 rounds to
  2.9999999999999996 and the 3-d corner offsets are *not* produced at radius
  sqrt(3)), sorted lexicographically.
* ``Star`` kernels (code_setup.py:224-263): the Full set with every offset
  removed whose direction tuple ``(atan2(x1, x0), atan2(x2, x0), ...)`` was
  already seen on a shorter offset.
* 2-d geocut weights (code_setup.py:163-197): offsets sorted by angle; each
  gets half the angular gap between its two angular neighbours, divided by
  ``2 * |offset|``.  The reference Star generator passes an unordered set to
  the weight routine, so its weight order is undefined; here the weight is
  always paired with its own offset.
* radius list (code_setup.py:84-88) and naming ``%s%dd_%d`` (code_setup.py:40),
  with duplicates of an already generated offset set becoming aliases
  (code_setup.py:369-399).

The 26-connected 3-d kernel is never produced by those rules; it is added
under the name ``Full3d_26`` the way ``addKernel(name=...)`` allows.
"""
import math
from itertools import product

# default radii: wscript:54-64 (2-d: 4, 3-d: 2) with code_setup.py:13
DEFAULT_MAX_RADIUS = {2: 4, 3: 2}
# opt-in dimensions of the reference build (options and defaults at
# wscript:49-67): --1d adds Full kernels at the integer radii
# 1 .. max_1d_radius - 1 (code_setup.py:81-92), --4d Full and Star kernels at
# the 4-d radius intervals up to max_4d_radius (code_setup.py:135-153)
OPTIONAL_1D_MAX_RADIUS = 8
OPTIONAL_4D_MAX_RADIUS = 1


def radius_intervals(dim, max_radius):
    """code_setup.py:84-88: distinct offset norms in (0, max_radius]."""
    vals = set()
    for loc in product(*([range(0, max_radius + 1)] * dim)):
        vals.add(math.sqrt(sum(x * x for x in loc)))
    return sorted(d for d in vals if 0 < d <= max_radius + 1e-8)


def full_offsets(dim, radius):
    lo, hi = int(math.floor(-radius)), int(math.ceil(radius))
    out = []
    for x in product(*([range(lo, hi + 1)] * dim)):
        s = sum(v * v for v in x)
        if 0 < s <= radius ** 2:
            out.append(tuple(x))
    return sorted(out)


def star_offsets(dim, radius):
    full = full_offsets(dim, radius)
    by_len = sorted(full, key=lambda e: sum(u * u for u in e))
    seen = set()
    keep = []
    for e in by_len:
        ang = tuple(math.atan2(u, e[0]) for u in e[1:])
        if ang in seen:
            continue
        seen.add(ang)
        keep.append(e)
    return sorted(keep)


def geocut_weights(dim, edges):
    """Returns (applicable, weights aligned with ``edges``)."""
    if dim != 2 or len(edges) < 4:
        return False, [1.0] * len(edges)
    angles = [math.atan2(e[1], e[0]) % (2 * math.pi) for e in edges]
    if len(set(angles)) != len(edges):
        return False, [1.0] * len(edges)
    info = sorted(zip(angles, edges))
    a = [p[0] for p in info]
    n = len(a)
    wmap = {}
    for i, (ang, e) in enumerate(info):
        a1 = a[(i - 1) % n]
        a2 = a[(i + 1) % n]
        if a2 < a1:
            a2 += 2 * math.pi
        width = (a2 - a1) / 2
        wmap[e] = width / (2.0 * math.sqrt(e[0] * e[0] + e[1] * e[1]))
    return True, [wmap[e] for e in edges]


class KernelSpec:
    def __init__(self, name, kind, dim, radius, offsets, geocut, weights, alias_of=None):
        self.name = name
        self.kind = kind
        self.dim = dim
        self.radius = radius
        self.offsets = offsets          # kernel order (lexicographic), all K offsets
        self.geocut = geocut
        self.weights = weights
        self.alias_of = alias_of

    @property
    def size(self):
        return len(self.offsets)

    def lattice_order(self):
        """Offsets in the order the lattice uses them.

        kernellattice.hpp:61-96 sorts the offsets by their linear jump in the
        padded row-major array; the jump order equals lexicographic order of
        the offset (|delta_i| is smaller than the padded stride of dim i), the
        positive half comes first in ascending order and index i + K/2 is the
        reverse of i.  Returns (offsets, weights) in that order.
        """
        pairs = list(zip(self.offsets, self.weights))
        K = len(pairs)
        zero = tuple([0] * self.dim)
        pos = sorted([p for p in pairs if p[0] > zero])
        out = pos + [(tuple(-v for v in o), w) for o, w in pos]
        wmap = dict(pairs)
        offs = [o for o, _ in out]
        assert len(offs) == K
        return offs, [wmap[o] for o in offs]


def generate(max_radius=None, optional=False):
    """All kernel specs, keyed by name, in generation order.  optional: also
    the kernels of the reference's opt-in 1-d and 4-d builds (--1d, --4d)."""
    if max_radius is None:
        max_radius = DEFAULT_MAX_RADIUS
    specs = {}
    seen_sets = {}

    def add(dim, r, kinds):
        for kind in kinds:
            offs = full_offsets(dim, r) if kind == "Full" else star_offsets(dim, r)
            if not offs:
                continue
            name = "%s%dd_%d" % (kind, dim, len(offs))
            key = frozenset(offs)
            if key in seen_sets:
                if name in specs:
                    continue
                base = specs[seen_sets[key]]
                specs[name] = KernelSpec(name, kind, dim, r, base.offsets,
                                         base.geocut, base.weights, alias_of=base.name)
                continue
            if name in specs:
                continue
            g, w = geocut_weights(dim, offs)
            specs[name] = KernelSpec(name, kind, dim, r, offs, g, w)
            seen_sets[key] = name

    if optional:
        for r in range(1, OPTIONAL_1D_MAX_RADIUS):
            add(1, r, ("Full",))
    for dim in sorted(max_radius):
        for r in radius_intervals(dim, max_radius[dim]):
            add(dim, r, ("Full", "Star"))
    # The full 3x3x3 neighbourhood comes out of the Star rule at radius 2
    # (Full3d_32 minus the six length-2 axis offsets) as "Star3d_26"; the name
    # "Full3d_26" is registered as an alias of it (code_setup.py:369-399
    # aliasing), or defined directly when 3-d radius 2 is not generated.
    offs26 = sorted(x for x in product(range(-1, 2), repeat=3) if any(x))
    base = seen_sets.get(frozenset(offs26))
    if base is not None:
        b = specs[base]
        specs["Full3d_26"] = KernelSpec("Full3d_26", "Full", 3, b.radius, b.offsets,
                                        b.geocut, b.weights, alias_of=base)
    else:
        specs["Full3d_26"] = KernelSpec("Full3d_26", "Full", 3, 2.0, offs26,
                                        False, [1.0] * 26)
    if optional:
        for r in radius_intervals(4, OPTIONAL_4D_MAX_RADIUS):
            add(4, r, ("Full", "Star"))
    return specs


if __name__ == "__main__":
    for name, s in generate().items():
        print(name, s.size, s.alias_of or "", s.geocut)
