"""Python surface of the GPU engine, mirroring the reference extension.

``LatticeFlow`` follows ``extensions/python/pylatticeflow.pyx:80-302``
(constructor arguments, ``addEnergy`` shapes and rounding, ``run``,
``runTime``, ``getCut`` and the properties), and the module functions follow
the factory helpers of ``solver/interface.hpp:186-191``.  Everything calls the
C ABI of ``include/latticeflow_gpu.h``; nothing here computes a cut.
"""
import ctypes

import numpy as np

from . import _native as N


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def isValidSolver(name):
    return bool(N.lib().lf_is_valid_solver(name.encode()))


def isValidKernel(name):
    return bool(N.lib().lf_is_valid_kernel(name.encode()))


def kernelDimension(kernel):
    d = N.lib().lf_kernel_dimension(kernel.encode())
    if d < 0:
        raise N.BadSolverOrKernelName("Bad Kernel or Solver Name: " + kernel)
    return d


def _names(fn):
    n = fn(None, 0)
    buf = ctypes.create_string_buffer(n)
    fn(buf, n)
    return [s for s in buf.value.decode().split("\n") if s]


def validKernelNames():
    return _names(N.lib().lf_valid_kernel_names)


def validSolverNames():
    return _names(N.lib().lf_valid_solver_names)


def kernelInfo(kernel):
    """(offsets[K, nd] in lattice order, geocut weights[K], geocut applicable)."""
    L = N.lib()
    nd = ctypes.c_int(0)
    K = L.lf_kernel_info(kernel.encode(), ctypes.byref(nd), None, None, None)
    if K < 0:
        raise N.BadSolverOrKernelName(N.last_error())
    d = np.zeros(K * nd.value, dtype=np.int32)
    w = np.zeros(K, dtype=np.float64)
    g = ctypes.c_int(0)
    L.lf_kernel_info(kernel.encode(), None, _p(d), _p(w), ctypes.byref(g))
    return d.reshape(K, nd.value), w, bool(g.value)


class LatticeFlow(object):
    """An interface to the lattice flow solvers (pylatticeflow.pyx:80-135).

    ``solver`` may be a reference solver name ("LatticeEnergyMinimizer",
    "LatticeLevelReductions") or its GPU name; both run on the GPU.
    """

    def __init__(self, kernel, solver, _dimensions, numerical_precision=1e-6):
        if not isValidSolver(solver):
            raise ValueError("'%s' not a valid solver name!  Valid solvers are: %s."
                             % (solver, ", ".join(validSolverNames())))
        if not isValidKernel(kernel):
            raise ValueError("Kernel '%s' not a valid kernel name!  Valid kernels are: %s."
                             % (kernel, ", ".join(validKernelNames())))
        dim = kernelDimension(kernel)
        self._dimensions = tuple(int(v) for v in _dimensions)
        self.n_nodes = int(np.prod(self._dimensions))
        if len(self._dimensions) != dim:
            raise ValueError("Kernel '%s' is %d-dimensional; a shape of %d dimensions was provided."
                             % (kernel, dim, len(self._dimensions)))
        self.kernel = kernel
        self.solver = solver
        self.numerical_precision_factor = 1.0 / numerical_precision
        dims = np.asarray(self._dimensions, dtype=np.uint64)
        h = ctypes.c_void_p()
        N.check(N.lib().lf_create(solver.encode(), kernel.encode(), dim, _p(dims), ctypes.byref(h)))
        self._h = h
        ne = N.lib().lf_n_filling_edges(h)
        e = np.zeros(ne * dim, dtype=np.int32)
        N.check(N.lib().lf_edge_deltas(h, _p(e)))
        self._edges = e.reshape(ne, dim)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            N.lib().lf_destroy(h)
            self._h = None

    # ---------------------------------------------------------- properties
    @property
    def ndim(self):
        return len(self._dimensions)

    @property
    def shape(self):
        return self._dimensions

    @property
    def size(self):
        return self.n_nodes

    @property
    def nFillingEdges(self):
        return self._edges.shape[0]

    @property
    def edges(self):
        return self._edges

    # -------------------------------------------------------------- filling
    def _check_arrays(self, unary_a, pairwise_a):
        ue = ("Unary energy must be either a 2d array with first dimension matching the number "
              "of nodes and second dimension containing E0 and E1, or (#dimensions + 1) with the "
              "first matching the lattice coordinates and the last containing E0 and E1.")
        if unary_a.ndim == 2:
            if unary_a.shape[0] != self.n_nodes:
                raise ValueError(ue + " (# nodes = %d; # unary_array_nodes = %d)"
                                 % (self.n_nodes, unary_a.shape[0]))
            if unary_a.shape[1] != 2:
                raise ValueError(ue + " (Second dimension has shape %d; 2 required.)"
                                 % unary_a.shape[1])
        elif unary_a.ndim == len(self._dimensions) + 1:
            for i, d in enumerate(self._dimensions):
                if unary_a.shape[i] != d:
                    raise ValueError(ue + " (dimension %d = %d; unary_array shape is %d)"
                                     % (i, d, unary_a.shape[i]))
            if unary_a.shape[-1] != 2:
                raise ValueError(ue + " (Last dimension has shape %d; 2 required.)"
                                 % unary_a.shape[-1])
        else:
            raise ValueError(ue + " (wrong number of dimensions)")
        pe = ("Pairwise energy must be either: (1) a 3d array with first dimension matching the "
              "number of nodes, second dimension containing the edge direction output, and third "
              "dimension containing E00, E01, E10, and E11 (with E01 being energy of source node "
              "off and dest node on.), or (2) a (#dimensions + 2) array with last two dimensions "
              "being the same and first dimensions corresponding to the lattice coordinates. ")
        ne = self.nFillingEdges
        if pairwise_a.ndim == 3:
            if pairwise_a.shape[0] != self.n_nodes:
                raise ValueError(pe + " (# nodes = %d; # nodes in pairwise_energy = %d)"
                                 % (self.n_nodes, pairwise_a.shape[0]))
        elif pairwise_a.ndim == len(self._dimensions) + 2:
            for i, d in enumerate(self._dimensions):
                if pairwise_a.shape[i] != d:
                    raise ValueError(pe + " (dimension %d shape is %d; pairwise_array shape is %d)"
                                     % (i, d, pairwise_a.shape[i]))
        else:
            raise ValueError(pe + " (Array has wrong number of dimensions.)")
        if pairwise_a.shape[-2] != ne:
            raise ValueError(pe + " (wrong number of edges specified in second-to-last dimension;"
                             " got %d, needed %d)." % (pairwise_a.shape[-2], ne))
        if pairwise_a.shape[-1] != 4:
            raise ValueError(pe + " (wrong number of pairwise energy terms; needed 4, got %d."
                             % pairwise_a.shape[-1])

    def addEnergy(self, unary_energy, pairwise_energy):
        """pylatticeflow.pyx:157-267: energies are scaled by 1/numerical_precision,
        rounded to int64 and accumulated into the lattice."""
        nf = self.numerical_precision_factor
        u = np.ascontiguousarray(np.round(nf * np.asarray(unary_energy)), dtype=np.int64)
        b = np.ascontiguousarray(np.round(nf * np.asarray(pairwise_energy)), dtype=np.int64)
        self._check_arrays(u, b)
        self.addEnergyPotentials(u, b)

    def addEnergyPotentials(self, unary, binary):
        """Integer form (interface.hpp:61): unary int64[N, 2], binary int64[N, K/2, 4]."""
        u = np.ascontiguousarray(unary, dtype=np.int64).reshape(-1)
        b = np.ascontiguousarray(binary, dtype=np.int64).reshape(-1)
        if u.size != 2 * self.n_nodes or b.size != 4 * self.nFillingEdges * self.n_nodes:
            raise ValueError("energy arrays do not match the lattice")
        N.check(N.lib().lf_add_energy_potentials(self._h, _p(u), _p(b)))

    def addCapacities(self, source=None, sink=None, edges=None):
        """Capacity form: source = cost of off, sink = cost of on, edges[N, K/2]."""
        args = []
        keep = []
        for a, n in ((source, self.n_nodes), (sink, self.n_nodes),
                     (edges, self.n_nodes * self.nFillingEdges)):
            if a is None:
                args.append(None)
                continue
            a = np.ascontiguousarray(a, dtype=np.int32).reshape(-1)
            if a.size != n:
                raise ValueError("capacity array has the wrong size")
            keep.append(a)
            args.append(_p(a))
        N.check(N.lib().lf_add_capacities(self._h, *args))

    # -------------------------------------------------------------- control
    def run(self):
        N.check(N.lib().lf_run(self._h))

    def runTime(self):
        """Device time of the last run, seconds."""
        return N.lib().lf_run_time(self._h)

    def clear(self):
        """Zero the accumulated energies (as a freshly created lattice)."""
        N.check(N.lib().lf_clear(self._h))

    def setProfiling(self, enable=True):
        N.check(N.lib().lf_set_profiling(self._h, 1 if enable else 0))

    def profile(self):
        """Per-category device milliseconds and counts of the last run."""
        ms = np.zeros(4, dtype=np.float64)
        c = np.zeros(6, dtype=np.int64)
        N.check(N.lib().lf_get_profile(self._h, _p(ms), _p(c)))
        return {"pr_ms": ms[0], "bfs_ms": ms[1], "reach_ms": ms[2], "run_ms": ms[3],
                "pr_launches": int(c[0]), "pr_tiles": int(c[1]), "bfs_passes": int(c[2]),
                "reach_passes": int(c[3]), "kernel_launches": int(c[4]), "bfs_tiles": int(c[5])}

    def stream(self):
        """The handle's cudaStream_t as an integer."""
        s = ctypes.c_void_p()
        N.check(N.lib().lf_get_stream(self._h, ctypes.byref(s)))
        return s.value or 0

    def layout(self):
        """Device layout of the last run: tile extents, padded extents, capacity bytes."""
        t = np.zeros(3, dtype=np.int32)
        pd = np.zeros(3, dtype=np.uint64)
        e = ctypes.c_int(0)
        N.check(N.lib().lf_get_layout(self._h, _p(t), _p(pd), ctypes.byref(e)))
        return tuple(int(v) for v in t), tuple(int(v) for v in pd), e.value

    def setParam(self, name, value):
        N.check(N.lib().lf_set_param(self._h, name.encode(), int(value)))

    def setTuning(self, tile_rows=0, local_sweeps=0, launches_per_relabel=0):
        N.check(N.lib().lf_set_tuning(self._h, tile_rows, local_sweeps, launches_per_relabel))

    # -------------------------------------------------------------- results
    def getCut(self):
        """int array shaped like the lattice, 1 = on (minimal on-set for binary cuts)."""
        out = np.empty(self.n_nodes, dtype=np.int32)
        N.check(N.lib().lf_get_cut(self._h, _p(out)))
        return out.reshape(self._dimensions)

    def getCutMax(self):
        out = np.empty(self.n_nodes, dtype=np.int32)
        N.check(N.lib().lf_get_cut_max(self._h, _p(out)))
        return out.reshape(self._dimensions)

    def flow(self):
        """(max-flow value, minimum energy), both int64."""
        f = ctypes.c_int64(0)
        e = ctypes.c_int64(0)
        N.check(N.lib().lf_get_flow(self._h, ctypes.byref(f), ctypes.byref(e)))
        return f.value, e.value

    def levels(self):
        out = np.empty(self.n_nodes, dtype=np.int64)
        N.check(N.lib().lf_get_levels(self._h, _p(out)))
        return out.reshape(self._dimensions)

    def levelSets(self):
        """Parametric solver: the level set of every node, numbered in the
        order ParametricFlowSolver::run returns the level sets
        (parametricflow/pf_solver.hpp:180-203)."""
        out = np.empty(self.n_nodes, dtype=np.int32)
        N.check(N.lib().lf_get_level_sets(self._h, _p(out)))
        return out.reshape(self._dimensions)

    def stats(self):
        a, b, c = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
        N.check(N.lib().lf_get_stats(self._h, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c)))
        return {"epochs": a.value, "pr_launches": b.value, "bfs_passes": c.value}


def calculate2dTV(f, lam, kernel="Full2d_4", return_levels=False, return_sets=False):
    """Single-lambda TV (tv/tv_solver.hpp:650-655) on the GPU.

    return_levels: also the final 2x-scaled values r; return_sets: also the
    level set of every pixel, numbered in the reference solver's order."""
    f = np.ascontiguousarray(f, dtype=np.float64)
    if f.ndim != 2:
        raise ValueError("calculate2dTV takes a 2-d array")
    nx, ny = f.shape
    out = np.empty((nx, ny), dtype=np.float64)
    lv = np.empty((nx, ny), dtype=np.int64)
    sets = np.empty((nx, ny), dtype=np.int32)
    N.check(N.lib().lf_tv_2d_level_sets(kernel.encode(), nx, ny, _p(f), float(lam), _p(out),
                                        _p(lv), _p(sets)))
    res = (out,)
    if return_levels:
        res += (lv,)
    if return_sets:
        res += (sets,)
    return res if len(res) > 1 else out


def calculate2dTVPath(f, lambdas, kernel="Full2d_4", return_stats=False):
    """The regularisation path (calculate2dTV with a lambda list,
    tv/tv_solver.hpp:657-681) -> array [len(lambdas), nx, ny].

    The reference's path tracker: one parametric solve at the largest
    lambda, then region segments followed down in lambda (joins, and splits
    found by region max-flow probes on the GPU); slice i is every pixel's
    segment line at lambdas[i], as the reference traces it.  These values
    are not the single-lambda solutions; for those use
    ``calculate2dTVBatch(f, lambdas)``.  Negative lambdas count as 0, as in
    the reference.  (The Cython wrappers also rescale their output,
    ``pylatticeflow.pyx:452`` by lambda and ``:482`` by a stale lambda;
    these functions return the C++ entries' values unscaled.)

    return_stats: also return {"segments", "probes", "events", "level_sets",
    "large_probes", "large_probe_s", "small_probe_s", "setup_s"}: path
    segments, region probes, events, initial level sets, probes of regions
    too large for one block and the seconds in them, in the one-block
    probes and in segment set-ups.
    """
    f = np.ascontiguousarray(f, dtype=np.float64)
    if f.ndim != 2:
        raise ValueError("calculate2dTVPath takes a 2-d array")
    lam = np.ascontiguousarray(np.atleast_1d(lambdas), dtype=np.float64)
    if lam.ndim != 1:
        raise ValueError("lambdas must be a 1-d sequence")
    nx, ny = f.shape
    out = np.empty((lam.size, nx, ny), dtype=np.float64)
    st = np.zeros(10, dtype=np.int64)
    N.check(N.lib().lf_tv_2d_path_stats(kernel.encode(), nx, ny, _p(f), lam.size, _p(lam),
                                        _p(out), _p(st)))
    if return_stats:
        return out, {"segments": int(st[0]), "probes": int(st[1]), "events": int(st[2]),
                     "level_sets": int(st[3]), "large_probes": int(st[4]),
                     "large_probe_s": st[5] * 1e-6, "small_probe_s": st[6] * 1e-6,
                     "setup_s": st[7] * 1e-6, "small_epochs": int(st[8]),
                     "small_bfs_levels": int(st[9])}
    return out


def calculate2dTVBatch(images, lambdas, kernel="Full2d_4", return_levels=False, max_nodes=0):
    """Many single-lambda TV problems of one shape solved together.

    ``images``: array [count, nx, ny] (or one [nx, ny] image shared by all
    problems); ``lambdas``: count values.  Result [count, nx, ny], slice p
    equal to ``calculate2dTV(images[p], lambdas[p])``.
    """
    f = np.ascontiguousarray(images, dtype=np.float64)
    lam = np.ascontiguousarray(np.atleast_1d(lambdas), dtype=np.float64)
    if f.ndim == 2:
        nx, ny = f.shape
        stride = 0
    elif f.ndim == 3:
        if f.shape[0] != lam.size:
            raise ValueError("one lambda per image")
        nx, ny = f.shape[1:]
        stride = nx * ny
    else:
        raise ValueError("images must be [nx, ny] or [count, nx, ny]")
    out = np.empty((lam.size, nx, ny), dtype=np.float64)
    lv = np.empty((lam.size, nx, ny), dtype=np.int64)
    N.check(N.lib().lf_tv_2d_batch(kernel.encode(), nx, ny, lam.size, _p(f), stride, _p(lam),
                                   _p(out), _p(lv), int(max_nodes)))
    return (out, lv) if return_levels else out


class LatticeBatch(object):
    """Many independent lattices solved together on the GPU (one instance pool).

    ``add(kernel, shape)`` returns the lattice's index; fill each lattice with
    ``addCapacities`` / ``addEnergyPotentials``; ``run()`` solves all of them;
    results per index.  Each lattice's result equals a plain ``LatticeFlow``
    solve of it.
    """

    def __init__(self):
        h = ctypes.c_void_p()
        N.check(N.lib().lf_batch_create(ctypes.byref(h)))
        self._h = h
        self._shapes = []
        self._edges = []

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            N.lib().lf_batch_destroy(h)
            self._h = None

    def __len__(self):
        return len(self._shapes)

    def add(self, kernel, shape):
        shape = tuple(int(v) for v in shape)
        dims = np.asarray(shape, dtype=np.uint64)
        idx = ctypes.c_int(-1)
        N.check(N.lib().lf_batch_add(self._h, kernel.encode(), len(shape), _p(dims), ctypes.byref(idx)))
        self._shapes.append(shape)
        self._edges.append(kernelInfo(kernel)[0].shape[0] // 2)
        return idx.value

    def setParam(self, name, value):
        N.check(N.lib().lf_batch_set_param(self._h, name.encode(), int(value)))

    def addCapacities(self, index, source=None, sink=None, edges=None):
        n = int(np.prod(self._shapes[index]))
        arrs = []
        for a, m in ((source, n), (sink, n), (edges, n * self._edges[index])):
            if a is None:
                arrs.append(None)
                continue
            a = np.ascontiguousarray(a, dtype=np.int32).reshape(-1)
            if a.size != m:
                raise ValueError("capacity array has the wrong size")
            arrs.append(a)
        N.check(N.lib().lf_batch_add_capacities(
            self._h, index, *[(_p(a) if a is not None else None) for a in arrs]))

    def addCapacitiesPacked(self, source=None, sink=None, edges=None):
        """Every lattice's capacities in one call: source / sink with all
        lattices' nodes back to back in index order, edges all lattices'
        filling edges back to back (lf_batch_add_capacities_packed)."""
        n = sum(int(np.prod(s)) for s in self._shapes)
        ne = sum(int(np.prod(s)) * e for s, e in zip(self._shapes, self._edges))
        arrs = []
        for a, m in ((source, n), (sink, n), (edges, ne)):
            if a is None:
                arrs.append(None)
                continue
            a = np.ascontiguousarray(a, dtype=np.int32).reshape(-1)
            if a.size != m:
                raise ValueError("packed capacity array has the wrong size")
            arrs.append(a)
        N.check(N.lib().lf_batch_add_capacities_packed(
            self._h, *[(_p(a) if a is not None else None) for a in arrs]))

    def getCutsPacked(self, maximal=False, out=None):
        """Every lattice's cut back to back in index order (one flat int32
        array; lf_batch_get_cuts_packed)."""
        n = sum(int(np.prod(s)) for s in self._shapes)
        if out is None:
            out = np.empty(n, dtype=np.int32)
        elif out.dtype != np.int32 or out.size != n or not out.flags.c_contiguous:
            raise ValueError("out must be a contiguous int32 array of the batch's node count")
        N.check(N.lib().lf_batch_get_cuts_packed(self._h, _p(out), 1 if maximal else 0))
        return out

    def flows(self):
        """(flow values, minimum energies) of every lattice, int64 arrays."""
        f = np.empty(len(self._shapes), dtype=np.int64)
        e = np.empty(len(self._shapes), dtype=np.int64)
        N.check(N.lib().lf_batch_get_flows(self._h, _p(f), _p(e)))
        return f, e

    def addEnergyPotentials(self, index, unary, binary):
        n = int(np.prod(self._shapes[index]))
        u = np.ascontiguousarray(unary, dtype=np.int64).reshape(-1)
        b = np.ascontiguousarray(binary, dtype=np.int64).reshape(-1)
        if u.size != 2 * n or b.size != 4 * n * self._edges[index]:
            raise ValueError("energy arrays do not match the lattice")
        N.check(N.lib().lf_batch_add_energy_potentials(self._h, index, _p(u), _p(b)))

    def clear(self):
        N.check(N.lib().lf_batch_clear(self._h))

    def run(self):
        N.check(N.lib().lf_batch_run(self._h))

    def runTime(self):
        return N.lib().lf_batch_run_time(self._h)

    def getCut(self, index):
        out = np.empty(int(np.prod(self._shapes[index])), dtype=np.int32)
        N.check(N.lib().lf_batch_get_cut(self._h, index, _p(out)))
        return out.reshape(self._shapes[index])

    def getCutMax(self, index):
        out = np.empty(int(np.prod(self._shapes[index])), dtype=np.int32)
        N.check(N.lib().lf_batch_get_cut_max(self._h, index, _p(out)))
        return out.reshape(self._shapes[index])

    def flow(self, index):
        f = ctypes.c_int64(0)
        e = ctypes.c_int64(0)
        N.check(N.lib().lf_batch_get_flow(self._h, index, ctypes.byref(f), ctypes.byref(e)))
        return f.value, e.value

    def stats(self):
        a, b, c = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
        N.check(N.lib().lf_batch_get_stats(self._h, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c)))
        return {"epochs": a.value, "pr_passes": b.value, "bfs_passes": c.value}


class LatticeServer(object):
    """Request server: TV-denoise and graph-cut requests admitted as they
    arrive and solved concurrently on the GPU (see ``lf_server_*``).

    ``submit_tv`` / ``submit_cut`` return a ticket at once; ``wait`` blocks
    until the request is finished and returns its latency in seconds;
    ``result`` returns the solution.  ``stats()`` gives p50 / p99 latency,
    throughput and the largest number of requests in flight together.
    TV requests of one shape waiting together are solved as one stacked
    problem (``max_group``, default 8; 1 turns grouping off).
    """

    def __init__(self, workers=4, hbm_budget_bytes=0, max_group=None):
        h = ctypes.c_void_p()
        N.check(N.lib().lf_server_create(int(workers), int(hbm_budget_bytes), ctypes.byref(h)))
        self._h = h
        self._meta = {}
        if max_group is not None:
            N.check(N.lib().lf_server_set_max_group(h, int(max_group)))

    def close(self):
        h = getattr(self, "_h", None)
        if h:
            N.lib().lf_server_destroy(h)
            self._h = None

    def __del__(self):
        self.close()

    def submit_tv(self, f, lam, kernel="Full2d_4"):
        f = np.ascontiguousarray(f, dtype=np.float64)
        t = ctypes.c_int64(0)
        N.check(N.lib().lf_server_submit_tv(self._h, kernel.encode(), f.shape[0], f.shape[1],
                                            _p(f), float(lam), ctypes.byref(t)))
        self._meta[t.value] = ("tv", f.shape)
        return t.value

    def submit_cut(self, kernel, shape, source, sink, edges):
        s = np.ascontiguousarray(source, dtype=np.int32).reshape(-1)
        k = np.ascontiguousarray(sink, dtype=np.int32).reshape(-1)
        e = np.ascontiguousarray(edges, dtype=np.int32).reshape(-1)
        t = ctypes.c_int64(0)
        N.check(N.lib().lf_server_submit_cut(self._h, kernel.encode(), shape[0], shape[1], _p(s),
                                             _p(k), _p(e), ctypes.byref(t)))
        self._meta[t.value] = ("cut", tuple(shape))
        return t.value

    def wait(self, ticket, timeout=600.0):
        lat = ctypes.c_double(0)
        N.check(N.lib().lf_server_wait(self._h, ctypes.c_int64(ticket), float(timeout),
                                       ctypes.byref(lat)))
        return lat.value

    def result(self, ticket):
        kind, shape = self._meta[ticket]
        if kind == "tv":
            out = np.empty(shape, dtype=np.float64)
            lv = np.empty(shape, dtype=np.int64)
            N.check(N.lib().lf_server_get_tv(self._h, ctypes.c_int64(ticket), _p(out), _p(lv)))
            return out, lv
        cut = np.empty(shape, dtype=np.int32)
        f = ctypes.c_int64(0)
        e = ctypes.c_int64(0)
        N.check(N.lib().lf_server_get_cut(self._h, ctypes.c_int64(ticket), _p(cut), ctypes.byref(f),
                                          ctypes.byref(e)))
        return cut, (f.value, e.value)

    def release(self, ticket):
        N.check(N.lib().lf_server_release(self._h, ctypes.c_int64(ticket)))
        self._meta.pop(ticket, None)

    def cancel(self, ticket):
        """Drop a request still waiting in the queue (its wait then raises
        LF_ERR_STATE); raises LF_ERR_STATE once it has been admitted."""
        N.check(N.lib().lf_server_cancel(self._h, ctypes.c_int64(ticket)))

    def inject_alloc_failures(self, count):
        """Fault injection on the host: the next `count` engine creations fail
        as a failed device allocation would (the request gets LF_ERR_OOM)."""
        N.check(N.lib().lf_server_inject_alloc_failures(self._h, int(count)))

    def stats(self):
        p50, p99, sps = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        c, m = ctypes.c_int64(), ctypes.c_int64()
        N.check(N.lib().lf_server_stats(self._h, ctypes.byref(p50), ctypes.byref(p99),
                                        ctypes.byref(sps), ctypes.byref(c), ctypes.byref(m)))
        g, gr = ctypes.c_int64(), ctypes.c_int64()
        N.check(N.lib().lf_server_group_stats(self._h, ctypes.byref(g), ctypes.byref(gr)))
        return {"p50_ms": p50.value, "p99_ms": p99.value, "solves_per_s": sps.value,
                "completed": c.value, "max_in_flight": m.value, "groups": g.value,
                "grouped_requests": gr.value}
