"""Python access to the oracles.  TEST INFRASTRUCTURE ONLY.

Two oracles live here, both CPU:

* the *port* (``oracle/lf_oracle.cpp`` -> ``oracle/liblf_oracle.so``): a
  step-for-step restatement of the reference push-relabel, parametric flow and
  single-lambda TV solver.  It is available wherever g++ is (including the
  GPU host) and is what the GPU tests compare against.
* the *compiled reference* (``oracle/_ref/libref_oracle.so``): the unmodified
  reference headers built by ``oracle/Makefile`` with small shims.  It exists
  only where the reference sources exist; it pins the port.

Only tests, the smoke check and the benchmark's CPU-baseline leg use this
module.
"""
import ctypes
import os
import subprocess

import numpy as np

from . import kernels as _kernels

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_SO = os.path.join(HERE, "liblf_oracle.so")
REF_SO = os.path.join(HERE, "_ref", "libref_oracle.so")
REF_SRC = os.environ.get("LATTICEFLOW_REFERENCE_SOLVER", "/root/reference/solver")

_SPECS = None
_ALL_SPECS = None
_port = None
_ref = None


def specs():
    global _SPECS
    if _SPECS is None:
        _SPECS = _kernels.generate()
    return _SPECS


def registry_specs():
    """The kernels the GPU registry serves: the reference's default build plus
    its opt-in 1-d kernels (the opt-in 4-d kernel is not served)."""
    return {k: v for k, v in all_specs().items() if v.dim <= 3}


def all_specs():
    """specs() plus the kernels of the reference's opt-in 1-d and 4-d builds."""
    global _ALL_SPECS
    if _ALL_SPECS is None:
        _ALL_SPECS = _kernels.generate(optional=True)
    return _ALL_SPECS


def lattice_offsets(kernel):
    """(offsets[K][nd], weights[K]) in lattice order (kernellattice.hpp:61-96)."""
    s = all_specs()[kernel]
    offs, w = s.lattice_order()
    return np.asarray(offs, dtype=np.int32), np.asarray(w, dtype=np.float64)


def build_port():
    subprocess.run(["make", "-s", "-C", HERE, "port"], check=True)


def build_ref():
    """Builds the compiled-reference oracle; returns False without sources."""
    if not os.path.isdir(REF_SRC):
        return False
    jobs = "-j%d" % max(1, min(5, os.cpu_count() or 1))  # the five parts of the driver at once
    subprocess.run(["make", "-s", jobs, "-C", HERE, "ref", "REF=" + REF_SRC], check=True)
    return True


def port():
    global _port
    if _port is None:
        if not os.path.exists(PORT_SO):
            build_port()
        lib = ctypes.CDLL(PORT_SO)
        P = ctypes.c_void_p
        lib.lfo_pr_solve.argtypes = [ctypes.c_int, P, ctypes.c_int, P, P, P, P, P]
        lib.lfo_pr_canonical.argtypes = [ctypes.c_int, P, ctypes.c_int, P, P, P, P, P, P, P]
        lib.lfo_pf_solve.argtypes = [ctypes.c_int, P, ctypes.c_int, P, P, P, P, P, P, P]
        lib.lfo_tv_single.argtypes = [ctypes.c_int64, ctypes.c_int64, ctypes.c_int, P, P, P,
                                      ctypes.c_double, P, P, P, P]
        lib.lfo_tv_path.argtypes = [ctypes.c_int64, ctypes.c_int64, ctypes.c_int, P, P, P,
                                    ctypes.c_int64, P, P, P, P]
        lib.lfo_tv_path.restype = ctypes.c_int
        _port = lib
    return _port


def ref_available():
    return os.path.exists(REF_SO)


def ref():
    global _ref
    if _ref is None:
        lib = ctypes.CDLL(REF_SO)
        P = ctypes.c_void_p
        lib.ref_solve.argtypes = [ctypes.c_char_p, ctypes.c_char_p, P, P, P, P, P, P, P]
        lib.ref_solve.restype = ctypes.c_int
        lib.ref_tv_single.argtypes = [ctypes.c_char_p, ctypes.c_size_t, ctypes.c_size_t, P,
                                      ctypes.c_double, P, P]
        lib.ref_tv_path.argtypes = [ctypes.c_char_p, ctypes.c_size_t, ctypes.c_size_t, P,
                                    ctypes.c_int, P, P, P]
        _ref = lib
    return _ref


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p) if a is not None else None


# ------------------------------------------------------------------ helpers

def energy(kernel, dims, unary, binary, labels):
    """E(labels) in int64 (interface.hpp:49-60 layout; in-bounds edges only)."""
    offs, _ = lattice_offsets(kernel)
    K = len(offs)
    nd = len(dims)
    x = np.asarray(labels).reshape(-1).astype(np.int64)
    N = int(np.prod(dims))
    u = np.asarray(unary, dtype=np.int64).reshape(N, 2)
    b = np.asarray(binary, dtype=np.int64).reshape(N, K // 2, 4)
    E = int(np.where(x == 1, u[:, 1], u[:, 0]).sum())
    coords = np.indices(dims).reshape(nd, -1)
    xs = x.reshape(dims)
    for e in range(K // 2):
        d = offs[e]
        c2 = coords + d[:, None]
        ok = np.all((c2 >= 0) & (c2 < np.asarray(dims)[:, None]), axis=0)
        idx1 = np.nonzero(ok)[0]
        x1 = x[idx1]
        x2 = xs[tuple(c2[:, idx1])]
        E += int(b[idx1, e, :][np.arange(len(idx1)), 2 * x1 + x2].sum())
    return E


def flip_problem(kernel, unary, binary):
    """The problem E'(x) = E(1 - x): its maximal on-set is the complement of
    the minimal on-set of E."""
    u = np.asarray(unary, dtype=np.int64).reshape(-1, 2)[:, ::-1]
    b = np.asarray(binary, dtype=np.int64).reshape(-1, 4)[:, ::-1]
    return np.ascontiguousarray(u), np.ascontiguousarray(b)


def port_pr(kernel, dims, unary, binary):
    """Reference push-relabel restated: returns (maximal on-set cut, seconds)."""
    lib = port()
    offs, _ = lattice_offsets(kernel)
    d = np.asarray(dims, dtype=np.int64)
    u = np.ascontiguousarray(unary, dtype=np.int64)
    b = np.ascontiguousarray(binary, dtype=np.int64)
    N = int(np.prod(dims))
    cut = np.zeros(N, dtype=np.int32)
    t = ctypes.c_double(0)
    lib.lfo_pr_solve(len(dims), _ptr(d), len(offs), _ptr(np.ascontiguousarray(offs)),
                     _ptr(u), _ptr(b), _ptr(cut), ctypes.byref(t))
    return cut.reshape(dims), t.value


def port_canonical(kernel, dims, unary, binary):
    """(energy, minimal on-set, maximal on-set, reference labelling, seconds).

    The minimal on-set is the forward residual closure of the excess nodes
    and the maximal on-set the complement of the backward closure of the
    deficit nodes, both read off the restated solver's final state.
    """
    lib = port()
    offs, _ = lattice_offsets(kernel)
    d = np.asarray(dims, dtype=np.int64)
    u = np.ascontiguousarray(unary, dtype=np.int64)
    b = np.ascontiguousarray(binary, dtype=np.int64)
    N = int(np.prod(dims))
    cpr = np.zeros(N, dtype=np.int32)
    cmin = np.zeros(N, dtype=np.int32)
    cmax = np.zeros(N, dtype=np.int32)
    t = ctypes.c_double(0)
    lib.lfo_pr_canonical(len(dims), _ptr(d), len(offs), _ptr(np.ascontiguousarray(offs)),
                         _ptr(u), _ptr(b), _ptr(cpr), _ptr(cmin), _ptr(cmax), ctypes.byref(t))
    E = energy(kernel, dims, unary, binary, cmin)
    return E, cmin.reshape(dims), cmax.reshape(dims), cpr.reshape(dims), t.value


def port_pf(kernel, dims, unary, binary, return_sets=False):
    """Restated parametric flow: (final r, reduction < 0 cut, seconds) and,
    with return_sets, the level set of every node in the reference's order."""
    lib = port()
    offs, _ = lattice_offsets(kernel)
    d = np.asarray(dims, dtype=np.int64)
    u = np.ascontiguousarray(unary, dtype=np.int64)
    b = np.ascontiguousarray(binary, dtype=np.int64)
    N = int(np.prod(dims))
    r = np.zeros(N, dtype=np.int64)
    cut = np.zeros(N, dtype=np.int32)
    sets = np.zeros(N, dtype=np.int32)
    t = ctypes.c_double(0)
    lib.lfo_pf_solve(len(dims), _ptr(d), len(offs), _ptr(np.ascontiguousarray(offs)),
                     _ptr(u), _ptr(b), _ptr(r), _ptr(cut), ctypes.byref(t), _ptr(sets))
    if return_sets:
        return r.reshape(dims), cut.reshape(dims), t.value, sets.reshape(dims)
    return r.reshape(dims), cut.reshape(dims), t.value


def port_tv_single(kernel, f, lam, return_sets=False):
    """Restated single-lambda TV: (out, raw r, seconds) and, with
    return_sets, the level set of every node in the reference's order."""
    lib = port()
    offs, w = lattice_offsets(kernel)
    f = np.ascontiguousarray(f, dtype=np.float64)
    nx, ny = f.shape
    out = np.zeros((nx, ny), dtype=np.float64)
    r = np.zeros((nx, ny), dtype=np.int64)
    sets = np.zeros((nx, ny), dtype=np.int32)
    t = ctypes.c_double(0)
    lib.lfo_tv_single(nx, ny, len(offs), _ptr(np.ascontiguousarray(offs)),
                      _ptr(np.ascontiguousarray(w)), _ptr(f), float(lam), _ptr(out), _ptr(r),
                      ctypes.byref(t), _ptr(sets))
    if return_sets:
        return out, r, t.value, sets
    return out, r, t.value


def port_tv_path(kernel, f, lams):
    """The reference's regularisation path restated (tv_solver.hpp:657-681):
    (out[n_lambda][nx][ny], seconds, segments).  Raises ValueError when the
    path tracker reports an error code."""
    lib = port()
    offs, w = lattice_offsets(kernel)
    f = np.ascontiguousarray(f, dtype=np.float64)
    nx, ny = f.shape
    lams = np.ascontiguousarray(lams, dtype=np.float64).reshape(-1)
    out = np.zeros((len(lams), nx, ny), dtype=np.float64)
    t = ctypes.c_double(0)
    st = np.zeros(2, dtype=np.int64)
    rc = lib.lfo_tv_path(nx, ny, len(offs), _ptr(np.ascontiguousarray(offs)),
                         _ptr(np.ascontiguousarray(w)), _ptr(f), len(lams), _ptr(lams), _ptr(out),
                         ctypes.byref(t), _ptr(st))
    if rc != 0:
        raise ValueError("port TV path failed: %d" % rc)
    return out, t.value, int(st[0])


def ref_solve(solver, kernel, dims, unary, binary):
    lib = ref()
    d = np.asarray(dims, dtype=np.uint64)
    u = np.ascontiguousarray(unary, dtype=np.int64)
    b = np.ascontiguousarray(binary, dtype=np.int64)
    N = int(np.prod(dims))
    cut = np.zeros(N, dtype=np.int32)
    w = ctypes.c_double(0)
    c = ctypes.c_double(0)
    rc = lib.ref_solve(solver.encode(), kernel.encode(), _ptr(d), _ptr(u), _ptr(b), _ptr(cut),
                       ctypes.byref(w), ctypes.byref(c), None)
    if rc < 0:
        raise ValueError("reference oracle has no %s:%s" % (solver, kernel))
    return cut.reshape(dims), w.value


def ref_filling_deltas(kernel, dims):
    lib = ref()
    d = np.asarray(dims, dtype=np.uint64)
    K = lattice_offsets(kernel)[0].shape[0]
    out = np.zeros((K // 2) * len(dims), dtype=np.int32)
    rc = lib.ref_solve(b"LatticeEnergyMinimizer", kernel.encode(), _ptr(d), None, None, None,
                       None, None, _ptr(out))
    if rc < 0:
        raise ValueError(kernel)
    return out.reshape(K // 2, len(dims))


def ref_tv_single(kernel, f, lam):
    lib = ref()
    f = np.ascontiguousarray(f, dtype=np.float64)
    nx, ny = f.shape
    out = np.zeros((nx, ny), dtype=np.float64)
    w = ctypes.c_double(0)
    rc = lib.ref_tv_single(kernel.encode(), nx, ny, _ptr(f), float(lam), _ptr(out), ctypes.byref(w))
    if rc < 0:
        raise ValueError(kernel)
    return out, w.value


def ref_tv_path(kernel, f, lams):
    lib = ref()
    f = np.ascontiguousarray(f, dtype=np.float64)
    nx, ny = f.shape
    lams = np.ascontiguousarray(lams, dtype=np.float64)
    out = np.zeros((len(lams), nx, ny), dtype=np.float64)
    w = ctypes.c_double(0)
    rc = lib.ref_tv_path(kernel.encode(), nx, ny, _ptr(f), len(lams), _ptr(lams), _ptr(out),
                         ctypes.byref(w))
    if rc < 0:
        raise ValueError(kernel)
    return out, w.value
