"""The C-ABI boundary on CPU: library loads, exports every declared symbol,
and the kernel registry / name validation need no GPU."""
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "latticeflow_gpu.h")


def declared_symbols():
    txt = open(HEADER).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(lf_[a-z0-9_]+)\s*\(", txt)))


def test_exports_every_declared_symbol(native):
    syms = declared_symbols()
    assert len(syms) >= 20
    for s in syms:
        assert hasattr(native, s), s


def test_binding_covers_header(native):
    from latticeflow_gb300 import _native
    assert sorted(_native.PROTOTYPES) == declared_symbols()


def test_registry_matches_oracle(native, oracle_port):
    import latticeflow_gb300 as lf
    O = oracle_port
    names = lf.validKernelNames()
    assert set(names) == set(O.registry_specs())
    for k in names:
        d, w, g = lf.kernelInfo(k)
        od, ow = O.lattice_offsets(k)
        assert np.array_equal(d, od) and np.array_equal(w, ow) and g == O.registry_specs()[k].geocut
        assert lf.kernelDimension(k) == O.registry_specs()[k].dim


def test_registry_matches_compiled_reference_deltas(native, oracle_port):
    O = oracle_port
    if not O.ref_available():
        pytest.skip("compiled reference not present")
    import latticeflow_gb300 as lf
    names = lf.validKernelNames()
    assert len(names) == 27  # the 20 of the default build and the 7 of the opt-in 1-d build
    for k in names:  # every name, aliases included (the compiled reference holds them all)
        dims = {1: (12,), 2: (9, 8), 3: (5, 6, 7)}[lf.kernelDimension(k)]
        d, _, _ = lf.kernelInfo(k)
        fd = O.ref_filling_deltas(k, dims)
        assert np.array_equal(fd, d[: len(d) // 2]), k


def test_names_validation(native):
    import latticeflow_gb300 as lf
    assert lf.isValidSolver("LatticeEnergyMinimizer")
    assert lf.isValidSolver("LatticeLevelReductions")
    assert not lf.isValidSolver("NoSuchSolver")
    assert lf.isValidKernel("Full2d_8") and not lf.isValidKernel("Full2d_5")
    with pytest.raises(lf.BadSolverOrKernelName):
        lf.kernelDimension("Full2d_5")
    with pytest.raises(ValueError):
        lf.LatticeFlow("Full2d_4", "NoSuchSolver", (4, 4))
    with pytest.raises(ValueError):
        lf.LatticeFlow("Full2d_4", "LatticeEnergyMinimizer", (4, 4, 4))


def test_no_cpu_fallback_in_package():
    """The product (package, native sources, C headers) never imports, loads
    or links anything of the oracle: no Python import of it, and no path to
    its libraries or sources in any product file, comments and docstrings
    aside."""
    roots = [os.path.join(ROOT, "latticeflow_gb300"), os.path.join(ROOT, "include")]
    bad = re.compile(r"\boracle\b|liblf_oracle|libref_oracle|lf_oracle\.cpp|lfo_\w+\(")
    for top in roots:
        for dirpath, _, files in os.walk(top):
            for f in files:
                path = os.path.join(dirpath, f)
                if f.endswith(".py"):
                    txt = re.sub(r'"""(.|\n)*?"""', "", open(path).read())
                    txt = "\n".join(l.split("#", 1)[0] for l in txt.splitlines())
                elif f.endswith((".cu", ".cuh", ".cpp", ".h", ".hpp")):
                    txt = re.sub(r"/\*(.|\n)*?\*/", "", open(path).read())
                    txt = "\n".join(l.split("//", 1)[0] for l in txt.splitlines())
                else:
                    continue
                m = bad.search(txt)
                assert m is None, (path, m.group(0) if m else None)
