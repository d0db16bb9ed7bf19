"""The compile-time stencils of the staged passes equal the registry's
lattice order, on the CPU.

The staged 2-d passes (lf_pool_pr2d.cuh, Stencil2d) and 3-d passes
(lf_pool_pr3d.cuh, Stencil3d) carry their neighbourhoods as packed
constants; a launcher only takes a lattice whose stencil matches the
table, so a wrong table would silently send every lattice to the generic
passes.  Each packed field holds offset + 1 in two bits per direction."""
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "latticeflow_gb300", "csrc")


def _tables(path, struct):
    txt = open(os.path.join(CSRC, path)).read()
    out = {}
    for m in re.finditer(r"template <> struct %s<(\d+)> \{(.*?)\};" % struct, txt, flags=re.S):
        K = int(m.group(1))
        fields = dict((n, int(v, 16)) for n, v in re.findall(r"(kD[ABC])\s*=\s*(0x[0-9a-fA-F]+|[0-9]+)", m.group(2)))
        # 2-d tables write the fields as or-ed shifts of disjoint bits: sum them
        if not fields:
            for n, expr in re.findall(r"(kD[BC])\s*=\s*(.*?);", m.group(2), flags=re.S):
                fields[n] = sum(int(v) << int(sh) for v, sh in re.findall(r"\((\d+)u << (\d+)\)", expr))
        out[K] = fields
    return out


def _decode(v, K):
    return [int((v >> (2 * k)) & 3) - 1 for k in range(K)]


@pytest.mark.parametrize("kernel", ["Full3d_6", "Full3d_18", "Full3d_26"])
def test_stencil3d_tables(native, kernel):
    import latticeflow_gb300 as lf
    d, _, _ = lf.kernelInfo(kernel)
    K = d.shape[0]
    t = _tables("lf_pool_pr3d.cuh", "Stencil3d")[K]
    got = np.stack([_decode(t["kDA"], K), _decode(t["kDB"], K), _decode(t["kDC"], K)], axis=1)
    assert np.array_equal(got, np.asarray(d)), kernel
    # entry k + K/2 is the reverse of entry k
    assert np.array_equal(got[K // 2:], -got[:K // 2])


@pytest.mark.parametrize("kernel", ["Full2d_4", "Full2d_8"])
def test_stencil2d_tables(native, kernel):
    import latticeflow_gb300 as lf
    d, _, _ = lf.kernelInfo(kernel)
    K = d.shape[0]
    t = _tables("lf_pool_pr2d.cuh", "Stencil2d")[K]
    got = np.stack([_decode(t["kDB"], K), _decode(t["kDC"], K)], axis=1)
    assert np.array_equal(got, np.asarray(d)), kernel
