"""The allocation-free cut entry point (lf_cut_2d_noalloc), checked against the
regular entry points and the oracle.

Callers that may not allocate device memory while they run (code inside
another framework's memory budget, hosts that forbid allocation after
start-up, plugins whose host owns every allocation) pass their own device
buffers; the solve keeps its intermediate state in a static device array.
This file is collected last so that a run stopping at the first failure has
already run every other test.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


def _call(lib, kernel, shape, src, snk, edge, cut, fe, stream):
    return lib.lf_cut_2d_noalloc(kernel.encode(), shape[0], shape[1], _ptr(src), _ptr(snk),
                                 _ptr(edge), _ptr(cut), _ptr(fe), ctypes.c_void_p(stream))


def test_no_alloc_cut_matches_regular_entry_point(native, gpu, oracle_port):
    import torch

    import latticeflow_gb300 as lf
    from latticeflow_gb300 import _native as N
    from latticeflow_gb300 import workloads as W
    lib = N.lib()
    stream = torch.cuda.current_stream().cuda_stream
    cases = [(11, "Full2d_4", (200, 181)), (12, "Full2d_8", (256, 256)), (13, "Full2d_8", (37, 250))]
    for seed, kernel, shape in cases:
        p = W.plain_cut(seed, shape, kernel)
        L = lf.LatticeFlow(kernel, "LatticeEnergyMinimizer", shape)
        L.addCapacities(p.source, p.sink, p.edge)
        L.run()
        want_cut, want_flow = L.getCut(), L.flow()
        u, b = p.energies()
        E, cmin, _, _, _ = oracle_port.port_canonical(kernel, shape, u, b)
        assert want_flow[1] == E and np.array_equal(want_cut, cmin)
        src = torch.from_numpy(np.ascontiguousarray(p.source)).cuda()
        snk = torch.from_numpy(np.ascontiguousarray(p.sink)).cuda()
        edge = torch.from_numpy(np.ascontiguousarray(p.edge.reshape(-1))).cuda()
        torch.cuda.synchronize()
        # two calls in a row on the same inputs: the shared scratch must not leak state
        for _ in range(2):
            cut = torch.full((p.n,), -1, dtype=torch.int32, device="cuda")
            fe = torch.zeros(2, dtype=torch.int64, device="cuda")
            rc = _call(lib, kernel, shape, src, snk, edge, cut, fe, stream)
            assert rc == 0, N.last_error()
            assert np.array_equal(cut.cpu().numpy().reshape(shape), want_cut)
            assert tuple(int(v) for v in fe.cpu().tolist()) == want_flow


def test_no_alloc_allocates_nothing(native, gpu):
    """A warm call changes neither torch's allocator counters nor the device's
    free memory (any device allocation takes at least one 2 MiB page)."""
    import torch

    from latticeflow_gb300 import _native as N
    from latticeflow_gb300 import workloads as W
    lib = N.lib()
    stream = torch.cuda.current_stream().cuda_stream
    shape, kernel = (128, 96), "Full2d_8"
    p = W.plain_cut(21, shape, kernel)
    src = torch.from_numpy(np.ascontiguousarray(p.source)).cuda()
    snk = torch.from_numpy(np.ascontiguousarray(p.sink)).cuda()
    edge = torch.from_numpy(np.ascontiguousarray(p.edge.reshape(-1))).cuda()
    cut = torch.zeros(p.n, dtype=torch.int32, device="cuda")
    fe = torch.zeros(2, dtype=torch.int64, device="cuda")
    assert _call(lib, kernel, shape, src, snk, edge, cut, fe, stream) == 0, N.last_error()
    torch.cuda.synchronize()
    alloc0, reserved0 = torch.cuda.memory_allocated(), torch.cuda.memory_reserved()
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(3):
        assert _call(lib, kernel, shape, src, snk, edge, cut, fe, stream) == 0, N.last_error()
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert torch.cuda.memory_allocated() == alloc0
    assert torch.cuda.memory_reserved() == reserved0
    assert free1 == free0, (free0, free1)


def test_no_alloc_rejects_oversize_and_bad_kernel(native, gpu):
    import torch

    from latticeflow_gb300 import _native as N
    lib = N.lib()
    buf = torch.zeros(300 * 300 * 4, dtype=torch.int32, device="cuda")
    fe = torch.zeros(2, dtype=torch.int64, device="cuda")
    rc = lib.lf_cut_2d_noalloc(b"Full2d_4", 300, 300, _ptr(buf), _ptr(buf), _ptr(buf), _ptr(buf),
                               _ptr(fe), None)
    assert rc == N.LF_ERR_RANGE and "at most 65536" in N.last_error()
    rc = lib.lf_cut_2d_noalloc(b"Full3d_6", 4, 4, _ptr(buf), _ptr(buf), _ptr(buf), _ptr(buf),
                               _ptr(fe), None)
    assert rc == N.LF_ERR_SHAPE


def test_no_alloc_range_errors_then_recovers(native, gpu):
    """A negative capacity and a capacity sum past the 32-bit range return
    LF_ERR_RANGE; the next call on valid inputs is still exact."""
    import torch

    from latticeflow_gb300 import _native as N
    from latticeflow_gb300 import workloads as W
    lib = N.lib()
    stream = torch.cuda.current_stream().cuda_stream
    shape, kernel = (64, 48), "Full2d_4"
    p = W.plain_cut(31, shape, kernel)
    cut = torch.zeros(p.n, dtype=torch.int32, device="cuda")
    fe = torch.zeros(2, dtype=torch.int64, device="cuda")
    edge = torch.from_numpy(np.ascontiguousarray(p.edge.reshape(-1))).cuda()
    bad = p.source.copy()
    bad[5] = -3
    src = torch.from_numpy(bad).cuda()
    snk = torch.from_numpy(np.ascontiguousarray(p.sink)).cuda()
    rc = _call(lib, kernel, shape, src, snk, edge, cut, fe, stream)
    assert rc == N.LF_ERR_RANGE and "non-negative" in N.last_error()
    big = np.full(p.n, 2 ** 30, dtype=np.int32)  # one node: 2^30 + 4 edges > INT_MAX
    rc = _call(lib, kernel, shape, torch.from_numpy(big).cuda(), snk,
               torch.from_numpy(np.full(p.edge.size, 2 ** 30, dtype=np.int32)).cuda(), cut, fe,
               stream)
    assert rc == N.LF_ERR_RANGE and "32-bit" in N.last_error()
    src = torch.from_numpy(np.ascontiguousarray(p.source)).cuda()
    rc = _call(lib, kernel, shape, src, snk, edge, cut, fe, stream)
    assert rc == 0, N.last_error()
    import latticeflow_gb300 as lf
    L = lf.LatticeFlow(kernel, "LatticeEnergyMinimizer", shape)
    L.addCapacities(p.source, p.sink, p.edge)
    L.run()
    assert np.array_equal(cut.cpu().numpy().reshape(shape), L.getCut())
    assert tuple(int(v) for v in fe.cpu().tolist()) == L.flow()
