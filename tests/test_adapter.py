"""The C++ adapter: it compiles against the reference's own interface.hpp and
links against the C ABI (CPU, where the reference's sources are), and it runs
on the GPU through the interface's virtual calls (GPU test)."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = os.environ.get("LATTICEFLOW_REFERENCE_SOLVER", "/root/reference/solver")


def test_adapter_compiles_against_reference_interface(native, tmp_path):
    if not os.path.isdir(REF):
        pytest.skip("reference sources not present")
    src = tmp_path / "use.cpp"
    src.write_text(
        '#include "latticeflow_gpu_interface.hpp"\n'
        "int main() {\n"
        "  size_t dims[2] = {4, 5};\n"
        "  latticeQBP::solver_ptr s;\n"
        "  if (dims[0] == 99) s = latticeQBP::getGPULatticeFlowInterface(\"LatticeEnergyMinimizer\", \"Full2d_4\", dims);\n"
        "  return s ? 1 : 0;\n"
        "}\n")
    exe = tmp_path / "use"
    lib = os.path.join(ROOT, "latticeflow_gb300", "_lib")
    cmd = ["g++", "-std=c++14", "-DNDEBUG", "-include", "numeric", "-w",
           "-I" + os.path.join(ROOT, "include"), "-I" + os.path.join(ROOT, "oracle", "shim"),
           "-I" + REF, str(src), "-L" + lib, "-llatticeflow_gpu", "-Wl,-rpath," + lib, "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]


@pytest.mark.gpu
def test_adapter_runs_on_gpu(native, gpu, tmp_path):
    """The adapter driven through the abstract interface's virtual calls on the
    GPU (factory with its BadSolverOrKernelName, metadata, addEnergyPotentials,
    run, getCut), against the compiled reference's BK labelling of a golden
    fixture.  Compiled against a test-only declaration of the interface
    (tests/native/interface_decl), as the reference's sources are absent on
    the GPU host."""
    import numpy as np
    z = np.load(os.path.join(ROOT, "tests", "golden", "cut_f8_seg.npz"))
    dims = tuple(int(v) for v in z["dims"])
    (tmp_path / "u.bin").write_bytes(np.ascontiguousarray(z["unary"], dtype=np.int64).tobytes())
    (tmp_path / "b.bin").write_bytes(np.ascontiguousarray(z["binary"], dtype=np.int64).tobytes())
    exe = tmp_path / "adapter_run"
    lib = os.path.join(ROOT, "latticeflow_gb300", "_lib")
    cmd = ["g++", "-std=c++14", "-O2", "-I" + os.path.join(ROOT, "include"),
           "-I" + os.path.join(ROOT, "tests", "native", "interface_decl"),
           os.path.join(ROOT, "tests", "native", "adapter_run.cpp"), "-L" + lib,
           "-llatticeflow_gpu", "-Wl,-rpath," + lib, "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    r = subprocess.run([str(exe), str(z["kernel"]), str(dims[0]), str(dims[1]),
                        str(tmp_path / "u.bin"), str(tmp_path / "b.bin"), str(tmp_path / "cut.bin")],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    cut = np.frombuffer((tmp_path / "cut.bin").read_bytes(), dtype=np.int32).reshape(dims)
    assert np.array_equal(cut, z["bk_cut"])
