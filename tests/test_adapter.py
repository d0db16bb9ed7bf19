"""The C++ adapter compiles against the reference's own interface.hpp and links
against the C ABI (CPU only: nothing is run)."""
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
