"""Writes the kernel header the compiled reference oracle needs.

TEST INFRASTRUCTURE ONLY.  The reference's solver/kernels/kernels.hpp is
generated at configure time and absent from the checkout; this script writes
an equivalent header from oracle/kernels.py (one KernelBase<d, K, geocut>
struct per kernel in the form of install/templates/kernels/code.hpp, aliases as
typedefs in the form of install/templates/kernels/duplicate_code.hpp).

usage: python oracle/gen_ref_kernels.py OUT_DIR   (writes OUT_DIR/kernels/kernels.hpp)
"""
import os
import sys

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
import kernels  # noqa: E402


def main(out_dir):
    specs = kernels.generate(optional=True)  # the default build plus --1d and --4d
    body = []
    for name, s in specs.items():
        if s.alias_of:
            body.append("typedef %s %s;" % (s.alias_of, name))
            continue
        edges = ",".join("{" + ",".join(str(v) for v in o) + "}" for o in s.offsets)
        w = ", ".join(("%1.16f" % x) if x != 1 else "1.0" for x in s.weights)
        g = 1 if s.geocut else 0
        body.append(
            "struct %s : public KernelBase<%d, %d, %d> {\n"
            "  %s() : KernelBase<%d, %d, %d>({%s}, {%s}) {}\n};"
            % (name, s.dim, s.size, g, name, s.dim, s.size, g, edges, w))
    d = os.path.join(out_dir, "kernels")
    os.makedirs(d, exist_ok=True)
    with open(os.path.join(d, "kernels.hpp"), "w") as f:
        f.write("// generated by oracle/gen_ref_kernels.py (oracle build only)\n")
        f.write("#ifndef _KERNELS_H_\n#define _KERNELS_H_\n#define MAX_KERNEL_DIMENSION 4\n")
        f.write('#include "kernels/kernel_base.hpp"\nnamespace latticeQBP {\n')
        f.write("\n".join(body))
        f.write("\n}\n#endif\n")


if __name__ == "__main__":
    main(sys.argv[1])
