"""Build recipe for the CPU oracle (test infrastructure only).

Compiles oracle/eb_oracle.c into oracle/_build/libeb_oracle.so with gcc, without
fused multiply-add contraction (-ffp-contract=off), so that the x86 and Arm builds round
alike (gcc contracts a*b+c on Arm by default). The reference itself is Fortran 77 and no Fortran compiler exists on either machine,
so there is no oracle/_ref build of the reference sources.
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libeb_oracle.so")


def build(force=False):
    src = os.path.join(HERE, "eb_oracle.c")
    hdr = os.path.join(HERE, "eb_oracle.h")
    if (not force and os.path.exists(LIB)
            and os.path.getmtime(LIB) >= max(os.path.getmtime(src), os.path.getmtime(hdr))):
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    tmp = LIB + ".tmp%d" % os.getpid()
    cmd = ["gcc", "-O3", "-std=gnu11", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
           "-fcx-fortran-rules", "-o", tmp, src, "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
