"""Build recipe for the CPU oracle (test infrastructure): liboracle.so.

The reference itself cannot be compiled here (it needs MADNESS, Boost, BTAS,
BLAS++ and MPI), so there is no oracle/_ref build; this compiles only the
C++ restatement in oracle.cpp.
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))


def build(force: bool = False) -> str:
    src = os.path.join(HERE, "oracle.cpp")
    out = os.path.join(HERE, "liboracle.so")
    if (not force and os.path.exists(out)
            and os.path.getmtime(out) >= os.path.getmtime(src)
            and os.path.getmtime(out) >= os.path.getmtime(os.path.join(HERE, "oracle.h"))):
        return out
    tmp = out + ".tmp"
    cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-pthread",
           "-ffp-contract=off", "-fno-fast-math", src, "-o", tmp]
    subprocess.run(cmd, check=True)
    os.replace(tmp, out)
    return out


if __name__ == "__main__":
    print(build(force=True))
