"""Build a program from a driver source and the GPU drop-in of the MCState
module (jmmonedmc_gb300/dropin/jmmMCState.cpp), linked to libjmmgpu.so.

    python -m jmmonedmc_gb300.dropin.build_dropin OUT DRIVER.cpp [more.cpp ...] [-I dir ...]

With the reference's own src/Main.cpp and src/readInput.cpp as the driver
sources (and -I pointing at the reference's src for its headers) this gives
the reference's program with the move loop on the GPU.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.dirname(HERE)
REPO = os.path.dirname(PKG)
LIBDIR = os.path.join(PKG, "_lib")


def build(out, sources, includes=(), extra=()):
    cmd = ["g++", "-O2", "-std=c++17", "-fopenmp", "-w", "-fpermissive",
           "-DVERSION=\"jmm-gpu-dropin\""]
    for inc in includes:
        cmd += ["-I", inc]
    cmd += ["-I", HERE, "-I", os.path.join(REPO, "include")]
    cmd += ["-o", out, *sources, os.path.join(HERE, "jmmMCState.cpp"),
            "-L", LIBDIR, "-ljmmgpu", f"-Wl,-rpath,{LIBDIR}", *extra]
    subprocess.run(cmd, check=True)
    return out


if __name__ == "__main__":
    args = sys.argv[1:]
    incs = [args[i + 1] for i, a in enumerate(args) if a == "-I"]
    rest = [a for i, a in enumerate(args) if a != "-I" and (i == 0 or args[i - 1] != "-I")]
    print(build(rest[0], rest[1:], incs))
