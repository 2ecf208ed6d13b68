"""Build recipe for the CPU oracle (test infrastructure, never the product).

Produces, under oracle/_build/:
  liboracle.so      strict FP64 restatement (-O2 -ffp-contract=off -fno-fast-math),
                    the parity checker;
  liboracle_omp.so  the same source with OpenMP over atoms, grid lines and FFT
                    lines (-O3 -fopenmp -ffp-contract=off), the timed CPU baseline.
The reference itself (Fortran 2008) cannot be compiled here: there is no
Fortran compiler on either machine, so oracle/_ref/ is never produced.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_build")
SRC = os.path.join(HERE, "dlpoly_oracle.cpp")


def build(verbose: bool = False) -> None:
    os.makedirs(OUT, exist_ok=True)
    jobs = [
        ["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared",
         SRC, "-o", os.path.join(OUT, "liboracle.so")],
        ["g++", "-std=c++17", "-O3", "-ffp-contract=off", "-fno-fast-math", "-fopenmp", "-DORACLE_OPENMP",
         "-fPIC", "-shared", SRC, "-o", os.path.join(OUT, "liboracle_omp.so")],
    ]
    procs = [subprocess.Popen(j, stdout=subprocess.PIPE, stderr=subprocess.STDOUT) for j in jobs]
    for j, p in zip(jobs, procs):
        out, _ = p.communicate()
        if p.returncode != 0:
            sys.stderr.write(out.decode())
            raise RuntimeError("oracle build failed: " + " ".join(j))
        if verbose and out:
            sys.stderr.write(out.decode())


if __name__ == "__main__":
    build(verbose=True)
