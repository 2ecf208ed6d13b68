"""Compile the GB300 library (csrc/*.cu -> libdlpoly_gb300.so) for sm_103a.

Each translation unit compiles in its own nvcc process, in parallel, then one
link step produces the shared library next to this file (in-tree, git-ignored).
Host code is built with -ffp-contract=off so the host-side geometry constants
(halo widths, link-cell sizes) round exactly as the FP64 restatement does on
both x86_64 and aarch64.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "csrc")
OBJ = os.path.join(os.path.dirname(HERE), "_build")
LIB = os.path.join(HERE, "libdlpoly_gb300.so")
SOURCES = ["gb_api.cu", "gb_list.cu", "gb_pair.cu", "gb_spme.cu", "gb_integrate.cu", "gb_thermostat.cu", "gb_metal.cu", "gb_mlp.cu",
           "gb_noalloc.cu", "gb_fft_f32.cu", "gb_fft_df.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC = os.environ.get("NVCC", "nvcc")


def flags(debug=False):
    f = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC,-ffp-contract=off", "--expt-relaxed-constexpr"]
    if os.environ.get("GB_PTXAS_V"):
        f += ["-Xptxas", "-v"]
    return ARCH + f


def build(verbose: bool = False) -> str:
    os.makedirs(OBJ, exist_ok=True)
    srcs = [s for s in SOURCES if os.path.exists(os.path.join(CSRC, s))]
    objs, procs = [], []
    for s in srcs:
        o = os.path.join(OBJ, s.replace(".cu", ".o"))
        objs.append(o)
        cmd = [NVCC] + flags() + ["-c", os.path.join(CSRC, s), "-o", o]
        procs.append((cmd, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
    failed = False
    for cmd, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0 or (verbose and out):
            sys.stderr.write(out.decode())
        if p.returncode != 0:
            failed = True
            sys.stderr.write("FAILED: " + " ".join(cmd) + "\n")
    if failed:
        raise RuntimeError("CUDA build failed")
    link = [NVCC] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart"]
    r = subprocess.run(link, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
    if r.returncode != 0:
        sys.stderr.write(r.stdout.decode())
        raise RuntimeError("link failed")
    return LIB


if __name__ == "__main__":
    print(build(verbose=True))
