"""Build recipes for the native parts of pilon_gb300.

libpilon_gb300.so — the CUDA engine and its C ABI, sm_103a only.
libpg_synth.so    — the host-side read simulator used by the benchmark.
libpg_bam.so      — BAM records <-> the packed read store and the BGZF inflate (host).

Everything is compiled in-tree into pilon_gb300/_build/ with nvcc / g++
directly (no cmake), the translation units in parallel.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
BUILD = os.path.join(HERE, "_build")
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(ROOT, "include")

ENGINE = os.path.join(BUILD, "libpilon_gb300.so")
SYNTH = os.path.join(BUILD, "libpg_synth.so")
BAMLIB = os.path.join(BUILD, "libpg_bam.so")

CU_SOURCES = ["pg_api.cu", "pg_pileup.cu", "pg_call.cu", "pg_kmer.cu", "pg_format.cu", "pg_noalloc.cu",
              "pg_breaks.cu", "pg_serve.cu"]
CPP_SOURCES = ["pg_assemble.cpp", "pg_fixes.cpp"]
NVCC_FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-lineinfo", "-std=c++17",
              "-Xcompiler", "-fPIC", "-Xcompiler", "-fwrapv", "--expt-relaxed-constexpr"]


def _nvcc():
    for p in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc"):
        if p and os.path.exists(p):
            return p
    return "nvcc"


def _newer(target, sources):
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(s) <= t for s in sources)


def _run_all(cmds):
    procs = [(c, subprocess.Popen(c, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)) for c in cmds]
    errs = []
    for c, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            errs.append(" ".join(c) + "\n" + out.decode(errors="replace"))
    if errs:
        raise RuntimeError("native build failed:\n" + "\n".join(errs))


def build(force=False, verbose=False):
    """Compiles the engine, the simulator and the BAM codec; returns the engine path."""
    os.makedirs(BUILD, exist_ok=True)
    headers = [os.path.join(INCLUDE, "pilon_gb300.h")] + [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith(".cuh")]
    nvcc = _nvcc()
    objs, cmds = [], []
    for s in CU_SOURCES:
        src = os.path.join(CSRC, s)
        obj = os.path.join(BUILD, s.replace(".cu", ".o"))
        objs.append(obj)
        if force or not _newer(obj, [src] + headers):
            cmds.append([nvcc] + NVCC_FLAGS + ["-I", INCLUDE, "-I", CSRC, "-c", src, "-o", obj])
    for s in CPP_SOURCES:  # host-only parts of the engine library
        src = os.path.join(CSRC, s)
        obj = os.path.join(BUILD, s.replace(".cpp", ".o"))
        objs.append(obj)
        if force or not _newer(obj, [src] + headers):
            cmds.append(["g++", "-O2", "-std=c++17", "-fPIC", "-pthread", "-fwrapv", "-I", INCLUDE, "-c", src,
                         "-o", obj])
    synth_src = os.path.join(CSRC, "synth.cpp")
    if force or not _newer(SYNTH, [synth_src]):
        cmds.append(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-pthread", synth_src, "-o", SYNTH])
    bam_srcs = [os.path.join(CSRC, "bam.cpp"), os.path.join(CSRC, "inflate.cpp")]
    if force or not _newer(BAMLIB, bam_srcs):
        cmds.append(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-pthread"] + bam_srcs + ["-o", BAMLIB])
    if cmds:
        if verbose:
            for c in cmds:
                print(" ".join(c), file=sys.stderr)
        _run_all(cmds)
    if force or not _newer(ENGINE, objs):
        _run_all([[nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-shared", "-o", ENGINE] + objs
                  + ["-lcudart", "-ldl", "-Xcompiler", "-pthread"]])
    return ENGINE


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
