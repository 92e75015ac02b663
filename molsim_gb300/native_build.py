"""Build the native library libmolsim_gb300.so for sm_103a with nvcc.

Each .cu file in csrc/ is compiled in parallel to an object, then the
objects are linked into a shared library next to this file.  Host code is
compiled without floating-point contraction so that the host-side set-up
(table, Ewald factors) carries the reference expressions' exact bits.
"""
import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libmolsim_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if c and (os.path.isabs(c) and os.path.exists(c) or not os.path.isabs(c)):
            return c
    return "nvcc"


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def _report(what):
    """Each compile or link step that runs is reported on stderr, so that a
    build log shows whether the library was compiled or found up to date."""
    sys.stderr.write(f"[molsim_gb300 build] {what}\n")


def _compile(src, verbose):
    obj = os.path.join(BUILD, os.path.basename(src)[:-3] + ".o")
    deps = [src] + [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cuh")]
    deps.append(os.path.join(HERE, "..", "include", "molsim_gb300.h"))
    if os.path.exists(obj) and all(os.path.getmtime(obj) >= os.path.getmtime(d) for d in deps):
        return obj
    cmd = [nvcc(), *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
           "-Xcompiler", "-ffp-contract=off", "-c", src, "-o", obj]
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    _report(" ".join(cmd))
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stderr}")
    if verbose and r.stderr:
        sys.stderr.write(r.stderr)
    return obj


def build(verbose=False, force=False):
    os.makedirs(BUILD, exist_ok=True)
    if force:
        for f in os.listdir(BUILD):
            os.remove(os.path.join(BUILD, f))
    srcs = sources()
    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose), srcs))
    if os.path.exists(LIB) and not force and all(os.path.getmtime(LIB) >= os.path.getmtime(o) for o in objs):
        _report(f"{LIB} up to date (objects newer than their sources)")
        build_harness()
        return LIB
    cmd = [nvcc(), *ARCH, "-shared", "-o", LIB, *objs, "-lcudart"]
    _report(" ".join(cmd))
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr}")
    build_harness()
    return LIB


def build_harness():
    """mg_replay: the compiled C++ caller of the ABI, linked against the
    library next to it (rpath $ORIGIN)."""
    src = os.path.join(HERE, "harness", "mg_replay.cpp")
    exe = os.path.join(HERE, "mg_replay")
    if os.path.exists(exe) and os.path.getmtime(exe) >= max(os.path.getmtime(src), os.path.getmtime(LIB)):
        return exe
    # no contraction: the harness restates the reference's arithmetic
    # (PBC, Metropolis) and must round as the Python and Fortran callers do
    cmd = ["g++", "-O2", "-std=c++17", "-Wall", "-ffp-contract=off", "-I", os.path.join(HERE, "..", "include"), src,
           "-L", HERE, "-lmolsim_gb300", "-Wl,-rpath,$ORIGIN", "-o", exe]
    _report(" ".join(cmd))
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"harness build failed:\n{r.stderr}")
    return exe


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
