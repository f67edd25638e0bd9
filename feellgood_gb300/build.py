"""Build recipe of the fggpu library (CUDA for sm_103a + C++ host code), in-tree.

Compiles every translation unit under csrc/ in parallel with nvcc / g++ and links
feellgood_gb300/_build/libfggpu.so. Used by __graft_entry__.build(); run directly with
``python -m feellgood_gb300.build``.
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libfggpu.so")
NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
           "--expt-relaxed-constexpr", "-I", os.path.join(HERE, "..", "include")]
CXXFLAGS = ["-O2", "-std=c++17", "-fPIC", "-I", os.path.join(HERE, "..", "include")]


MAIN = "fg_main.cpp"  # the command-line driver, linked as an executable
EXE = os.path.join(OUT, "fggpu")


def _sources():
    cu = sorted(f for f in os.listdir(CSRC) if f.endswith(".cu"))
    cpp = sorted(f for f in os.listdir(CSRC) if f.endswith(".cpp") and f != MAIN)
    return cu, cpp


def _newest_input():
    t = 0.0
    for d in (CSRC, os.path.join(HERE, "..", "include")):
        for f in os.listdir(d):
            t = max(t, os.path.getmtime(os.path.join(d, f)))
    return t


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    return r.returncode, " ".join(cmd) + "\n" + r.stdout + r.stderr


def build(force=False, verbose=False, ptxas_info=False):
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= _newest_input():
        return LIB
    os.makedirs(OUT, exist_ok=True)
    cu, cpp = _sources()
    jobs = []
    for f in cu:
        extra = ["-Xptxas", "-v"] if ptxas_info else []
        jobs.append([NVCC] + ARCH + NVFLAGS + extra + ["-c", os.path.join(CSRC, f), "-o",
                                                       os.path.join(OUT, f + ".o")])
    for f in cpp:
        jobs.append(["g++"] + CXXFLAGS + ["-c", os.path.join(CSRC, f), "-o", os.path.join(OUT, f + ".o")])
    with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        results = list(ex.map(_run, jobs))
    failed = [log for rc, log in results if rc != 0]
    if verbose or ptxas_info:
        for rc, log in results:
            sys.stderr.write(log)
    if failed:
        sys.stderr.write("\n".join(failed))
        raise RuntimeError("fggpu build failed")
    objs = [os.path.join(OUT, f + ".o") for f in cu + cpp]
    rc, log = _run([NVCC] + ARCH + ["-shared", "-o", LIB + ".tmp"] + objs + ["-lcudart"])
    if rc != 0:
        sys.stderr.write(log)
        raise RuntimeError("fggpu link failed")
    os.replace(LIB + ".tmp", LIB)
    rc, log = _run(["g++"] + CXXFLAGS + [os.path.join(CSRC, MAIN), "-o", EXE, "-L", OUT, "-lfggpu",
                                        "-Wl,-rpath,$ORIGIN"])
    if rc != 0:
        sys.stderr.write(log)
        raise RuntimeError("fggpu driver link failed")
    return LIB


if __name__ == "__main__":
    print(build(force=True, verbose="-v" in sys.argv, ptxas_info="--ptxas" in sys.argv))
