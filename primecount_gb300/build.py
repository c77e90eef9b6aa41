"""In-tree build of libpcgpu.so (sm_103a) and of the CPU oracle.

    python -m primecount_gb300.build          # library + oracle
    python -m primecount_gb300.build --lib    # library only

The library is compiled with nvcc for sm_103a only (one -gencode), host
sources with the same nvcc/g++ driver, translation units in parallel.  The
oracle (oracle/pcg_oracle.c) is test infrastructure and is built into
oracle/liboracle.so; the library never links it.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INC = os.path.join(ROOT, "include")
BUILD = os.path.join(ROOT, "_build")
LIB = os.path.join(PKG, "libpcgpu.so")
ORACLE_DIR = os.path.join(ROOT, "oracle")
ORACLE_LIB = os.path.join(ORACLE_DIR, "liboracle.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-O2", "--expt-relaxed-constexpr",
              "-I" + INC, "-I" + CSRC]


def _nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    return r


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cu", ".cpp")))


def build_lib(verbose=False):
    os.makedirs(BUILD, exist_ok=True)
    nvcc = _nvcc()
    objs = []
    jobs = []
    for src in sources():
        obj = os.path.join(BUILD, os.path.basename(src) + ".o")
        objs.append(obj)
        if src.endswith(".cu"):
            cmd = [nvcc] + ARCH + NVCC_FLAGS + ["-c", src, "-o", obj]
        else:
            cmd = [nvcc] + NVCC_FLAGS + ["-x", "cu"] + ARCH + ["-c", src, "-o", obj]
        jobs.append(cmd)
    with cf.ThreadPoolExecutor(max_workers=min(8, len(jobs))) as ex:
        for r in ex.map(_run, jobs):
            if verbose and r.stderr:
                print(r.stderr, file=sys.stderr)
    tmp = LIB + ".tmp"
    _run([nvcc] + ARCH + ["-shared", "-o", tmp] + objs + ["-lpthread"])
    os.replace(tmp, LIB)
    return LIB


def build_oracle():
    cc = shutil.which("gcc") or shutil.which("cc")
    tmp = ORACLE_LIB + ".tmp"
    _run([cc, "-O2", "-fopenmp", "-shared", "-fPIC", os.path.join(ORACLE_DIR, "pcg_oracle.c"),
          "-o", tmp, "-lm"])
    os.replace(tmp, ORACLE_LIB)
    return ORACLE_LIB


def main(argv=None):
    argv = sys.argv[1:] if argv is None else argv
    if "--oracle" not in argv or "--lib" in argv:
        print(build_lib(verbose="-v" in argv))
    if "--lib" not in argv or "--oracle" in argv:
        print(build_oracle())


if __name__ == "__main__":
    main()
