"""Build recipe of libfmf_gb300.so (sm_103a only).

Compiles every ``csrc/*.cu`` in parallel with nvcc and links one shared
library into ``fast_matched_filter_gb300/lib``.  The CUDA runtime is linked
statically, so the library needs only the NVIDIA driver at run time.

    python -m fast_matched_filter_gb300.build [--verbose]
"""
import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
LIBDIR = os.path.join(HERE, "lib")
LIB = os.path.join(LIBDIR, "libfmf_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-O2,-fvisibility=hidden",
         "-Xptxas", "-v", "--expt-relaxed-constexpr"]


def nvcc():
    exe = shutil.which("nvcc")
    if exe is None and os.path.exists("/usr/local/cuda/bin/nvcc"):
        exe = "/usr/local/cuda/bin/nvcc"
    if exe is None:
        raise RuntimeError("nvcc not found")
    return exe


def _compile(src):
    obj = os.path.join(OBJ, os.path.basename(src)[:-3] + ".o")
    cmd = [nvcc()] + ARCH + FLAGS + ["-c", src, "-o", obj]
    p = subprocess.run(cmd, capture_output=True, text=True)
    if p.returncode != 0:
        raise RuntimeError("nvcc failed on %s:\n%s\n%s" % (src, p.stdout, p.stderr))
    return obj, p.stderr


def _stale(sources):
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = sources + glob.glob(os.path.join(CSRC, "*.cuh")) + [
        os.path.join(HERE, "..", "include", "fmf_gb300.h"), __file__]
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build(force=False, verbose=False):
    """Compile the library if any source is newer than it; return its path."""
    sources = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    if not force and not _stale(sources):
        return LIB
    os.makedirs(OBJ, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(sources), os.cpu_count() or 4))) as ex:
        results = list(ex.map(_compile, sources))
    log = []
    for (obj, err), src in zip(results, sources):
        log.append("== %s\n%s" % (os.path.basename(src), err))
    tmp = LIB + ".tmp"
    cmd = [nvcc()] + ARCH + ["-shared", "-o", tmp] + [o for o, _ in results] + ["-lcuda"]
    p = subprocess.run(cmd, capture_output=True, text=True)
    if p.returncode != 0:
        raise RuntimeError("link failed:\n%s\n%s" % (p.stdout, p.stderr))
    os.replace(tmp, LIB)
    with open(os.path.join(OBJ, "ptxas.log"), "w") as f:
        f.write("\n".join(log))
    if verbose:
        print("\n".join(log))
    return LIB


if __name__ == "__main__":
    print(build(force=True, verbose="--verbose" in sys.argv))
