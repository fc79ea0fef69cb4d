"""In-tree build of ``libfockgb300.so`` (the C-ABI CUDA library).

Compiles every ``csrc/*.cu`` for sm_103a only, in parallel, and links them into
one shared library next to this file.  Objects are rebuilt only when a source
or header is newer.  ``python -m strawberryfields_gb300.build`` runs it.
"""

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
OBJDIR = os.path.join(HERE, "_build")
LIBNAME = "libfockgb300.so"
LIBPATH = os.path.join(HERE, LIBNAME)

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
              "-I", INCLUDE, "-I", CSRC]


def _nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build the Fock GB300 library")


def _newest(paths):
    return max((os.path.getmtime(p) for p in paths), default=0.0)


def build(verbose=False, jobs=None, extra_flags=()):
    """Compile and link the library; return its path."""
    nvcc = _nvcc()
    os.makedirs(OBJDIR, exist_ok=True)
    # largest translation units first, so the slowest file starts at once.
    # (nvcc --split-compile would shorten the build further but measured a 5x
    # slower plane_adjoint_kernel on GB300 at the same register count.)
    sources = sorted(glob.glob(os.path.join(CSRC, "*.cu")), key=lambda s: -os.path.getsize(s))
    headers = glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(INCLUDE, "*.h"))
    hdr_time = _newest(headers)
    flags = NVCC_FLAGS + ARCH + list(extra_flags)

    def compile_one(src):
        obj = os.path.join(OBJDIR, os.path.basename(src) + ".o")
        if os.path.exists(obj) and os.path.getmtime(obj) >= max(os.path.getmtime(src), hdr_time):
            return obj, None
        cmd = [nvcc, "-c", src, "-o", obj] + flags
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            return obj, r.stderr + r.stdout
        if verbose and (r.stderr or r.stdout):
            print(r.stderr + r.stdout)
        return obj, None

    jobs = jobs or min(len(sources), os.cpu_count() or 4)
    with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
        results = list(ex.map(compile_one, sources))
    errors = [e for _, e in results if e]
    if errors:
        raise RuntimeError("nvcc failed:\n" + "\n".join(errors))
    objs = [o for o, _ in results]
    if not os.path.exists(LIBPATH) or os.path.getmtime(LIBPATH) < _newest(objs):
        tmp = LIBPATH + ".tmp"
        cmd = [nvcc, "-shared", "-o", tmp] + objs + ARCH + ["-lcudart_static", "-lrt", "-lpthread", "-ldl"]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n" + r.stderr + r.stdout)
        os.replace(tmp, LIBPATH)
    return LIBPATH


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
