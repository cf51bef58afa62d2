"""Builds the CUDA library libmfem_gb300.so in-tree for sm_103a (GB300).

The translation units compile in parallel with nvcc and link into
mfem_gb300/_build/libmfem_gb300.so.  No CMake, no torch extension machinery.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_build")
LIB_NAME = "libmfem_gb300.so"
SOURCES = ["k_elem.cu", "k_rows.cu", "k_minres.cu", "k_noalloc.cu", "tri2d.cu", "host.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc():
    path = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(path):
        raise RuntimeError("nvcc not found")
    return path


def _flags(verbose_ptxas=False):
    f = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
         "--expt-relaxed-constexpr", "-I", CSRC] + ARCH
    if verbose_ptxas:
        f += ["-Xptxas", "-v"]
    return f


def lib_path():
    return os.path.join(OUT_DIR, LIB_NAME)


def _stale():
    lib = lib_path()
    if not os.path.exists(lib):
        return True
    t = os.path.getmtime(lib)
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    deps.append(os.path.join(HERE, "..", "include", "mfem_gb300.h"))
    deps.append(os.path.abspath(__file__))
    return any(os.path.getmtime(p) > t for p in deps if os.path.exists(p))


def build(force=False, verbose_ptxas=False, quiet=False):
    """Compiles the library if any source is newer than it; returns its path."""
    if not force and not _stale():
        return lib_path()
    os.makedirs(OUT_DIR, exist_ok=True)
    cc = nvcc()
    flags = _flags(verbose_ptxas)

    def compile_one(src):
        obj = os.path.join(OUT_DIR, os.path.splitext(src)[0] + ".o")
        cmd = [cc, *flags, "-c", os.path.join(CSRC, src), "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
        return obj, r.stderr

    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        results = list(ex.map(compile_one, SOURCES))
    if verbose_ptxas and not quiet:
        for _, err in results:
            sys.stderr.write(err)
    objs = [o for o, _ in results]
    tmp = lib_path() + ".tmp"
    cmd = [cc, "-shared", *ARCH, "-o", tmp, *objs, "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, lib_path())
    return lib_path()


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose_ptxas="-v" in sys.argv))
