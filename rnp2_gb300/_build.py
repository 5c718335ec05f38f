"""In-tree build of the GB300 QR library (libqr_gb300.so) for sm_103a.

Each CUDA translation unit is compiled by its own nvcc process, in parallel,
then linked into rnp2_gb300/_lib/libqr_gb300.so with the CUDA runtime linked
statically.  Objects go to rnp2_gb300/_build/ (git-ignored).
"""
import concurrent.futures as cf
import glob
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OBJDIR = os.path.join(HERE, "_build")
LIBDIR = os.path.join(HERE, "_lib")
LIBNAME = "libqr_gb300.so"
LIBPATH = os.path.join(LIBDIR, LIBNAME)
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2", "--expt-relaxed-constexpr", "-I" + INCLUDE]

UNITS = ["api_context.cu", "qr_s.cu", "qr_d.cu", "qr_c.cu", "qr_z.cu", "qr_noalloc.cu", "batched.cu", "batched_s.cu", "batched_d.cu", "batched_c.cu", "batched_z.cu"]


def _nvcc():
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    p = os.path.join(cuda, "bin", "nvcc")
    return p if os.path.exists(p) else (shutil.which("nvcc") or "nvcc")


def _newest_input():
    files = glob.glob(os.path.join(CSRC, "*")) + glob.glob(os.path.join(INCLUDE, "rnp_gpu", "*")) + [__file__]
    return max(os.path.getmtime(f) for f in files)


def _compile(unit):
    src = os.path.join(CSRC, unit)
    obj = os.path.join(OBJDIR, unit.replace(".cu", ".o"))
    cmd = [_nvcc()] + NVFLAGS + ["-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (unit, " ".join(cmd), r.stderr[-4000:]))
    return obj


def build(force=False, verbose=False):
    """Compile and link the library if any source is newer than it."""
    if not force and os.path.exists(LIBPATH) and os.path.getmtime(LIBPATH) >= _newest_input():
        return LIBPATH
    os.makedirs(OBJDIR, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=min(len(UNITS), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(_compile, UNITS))
    tmp = LIBPATH + ".tmp"
    cmd = [_nvcc()] + ARCH + ["-shared", "-o", tmp] + objs + ["-Xcompiler", "-fPIC"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s\n%s" % (" ".join(cmd), r.stderr[-4000:]))
    os.replace(tmp, LIBPATH)
    if verbose:
        print("built", LIBPATH)
    return LIBPATH


if __name__ == "__main__":
    build(force=True, verbose=True)
