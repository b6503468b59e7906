"""Build recipe of libpicgpu.so (CUDA for sm_103a + host C++), in-tree.

Each translation unit is compiled by nvcc in parallel and linked into
picfoam_gb300/_build/libpicgpu.so.  Kernels whose results are compared bit
for bit with the CPU oracle are compiled with --fmad=false; host code is
compiled with -ffp-contract=off so the mesh geometry rounds identically on
x86 and Arm hosts.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
SRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libpicgpu.so")
DRIVER = os.path.join(OUT, "picgpu_rts_driver")
INCLUDE = os.path.join(ROOT, "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-ffp-contract=off,-fno-fast-math",
          "-I", INCLUDE, "-I", SRC, "--expt-relaxed-constexpr"]
# translation unit -> extra flags
UNITS = {
    "move_fp64.cu": ["--fmad=false"],
    "move_fp32.cu": ["--use_fast_math"],
    "fields.cu": ["--fmad=false"],
    "particles.cu": [],
    "collide.cu": ["--fmad=false"],
    "mcc_fp32.cu": ["--use_fast_math"],
    "library.cu": [],
    "pcg_static.cu": ["--fmad=false"],
    "unet_conv.cu": [],
    "unet.cu": [],
    "learned.cu": [],
    "mg.cu": [],
    "init.cu": ["--fmad=false"],
    "unet_api.cu": [],
}
HEADERS = [os.path.join(SRC, f) for f in os.listdir(SRC) if f.endswith((".h", ".cuh", ".hpp"))] + [
    os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")]


def nvcc():
    exe = shutil.which("nvcc")
    if exe is None and os.path.exists("/usr/local/cuda/bin/nvcc"):
        exe = "/usr/local/cuda/bin/nvcc"
    if exe is None:
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libpicgpu.so")
    return exe


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def _compile(unit, flags):
    src = os.path.join(SRC, unit)
    obj = os.path.join(OUT, unit.replace(".cu", ".o"))
    if not _stale(obj, [src] + HEADERS):
        return obj, None
    cmd = [nvcc()] + ARCH + COMMON + flags + ["-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        return obj, f"{' '.join(cmd)}\n{r.stdout}\n{r.stderr}"
    return obj, None


def build(verbose=False):
    """Compile (incrementally) and link libpicgpu.so; returns its path."""
    os.makedirs(OUT, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=min(len(UNITS), os.cpu_count() or 4)) as ex:
        results = list(ex.map(lambda kv: _compile(*kv), UNITS.items()))
    errors = [e for _, e in results if e]
    if errors:
        raise RuntimeError("nvcc failed:\n" + "\n".join(errors))
    objs = [o for o, _ in results]
    if _stale(LIB, objs):
        cmd = [nvcc()] + ARCH + ["-shared", "--cudart", "static", "-o", LIB] + objs
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    # the C++ host driver over the run-time selection header (picgpu_rts.hpp)
    drv_src = os.path.join(HERE, "host", "rts_driver.cpp")
    if os.path.exists(drv_src) and _stale(DRIVER, [drv_src, LIB] + HEADERS):
        cxx = shutil.which("g++") or "g++"
        cmd = [cxx, "-O2", "-std=c++17", "-I", INCLUDE, drv_src, "-o", DRIVER, "-L", OUT, "-lpicgpu",
               "-Wl,-rpath,$ORIGIN"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"driver build failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    if verbose:
        print(LIB)
    return LIB


if __name__ == "__main__":
    build(verbose=True)
    sys.exit(0)
