"""Build recipe of the pfast_gb300 CUDA library (sm_103a only).

Compiles pfast_gb300/csrc/*.cu in parallel with nvcc and links
pfast_gb300/lib/libpfast_gb300.so (CUDA runtime linked statically, cuFFT
dynamically from the toolkit, C ABI in include/pfast_gb300.h).  -fmad=false: no FMA contraction anywhere, so the plain
FP64 kernels evaluate the reference's expressions exactly; the fast kernels
request FMA explicitly with fma().
"""
import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
LIBDIR = os.path.join(HERE, "lib")
LIB = os.path.join(LIBDIR, "libpfast_gb300.so")
SOURCES = ["kernels3d.cu", "kernels3d_s84.cu", "kernels2d.cu", "engine.cu", "engine2d.cu", "multi3d.cu", "noalloc.cu", "invert.cu", "serve.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-std=c++17", "-O3", "-lineinfo", "-fmad=false", "-Xcompiler", "-fPIC,-O2",
              "--expt-relaxed-constexpr", "-Xptxas", "-warn-spills"] + ARCH


def nvcc():
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build pfast_gb300")
    return cand


def cuda_libdir():
    """Directory of the toolkit's shared libraries (libcufft), recorded as the library's rpath."""
    root = os.path.dirname(os.path.dirname(os.path.realpath(nvcc())))
    for sub in ("lib64", "lib"):
        d = os.path.join(root, sub)
        if os.path.exists(os.path.join(d, "libcufft.so")):
            return d
    raise RuntimeError("libcufft.so not found under " + root)


def _stale(out, deps):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose=False, force=False):
    os.makedirs(OBJ, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    headers.append(os.path.join(HERE, "..", "include", "pfast_gb300.h"))
    cc = nvcc()
    jobs = []
    objs = []
    for src in SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OBJ, src.replace(".cu", ".o"))
        objs.append(o)
        if force or _stale(o, [s] + headers):
            jobs.append([cc] + NVCC_FLAGS + ["-c", s, "-o", o])

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
        return r.stderr

    with ThreadPoolExecutor(max(1, len(jobs))) as ex:
        for err in ex.map(run, jobs):
            if verbose and err.strip():
                print(err)
    if force or jobs or _stale(LIB, objs):
        libdir = cuda_libdir()
        run([cc] + ARCH + ["-shared", "-o", LIB] + objs +
            ["-L" + libdir, "-lcufft", "-lpthread", "-Xlinker", "-rpath", "-Xlinker", libdir])
    build_drivers(verbose=verbose, force=force)
    return LIB


# Drop-in executables: (binary name, source, extra defines)
DRIVERS = [("T_PFAST3D_FW", "t_pfast3d_fw.cpp", []),
           ("RT_PFAST2D_FW", "rt_pfast2d_fw.cpp", []),
           ("RT_PFAST2D_FW_NoS", "rt_pfast2d_fw.cpp", ["-DNoShotGather"]),
           ("T_PFAST3D", "t_pfast3d.cpp", []),
           ("RT_PFAST2D", "rt_pfast2d.cpp", [])]
BINDIR = os.path.join(HERE, "bin")


def build_drivers(verbose=False, force=False):
    os.makedirs(BINDIR, exist_ok=True)
    ddir = os.path.join(HERE, "drivers")
    inc = os.path.join(HERE, "..", "include")
    jobs = []
    for name, src, defs in DRIVERS:
        out = os.path.join(BINDIR, name)
        deps = [os.path.join(ddir, src), os.path.join(ddir, "driver_io.h"), LIB]
        if force or _stale(out, deps):
            jobs.append(["g++", "-O2", "-std=c++17", "-I", inc] + defs +
                        [os.path.join(ddir, src), "-o", out, "-L", LIBDIR, "-lpfast_gb300",
                         "-Wl,-rpath,$ORIGIN/../lib"])

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("driver build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)

    with ThreadPoolExecutor(max(1, len(jobs))) as ex:
        list(ex.map(run, jobs))
    return BINDIR


if __name__ == "__main__":
    print(build(verbose=True))
