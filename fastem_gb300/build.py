"""Build recipe of the in-tree native libraries (no cmake, no setup.py).

  libfastem_gpu.so   CUDA kernels + the C-ABI of include/fastem_gpu.h,
                     compiled for sm_103a only.
  libfastem_host.so  C++ host classes mirroring the reference's EMAlgorithm /
                     GaussianMixture / KMeansAlgorithm interfaces on top of
                     the C-ABI, plus the .bin / .cmp formats.
  em2gpu             command-line driver mirroring the reference's em2.
  eminitgpu          command-line driver mirroring the reference's eminit.

Translation units compile in parallel; a unit is rebuilt when it or any
header is newer than its object file.
"""
import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
HOST = os.path.join(HERE, "host")
OBJ = os.path.join(HERE, "_build")
GPU_LIB = os.path.join(HERE, "libfastem_gpu.so")
HOST_LIB = os.path.join(HERE, "libfastem_host.so")
EM2GPU = os.path.join(HERE, "em2gpu")
EMINITGPU = os.path.join(HERE, "eminitgpu")
DRIVERS = {"em2gpu.cpp": EM2GPU, "eminitgpu.cpp": EMINITGPU}   # source -> program

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr",
                     "-Xcompiler", "-fPIC,-O3", "-I" + os.path.join(ROOT, "include")]


def nvcc():
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found: the CUDA 13 toolkit is required to build fastem_gb300")


def _newest(paths):
    return max((os.path.getmtime(p) for p in paths), default=0.0)


_ELF_MACHINE = {"x86_64": 62, "aarch64": 183}


def foreign_binary(path):
    """True if `path` is an ELF file built for another CPU (x86 objects
    copied to the Arm GPU host, or the reverse)."""
    import platform
    want = _ELF_MACHINE.get(platform.machine())
    try:
        with open(path, "rb") as f:
            head = f.read(20)
    except OSError:
        return False
    if want is None or len(head) < 20 or head[:4] != b"\x7fELF":
        return False
    return int.from_bytes(head[18:20], "little") != want


def _drop_foreign(paths):
    for p in paths:
        if os.path.exists(p) and foreign_binary(p):
            os.remove(p)


def _run(cmd, verbose):
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    if verbose and (r.stdout or r.stderr):
        print(r.stdout + r.stderr, flush=True)
    return r


def build_gpu(verbose=False, jobs=None, extra_flags=()):
    os.makedirs(OBJ, exist_ok=True)
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    hdrs = glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(ROOT, "include", "*.h"))
    hdr_time = _newest(hdrs)
    _drop_foreign(glob.glob(os.path.join(OBJ, "*.o")) + [GPU_LIB])
    cc = nvcc()
    objs, todo = [], []
    for s in srcs:
        o = os.path.join(OBJ, os.path.basename(s)[:-3] + ".o")
        objs.append(o)
        if not os.path.exists(o) or os.path.getmtime(o) < max(os.path.getmtime(s), hdr_time):
            todo.append((s, o))
    with cf.ThreadPoolExecutor(max_workers=jobs or min(8, os.cpu_count() or 4)) as ex:
        futs = [ex.submit(_run, [cc] + NVCC_FLAGS + list(extra_flags) + ["-c", s, "-o", o], verbose)
                for s, o in todo]
        for f in futs:
            f.result()
    if todo or not os.path.exists(GPU_LIB) or os.path.getmtime(GPU_LIB) < _newest(objs):
        _run([cc] + ARCH + ["-shared", "-o", GPU_LIB] + objs, verbose)
    return GPU_LIB


def build_host(verbose=False):
    srcs = sorted(glob.glob(os.path.join(HOST, "*.cpp")))
    if not srcs:
        return None
    hdrs = glob.glob(os.path.join(HOST, "*.h")) + glob.glob(os.path.join(ROOT, "include", "*.h"))
    lib_srcs = [s for s in srcs if os.path.basename(s) not in DRIVERS]
    cxx = os.environ.get("CXX", "g++")
    _drop_foreign([HOST_LIB] + list(DRIVERS.values()))
    common = ["-O2", "-std=c++17", "-fPIC", "-I" + os.path.join(ROOT, "include"), "-I" + HOST]
    newest = _newest(srcs + hdrs + [GPU_LIB])
    if not os.path.exists(HOST_LIB) or os.path.getmtime(HOST_LIB) < newest:
        _run([cxx] + common + ["-shared", "-o", HOST_LIB] + lib_srcs +
             ["-L" + HERE, "-lfastem_gpu", "-Wl,-rpath,$ORIGIN"], verbose)
    for src, exe in DRIVERS.items():
        drv = os.path.join(HOST, src)
        if os.path.exists(drv) and (not os.path.exists(exe) or os.path.getmtime(exe) < newest):
            _run([cxx] + common + ["-o", exe, drv, "-L" + HERE, "-lfastem_host", "-lfastem_gpu",
                                   "-Wl,-rpath,$ORIGIN"], verbose)
    return HOST_LIB


def build(verbose=False):
    build_gpu(verbose=verbose)
    build_host(verbose=verbose)


if __name__ == "__main__":
    build(verbose="-v" in sys.argv)
    print("built", GPU_LIB)
