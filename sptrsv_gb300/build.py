"""Build recipe for the in-tree native libraries.

libsptrsv_gb300.so  -- the CUDA solver (sm_103a only) and its C ABI (include/*.h);
libsptrsv_gen.so    -- the host-only synthetic matrix generators.

nvcc compiles each translation unit for `-gencode arch=compute_103a,code=sm_103a` in
parallel, then links one shared library with the static CUDA runtime.  Objects go to
sptrsv_gb300/_build/ and are rebuilt when a source or header is newer.
"""
import concurrent.futures as cf
import glob
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
ROOT = os.path.dirname(HERE)
LIB = os.path.join(HERE, "libsptrsv_gb300.so")
GEN = os.path.join(HERE, "libsptrsv_gen.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc():
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return cand


def _newest(paths):
    return max((os.path.getmtime(p) for p in paths), default=0.0)


def build(verbose=False, force=False):
    os.makedirs(BUILD, exist_ok=True)
    headers = glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(ROOT, "include", "*.h"))
    hdr_time = _newest(headers)
    # CUDA translation units plus host-only C++ ones (gen.cpp goes into the generator library)
    sources = sorted(glob.glob(os.path.join(CSRC, "*.cu")) +
                     [p for p in glob.glob(os.path.join(CSRC, "*.cpp")) if os.path.basename(p) != "gen.cpp"])
    nvcc = _nvcc()
    flags = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-fvisibility=hidden",
                    "-I" + os.path.join(ROOT, "include"), "--expt-relaxed-constexpr"]
    jobs = []
    objs = []
    for src in sources:
        obj = os.path.join(BUILD, os.path.basename(src) + ".o")
        objs.append(obj)
        if force or not os.path.exists(obj) or os.path.getmtime(obj) < max(os.path.getmtime(src), hdr_time):
            jobs.append([nvcc] + flags + ["-c", src, "-o", obj])
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        results = list(ex.map(lambda c: subprocess.run(c, capture_output=True, text=True), jobs))
    for cmd, r in zip(jobs, results):
        if verbose or r.returncode:
            print(" ".join(cmd))
            print(r.stdout, r.stderr)
        if r.returncode:
            raise RuntimeError("nvcc failed for " + cmd[-3])
    if force or jobs or not os.path.exists(LIB) or os.path.getmtime(LIB) < _newest(objs):
        link = [nvcc] + ARCH + ["-shared", "-o", LIB] + objs + ["-cudart", "static"]
        r = subprocess.run(link, capture_output=True, text=True)
        if r.returncode:
            print(" ".join(link), r.stdout, r.stderr)
            raise RuntimeError("link failed")
    gsrc = os.path.join(CSRC, "gen.cpp")
    if force or not os.path.exists(GEN) or os.path.getmtime(GEN) < os.path.getmtime(gsrc):
        cmd = ["g++", "-O3", "-ffp-contract=off", "-std=c++17", "-fPIC", "-shared", "-pthread", "-o", GEN, gsrc]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode:
            print(" ".join(cmd), r.stdout, r.stderr)
            raise RuntimeError("generator build failed")
    return LIB


if __name__ == "__main__":
    build(verbose=True)
