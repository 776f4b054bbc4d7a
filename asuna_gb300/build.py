"""Build recipe of the native library ``asuna_gb300/_build/libasuna_rt.so``.

sm_103a only (``-gencode arch=compute_103a,code=sm_103a``).  The shading
translation unit is compiled with ``-fmad=false`` so its float arithmetic
rounds operation by operation like the reference's GLSL; the traversal unit
keeps FMA contraction for box tests and spells its exact operations with
``__f*_rn`` intrinsics.  Host C++ is compiled with g++; CUDA runtime is linked
statically.  Translation units build in parallel.
"""
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libasuna_rt.so")
CUDA = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA, "bin", "nvcc") if os.path.exists(os.path.join(CUDA, "bin", "nvcc")) else "nvcc"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

CU = {"trace.cu": [], "shade.cu": ["-fmad=false"], "engine.cu": [], "noalloc.cu": [], "denoise.cu": [], "post.cu": [],
      "conv_tc.cu": [], "queue_sort.cu": [], "bvh_device.cu": ["-fmad=false"]}
CPP = ["host_scene.cpp", "json.cpp", "bvh_build.cpp", "server.cpp"]


def _deps():
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    files.append(os.path.join(REPO, "include", "asuna_rt.h"))
    files.append(os.path.abspath(__file__))
    return files


def up_to_date():
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(f) <= t for f in _deps())


def build(force=False, verbose=False):
    if not force and up_to_date():
        return LIB
    os.makedirs(OUT, exist_ok=True)
    jobs = []
    for src, extra in CU.items():
        obj = os.path.join(OUT, src + ".o")
        cmd = [NVCC, *ARCH, "-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC", *extra,
               "-c", os.path.join(CSRC, src), "-o", obj]
        jobs.append((cmd, obj))
    for src in CPP:
        obj = os.path.join(OUT, src + ".o")
        cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-Wall", "-I", os.path.join(CUDA, "include"),
               "-c", os.path.join(CSRC, src), "-o", obj]
        jobs.append((cmd, obj))
    procs = [(subprocess.Popen(c, stdout=subprocess.PIPE, stderr=subprocess.STDOUT), c) for c, _ in jobs]
    failed = []
    for p, c in procs:
        out, _ = p.communicate()
        if p.returncode != 0 or verbose:
            sys.stderr.write(out.decode(errors="replace"))
        if p.returncode != 0:
            failed.append(" ".join(c))
    if failed:
        raise RuntimeError("native build failed:\n" + "\n".join(failed))
    tmp = LIB + ".tmp"
    cmd = [NVCC, *ARCH, "-shared", "-Xcompiler", "-fPIC", "-o", tmp, *[o for _, o in jobs], "-lpthread"]
    subprocess.check_call(cmd)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
