"""Build recipe of the CPU oracle (test infrastructure).

* ``oracle/_build/libasuna_oracle.so`` — the C++ restatement
  (``oracle/asuna_oracle.cpp``); builds on any host with g++.
* ``oracle/_ref/libasuna_ref.so`` — the reference's own shader source
  translated by ``oracle/gen_ref.py`` and run by ``oracle/ref_harness.cpp``;
  built only where the reference tree is available.

Both are compiled with ``-ffp-contract=off`` so float arithmetic is rounded
operation by operation, as the GLSL source spells it, on x86-64 and AArch64.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
PORT_SO = os.path.join(HERE, "_build", "libasuna_oracle.so")
REF_SO = os.path.join(HERE, "_ref", "libasuna_ref.so")
REF_TREE = "/root/reference"
CXXFLAGS = ["-std=c++20", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared", "-pthread"]


def _newer(out, srcs):
    if not os.path.exists(out):
        return False
    t = os.path.getmtime(out)
    return all(os.path.getmtime(s) <= t for s in srcs)


def build_port(force=False):
    src = os.path.join(HERE, "asuna_oracle.cpp")
    deps = [src, os.path.join(HERE, "asuna_oracle.h"), os.path.join(REPO, "include", "asuna_rt.h")]
    if not force and _newer(PORT_SO, deps):
        return PORT_SO
    os.makedirs(os.path.dirname(PORT_SO), exist_ok=True)
    tmp = PORT_SO + ".tmp"
    subprocess.check_call(["g++", *CXXFLAGS, "-Wall", "-o", tmp, src])
    os.replace(tmp, PORT_SO)
    return PORT_SO


def build_ref(ref_tree=REF_TREE, force=False):
    """Returns the path of the reference-shader library, or None without the tree."""
    if not os.path.isdir(os.path.join(ref_tree, "src", "shaders")):
        return None
    gen = os.path.join(HERE, "_ref", "gen")
    subprocess.check_call([sys.executable, os.path.join(HERE, "gen_ref.py"), "--ref", ref_tree, "--out", gen])
    srcs = [os.path.join(HERE, "ref_harness.cpp"), os.path.join(HERE, "asuna_oracle.cpp")]
    tmp = REF_SO + ".tmp"
    subprocess.check_call(["g++", *CXXFLAGS, "-Wno-return-type", "-Wno-unused-variable", "-Wno-unused-function",
                           "-I", HERE, "-I", os.path.join(HERE, "shim"), "-I", gen,
                           "-I", os.path.join(ref_tree, "src"), "-o", tmp, *srcs])
    os.replace(tmp, REF_SO)
    return REF_SO


if __name__ == "__main__":
    print(build_port(force=True))
    print(build_ref(force=True))
