"""Build recipe of the CPU oracle (test infrastructure).

* ``oracle/_build/libasuna_oracle.so`` — the C++ restatement
  (``oracle/asuna_oracle.cpp``); builds on any host with g++.
* ``oracle/_ref/libasuna_ref.so`` — the reference's own shader source
  translated by ``oracle/gen_ref.py`` and run by ``oracle/ref_harness.cpp``.
  Where the reference checkout is present (``gen_ref.find_ref_tree``) the
  translation is made afresh; elsewhere (the GPU host) the library is built
  from a translation made earlier in ``oracle/_ref/gen/``, which carries the
  reference's shared headers with it.  Without either, it is not built.

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
GEN_DIR = os.path.join(HERE, "_ref", "gen")
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


def _gen_complete(gen):
    """An earlier translation with its shared headers (gen_ref writes the
    manifest last)."""
    return os.path.exists(os.path.join(gen, "GENERATED_FROM")) and os.path.isdir(os.path.join(gen, "shared"))


def build_ref(ref_tree=None, force=False):
    """Returns the path of the reference-shader library, or None where neither
    the reference checkout nor an earlier translation of it is available."""
    sys.path.insert(0, HERE)
    import gen_ref

    if ref_tree is None:
        ref_tree = gen_ref.find_ref_tree()
    gen = GEN_DIR
    srcs = [os.path.join(HERE, "ref_harness.cpp"), os.path.join(HERE, "post_harness.cpp"),
            os.path.join(HERE, "asuna_oracle.cpp")]
    deps = srcs + [os.path.join(HERE, "asuna_oracle.h"), os.path.join(HERE, "glsl_shim.h"),
                   os.path.join(REPO, "include", "asuna_rt.h"), os.path.join(REPO, "include", "asuna_math.h")]
    if ref_tree is not None:
        subprocess.check_call([sys.executable, os.path.join(HERE, "gen_ref.py"), "--ref", ref_tree, "--out", gen])
    elif not _gen_complete(gen):
        return None
    elif not force and _newer(REF_SO, deps):
        return REF_SO
    tmp = REF_SO + ".tmp"
    subprocess.check_call(["g++", *CXXFLAGS, "-Wno-return-type", "-Wno-unused-variable", "-Wno-unused-function",
                           "-I", HERE, "-I", os.path.join(HERE, "shim"), "-I", gen, "-o", tmp, *srcs])
    os.replace(tmp, REF_SO)
    return REF_SO


if __name__ == "__main__":
    print(build_port(force=True))
    print(build_ref(force=True))
