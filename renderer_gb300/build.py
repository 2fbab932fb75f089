"""Builds the in-tree CUDA library renderer_gb300/_build/libgbrt.so for sm_103a.

Every translation unit is compiled by nvcc in parallel (one -gencode, sm_103a
only) and linked into one shared library with the CUDA runtime linked
statically, so the library carries no dependency on torch.
"""
import concurrent.futures
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libgbrt.so")

SOURCES = ["scene.cpp", "bvh_build.cpp", "bvh_gpu.cu", "scene_parse.cpp", "image_png.cpp", "image_jpeg.cpp",
           "image_out.cu", "trace.cu", "pathtrace.cu", "guide.cu"]

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
          "-Xcompiler", "-fno-strict-aliasing", "-I", os.path.join(HERE, "..", "include")]


def nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


# The checked build (build(checked=True)): the kernels test the indices they
# follow and report failures in the call's status (GBRT_CHECKED in
# csrc/gbrt_scene.h); a separate library for tests, not the product path.
OUT_CHECKED = os.path.join(HERE, "_build_checked")
LIB_CHECKED = os.path.join(OUT_CHECKED, "libgbrt.so")


def _compile(src, out=OUT, extra=()):
    obj = os.path.join(out, os.path.splitext(src)[0] + ".o")
    path = os.path.join(CSRC, src)
    lang = [] if src.endswith(".cu") else ["-x", "c++"]
    cmd = [nvcc()] + ARCH + COMMON + list(extra) + lang + ["-c", path, "-o", obj]
    if src.endswith(".cu"):
        cmd += ["-Xptxas", "-v"] if os.environ.get("GBRT_PTXAS_VERBOSE") else []
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, r.stdout, r.stderr))
    return obj, r.stderr


def build(verbose=False, checked=False):
    out, lib = (OUT_CHECKED, LIB_CHECKED) if checked else (OUT, LIB)
    extra = ("-DGBRT_CHECKED",) if checked else ()
    os.makedirs(out, exist_ok=True)
    with concurrent.futures.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        results = list(ex.map(lambda src: _compile(src, out, extra), SOURCES))
    objs = [o for o, _ in results]
    if verbose:
        for _, err in results:
            if err:
                print(err, file=sys.stderr)
    tmp = lib + ".tmp"
    cmd = [nvcc()] + ARCH + ["-shared", "-o", tmp] + objs + ["-cudart", "static", "-Xcompiler", "-pthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s\n%s" % (r.stdout, r.stderr))
    os.replace(tmp, lib)
    return lib


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, checked="--checked" in sys.argv))
