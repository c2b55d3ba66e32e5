"""Build the C-ABI shared library libvhsdecode_gb300.so for sm_103a.

Every translation unit is compiled by nvcc in parallel (``.cu`` with the
sm_103a target, ``.cpp`` as host code) and linked into
``vhs-decode-dotnet_gb300/lib/libvhsdecode_gb300.so`` against the CUDA
runtime.  No cmake; one ``-gencode``.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess

PKG = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(PKG, "csrc")
LIB_DIR = os.path.join(PKG, "lib")
LIB = os.path.join(LIB_DIR, "libvhsdecode_gb300.so")
OBJ = os.path.join(LIB_DIR, "obj")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = ["demod_fp32.cu", "demod_fp64.cu", "field_kernels.cu", "test_entries.cu", "decimate.cu",
           "abi.cpp", "control.cpp", "filters.cpp", "noalloc.cu",
           "server.cpp", "run.cpp", "flac.cu", "chroma.cu", "chroma_design.cpp"]


def nvcc():
    path = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(path):
        raise RuntimeError("nvcc not found; the CUDA toolkit is required to build the library")
    return path


def _compile(src):
    out = os.path.join(OBJ, os.path.splitext(src)[0] + ".o")
    srcp = os.path.join(CSRC, src)
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    deps.append(os.path.join(os.path.dirname(PKG), "include", "vhsdecode_gb300.h"))
    if os.path.exists(out) and os.path.getmtime(out) >= max(os.path.getmtime(d) for d in deps):
        return out
    # host floating point exactly as written (no fused multiply-adds on Arm)
    common = ["-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-fvisibility=hidden",
              "-Xcompiler", "-ffp-contract=off", "-I", CSRC]
    if src.endswith(".cu"):
        cmd = [nvcc()] + ARCH + common + ["-lineinfo", "-c", srcp, "-o", out]
    else:
        cmd = [nvcc()] + common + ["-x", "c++", "-c", srcp, "-o", out]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("compile failed: %s\n%s\n%s" % (" ".join(cmd), r.stdout, r.stderr))
    return out


def build(force: bool = False) -> str:
    os.makedirs(OBJ, exist_ok=True)
    if force:
        for f in os.listdir(OBJ):
            os.remove(os.path.join(OBJ, f))
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(_compile, SOURCES))
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < max(os.path.getmtime(o) for o in objs):
        cmd = [nvcc()] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart", "-ldl"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed: %s\n%s\n%s" % (" ".join(cmd), r.stdout, r.stderr))
    return LIB


if __name__ == "__main__":
    print(build())
