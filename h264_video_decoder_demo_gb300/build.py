"""Build recipe for the engine's shared libraries (in-tree, no cmake).

  libh264r.so   the CUDA engine (sm_103a) behind include/h264r.h
  liboracle.so  the CPU oracle (test infrastructure, oracle/ Makefile)

`python -m h264_video_decoder_demo_gb300.build` compiles both; the CUDA
translation units compile in parallel with one -gencode for sm_103a.
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libh264r.so")

CU_SOURCES = ["h264r_kernels.cu", "h264r_api.cu", "h264r_noalloc.cu", "h264r_server.cu", "h264r_decoder.cu"]
CXX_SOURCES = ["h264r_synth.cpp", "h264r_order.cpp", "h264r_syntax.cpp", "h264r_cavlc.cpp", "h264r_parser.cpp", "h264r_writer.cpp", "h264r_cabac.cpp"]
NVCC_FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-lineinfo", "-std=c++17",
              "-Xcompiler", "-fPIC", "-Xcompiler", "-O2"]


def _nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.sep not in cand or os.path.exists(cand)):
            return cand
    return "nvcc"


def _newer(target, sources):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in sources)


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed: %s\n%s" % (" ".join(cmd), r.stdout))
    return r.stdout


def build_engine(force=False, verbose=False):
    os.makedirs(BUILD, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    headers += [os.path.join(ROOT, "include", f) for f in os.listdir(os.path.join(ROOT, "include"))]
    jobs = []
    objs = []
    for src in CU_SOURCES + CXX_SOURCES:
        path = os.path.join(CSRC, src)
        obj = os.path.join(BUILD, src + ".o")
        objs.append(obj)
        if force or _newer(obj, [path] + headers):
            if src.endswith(".cu"):
                cmd = [_nvcc()] + NVCC_FLAGS + ["-c", path, "-o", obj]
            else:
                cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-Wall", "-c", path, "-o", obj]
            jobs.append(cmd)
    if jobs:
        with ThreadPoolExecutor(max_workers=len(jobs)) as ex:
            for out in ex.map(_run, jobs):
                if verbose and out:
                    print(out)
    if force or jobs or _newer(LIB, objs):
        _run([_nvcc(), "-shared", "-gencode", "arch=compute_103a,code=sm_103a", "-o", LIB] + objs + ["-lcudart"])
    return LIB


def build_oracle(force=False):
    odir = os.path.join(ROOT, "oracle")
    cmd = ["make", "-C", odir, "-s", "liboracle.so", "check_dump"]
    if force:
        cmd.insert(3, "-B")
    _run(cmd)
    # the reference decoder from its own sources, where they are present
    # (H264R_REFERENCE_DIR, or the recipe's default location)
    _run(["make", "-C", odir, "-s", "-j8", "ref-if-present"])
    return os.path.join(odir, "liboracle.so")


def main(argv):
    force = "--force" in argv
    print(build_engine(force=force, verbose="-v" in argv))
    print(build_oracle(force=force))


if __name__ == "__main__":
    main(sys.argv[1:])
