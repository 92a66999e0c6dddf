"""Build the lrt engine shared library (CUDA for sm_103a + host C++) in-tree.

Output: litert_gb300/_build/liblrt_gb300.so.  Translation units compile in
parallel; the whole build takes well under a minute.  Kernels are compiled with
--fmad=false so their float arithmetic follows the reference's evaluation order
exactly (except trace_fused.cu, the opt-in contracted render kernels); host code with -ffp-contract=off so x86-64 and aarch64 hosts agree.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "liblrt_gb300.so")
CUDA = os.environ.get("CUDA_HOME", "/usr/local/cuda")
GENCODE = "-gencode=arch=compute_103a,code=sm_103a"

CU_SOURCES = ["trace.cu", "trace_fused.cu", "trace_ref.cu", "trace_inst.cu", "trace_pkt.cu", "dr.cu", "proposal.cu", "build_gpu.cu", "bvh_gpu.cu"]
# translation units compiled with floating-point contraction (the opt-in "fma" kernels)
CONTRACTED = {"trace_fused.cu"}
CPP_SOURCES = ["lrt_api.cpp", "scene_build.cpp", "scene_io.cpp", "bvh_build.cpp", "dr_api.cpp", "proposal_api.cpp"]


def _nvcc():
    p = os.path.join(CUDA, "bin", "nvcc")
    return p if os.path.exists(p) else "nvcc"


def _cmds():
    inc = ["-I" + os.path.join(ROOT, "include"), "-I" + CSRC, "-I" + os.path.join(CUDA, "include")]
    cmds = []
    objs = []
    for src in CU_SOURCES:
        obj = os.path.join(OUT, src.replace(".cu", ".o"))
        objs.append(obj)
        fmad = "--fmad=true" if src in CONTRACTED else "--fmad=false"
        cmds.append([_nvcc(), GENCODE, "-O3", "-lineinfo", fmad, "-std=c++17", "-Xptxas", "-v",
                     "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off", *inc, "-c",
                     os.path.join(CSRC, src), "-o", obj])
    for src in CPP_SOURCES:
        obj = os.path.join(OUT, src.replace(".cpp", ".o"))
        objs.append(obj)
        cmds.append(["g++", "-O2", "-std=c++17", "-fPIC", "-fopenmp", "-ffp-contract=off", "-Wall",
                     "-Wno-unused-function", *inc, "-c", os.path.join(CSRC, src), "-o", obj])
    link = ["g++", "-shared", "-o", LIB, *objs, "-L" + os.path.join(CUDA, "lib64"),
            "-Wl,-rpath," + os.path.join(CUDA, "lib64"), "-lcudart", "-fopenmp"]
    return cmds, link


def build(verbose=False):
    os.makedirs(OUT, exist_ok=True)
    cmds, link = _cmds()
    procs = [(c, subprocess.Popen(c, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)) for c in cmds]
    logs = []
    failed = False
    for c, p in procs:
        out, _ = p.communicate()
        logs.append(" ".join(c) + "\n" + out)
        if p.returncode != 0:
            failed = True
            sys.stderr.write(out)
    with open(os.path.join(OUT, "build.log"), "w") as f:
        f.write("\n".join(logs))
    if failed:
        raise RuntimeError("lrt build failed; see " + os.path.join(OUT, "build.log"))
    r = subprocess.run(link, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        sys.stderr.write(r.stdout)
        raise RuntimeError("lrt link failed")
    if verbose:
        print("\n".join(logs))
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
