"""Compile the reference's ray-query translation units in place (oracle pinning).

Builds oracle/_ref/libref_bvh.so from the reference tree's own
BVH/BVH2Common.cpp and diff_render/BVH2DR.cpp (read where they lie; nothing is
copied) plus
oracle/ref_driver.cpp, against the project's shims for the reference's missing
dependencies (oracle/ref_shim/: a LiteMath stand-in and the CrossRT
ISceneObject interface).  Leaf types off the path are compiled out with the
reference's own DISABLE_* switches.  Runs only where the reference tree exists
(LRT_REFERENCE_TREE); machines without it skip this step, nothing in the engine,
the benchmark or the GPU tests needs this library.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
# The reference tree: LRT_REFERENCE_TREE, else the checkout this recipe was written
# against.  This recipe is the only file that locates it; tests ask it.
REF = os.environ.get("LRT_REFERENCE_TREE", "/root/reference")
OUT = os.path.join(HERE, "_ref")
LIB = os.path.join(OUT, "libref_bvh.so")
DEFINES = ["ON_CPU=1", "DISABLE_OPENVDB", "DISABLE_RF_GRID", "DISABLE_GS_PRIMITIVE", "DISABLE_NURBS",
           "DISABLE_CATMUL_CLARK", "DISABLE_RIBBON", "DISABLE_GRAPHICS_PRIM", "DISABLE_SDF_FRAME_OCTREE_COMPACT",
           "DISABLE_SDF_GRID", "DISABLE_SDF_FRAME_OCTREE", "DISABLE_SDF_FRAME_OCTREE_TEX", "DISABLE_SDF_SBS_ADAPT"]


def available():
    return os.path.exists(os.path.join(REF, "BVH", "BVH2Common.cpp"))


def build():
    if not available():
        return None
    os.makedirs(OUT, exist_ok=True)
    flags = ["-std=c++17", "-O2", "-ffp-contract=off", "-fPIC", "-w", "-I" + os.path.join(HERE, "ref_shim"),
             "-I" + REF] + ["-D" + d for d in DEFINES]
    objs = []
    for src, obj in ((os.path.join(REF, "BVH", "BVH2Common.cpp"), "bvh2common.o"),
                     (os.path.join(REF, "diff_render", "BVH2DR.cpp"), "bvh2dr.o"),
                     (os.path.join(HERE, "ref_driver.cpp"), "ref_driver.o")):
        o = os.path.join(OUT, obj)
        r = subprocess.run(["g++", *flags, "-c", src, "-o", o], stdout=subprocess.PIPE, stderr=subprocess.STDOUT,
                           text=True)
        if r.returncode != 0:
            sys.stderr.write(r.stdout)
            raise RuntimeError("reference in-place build failed: " + src)
        objs.append(o)
    r = subprocess.run(["g++", "-shared", "-Wl,--no-undefined", "-o", LIB, *objs], stdout=subprocess.PIPE,
                       stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        sys.stderr.write(r.stdout)
        raise RuntimeError("reference in-place link failed")
    return LIB


if __name__ == "__main__":
    print(build())
