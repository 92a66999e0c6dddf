"""Compile the reference's ray-query translation units in place (oracle pinning).

Builds oracle/_ref/libref_bvh.so from the reference tree's own
BVH/BVH2Common.cpp and diff_render/BVH2DR.cpp (read where they lie; nothing is
copied) plus
oracle/ref_driver.cpp, and oracle/_ref/libref_dr.so from those two plus
Renderer/eye_ray.cpp, diff_render/MultiRendererDR.cpp, diff_render/DR_common.cpp
and utils/sparse_octree_builder.cpp with oracle/ref_driver_dr.cpp, against the
project's shims for the reference's missing dependencies (oracle/ref_shim/: a
LiteMath stand-in, the CrossRT ISceneObject interface, LiteImage's Image2D and
LiteScene's SimpleMesh).  Leaf types off the path are compiled out with the
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


# the differentiable renderer and the builders need the graphics-primitive
# members of BVHRT (MultiRendererDR.cpp reads them in its debug paths), so that
# library is built with them, every unit alike
DR_DEFINES = [d for d in DEFINES if d != "DISABLE_GRAPHICS_PRIM"]
DR_SOURCES = [("BVH/BVH2Common.cpp", "dr_bvh2common.o"), ("diff_render/BVH2DR.cpp", "dr_bvh2dr.o"),
              ("Renderer/eye_ray.cpp", "dr_eye_ray.o"), ("diff_render/MultiRendererDR.cpp", "dr_multirendererdr.o"),
              ("diff_render/DR_common.cpp", "dr_common.o"), ("utils/sparse_octree_builder.cpp", "dr_sob.o")]
DR_LIB = os.path.join(OUT, "libref_dr.so")


def build_dr():
    """libref_dr.so: MultiRendererDR, create_grid_sbs and the SBS/SVS builders in place."""
    if not available():
        return None
    os.makedirs(OUT, exist_ok=True)
    flags = ["-std=c++17", "-O2", "-ffp-contract=off", "-fPIC", "-w", "-fopenmp", "-I" + os.path.join(HERE, "ref_shim"),
             "-I" + REF] + ["-D" + d for d in DR_DEFINES]
    jobs = [(os.path.join(REF, src), os.path.join(OUT, obj)) for src, obj in DR_SOURCES]
    jobs.append((os.path.join(HERE, "ref_driver_dr.cpp"), os.path.join(OUT, "dr_driver.o")))
    procs = [(src, subprocess.Popen(["g++", *flags, "-c", src, "-o", obj], stdout=subprocess.PIPE,
                                    stderr=subprocess.STDOUT, text=True)) for src, obj in jobs]
    for src, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            sys.stderr.write(out)
            raise RuntimeError("reference in-place build failed: " + src)
    r = subprocess.run(["g++", "-shared", "-fopenmp", "-Wl,--no-undefined", "-o", DR_LIB, *[o for _, o in jobs]],
                       stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        sys.stderr.write(r.stdout)
        raise RuntimeError("reference in-place link failed (differentiable renderer)")
    return DR_LIB


ADAPTER = os.path.join(OUT, "adapter_check")


def build_adapter_check(engine_lib):
    """oracle/_ref/adapter_check: the reference-side binding
    (litert_gb300/ref_side/lrt_bvhrt_gpu.h) compiled against the reference's own
    headers and linked with the engine and the in-place renderer."""
    if not available():
        return None
    build_dr()
    root = os.path.dirname(HERE)
    flags = ["-std=c++17", "-O1", "-w", "-fopenmp", "-I" + os.path.join(HERE, "ref_shim"), "-I" + REF,
             "-I" + os.path.join(root, "include"), "-I" + os.path.join(root, "litert_gb300", "ref_side")] + \
            ["-D" + d for d in DR_DEFINES]
    objs = [os.path.join(OUT, o) for _, o in DR_SOURCES] + [os.path.join(OUT, "dr_driver.o")]
    r = subprocess.run(["g++", *flags, os.path.join(HERE, "ref_adapter_check.cpp"), *objs, engine_lib,
                        "-Wl,-rpath," + os.path.dirname(engine_lib), "-o", ADAPTER],
                       stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        sys.stderr.write(r.stdout)
        raise RuntimeError("reference-side binding does not build against the reference headers")
    return ADAPTER


def build():
    if not available():
        return None
    build_dr()
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
