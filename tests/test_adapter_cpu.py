"""CPU: the reference-side binding (litert_gb300/ref_side/lrt_bvhrt_gpu.h) --
BVHRT_GPU : ISceneObject and MultiRendererGPU : MultiRenderer -- compiles
against the reference's own BVH/BVH2Common.h and Renderer/eye_ray.h, links with
the engine library and the reference's renderer compiled in place, and runs:
without a GPU the engine context fails cleanly, with one it renders.  Where the
reference tree is absent the check is skipped (tests/test_adapter_render_gpu.py
drives the engine exactly as the binding does and pins its image to the
reference's)."""
import subprocess

import pytest

from litert_gb300 import build
from oracle import build_ref

pytestmark = pytest.mark.skipif(not build_ref.available(), reason="reference tree not present")


def test_binding_builds_against_reference_headers_and_runs():
    exe = build_ref.build_adapter_check(build.LIB)
    r = subprocess.run([exe], stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True, timeout=120)
    assert r.returncode == 0, r.stdout
    assert r.stdout.startswith("no-device BVHRT_GPU") or r.stdout.startswith("rendered BVHRT_GPU"), r.stdout
