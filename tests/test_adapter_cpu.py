"""CPU: the reference-side bindings (litert_gb300/ref_side/lrt_bvhrt_gpu.h:
BVHRT_GPU : ISceneObject and MultiRendererGPU : MultiRenderer;
lrt_multirenderer_dr_gpu.h: MultiRendererDR_GPU : dr::MultiRendererDR) compile
against the reference's own BVH/BVH2Common.h, Renderer/eye_ray.h and
diff_render/MultiRendererDR.h, link with the engine library and the reference's
renderer compiled in place, and run: without a GPU the engine contexts fail
cleanly, with one they render and optimise.  Where the
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
    lines = r.stdout.splitlines()
    assert len(lines) >= 2 and (lines[1].startswith("no-device MultiRendererDR_GPU") or
                                lines[1].startswith("optimised MultiRendererDR_GPU")), r.stdout
