"""gr_render_static: the render entry point that allocates nothing.

Some callers of this library cannot let it allocate device memory: an application that
manages all GPU memory through its own pool, or a frame loop that a cudaMalloc /
cudaFree (which synchronise the device) would stall.  gr_render_static runs the same
passes as gr_render with its scratch in a fixed array inside the library and writes into
a film the caller owns.  This test calls it twice in a row through the C ABI (passes 0
and 1 into the same caller-owned buffer) and checks the film against gr_render's after
each call.  Tolerance: 1e-6 relative (the two entry points run the same kernels in the
same order, so the sums are expected to be identical).

The file is named so pytest collects it last.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RTOL = 1e-6


def test_render_static_matches_render(gpu):
    import torch

    import gammaray_gb300 as g
    from gammaray_gb300 import scenes

    w = scenes.cornell_spheres(96, 80, 2)  # 7680 pixels, below the 131072-pixel limit
    st = g.Stage(w.prims, lib=gpu, environment=w.environment, seed=9)
    cam = w.camera.desc()
    out = torch.zeros((w.height, w.width, 4), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    for k in range(2):
        p = st.params(w.integrator, 1, first_pass=k)
        gpu.call("gr_render_static", st.handle, C.byref(cam), C.byref(p), w.width, w.height,
                 C.c_void_p(out.data_ptr()), None)
        torch.cuda.synchronize()
        ref = g.Film(w.width, w.height, lib=gpu)
        p_ref = st.params(w.integrator, k + 1, first_pass=0)
        gpu.call("gr_render", st.handle, C.byref(cam), C.byref(p_ref), ref.handle)
        acc, wt = ref.read()
        got = out.cpu().numpy()
        np.testing.assert_allclose(got[..., :3], acc, rtol=RTOL, atol=1e-7)
        np.testing.assert_allclose(got[..., 3], wt, rtol=RTOL, atol=1e-7)
        assert np.abs(acc).sum() > 0


def test_render_static_rejects_oversize(gpu):
    import gammaray_gb300 as g
    from gammaray_gb300 import _abi, scenes

    import torch

    w = scenes.cornell_spheres(8, 8, 1)
    st = g.Stage(w.prims, lib=gpu)
    cam = w.camera.desc()
    p = st.params(w.integrator, 1)
    out = torch.zeros((512, 512, 4), dtype=torch.float32, device="cuda")
    with pytest.raises(_abi.GrError) as e:
        # 512 x 512 > 131072 pixels: rejected before any device work.
        gpu.call("gr_render_static", st.handle, C.byref(cam), C.byref(p), 512, 512, C.c_void_p(out.data_ptr()),
                 None)
    assert e.value.status == 1
    assert "exceeds the fixed maximum" in str(e.value)
