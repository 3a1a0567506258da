"""gr_render_static: the render entry point that allocates nothing.

Some callers of this library cannot let it allocate device memory.  Examples are an
application that manages all GPU memory through its own pool, and a frame loop that a
cudaMalloc / cudaFree would stall, since both synchronise the device.
gr_render_static runs the same passes as gr_render, with its scratch in a fixed array
inside the library, and writes into a film the caller owns.

These tests call it through the C ABI twice in a row (passes 0 and 1, into the same
caller-owned buffer, on a stream of the caller's) and check the film against gr_render's
after each call.  They cover:
  - the path tracer with a depth cap;
  - the path tracer with the reference's unbounded depth;
  - the display-colour integrator.
Tolerance: 1e-6 relative.  The two entry points run the same kernels in the same order,
so the sums are expected to be identical.  Around the second call, the device's free
memory must not change.

Other tests:
  - a traversal step budget that every ray exceeds (set on the host through
    GR_STEP_BUDGET; no GPU fault) is reported as GR_ERR_TIMEOUT, and the next call works;
  - settings that apply to BDPT only are rejected;
  - sizes above the fixed maximum are rejected.

The file is named so pytest collects it last.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RTOL = 1e-6


def _call_static(gpu, st, cam, p, width, height, out, stream):
    gpu.call("gr_render_static", st.handle, C.byref(cam), C.byref(p), width, height, C.c_void_p(out.data_ptr()),
             C.c_void_p(stream.cuda_stream))


@pytest.mark.parametrize("case", ["depth_8", "unbounded_depth", "display_color"])
def test_render_static_matches_render(gpu, case):
    import torch

    import gammaray_gb300 as g
    from gammaray_gb300 import scenes

    w = scenes.cornell_spheres(96, 80, 2)  # 7680 pixels, below the 131072-pixel limit
    integ = {"depth_8": w.integrator, "unbounded_depth": g.PathTracerIntegrator(),
             "display_color": g.DisplayColorIntegrator()}[case]
    st = g.Stage(w.prims, lib=gpu, environment=w.environment, seed=9)
    cam = w.camera.desc()
    stream = torch.cuda.Stream()
    out = torch.zeros((w.height, w.width, 4), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    for k in range(2):
        p = st.params(integ, 1, first_pass=k)
        free_before = torch.cuda.mem_get_info()[0]
        _call_static(gpu, st, cam, p, w.width, w.height, out, stream)
        stream.synchronize()
        if k == 1:  # the first call may load kernels; later ones must leave memory alone
            assert torch.cuda.mem_get_info()[0] == free_before
        ref = g.Film(w.width, w.height, lib=gpu)
        p_ref = st.params(integ, k + 1, first_pass=0)
        gpu.call("gr_render", st.handle, C.byref(cam), C.byref(p_ref), ref.handle)
        acc, wt = ref.read()
        got = out.cpu().numpy()
        np.testing.assert_allclose(got[..., :3], acc, rtol=RTOL, atol=1e-7)
        np.testing.assert_allclose(got[..., 3], wt, rtol=RTOL, atol=1e-7)
        assert np.abs(acc).sum() > 0


def test_render_static_reports_the_step_budget(gpu, monkeypatch):
    import torch

    import gammaray_gb300 as g
    from gammaray_gb300 import _abi, scenes

    w = scenes.cornell_spheres(32, 32, 1)
    monkeypatch.setenv("GR_STEP_BUDGET", "1")  # read at scene creation
    st = g.Stage(w.prims, lib=gpu, environment=w.environment, seed=1)
    monkeypatch.delenv("GR_STEP_BUDGET")
    ok = g.Stage(w.prims, lib=gpu, environment=w.environment, seed=1)
    cam = w.camera.desc()
    stream = torch.cuda.Stream()
    out = torch.zeros((32, 32, 4), dtype=torch.float32, device="cuda")
    with pytest.raises(_abi.GrError) as e:
        _call_static(gpu, st, cam, st.params(w.integrator, 1), 32, 32, out, stream)
    assert e.value.status == 5  # GR_ERR_TIMEOUT
    assert "step budget" in str(e.value)
    out.zero_()
    _call_static(gpu, ok, cam, ok.params(w.integrator, 1), 32, 32, out, stream)  # the context stays usable
    stream.synchronize()
    assert float(out[..., 3].sum()) > 0


def test_render_static_rejects_bad_settings(gpu):
    import torch

    import gammaray_gb300 as g
    from gammaray_gb300 import _abi, scenes

    w = scenes.cornell_spheres(8, 8, 1)
    st = g.Stage(w.prims, lib=gpu)
    cam = w.camera.desc()
    stream = torch.cuda.Stream()
    out = torch.zeros((512, 512, 4), dtype=torch.float32, device="cuda")
    with pytest.raises(_abi.GrError) as e:
        # 512 x 512 > 131072 pixels: rejected before any device work.
        _call_static(gpu, st, cam, st.params(w.integrator, 1), 512, 512, out, stream)
    assert e.value.status == 1
    assert "exceeds the fixed maximum" in str(e.value)
    p = st.params(w.integrator, 1)
    p.mis = 1  # a BDPT setting on the path tracer
    with pytest.raises(_abi.GrError) as e:
        _call_static(gpu, st, cam, p, 8, 8, out, stream)
    assert e.value.status == 1
