"""Batched rendering and the serving loop on the GPU, against the per-image render."""
from __future__ import annotations

import numpy as np
import pytest

import gammaray_gb300 as g
from gammaray_gb300 import batch, scenes, serve

pytestmark = pytest.mark.gpu


def small_workloads(n=6, seed=3):
    out = []
    for k, w in enumerate(scenes.batch_scenes(n, seed=seed)):
        res = [(64, 48), (32, 32), (80, 40), (24, 56)][k % 4]
        w.width, w.height = res
        w.spp = 2 + k % 4
        out.append(w)
    return out


def test_batch_equals_per_image(gpu):
    ws = small_workloads()
    jobs, ref = [], []
    for k, w in enumerate(ws):
        st = g.Stage(w.prims, lib=gpu, environment=w.environment, seed=k)
        jobs.append(batch.Job(st, w.camera, w.integrator, g.Film(w.width, w.height, lib=gpu), w.spp))
        f = g.Film(w.width, w.height, lib=gpu)
        st.render(w.camera, w.integrator, f, w.spp)
        ref.append(f.read())
    stats = batch.render_batch(jobs, gpu, path_capacity=1 << 16)
    assert stats.samples == sum(w.width * w.height * w.spp for w in ws)
    for j, (acc, wt) in zip(jobs, ref):
        a, b = j.film.read()
        np.testing.assert_allclose(a, acc, rtol=1e-6, atol=1e-7)
        np.testing.assert_allclose(b, wt, rtol=1e-6, atol=1e-7)
        assert j.film.passes() == j.spp


def test_batch_autotune_and_display(gpu):
    ws = small_workloads(3)
    jobs = []
    for k, w in enumerate(ws):
        st = g.Stage(w.prims, lib=gpu, environment=w.environment)
        integ = g.DisplayColorIntegrator() if k == 0 else w.integrator
        jobs.append(batch.Job(st, w.camera, integ, g.Film(w.width, w.height, lib=gpu), w.spp))
    opt = batch.autotune(jobs, gpu)
    assert opt.path_capacity in (1 << 21, 1 << 23, 1 << 24) and opt.block_size in (128, 256)
    for j in jobs:
        assert j.film.passes() == 0  # trials render into scratch films
    batch.render_batch(jobs, gpu, opt.path_capacity, opt.block_size)
    ref = g.Film(ws[0].width, ws[0].height, lib=gpu)
    jobs[0].stage.render(ws[0].camera, g.DisplayColorIntegrator(), ref, ws[0].spp)
    np.testing.assert_array_equal(jobs[0].film.read()[0], ref.read()[0])


def test_server_alone_equals_mixed(gpu):
    ws = small_workloads(5, seed=9)
    stages = [g.Stage(w.prims, lib=gpu, environment=w.environment, seed=k) for k, w in enumerate(ws)]
    w0 = ws[0]
    alone = serve.Server(gpu, path_capacity=1 << 16)
    rid = alone.submit(stages[0], w0.camera, w0.integrator, w0.width, w0.height, 4)
    alone.run_until_done([rid])
    a_acc, a_w = alone.take(rid)
    mixed = serve.Server(gpu, path_capacity=1 << 16)
    ids = [mixed.submit(stages[k], ws[k].camera, ws[k].integrator, ws[k].width, ws[k].height, 3) for k in (1, 2)]
    mixed.step(1.0)
    rid0 = mixed.submit(stages[0], w0.camera, w0.integrator, w0.width, w0.height, 4)  # arrives mid-flight
    ids += [mixed.submit(stages[k], ws[k].camera, ws[k].integrator, ws[k].width, ws[k].height, 5) for k in (3, 4)]
    mixed.run_until_done(ids + [rid0])
    st = mixed.poll(rid0)
    assert st.state == 2 and st.passes_done == 4 and st.finish_ms >= st.submit_ms
    m_acc, m_w = mixed.take(rid0)
    np.testing.assert_array_equal(m_w, a_w)
    np.testing.assert_allclose(m_acc, a_acc, rtol=1e-6, atol=1e-7)
    ref = g.Film(w0.width, w0.height, lib=gpu)
    stages[0].render(w0.camera, w0.integrator, ref, 4)
    np.testing.assert_allclose(ref.read()[0], a_acc, rtol=1e-6, atol=1e-7)


def test_server_admission_and_cancel(gpu):
    w = small_workloads(1)[0]
    st = g.Stage(w.prims, lib=gpu, environment=w.environment)
    film_bytes = w.width * w.height * 16
    s = serve.Server(gpu, memory_budget_bytes=film_bytes, path_capacity=1 << 16)  # one film at a time
    a = s.submit(st, w.camera, w.integrator, w.width, w.height, 3)
    b = s.submit(st, w.camera, w.integrator, w.width, w.height, 3)
    c = s.submit(st, w.camera, w.integrator, w.width, w.height, 3)
    s.cancel(c)
    s.step(0.5)
    assert s.poll(c).state == 3
    s.run_until_done([a])
    assert s.poll(a).state == 2
    assert s.poll(b).state == 0  # queued: a's film still holds the whole budget
    fin_a = s.poll(a).finish_ms
    s.take(a)  # releases a's film
    s.run_until_done([b])
    sb = s.poll(b)
    assert sb.state == 2 and sb.start_ms >= fin_a
    s.take(b)
    s.take(c)
    with pytest.raises(Exception):
        s.submit(st, w.camera, w.integrator, w.width * 4, w.height * 4, 1)  # film larger than the budget
