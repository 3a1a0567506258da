"""Batched rendering and the serving loop on the GPU, against the per-image render."""
from __future__ import annotations

import math

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


def test_batch_release_frees_the_engine(gpu):
    import torch
    ws = small_workloads(2)
    jobs = [batch.Job(g.Stage(w.prims, lib=gpu, environment=w.environment), w.camera, w.integrator,
                      g.Film(w.width, w.height, lib=gpu), w.spp) for w in ws]
    batch.render_batch(jobs, gpu, path_capacity=1 << 23)  # about 2.4 GB of queues and ring
    torch.cuda.synchronize()
    held = torch.cuda.mem_get_info()[0]
    batch.release(gpu)
    freed = torch.cuda.mem_get_info()[0] - held
    assert freed > 1 << 30, freed
    batch.render_batch(jobs, gpu, path_capacity=1 << 23)  # set up again
    assert all(j.film.passes() == 2 * j.spp for j in jobs)


def test_batch_autotune_and_display(gpu):
    ws = small_workloads(3)
    jobs = []
    for k, w in enumerate(ws):
        st = g.Stage(w.prims, lib=gpu, environment=w.environment)
        integ = g.DisplayColorIntegrator() if k == 0 else w.integrator
        jobs.append(batch.Job(st, w.camera, integ, g.Film(w.width, w.height, lib=gpu), w.spp))
    opt = batch.autotune(jobs, gpu)
    assert opt.path_capacity in (1 << 23, 1 << 25, 1 << 26) and opt.block_size in (128, 256)
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


def test_server_snapshot_shows_the_film_so_far(gpu):
    w = small_workloads(1, seed=14)[0]
    st = g.Stage(w.prims, lib=gpu, environment=w.environment, seed=5)
    s = serve.Server(gpu, path_capacity=1 << 16)
    rid = s.submit(st, w.camera, w.integrator, w.width, w.height, 64)
    acc0, wt0, n0 = s.snapshot(rid)  # not admitted yet: zeros
    assert n0 == 0 and not wt0.any()
    seen, part = [], {}
    for _ in range(400):
        s.step(0.5)
        acc, wt, n = s.snapshot(rid)
        seen.append(n)
        if 0 < n < 64:
            part[n] = (acc, wt)
        if s.poll(rid).state == 2:
            break
    assert seen == sorted(seen) and seen[-1] == 64
    assert part  # a film part-way through
    acc, wt, n = s.snapshot(rid)
    a2, w2 = s.take(rid)
    np.testing.assert_array_equal(acc, a2)
    np.testing.assert_array_equal(wt, w2)
    # a part-way film is the film of the first k passes
    k = min(part)
    ref = g.Film(w.width, w.height, lib=gpu)
    st.render(w.camera, w.integrator, ref, k)
    racc, rwt = ref.read()
    np.testing.assert_array_equal(part[k][1], rwt)
    np.testing.assert_allclose(part[k][0], racc, rtol=1e-6, atol=1e-7)


def test_server_rejects_an_image_too_large_for_its_ring(gpu):
    # The check is at submission: an oversized request must not fail the steps that
    # serve the others.  A 64 k-path server keeps an 8 M-slot ring (images up to 4 M px).
    w = small_workloads(1)[0]
    st = g.Stage(w.prims, lib=gpu, environment=w.environment)
    s = serve.Server(gpu, path_capacity=1 << 16)
    ok = s.submit(st, w.camera, w.integrator, w.width, w.height, 2)
    with pytest.raises(Exception, match="path ring"):
        s.submit(st, w.camera, w.integrator, 4096, 2048, 1)
    s.run_until_done([ok])
    assert s.poll(ok).state == 2


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


def half_films(st, w, passes, gpu):
    """Even and odd passes rendered pass by pass into two films, as a progressive request
    splits them."""
    import ctypes as C
    films = [g.Film(w.width, w.height, lib=gpu), g.Film(w.width, w.height, lib=gpu)]
    cam = w.camera.desc()
    for p in range(passes):
        prm = st.params(w.integrator, 1, p)
        gpu.call("gr_render", st.handle, C.byref(cam), C.byref(prm), films[p % 2].handle)
    return [f.read() for f in films]


def rel_mse_estimate(fa, fb):
    (aa, wa), (ab, wb) = fa, fb
    ok = (wa > 0) & (wb > 0)
    a = aa[ok].astype(np.float64) / wa[ok, None]
    b = ab[ok].astype(np.float64) / wb[ok, None]
    f = (aa[ok].astype(np.float64) + ab[ok]) / (wa[ok, None].astype(np.float64) + wb[ok, None])
    return float(np.sum((a - b) ** 2) / 4 / np.sum(f ** 2))


def test_server_progressive_stops_at_a_checkpoint(gpu):
    w = small_workloads(1, seed=11)[0]
    st = g.Stage(w.prims, lib=gpu, environment=w.environment, seed=2)
    s = serve.Server(gpu, path_capacity=1 << 16)
    loose = s.submit(st, w.camera, w.integrator, w.width, w.height, 256, target_rel_mse=10.0)
    tight = s.submit(st, w.camera, w.integrator, w.width, w.height, 48, target_rel_mse=1e-12)
    s.run_until_done([loose, tight])
    sl, stt = s.poll(loose), s.poll(tight)
    assert sl.state == 2 and sl.passes_done == 8 and 0 < sl.rel_mse <= 10.0
    assert stt.state == 2 and stt.passes_done == 48 and stt.rel_mse > 1e-12  # capped by spp
    # The estimate is the two half-films' (even and odd passes) and falls with more passes.
    est8 = rel_mse_estimate(*half_films(st, w, 8, gpu))
    np.testing.assert_allclose(sl.rel_mse, est8, rtol=1e-4)
    fa, fb = half_films(st, w, 48, gpu)
    np.testing.assert_allclose(stt.rel_mse, rel_mse_estimate(fa, fb), rtol=1e-4)
    assert stt.rel_mse < sl.rel_mse
    # take() returns the sum of the half-films.
    acc, wt = s.take(tight)
    np.testing.assert_allclose(acc, fa[0] + fb[0], rtol=1e-6, atol=1e-7)
    np.testing.assert_allclose(wt, fa[1] + fb[1], rtol=1e-6, atol=1e-7)


def next_checkpoint(done, est, target, cap):
    """The server's checkpoint rule (batch.cu next_checkpoint), restated: the pass count
    at which an estimate falling as 1 / passes meets the target with a 10% margin, within
    1.25x to 8x the passes so far, rounded up to a multiple of 8, at most cap."""
    want = done * float(np.float32(est)) / float(np.float32(target)) * 1.1
    want = min(max(want, 1.25 * done), 8.0 * done)
    return min((math.ceil(want) + 7) // 8 * 8, cap)


def test_server_progressive_target_and_mix(gpu):
    ws = small_workloads(3, seed=12)
    stages = [g.Stage(w.prims, lib=gpu, environment=w.environment, seed=k) for k, w in enumerate(ws)]
    w0 = ws[0]
    cache = {}

    def est(n):
        if n not in cache:
            cache[n] = rel_mse_estimate(*half_films(stages[0], w0, n, gpu))
        return cache[n]

    target = est(32) * 1.01  # met by 64 passes
    want = 8  # the checkpoints the server visits, replayed on the same estimates
    while est(want) > target and want < 64:
        want = next_checkpoint(want, est(want), target, 64)
    assert want > 8
    alone = serve.Server(gpu, path_capacity=1 << 16)
    rid = alone.submit(stages[0], w0.camera, w0.integrator, w0.width, w0.height, 64, target_rel_mse=target)
    alone.run_until_done([rid])
    sa = alone.poll(rid)
    assert sa.passes_done == want and sa.rel_mse <= target
    a_acc, a_w = alone.take(rid)
    mixed = serve.Server(gpu, path_capacity=1 << 16)
    ids = [mixed.submit(stages[k], ws[k].camera, ws[k].integrator, ws[k].width, ws[k].height, 6) for k in (1, 2)]
    mixed.step(1.0)
    rid0 = mixed.submit(stages[0], w0.camera, w0.integrator, w0.width, w0.height, 64, target_rel_mse=target)
    ids.append(mixed.submit(stages[1], ws[1].camera, ws[1].integrator, ws[1].width, ws[1].height, 64,
                            target_rel_mse=1e-12))
    mixed.run_until_done(ids + [rid0])
    sm = mixed.poll(rid0)
    assert sm.passes_done == sa.passes_done and sm.rel_mse == sa.rel_mse
    m_acc, m_w = mixed.take(rid0)
    np.testing.assert_array_equal(m_w, a_w)
    np.testing.assert_allclose(m_acc, a_acc, rtol=1e-6, atol=1e-7)
    assert mixed.poll(ids[-1]).passes_done == 64


def test_server_progressive_cancel_and_budget(gpu):
    w = small_workloads(1, seed=13)[0]
    st = g.Stage(w.prims, lib=gpu, environment=w.environment)
    film_bytes = w.width * w.height * 16
    s = serve.Server(gpu, memory_budget_bytes=2 * film_bytes, path_capacity=1 << 16)
    a = s.submit(st, w.camera, w.integrator, w.width, w.height, 64, target_rel_mse=1e-12)
    b = s.submit(st, w.camera, w.integrator, w.width, w.height, 4)  # waits: a holds two films
    s.step(0.5)
    assert s.poll(b).state == 0
    s.cancel(a)
    assert s.poll(a).state == 3
    s.take(a)  # releases both half-films
    s.run_until_done([b])
    assert s.poll(b).state == 2
    s.take(b)
    with pytest.raises(Exception):
        s.submit(st, w.camera, w.integrator, w.width, w.height, 4, target_rel_mse=-1.0)


def test_server_keeps_a_closed_scene_until_its_requests_let_go(gpu):
    # gr_scene_destroy of a scene that server requests still use defers the free: a
    # request queued when its scene is closed still renders the same image, and one
    # cancelled while running drains against the scene before it is freed.
    w = small_workloads(1, seed=15)[0]
    keep = g.Stage(w.prims, lib=gpu, environment=w.environment, seed=2)
    ref = g.Film(w.width, w.height, lib=gpu)
    keep.render(w.camera, w.integrator, ref, 3)
    ref_acc, ref_w = ref.read()
    s = serve.Server(gpu, path_capacity=1 << 16)
    st = g.Stage(w.prims, lib=gpu, environment=w.environment, seed=2)
    a = s.submit(st, w.camera, w.integrator, w.width, w.height, 3)
    st.close()  # queued: the request holds the scene
    s.run_until_done([a])
    acc, wt = s.take(a)  # the last holder: the scene is freed here
    np.testing.assert_array_equal(wt, ref_w)
    np.testing.assert_allclose(acc, ref_acc, rtol=1e-6, atol=1e-7)
    st2 = g.Stage(w.prims, lib=gpu, environment=w.environment, seed=3)
    b = s.submit(st2, w.camera, w.integrator, w.width, w.height, 1024)
    s.step(0.5)
    assert s.poll(b).state == 1  # running
    s.cancel(b)
    st2.close()
    s.take(b)  # its paths may still be queued: the scene waits for the engine to drain
    c = s.submit(keep, w.camera, w.integrator, w.width, w.height, 3)
    s.run_until_done([c])
    acc, wt = s.take(c)
    np.testing.assert_array_equal(wt, ref_w)
    np.testing.assert_allclose(acc, ref_acc, rtol=1e-6, atol=1e-7)
    s.close()


@pytest.mark.parametrize("policy", [0, 1])
def test_server_resets_its_tables_at_idle(gpu, policy):
    # The step that finds nothing running and every appended pass gathered clears the
    # engine's job and unit tables (in the same gr_server_step that finishes the last
    # request); a request served after the reset gets the same film as a plain render,
    # under either scheduling policy.
    ws = small_workloads(3, seed=21)
    stages = [g.Stage(w.prims, lib=gpu, environment=w.environment, seed=k) for k, w in enumerate(ws)]
    s = serve.Server(gpu, path_capacity=1 << 16, policy=policy)
    ids = [s.submit(stages[k], ws[k].camera, ws[k].integrator, ws[k].width, ws[k].height, 3) for k in range(2)]
    # 256 passes of 3072 pixels need at least 12 fills of the 64 k-path pool, more than
    # the 8 iterations of one step: the request is still running after it.
    w2 = ws[2]
    long_id = s.submit(stages[2], w2.camera, w2.integrator, 64, 48, 256)
    s.step(0.0)
    during = s.info()
    assert during.running >= 1 and during.engine_jobs == 3 and during.engine_units > 0 and during.resets == 0
    s.run_until_done(ids + [long_id])
    after = s.info()
    assert after.engine_jobs == 0 and after.engine_units == 0 and after.resets == 1
    assert after.finished == 3 and after.running == 0  # finished films stay until taken
    for rid in ids + [long_id]:
        s.take(rid)
    w = ws[1]
    rid = s.submit(stages[1], w.camera, w.integrator, w.width, w.height, 4)
    s.run_until_done([rid])
    assert s.info().resets == 2
    acc, wt = s.take(rid)
    ref = g.Film(w.width, w.height, lib=gpu)
    stages[1].render(w.camera, w.integrator, ref, 4)
    racc, rwt = ref.read()
    np.testing.assert_array_equal(wt, rwt)
    np.testing.assert_allclose(acc, racc, rtol=1e-6, atol=1e-7)


def test_progressive_estimate_matches_the_actual_error(gpu):
    # A progressive request stops at the first checkpoint whose half-film estimate of its
    # relMSE is at most the target.  The estimate is checked against the relMSE its image
    # actually has against a converged render of the same view (65536 spp, other random
    # streams, whose own noise is about 1.6e-5 here): within a factor of 1.5.
    w = scenes.cornell_spheres(64, 64, 1)
    st = g.Stage(w.prims, lib=gpu, seed=3)
    s = serve.Server(gpu, path_capacity=1 << 20)
    rid = s.submit(st, w.camera, w.integrator, 64, 64, 4096, target_rel_mse=2e-3)
    s.run_until_done([rid])
    stat = s.poll(rid)
    acc, wt = s.take(rid)
    assert stat.state == 2 and 0 < stat.rel_mse <= 2e-3 and stat.passes_done < 4096
    img = acc / wt[..., None]
    conv_stage = g.Stage(w.prims, lib=gpu, seed=99)
    conv = g.Film(64, 64, lib=gpu)
    conv_stage.render(w.camera, w.integrator, conv, 65536)
    ref = conv.resolve().astype(np.float64)
    actual = float(np.mean((img - ref) ** 2) / np.mean(ref ** 2))
    assert actual / 1.5 <= stat.rel_mse <= actual * 1.5, (stat.passes_done, stat.rel_mse, actual)
