"""Wavefront form (crg_render_batch) versus the megakernel (crg_render).

Both run the same per-bounce shading code with the same random numbers, and
the wavefront resolves each sample into the film in sample order, so the FP32
and FP64 film sums must be bit-identical — for one view, for batches of views
over several scenes with uneven resolution and spp, and with a path pool and
chunks small enough to force regeneration and several resolves.  The device
loop is bounded: a tiny iteration cap must end the frame with TIMEOUT and
leave the context usable."""
import numpy as np
import pytest

from crender_gb300 import CrgError, api, scenes
from test_gpu_c_render import _box_variant

pytestmark = pytest.mark.gpu


def _mega(ctx, scene, cam, st, passes=1):
    f = api.Film(ctx, st.width, st.height, f64=True)
    for _ in range(passes):
        api.render(scene, cam, st, f)
    out = f.download(f64=True)
    f.close()
    return out


def _same(a, b):
    for k in ("sum", "sum64", "sumsq64"):
        bad = int((a[k].view(np.uint8).reshape(a[k].size, -1) != b[k].view(np.uint8).reshape(b[k].size, -1)).any(1).sum())
        assert bad == 0, f"{k}: {bad} values differ"


OFF = 0xFFFFFFFF  # refill off: static per-warp fetch


@pytest.mark.parametrize("mode,rr", [(1, 3), (0, 0)])
@pytest.mark.parametrize("opts", [None, dict(path_pool=1000, chunk_samples=5000, fetch=32, block_size=64, refill=OFF),
                                  dict(path_pool=4096, chunk_samples=20000, host_loop=1, refill=OFF, fetch=64),
                                  dict(path_pool=1000, chunk_samples=5000, fuse=2),
                                  dict(path_pool=1000, chunk_samples=5000, fuse=3, fetch=32, block_size=256),
                                  dict(path_pool=4096, chunk_samples=20000, host_loop=1, fuse=3),
                                  dict(path_pool=1000, chunk_samples=5000, refill=8),
                                  dict(path_pool=1000, chunk_samples=5000, refill=1, fuse=2, block_size=256),
                                  dict(path_pool=4096, chunk_samples=20000, refill=32, host_loop=1)])
def test_single_view_matches_megakernel(ctx, mode, rr, opts):
    sc = _box_variant("materials")
    s = api.Scene(ctx, sc["verts"], sc["mat_idx"], sc["mats"]).build()
    st = api.make_settings(40, 30, 6, max_bounces=8, rr_depth=rr, mode=mode, seed=21, aspect=40 / 30)
    try:
        ref = _mega(ctx, s, sc["camera"], st)
        f = api.Film(ctx, 40, 30, f64=True)
        ctx.check(api.render_batch([s], [(0, sc["camera"], st)], [f], opts))
        assert f.spp == 6
        _same(f.download(f64=True), ref)
        f.close()
    finally:
        s.close()


def test_batch_of_uneven_views_and_scenes(ctx):
    a = _box_variant("plain")
    b = _box_variant("materials")
    sa = api.Scene(ctx, a["verts"], a["mat_idx"], a["mats"]).build()
    sb = api.Scene(ctx, b["verts"], b["mat_idx"], b["mats"]).build()
    sb.set_skybox(np.array([[[0.3, 0.4, 0.5, 1.0]]], np.float32))
    views = [
        (0, a["camera"], api.make_settings(32, 32, 4, 8, 3, 1, 1)),
        (1, dict(position=(0.5, 0.6, -1.2), rotation=(6.0, -4.0, 0.0), fov=50.0), api.make_settings(48, 20, 9, 10, 3, 1, 2, 48 / 20)),
        (0, a["camera"], api.make_settings(16, 24, 16, 6, 0, 0, 3)),
        (1, b["camera"], api.make_settings(8, 8, 33, 12, 4, 1, 4)),
    ]
    try:
        refs = [_mega(ctx, (sa, sb)[si], cam, st) for si, cam, st in views]
        counts = set()
        for fuse in (1, 2, 3):
            films = [api.Film(ctx, st.width, st.height, f64=True) for _, _, st in views]
            ctx.check(api.render_batch([sa, sb], views, films, dict(path_pool=2048, chunk_samples=4096, fuse=fuse,
                                                                     refill=(OFF, 4, 8)[fuse - 1])))
            for f, r in zip(films, refs):
                _same(f.download(f64=True), r)
                f.close()
            stats = api.batch_stats(ctx)
            assert stats["samples"] == sum(st.width * st.height * st.spp for _, _, st in views)
            assert stats["segments"] >= stats["samples"]
            counts.add((stats["segments"], stats["shadow_rays"]))
        assert len(counts) == 1, counts  # same rays traced at every fusion level
    finally:
        sa.close()
        sb.close()


@pytest.mark.parametrize("refill", [OFF, 8])
def test_faithful_sun_matches_megakernel(ctx, refill):
    """Sun requests (closest hits stepping past alpha-zero surfaces) keep the
    static shadow stage even when per-lane refill is asked for."""
    sc = _box_variant("materials")
    s = api.Scene(ctx, sc["verts"], sc["mat_idx"], sc["mats"]).build()
    s.set_sun(True, dict(direction=(0.3, -1.0, 0.2)))
    st = api.make_settings(32, 24, 5, max_bounces=6, rr_depth=0, mode=0, seed=4, aspect=32 / 24)
    try:
        ref = _mega(ctx, s, sc["camera"], st)
        assert ref["sum"].sum() > 0
        f = api.Film(ctx, 32, 24, f64=True)
        ctx.check(api.render_batch([s], [(0, sc["camera"], st)], [f], dict(refill=refill, path_pool=700)))
        _same(f.download(f64=True), ref)
        f.close()
    finally:
        s.close()


def test_accumulates_after_megakernel_passes(ctx):
    """A film that already holds megakernel samples continues with the next
    sample indices, exactly like a further megakernel pass."""
    sc = _box_variant("plain")
    s = api.Scene(ctx, sc["verts"], sc["mat_idx"], sc["mats"]).build()
    st = api.make_settings(24, 24, 3, 8, 3, 1, 5)
    try:
        ref = _mega(ctx, s, sc["camera"], st, passes=2)
        f = api.Film(ctx, 24, 24, f64=True)
        api.render(s, sc["camera"], st, f)
        ctx.check(api.render_batch([s], [(0, sc["camera"], st)], [f]))
        assert f.spp == 6
        _same(f.download(f64=True), ref)
        f.close()
    finally:
        s.close()


def test_iteration_cap_times_out_and_context_survives(ctx):
    sc = _box_variant("plain")
    s = api.Scene(ctx, sc["verts"], sc["mat_idx"], sc["mats"]).build()
    st = api.make_settings(32, 32, 8, 8, 3, 1, 6)
    try:
        f = api.Film(ctx, 32, 32)
        rc = api.render_batch([s], [(0, sc["camera"], st)], [f], dict(max_iterations=3))
        assert rc == 4  # CRG_ERR_TIMEOUT
        f.close()
        # the context still renders
        ref = _mega(ctx, s, sc["camera"], st)
        g = api.Film(ctx, 32, 32, f64=True)
        ctx.check(api.render_batch([s], [(0, sc["camera"], st)], [g]))
        _same(g.download(f64=True), ref)
        g.close()
    finally:
        s.close()


def test_displaced_scene_small(ctx, orc):
    """The displaced-icosphere scene (4,195,280 + 1,282 triangles): megakernel
    bit-identical to the oracle and to the wavefront at a small resolution."""
    sc = scenes.displaced_scene()
    s = api.Scene(ctx, sc["verts"], sc["mat_idx"], sc["mats"]).build()
    s.set_skybox(sc["skybox"])
    st = api.make_settings(24, 14, 2, 16, 3, 1, 7, 24 / 14)
    try:
        ref = _mega(ctx, s, sc["camera"], st)
        f = api.Film(ctx, 24, 14, f64=True)
        ctx.check(api.render_batch([s], [(0, sc["camera"], st)], [f]))
        _same(f.download(f64=True), ref)
        f.close()
    finally:
        s.close()
    o = orc.render(sc, sc["camera"], st, skybox=sc["skybox"])
    _same(ref, o)
    assert np.isfinite(ref["sum"]).all() and ref["sum"].mean() > 0


def test_autotune_picks_options_that_render_identically(ctx):
    """The autotuner's trials run on scratch films; its pick (and the BVH width
    it leaves the scenes at) renders the same films as the megakernel; a
    second call for the same batch shape is answered from the cache."""
    a = _box_variant("plain")
    b = _box_variant("materials")
    sa = api.Scene(ctx, a["verts"], a["mat_idx"], a["mats"]).build(8, 1)
    sb = api.Scene(ctx, b["verts"], b["mat_idx"], b["mats"]).build(8, 1)
    views = [(0, a["camera"], api.make_settings(64, 48, 16, 8, 3, 1, 1, 64 / 48)),
             (1, b["camera"], api.make_settings(32, 32, 64, 10, 3, 1, 2)),
             (0, a["camera"], api.make_settings(40, 40, 8, 6, 0, 0, 3))]
    try:
        opts, width, trials = api.autotune_batch([sa, sb], views, sample_budget=1 << 17, widths=4 | 8)
        assert width in (4, 8) and sa.info()["width"] == width and sb.info()["width"] == width
        assert len(trials) >= 7 and all(t["ms"] > 0 for t in trials)
        fastest = min(trials, key=lambda t: t["ms"])
        assert fastest["width"] == width
        assert all(fastest[k] == opts[k] for k in ("fuse", "refill", "fetch", "block_size", "path_pool"))
        refs = [_mega(ctx, (sa, sb)[si], cam, st) for si, cam, st in views]
        films = [api.Film(ctx, st.width, st.height, f64=True) for _, _, st in views]
        ctx.check(api.render_batch([sa, sb], views, films, opts))
        for f, r in zip(films, refs):
            _same(f.download(f64=True), r)
            f.close()
        again, width2, trials2 = api.autotune_batch([sa, sb], views, sample_budget=1 << 17, widths=4 | 8)
        assert again == opts and width2 == width and trials2 == []
    finally:
        sa.close()
        sb.close()


def test_autotune_leaf_sizes(ctx):
    """With leaves set, the autotuner also picks each scene's leaf size, leaves
    the scenes built with it, and renders identical films; a cached answer
    rebuilds scenes whose leaf size has been changed since."""
    a = _box_variant("plain")
    b = _box_variant("materials")
    sa = api.Scene(ctx, a["verts"], a["mat_idx"], a["mats"]).build(8, 1)
    sb = api.Scene(ctx, b["verts"], b["mat_idx"], b["mats"]).build(8, 1)
    views = [(0, a["camera"], api.make_settings(48, 48, 16, 8, 3, 1, 1)),
             (1, b["camera"], api.make_settings(32, 32, 32, 8, 3, 1, 2))]
    leaves = (1 << 1) | (1 << 2) | (1 << 3)
    try:
        opts, width, trials = api.autotune_batch([sa, sb], views, sample_budget=1 << 16, widths=8, leaves=leaves)
        la, lb = sa.info()["leaf_max"], sb.info()["leaf_max"]
        assert la in (1, 2, 3) and lb in (1, 2, 3)
        assert len(trials) >= 1 + 2 + 2  # defaults, two more leaf sizes per scene
        refs = [_mega(ctx, (sa, sb)[si], cam, st) for si, cam, st in views]
        films = [api.Film(ctx, st.width, st.height, f64=True) for _, _, st in views]
        ctx.check(api.render_batch([sa, sb], views, films, opts))
        for f, r in zip(films, refs):
            _same(f.download(f64=True), r)
            f.close()
        sa.build(8, 1, 3 if la != 3 else 1)
        again, width2, trials2 = api.autotune_batch([sa, sb], views, sample_budget=1 << 16, widths=8, leaves=leaves)
        assert again == opts and trials2 == [] and sa.info()["leaf_max"] == la
    finally:
        sa.close()
        sb.close()


def test_autotune_cache_file(ctx, tmp_path):
    """The autotuner's answers survive the process: saved to a file, loaded by
    a fresh context, they answer the same batch shape without trials (scenes
    rebuilt at the saved width and leaf sizes); a file from another kind of
    device reads nothing; a malformed file is refused and adds nothing."""
    a = _box_variant("plain")
    views = [(0, a["camera"], api.make_settings(48, 48, 16, 8, 3, 1, 1))]
    leaves = (1 << 1) | (1 << 2) | (1 << 3)
    path = str(tmp_path / "tune.txt")
    sa = api.Scene(ctx, a["verts"], a["mat_idx"], a["mats"]).build(8, 1)
    try:
        opts, width, _ = api.autotune_batch([sa], views, sample_budget=1 << 15, widths=4 | 8, leaves=leaves)
        leaf = sa.info()["leaf_max"]
        api.autotune_cache_save(ctx, path)
    finally:
        sa.close()
    text = open(path).read().splitlines()
    assert text[0] == "crg-autotune-cache 1" and text[1].startswith("device ") and len(text) >= 3
    ctx2 = api.Context(0)
    try:
        assert api.autotune_cache_load(ctx2, path) == len(text) - 2
        s2 = api.Scene(ctx2, a["verts"], a["mat_idx"], a["mats"]).build(2 if width != 2 else 4, 1, 3)
        try:
            again, width2, trials = api.autotune_batch([s2], views, sample_budget=1 << 15, widths=4 | 8, leaves=leaves)
            assert trials == [] and again == opts and width2 == width
            assert s2.info()["width"] == width and s2.info()["leaf_max"] == leaf
        finally:
            s2.close()
        other = tmp_path / "other.txt"
        other.write_text("\n".join([text[0], "device Some_Other_GPU|8"] + text[2:]) + "\n")
        assert api.autotune_cache_load(ctx2, str(other)) == 0
        bad = tmp_path / "bad.txt"
        bad.write_text("\n".join(text[:2] + ["shape-without-fields"]) + "\n")
        with pytest.raises(CrgError):
            api.autotune_cache_load(ctx2, str(bad))
        with pytest.raises(CrgError):
            api.autotune_cache_load(ctx2, str(tmp_path / "missing.txt"))
    finally:
        ctx2.close()


@pytest.mark.parametrize("fuse", [1, 2])
def test_stage_timing_and_shadow_work_split(ctx, fuse):
    """host_loop 2 times every stage with CUDA events (crg_batch_stage_times_get)
    and renders the megakernel's film; with count_work the shadow stage's share
    of the traversal work is reported apart from the closest hits'."""
    sc = scenes.box_scene()
    s = api.Scene(ctx, sc["verts"], sc["mat_idx"], sc["mats"]).build(8, 1)
    st = api.make_settings(64, 48, 8, 8, 3, 1, 11, 64 / 48)
    f = api.Film(ctx, st.width, st.height, f64=True)
    ctx.check(api.render_batch([s], [(0, sc["camera"], st)], [f], dict(host_loop=2, count_work=1, fuse=fuse,
                                                                       path_pool=4096)))
    work, t = api.batch_stats(ctx), api.stage_times(ctx)
    _same(f.download(f64=True), _mega(ctx, s, sc["camera"], st))
    assert 0 < t["shadow_nodes"] < work["nodes_visited"] and 0 < t["shadow_tris"] < work["tris_tested"]
    assert t["iterations"] >= work["iterations"] - 8
    assert t["extend_ms"] > 0 and t["shade_ms"] > 0 and t["other_ms"] > 0
    assert (t["shadow_ms"] > 0) == (fuse == 1)  # fuse 2 tests the shadow rays inside shade
    ctx.check(api.render_batch([s], [(0, sc["camera"], st)], [f], dict(path_pool=4096)))
    assert api.stage_times(ctx)["extend_ms"] == 0  # only host_loop 2 times stages
    f.close()
    s.close()


def test_async_batches_overlap_the_host_and_match_the_synchronous_form(ctx):
    """crg_render_batch_async returns once the batch is enqueued: two batches in
    a row on one stream leave the stream busy when the second call returns,
    crg_batch_wait then reports success, and the films equal those of the
    synchronous form (the cached graph relaunched with a new plan)."""
    import ctypes as C
    import time

    from test_zz_no_alloc import _cudart

    rt = _cudart()
    sc = scenes.box_scene()
    s = api.Scene(ctx, sc["verts"], sc["mat_idx"], sc["mats"]).build(8, 1, 3)
    sts = [api.make_settings(512, 512, 32, 8, 3, 1, 21 + k) for k in range(2)]
    ref = []
    for st in sts:
        f = api.Film(ctx, 512, 512)
        ctx.check(api.render_batch([s], [(0, sc["camera"], st)], [f]))
        ref.append(f.download()["sum"])
        f.close()
    films = [api.Film(ctx, 512, 512) for _ in sts]
    assert rt.cudaDeviceSynchronize() == 0
    t0 = time.perf_counter()
    for st, f in zip(sts, films):
        ctx.check(api.render_batch([s], [(0, sc["camera"], st)], [f], wait=False))
    enqueue_s = time.perf_counter() - t0
    busy = rt.cudaStreamQuery(None)
    assert api.batch_wait(ctx) == 0
    assert busy == 600, busy  # cudaErrorNotReady: the host returned while the GPU was rendering
    for f, r in zip(films, ref):
        assert np.array_equal(f.download()["sum"].view(np.uint32), r.view(np.uint32))
        f.close()
    assert enqueue_s < 1.0
    s.close()


def test_async_errors_arrive_with_the_wait(ctx):
    sc = scenes.box_scene()
    s = api.Scene(ctx, sc["verts"], sc["mat_idx"], sc["mats"]).build(8, 1)
    st = api.make_settings(64, 64, 16, 8, 3, 1, 5)
    f = api.Film(ctx, 64, 64)
    assert api.render_batch([s], [(0, sc["camera"], st)], [f], dict(max_iterations=2, path_pool=256), wait=False) == 0
    assert api.batch_wait(ctx) == 4  # CRG_ERR_TIMEOUT, found on the device
    assert b"iteration cap" in ctx.lib.crg_last_error_string(ctx.h)
    assert api.batch_wait(ctx) == 0  # reported once
    f.reset()
    ctx.check(api.render_batch([s], [(0, sc["camera"], st)], [f]))
    assert np.array_equal(f.download()["sum"].view(np.uint32), _mega(ctx, s, sc["camera"], st)["sum"].view(np.uint32))
    f.close()
    s.close()


def test_small_batch_call_overhead(ctx, capsys):
    """Per-call cost of a small batch (one 64x64 view, 1 spp): the synchronous
    call against enqueueing alone; the loop's graph is instantiated once and
    relaunched by every later call of the same shape."""
    import time

    sc = scenes.box_scene()
    s = api.Scene(ctx, sc["verts"], sc["mat_idx"], sc["mats"]).build(8, 1)
    st = api.make_settings(64, 64, 1, 8, 3, 1, 5)
    f = api.Film(ctx, 64, 64)
    view = [(0, sc["camera"], st)]
    for _ in range(3):
        ctx.check(api.render_batch([s], view, [f]))
    n = 50
    t0 = time.perf_counter()
    for _ in range(n):
        ctx.check(api.render_batch([s], view, [f]))
    sync_us = (time.perf_counter() - t0) / n * 1e6
    # the host's own cost of an enqueue, with the device idle (a long run of enqueues
    # is paced by the device once the host is two batches ahead)
    enq = []
    for _ in range(n):
        assert api.batch_wait(ctx) == 0
        t0 = time.perf_counter()
        ctx.check(api.render_batch([s], view, [f], wait=False))
        enq.append(time.perf_counter() - t0)
    assert api.batch_wait(ctx) == 0
    enq_us = float(np.median(enq)) * 1e6
    with capsys.disabled():
        print(f"\nsmall batch: {sync_us:.0f} us per synchronous call, {enq_us:.0f} us of host time per enqueue")
    assert enq_us < sync_us
    f.close()
    s.close()
