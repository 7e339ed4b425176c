"""Batched and served forms: every frame's image equals the image the plain
per-frame entry point gives, alone or in a mix of concurrent requests."""
import numpy as np
import pytest

from contour3d_gb300 import workloads

pytestmark = pytest.mark.gpu


def _small_set(gpu, n=7, seed=7):
    import torch
    rng = np.random.default_rng(seed)
    fields, frames = [], []
    for q in range(n):
        shape = tuple(int(x) for x in rng.integers(24, 72, size=3))
        if q % 2 == 0:
            f = workloads.blobs_device(gpu, shape, int(rng.integers(3, 9)), seed=50 + q)
        else:
            f, _ = workloads.modes_device(gpu, shape, nmodes=24, kmin=1, kmax=6, seed=80 + q, dtype=torch.float32)
        fields.append(f)
        nlev = int(rng.integers(1, 4))
        frames.append(workloads.FrameSpec(q, workloads.quantile_levels(f, rng, nlev), workloads.PALETTE[:nlev],
                                          workloads.random_camera(rng), 160, 120))
    return fields, frames


def _single(gpu, fields, spec):
    import torch
    out = torch.zeros(spec.width * spec.height * 3, dtype=torch.uint8, device="cuda")
    assert gpu.render_pack(workloads.frame_pack(gpu, fields[spec.field], spec, out)) == 0
    torch.cuda.synchronize()
    return out.cpu().numpy()


@pytest.mark.parametrize("batch_classify", [True, False], ids=["one-classify-launch", "per-frame-classify"])
def test_batch_matches_single_frames(gpu, batch_classify):
    import torch
    fields, frames = _small_set(gpu)
    ref = [_single(gpu, fields, s) for s in frames]
    outs = [torch.zeros(s.width * s.height * 3, dtype=torch.uint8, device="cuda") for s in frames]
    packs = [workloads.frame_pack(gpu, fields[s.field], s, o) for s, o in zip(frames, outs)]
    gpu.set_batch_classify(batch_classify)
    try:
        ms = gpu.render_batch(packs, workers=3)
        torch.cuda.synchronize()
    finally:
        gpu.set_batch_classify(True)
    assert len(ms) == len(frames) and all(m > 0 for m in ms)
    for a, o in zip(ref, outs):
        assert np.array_equal(a, o.cpu().numpy())


def test_unsynchronised_workers_match_single_frames(gpu):
    """Worker contexts that render without per-pass synchronisation
    (contour3d_gb300_set_server_async): each context sizes a frame's buffers
    from the frames it rendered before, of other sizes, so overflows and
    frames rendered again are common; every image still equals the plain
    single-frame image."""
    import torch
    fields, frames = _small_set(gpu, n=12, seed=23)
    ref = [_single(gpu, fields, s) for s in frames]
    outs = [torch.zeros(s.width * s.height * 3, dtype=torch.uint8, device="cuda") for s in frames]
    packs = [workloads.frame_pack(gpu, fields[s.field], s, o) for s, o in zip(frames, outs)]
    assert gpu.lib.contour3d_gb300_set_server_async(1) == 0
    try:
        for _ in range(2):
            for o in outs:
                o.zero_()
            gpu.render_batch(packs, workers=3)
            torch.cuda.synchronize()
            for q, (a, o) in enumerate(zip(ref, outs)):
                assert np.array_equal(a, o.cpu().numpy()), f"frame {q}"
    finally:
        gpu.lib.contour3d_gb300_set_server_async(0)


def test_server_result_same_alone_and_in_the_mix(gpu):
    import torch
    fields, frames = _small_set(gpu, n=9, seed=11)
    ref = [_single(gpu, fields, s) for s in frames]
    target = 4
    with gpu.server(slots=4) as sv:
        out = torch.zeros(frames[target].width * frames[target].height * 3, dtype=torch.uint8, device="cuda")
        t = sv.submit(workloads.frame_pack(gpu, fields[target], frames[target], out))
        st_alone = sv.wait(t)
        torch.cuda.synchronize()
        alone = out.cpu().numpy()
        outs = [torch.zeros(s.width * s.height * 3, dtype=torch.uint8, device="cuda") for s in frames]
        order = np.random.default_rng(3).permutation(len(frames))
        tickets = {int(q): sv.submit(workloads.frame_pack(gpu, fields[frames[q].field], frames[q], outs[q]))
                   for q in order}
        stats = {q: sv.wait(t) for q, t in tickets.items()}
        torch.cuda.synchronize()
    assert np.array_equal(alone, ref[target])
    for q in range(len(frames)):
        assert np.array_equal(outs[q].cpu().numpy(), ref[q]), f"frame {q} differs in the mix"
        assert stats[q].latency_ms >= stats[q].queue_ms >= 0
    assert st_alone.latency_ms > 0


def test_server_admits_against_a_budget(gpu):
    """A budget that fits one request at a time serialises them; results stay exact."""
    import torch
    fields, frames = _small_set(gpu, n=5, seed=19)
    ref = [_single(gpu, fields, s) for s in frames]
    with gpu.server(slots=3, budget_bytes=1, resident_bytes=0) as sv:
        outs = [torch.zeros(s.width * s.height * 3, dtype=torch.uint8, device="cuda") for s in frames]
        ts = [sv.submit(workloads.frame_pack(gpu, fields[s.field], s, o)) for s, o in zip(frames, outs)]
        stats = [sv.wait(t) for t in ts]
        torch.cuda.synchronize()
    for q in range(len(frames)):
        assert np.array_equal(outs[q].cpu().numpy(), ref[q])
    # with one request admitted at a time, each later request waited for the earlier ones
    assert stats[-1].queue_ms >= 0 and all(s.estimate_bytes > 0 for s in stats)


def test_server_charges_buffer_growth_against_the_budget(gpu):
    """Buffer growth of running requests is charged against the budget when
    it is sized (the triangle buffers from each slab's triangle count): with a
    budget that holds about one and a half requests' buffers, the memory held
    stays within the budget except for growths that had to go ahead because
    every other running request was waiting (counted), and every image is
    still the plain path's."""
    import torch
    fields, frames = _small_set(gpu, n=8, seed=23)
    ref = [_single(gpu, fields, s) for s in frames]
    # one request's peak: run it alone on a one-slot server without a budget
    with gpu.server(slots=1) as sv:
        outs = [torch.zeros(s.width * s.height * 3, dtype=torch.uint8, device="cuda") for s in frames]
        held = [sv.wait(sv.submit(workloads.frame_pack(gpu, fields[s.field], s, o))).held_bytes
                for s, o in zip(frames, outs)]
        assert sv.memory().overcommits == 0
    budget = int(1.5 * max(held))
    with gpu.server(slots=4, budget_bytes=budget, resident_bytes=0) as sv:
        outs = [torch.zeros(s.width * s.height * 3, dtype=torch.uint8, device="cuda") for s in frames]
        ts = [sv.submit(workloads.frame_pack(gpu, fields[s.field], s, o)) for s, o in zip(frames, outs)]
        stats = [sv.wait(t) for t in ts]
        mem = sv.memory()
        torch.cuda.synchronize()
    for q in range(len(frames)):
        assert np.array_equal(outs[q].cpu().numpy(), ref[q])
    assert all(s.held_bytes > 0 for s in stats)
    # the invariant: above the budget only through counted go-aheads
    assert mem.peak_bytes <= budget or mem.overcommits > 0
    assert mem.used_bytes <= mem.peak_bytes
