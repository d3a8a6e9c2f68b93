"""The native scene server (gsph_server_*): requests submitted while others
are stepped, admitted between chunks, retired at different frames; every
result equals the scene stepped alone, bit for bit. Also: submission from
another thread, rejection of a request larger than the capacity, stats."""
import threading

import numpy as np
import pytest

from gpu_helpers import dam_scene, shuffled

pytestmark = pytest.mark.gpu

SPECS = [(9, (0.5, 0.4, 0.4), 13), (12, (0.7, 0.5, 0.5), 8), (7, (0.3, 0.3, 0.4), 17),
         (14, (0.8, 0.5, 0.5), 6), (8, (0.4, 0.4, 0.4), 11), (10, (0.6, 0.4, 0.4), 3)]


def _requests(gsph):
    reqs = []
    for k, (n_side, box, frames) in enumerate(SPECS):
        _, p, pos = dam_scene(gsph, n_side=n_side, box=box, seed=40 + k)
        reqs.append((k, p, shuffled(pos, seed=k), frames))
    return reqs


def _alone(gsph, reqs):
    out = {}
    for rid, p, pos, frames in reqs:
        with gsph.HybridSystem(params=p, positions=pos) as h:
            h.step(frames)
            out[rid] = (h.copy_out(gsph.FIELD_POSITION), h.copy_out(gsph.FIELD_VELOCITY))
    return out


def test_native_server_results_identical_alone(gsph, cuda_device):
    reqs = _requests(gsph)
    alone = _alone(gsph, reqs)
    got = {}
    with gsph.NativeSceneServer(1 << 34, (200000, 400000, 4), chunk=4) as srv:
        pending = list(reqs)
        # two requests first, the rest arrive one per step
        for r in pending[:2]:
            srv.submit(r[0], r[1], r[2], r[3])
        pending = pending[2:]
        steps = 0
        while True:
            k = srv.step()
            got.update(srv.results())
            steps += 1
            if pending:
                r = pending.pop(0)
                srv.submit(r[0], r[1], r[2], r[3])
            elif k == 0 and srv.stats()["queued"] == 0 and srv.stats()["resident"] == 0:
                break
            assert steps < 1000
        st = srv.stats()
    assert sorted(got) == [r[0] for r in reqs]
    for rid, (pos, vel) in got.items():
        assert np.array_equal(pos.view(np.uint32), alone[rid][0].view(np.uint32)), rid
        assert np.array_equal(vel.view(np.uint32), alone[rid][1].view(np.uint32)), rid
    assert st["submitted"] == len(reqs) and st["finished"] == len(reqs)
    assert st["particle_steps"] == sum(len(r[2]) * r[3] for r in reqs)
    # capacity of 4 scenes: some requests waited, frames were shared
    assert st["frames"] < sum(r[3] for r in reqs)


def test_native_server_threads_and_rejection(gsph, cuda_device):
    reqs = _requests(gsph)
    alone = _alone(gsph, reqs[:3])
    big = reqs[3]   # 2,744 particles: larger than the particle capacity below
    with gsph.NativeSceneServer(1 << 34, (2000, 400000, 8), chunk=5) as srv:
        def client():
            for r in (reqs[0], big, reqs[1], reqs[2]):
                srv.submit(r[0], r[1], r[2], r[3])
        t = threading.Thread(target=client)
        t.start()
        got = {}
        for _ in range(200):
            srv.step()
            got.update(srv.results())
            st = srv.stats()
            if not t.is_alive() and st["queued"] == 0 and st["resident"] == 0:
                break
        t.join()
        st = srv.stats()
    assert st["rejected"] == 1
    assert sorted(got) == [reqs[0][0], reqs[1][0], reqs[2][0]]
    for rid, (pos, vel) in got.items():
        assert np.array_equal(pos.view(np.uint32), alone[rid][0].view(np.uint32)), rid


def test_native_server_spreads_over_batches(gsph, cuda_device):
    """Each batch's cell capacity holds about two of these scenes; with up to
    three batches the server keeps more scenes resident (stepped together on
    three streams) and every result still equals the scene stepped alone."""
    reqs = _requests(gsph)
    alone = _alone(gsph, reqs)
    cells = max(int(r[1].numc) for r in reqs)
    got = {}
    peak_batches = 0
    with gsph.NativeSceneServer(1 << 34, (200000, 2 * cells + 1, 8), chunk=4,
                                max_batches=3) as srv:
        for r in reqs:
            srv.submit(r[0], r[1], r[2], r[3])
        for _ in range(400):
            srv.step()
            got.update(srv.results())
            st = srv.stats()
            peak_batches = max(peak_batches, st["batches"])
            if st["queued"] == 0 and st["resident"] == 0:
                break
    assert peak_batches >= 2
    assert sorted(got) == [r[0] for r in reqs]
    for rid, (pos, vel) in got.items():
        assert np.array_equal(pos.view(np.uint32), alone[rid][0].view(np.uint32)), rid
        assert np.array_equal(vel.view(np.uint32), alone[rid][1].view(np.uint32)), rid
