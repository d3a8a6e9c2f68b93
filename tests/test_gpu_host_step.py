"""gsph_step_host_async: a step on host-resident state (upload the three
state arrays, run the frames, download them into the same arrays) gives the
same state, bit for bit, as stepping with the state resident on the device;
consecutive calls overlap one call's downloads with the next call's uploads,
and any other call on the handle waits for the downloads first."""
import numpy as np
import pytest

from gpu_helpers import dam_scene, dense_scene

pytestmark = pytest.mark.gpu

K = 6


def _fields(gsph):
    return (gsph.FIELD_POSITION, gsph.FIELD_VELOCITY, gsph.FIELD_EVAL_VELOCITY)


@pytest.mark.parametrize("builder", [lambda g: dam_scene(g, n_side=16),
                                     lambda g: dense_scene(g, n_side=20)],
                         ids=["sparse", "dense"])
@pytest.mark.parametrize("graph", [0, 2])
def test_host_steps_match_device_steps(gsph, cuda_device, builder, graph):
    import torch
    _, p, pos = builder(gsph)
    with gsph.HybridSystem(params=p, positions=pos) as h:
        h.set_graph_mode(graph)
        h.step(1)
        n = h.n
        host = [torch.empty((n, 4), dtype=torch.float32, pin_memory=True) for _ in range(3)]
        for t, f in zip(host, _fields(gsph)):
            t.numpy()[:] = h.copy_out(f)
        for _ in range(K):
            h.step_host_async(1 if graph == 0 else 2, *(t.data_ptr() for t in host))
        h.sync()
        got = [t.numpy().copy() for t in host]
        # the device state is the state downloaded last (another call joins
        # the pending downloads before it reads)
        dev = [h.copy_out(f) for f in _fields(gsph)]
    frames = 1 + K * (1 if graph == 0 else 2)
    with gsph.HybridSystem(params=p, positions=pos) as r:
        r.step(frames)
        ref = [r.copy_out(f) for f in _fields(gsph)]
    for a, b, c in zip(got, ref, dev):
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
        assert np.array_equal(c.view(np.uint32), b.view(np.uint32))


def test_host_step_rejects_bad_arguments(gsph, cuda_device):
    _, p, pos = dam_scene(gsph, n_side=8)
    with gsph.HybridSystem(params=p, positions=pos) as h:
        with pytest.raises(gsph.GsphError) as ei:
            h.step_host_async(1, 0, 0, 0)
        assert ei.value.status == gsph.ERR_INVALID_ARG
