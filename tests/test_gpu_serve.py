"""The request loop on the GPU: a deck's bases are the same when it is solved
alone and when it is solved among other decks of different sizes arriving
while it runs (continuous batching with overlapping work)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ACC = 1e-9
V = 1e4


def _board(seed, shape, n):
    from ion_gym_gb300.workloads import planar_board
    masks, box = planar_board(seed, shape=shape, n_electrodes=n)
    masks = {i: m for i, m in masks.items() if m.any()}
    masks[max(masks) + 1] = box
    return masks


def test_result_same_alone_and_in_the_mix():
    from ion_gym_gb300.serve import FieldServer
    target = _board(1, (96, 48, 40), 8)
    others = [_board(s, shp, k) for s, shp, k in
              [(2, (128, 64, 48), 12), (3, (64, 40, 32), 6),
               (4, (160, 64, 48), 16), (5, (96, 48, 40), 8)]]
    srv = FieldServer(workers=3)
    alone = srv.submit(target, V, ACC).result(timeout=300)
    futs = [srv.submit(o, V, ACC) for o in others[:2]]
    mixed = srv.submit({i: m.copy() for i, m in target.items()}, V, ACC)
    futs += [srv.submit(o, V, ACC) for o in others[2:]]
    in_mix = mixed.result(timeout=300)
    for f in futs:
        f.result(timeout=300)
    srv.close()
    assert sorted(alone) == sorted(in_mix)
    for i in alone:
        assert np.abs(alone[i] - in_mix[i]).max() <= ACC * V
        assert np.all(alone[i][target[i]] == V)
    lat = srv.latencies()
    assert len(lat) == 6 and all(t >= 0 for row in lat for t in row)


def test_device_results_match_host_results():
    """results="device" returns the same bases as CUDA tensors that stay in
    HBM (no device-to-host copy in the request)."""
    import torch
    from ion_gym_gb300.serve import FieldServer
    deck = _board(6, (80, 48, 40), 6)
    host = FieldServer(workers=1)
    ref = host.submit(deck, V, ACC).result(timeout=300)
    host.close()
    dev = FieldServer(workers=1, results="device")
    got = dev.submit(deck, V, ACC).result(timeout=300)
    dev.close()
    assert sorted(got) == sorted(ref)
    for i in ref:
        assert isinstance(got[i], torch.Tensor) and got[i].is_cuda
        assert np.array_equal(got[i].cpu().numpy(), ref[i])
