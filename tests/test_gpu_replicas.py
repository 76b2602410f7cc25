"""Replica correctness on one GPU: ranks that render the disjoint global
sample ranges of replicas.sample_range (as bench.py's replicas do) produce,
summed, the accumulation of one rank rendering all the samples.

Per-sample radiance depends only on the pixel and the global sample index
(deviation D1), so each replica's samples are bit-identical to the same
samples of the single run, and the summed accumulators agree up to the order
of the FP32 additions."""
import numpy as np
import pytest

from rustracer_gb300 import replicas, scenes

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("world", [2, 3])
def test_replica_ranges_sum_to_single_accumulation(gpu_ctx, world):
    from rustracer_gb300 import gbrt
    sd = scenes.icosphere_scene(subdiv=3)
    W, H, spp, steps = 64, 48, 4, 2
    sc = gbrt.Scene(gpu_ctx, sd)
    total = world * spp * steps
    single = gbrt.Accum(gpu_ctx, W, H)
    r1 = sc.render(sd.ubo(W, H, samples=total, total=total, bounces=8, exposure=1.0), single, want_samples=True)
    acc_sum = np.zeros((H, W, 4), np.float64)
    for rank in range(world):
        acc = gbrt.Accum(gpu_ctx, W, H)
        for k in range(steps):
            first, last = replicas.sample_range(rank, world, k, spp)
            r = sc.render(sd.ubo(W, H, samples=spp, total=last, bounces=8, exposure=1.0), acc, want_samples=True)
            # the replica's samples are the single run's samples [first, last), bit for bit
            assert np.array_equal(r["samples"].view(np.uint32), r1["samples"][:, first:last].view(np.uint32))
        acc_sum += acc.download().reshape(H, W, 4).astype(np.float64)
    ref = single.download().reshape(H, W, 4).astype(np.float64)
    assert ref[..., :3].sum() > 0
    # FP32 sums of `total` positive samples in two different orders
    np.testing.assert_allclose(acc_sum[..., :3], ref[..., :3], rtol=total * 2.0 ** -23, atol=1e-6)
