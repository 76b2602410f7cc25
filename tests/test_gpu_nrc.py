"""Radiance cache on the GPU vs the float64 oracle (oracle/nrc_ref.py).

* queries (FP16 table, BF16 tensor-core MLP with FP32 accumulation) agree
  with the float64 forward within 3% of the output scale, on tcgen05 (the
  default) and on mma.sync, and the two agree with each other within 1%;
* the tensor-core training pass (BF16 operands, FP32 accumulation) gives
  the loss and gradients of the oracle run with the same BF16 roundings
  (1e-3 relative L2 per block), and stands no further from the exact
  float64 gradients than that BF16 oracle does (the operand precision);
* the FP32 training pass (GBRT_NRC_TRAIN_FP32) gives the oracle's loss
  (1e-4 relative) and its gradients: per layer and for the table, 1e-3
  relative L2 error and every entry within 1e-3 of the block's largest
  gradient;
* one Adam step from zero moments moves every parameter with a non-zero
  gradient by -lr * sign(g);
* online training on a smooth target field lowers the loss 10x.
"""
import numpy as np
import pytest

import nrc_ref as N

pytestmark = pytest.mark.gpu

LOG2T, BASE, GROWTH = 12, 16, 1.447
LO, HI = (-1.0, -2.0, -1.5), (3.0, 2.0, 2.5)


def _cache(gpu_ctx, lr=1e-2, flags=0):
    from rustracer_gb300 import gbrt
    return gbrt.Nrc(gpu_ctx, LO, HI, log2_table=LOG2T, base_resolution=BASE, growth=GROWTH, learning_rate=lr,
                    flags=flags)


def _random_params(rng):
    fan = np.repeat([np.sqrt(6 / 32)] + [np.sqrt(6 / 64)] * 5, [2048, 4096, 4096, 4096, 4096, 192])
    mlp = (rng.uniform(-1, 1, 18624) * fan).astype(np.float32)
    grid = rng.uniform(-0.5, 0.5, 16 * (1 << LOG2T) * 2).astype(np.float32)
    return mlp, grid


def _points(rng, n):
    lo, hi = np.array(LO), np.array(HI)
    return (lo + rng.random((n, 3)) * (hi - lo)).astype(np.float32)


def _p01(pos):
    lo, hi = np.array(LO, np.float32), np.array(HI, np.float32)
    inv = (np.float32(1.0) / (hi - lo)).astype(np.float32)
    return np.clip((pos - lo) * inv, 0, 1).astype(np.float32)


@pytest.mark.parametrize("flags", [0, 1], ids=["tcgen05", "mma_sync"])
@pytest.mark.parametrize("n", [5000, 1, 128])
def test_query_matches_oracle(gpu_ctx, flags, n):
    rng = np.random.default_rng(3)
    c = _cache(gpu_ctx, flags=flags)
    mlp, grid = _random_params(rng)
    c.set_params(mlp, grid)
    pos = _points(rng, 5000)
    ref, _ = N.forward(mlp, grid, _p01(pos), N.level_table(BASE, GROWTH, LOG2T), LOG2T)
    scale = np.abs(ref).max()  # of the 5000 points, so that n = 1 and 128 are compared on the same scale
    y = c.query(pos[:n])
    err = np.abs(y - ref[:n])
    assert np.all(np.isfinite(y))
    assert err.max() <= 0.03 * scale, (err.max(), scale)
    assert np.median(err) <= 0.005 * scale


def test_tcgen05_matches_mma_sync(gpu_ctx):
    """Both tensor-core paths over many tiles per CTA and a ragged last tile."""
    from rustracer_gb300 import gbrt
    rng = np.random.default_rng(11)
    mlp, grid = _random_params(rng)
    pos = _points(rng, 152 * 4 * 128 * 3 + 77)
    ys = []
    for flags in (0, gbrt.NRC_QUERY_MMA_SYNC):
        c = _cache(gpu_ctx, flags=flags)
        c.set_params(mlp, grid)
        ys.append(c.query(pos))
    scale = np.abs(ys[1]).max()
    assert np.all(np.isfinite(ys[0]))
    assert np.abs(ys[0] - ys[1]).max() <= 0.01 * scale


def test_tcgen05_follows_training(gpu_ctx):
    """The BF16 tcgen05 weight copy is refreshed by every Adam step."""
    from rustracer_gb300 import gbrt
    rng = np.random.default_rng(12)
    mlp, grid = _random_params(rng)
    pos = _points(rng, 4096)
    tgt = rng.random((4096, 3)).astype(np.float32)
    ys = []
    for flags in (0, gbrt.NRC_QUERY_MMA_SYNC):
        c = _cache(gpu_ctx, flags=flags)
        c.set_params(mlp, grid)
        for step in range(3):
            c.train(pos, tgt)
        ys.append(c.query(pos))
    scale = np.abs(ys[1]).max()
    assert np.abs(ys[0] - ys[1]).max() <= 0.01 * scale


def _kink_free(mlp, grid, pos, bf16_ops):
    """Samples whose pre-activations all sit away from the ReLU kink (1e-5
    of the layer's scale): FP32 and float64 may take different sides there."""
    lv = N.level_table(BASE, GROWTH, LOG2T)
    fwd = N.forward_bf16 if bf16_ops else N.forward
    _, (_, _, hs, Ws) = fwd(mlp, grid, _p01(pos), lv, LOG2T)
    keep = np.ones(len(pos), bool)
    for l in range(5):
        z = np.abs(hs[l] @ Ws[l].T)
        keep &= z.min(axis=1) > 1e-5 * z.max(axis=1)
    return keep


def _grad_blocks(gm, gg, rgm, rgg):
    bounds = [0, 2048, 6144, 10240, 14336, 18432, 18624]
    blocks = [(gm[a:b], rgm[a:b], f"W{k}") for k, (a, b) in enumerate(zip(bounds[:-1], bounds[1:]))]
    blocks.append((gg, rgg, "table"))
    return {name: (np.linalg.norm(g - r) / np.linalg.norm(r), np.abs(g - r).max() / np.abs(r).max())
            for g, r, name in blocks}


def test_tc_gradients_match_oracle(gpu_ctx):
    """Default training path: forward, backward and weight gradient on the
    tensor cores (mma.sync, BF16 operands, FP32 accumulation)."""
    rng = np.random.default_rng(14)
    c = _cache(gpu_ctx)
    mlp, grid = _random_params(rng)
    c.set_params(mlp, grid)
    pos = _points(rng, 5000)
    tgt = rng.random((5000, 3)).astype(np.float32)
    keep = _kink_free(mlp, grid, pos, True)
    assert keep.mean() > 0.9
    pos, tgt = pos[keep], tgt[keep]
    loss, gm, gg = c.train(pos, tgt, step=False, grads=True)
    lv = N.level_table(BASE, GROWTH, LOG2T)
    bl, bgm, bgg = N.loss_and_grads(mlp, grid, _p01(pos), tgt, lv, LOG2T, bf16_ops=True)
    assert abs(loss - bl) <= 1e-4 * abs(bl)
    errs = _grad_blocks(gm, gg, bgm, bgg)
    assert all(rel < 1e-3 and worst < 1e-2 for rel, worst in errs.values()), errs
    # against the exact float64 gradients: no further than the BF16-operand
    # oracle itself (the precision BF16 operands give), plus the 1e-3 above
    rl, rgm, rgg = N.loss_and_grads(mlp, grid, _p01(pos), tgt, lv, LOG2T)
    assert abs(loss - rl) <= 1e-2 * abs(rl)
    errs = _grad_blocks(gm, gg, rgm, rgg)
    prec = _grad_blocks(bgm, bgg, rgm, rgg)
    assert all(errs[k][0] <= 1.1 * prec[k][0] + 1e-3 for k in errs), (errs, prec)
    assert all(prec[k][0] < 0.1 for k in prec), prec


def test_gradients_match_oracle(gpu_ctx):
    from rustracer_gb300 import gbrt
    rng = np.random.default_rng(4)
    c = _cache(gpu_ctx, flags=gbrt.NRC_TRAIN_FP32)
    mlp, grid = _random_params(rng)
    c.set_params(mlp, grid)
    pos = _points(rng, 3000)
    tgt = rng.random((3000, 3)).astype(np.float32)
    keep = _kink_free(mlp, grid, pos, False)
    assert keep.mean() > 0.9
    pos, tgt = pos[keep], tgt[keep]
    loss, gm, gg = c.train(pos, tgt, step=False, grads=True)
    rl, rgm, rgg = N.loss_and_grads(mlp, grid, _p01(pos), tgt, N.level_table(BASE, GROWTH, LOG2T), LOG2T)
    assert abs(loss - rl) <= 1e-4 * abs(rl)
    # per layer and for the table: relative L2 error 1e-3, every entry within
    # 1e-3 of that block's largest gradient (FP32 sums over 3000 samples in
    # atomic order against float64)
    errs = _grad_blocks(gm, gg, rgm, rgg)
    assert all(rel < 1e-3 and worst < 1e-3 for rel, worst in errs.values()), errs


def test_adam_first_step(gpu_ctx):
    rng = np.random.default_rng(5)
    lr = 1e-3
    c = _cache(gpu_ctx, lr=lr)
    mlp, grid = _random_params(rng)
    c.set_params(mlp, grid)
    pos = _points(rng, 2000)
    tgt = rng.random((2000, 3)).astype(np.float32)
    _, gm, gg = c.train(pos, tgt, step=True, grads=True)
    m2, g2 = c.params()
    for w0, w1, g in ((mlp, m2, gm), (grid, g2, gg)):
        moved = np.abs(g) > 1e-12
        np.testing.assert_allclose(w1[moved], w0[moved] - lr * np.sign(g[moved]), rtol=0, atol=2e-6)
        assert np.array_equal(w1[~moved], w0[~moved])


def test_training_fits_smooth_field(gpu_ctx):
    rng = np.random.default_rng(6)
    c = _cache(gpu_ctx, lr=1e-2)

    def field(p):
        return np.stack([0.6 + 0.4 * np.sin(1.5 * p[:, 0]), 0.5 + 0.3 * np.cos(p[:, 1] + p[:, 2]),
                         0.4 + 0.2 * p[:, 2] / 2.5], 1).astype(np.float32)

    test = _points(rng, 4096)
    first = None
    for k in range(300):
        pos = _points(rng, 1 << 14)
        loss = c.train(pos, field(pos))
        first = loss if first is None else first
    assert loss < first / 10, (first, loss)
    err = np.abs(c.query(test) - field(test))
    assert np.mean(err) < 0.05


def _scene_box(sd, pad=0.05):
    p = sd.vertices["pos"][:, :3]
    lo, hi = p.min(0) - pad, p.max(0) + pad
    return tuple(map(float, lo)), tuple(map(float, hi))


def test_render_disabled_equals_path_tracing(gpu_ctx):
    """With no path stopping at the cache, gbrt_render_nrc is the plain
    wavefront render bit for bit (the training snapshots change nothing)."""
    from rustracer_gb300 import gbrt, scenes
    sd = scenes.icosphere_scene(subdiv=3)
    sc = gbrt.Scene(gpu_ctx, sd)
    lo, hi = _scene_box(sd)
    c = gbrt.Nrc(gpu_ctx, lo, hi, log2_table=16)
    ubo = sd.ubo(96, 64, samples=4, bounces=8, exposure=1.0)
    a1, a2 = gbrt.Accum(gpu_ctx, 96, 64), gbrt.Accum(gpu_ctx, 96, 64)
    ref = sc.render(ubo, a1, mode=gbrt.MODE_WAVEFRONT)
    r = c.render(sc, ubo, a2, disabled=True, train_samples=4096)
    assert np.array_equal(r["image"], ref["image"])
    assert np.array_equal(a1.download(), a2.download())
    assert r["loss"] > 0


def _relmse(x, ref):
    return float(np.mean((x - ref) ** 2 / (ref ** 2 + 1e-2)))


def test_render_with_cache_converges(gpu_ctx):
    """Icosphere scene (point lights, so next-event estimation carries the
    direct light), 1 spp per frame, 128x128: the running mean of 64 frames
    that stop at the cache after the first bounce is closer to a 2048-spp
    path-traced reference than 64 plain path-traced frames, and the cache's
    loss falls while it trains."""
    from rustracer_gb300 import gbrt, scenes
    sd = scenes.icosphere_scene(subdiv=4)
    sc = gbrt.Scene(gpu_ctx, sd)
    W, H = 128, 128
    ref_acc = gbrt.Accum(gpu_ctx, W, H)
    sc.render(sd.ubo(W, H, samples=2048, bounces=8, exposure=1.0), ref_acc, image=False, mode=gbrt.MODE_WAVEFRONT)
    ref = ref_acc.download()[..., :3] / 2048.0
    lo, hi = _scene_box(sd)
    c = gbrt.Nrc(gpu_ctx, lo, hi, log2_table=16, learning_rate=1e-3)
    acc_c, acc_p = gbrt.Accum(gpu_ctx, W, H), gbrt.Accum(gpu_ctx, W, H)
    losses = []
    for f in range(64):
        u = sd.ubo(W, H, samples=1, total=f + 1, bounces=8, exposure=1.0)
        losses.append(c.render(sc, u, acc_c, image=False, train_samples=4096, train_steps=4)["loss"])
        sc.render(u, acc_p, image=False, mode=gbrt.MODE_WAVEFRONT)
    img_c = acc_c.download()[..., :3] / 64.0
    img_p = acc_p.download()[..., :3] / 64.0
    assert np.all(np.isfinite(img_c))
    e_c, e_p = _relmse(img_c, ref), _relmse(img_p, ref)
    assert e_c < e_p, (e_c, e_p, losses[:3], losses[-3:])
    assert np.mean(losses[-10:]) < np.mean(losses[:5]) / 10


def test_primary_indirect_mode_converges(gpu_ctx):
    """GBRT_NRC_MODE_PRIMARY_INDIRECT on the icosphere scene, 128x128, 1 spp
    per frame: after 8 warm-up frames of plain path tracing that train the
    cache (disabled = 1), frames that shade the camera hit and take the rest
    of the path from the cache trace under 70% of the plain frames' rays,
    their running mean keeps converging towards a 2048-spp reference, and
    after 64 frames it is within 1.5x of the plain running mean's error (the
    cache's bias; on this scene the two measure within 5% of each other)."""
    from rustracer_gb300 import gbrt, scenes
    sd = scenes.icosphere_scene(subdiv=4)
    sc = gbrt.Scene(gpu_ctx, sd)
    W, H = 128, 128
    ref_acc = gbrt.Accum(gpu_ctx, W, H)
    sc.render(sd.ubo(W, H, samples=2048, bounces=8, exposure=1.0), ref_acc, image=False, mode=gbrt.MODE_WAVEFRONT)
    ref = ref_acc.download()[..., :3] / 2048.0
    lo, hi = _scene_box(sd)
    c = gbrt.Nrc(gpu_ctx, lo, hi, log2_table=16, learning_rate=1e-3)
    acc_c, acc_p = gbrt.Accum(gpu_ctx, W, H), gbrt.Accum(gpu_ctx, W, H)
    rays_c = rays_p = 0
    e16 = None
    for f in range(64):
        u = sd.ubo(W, H, samples=1, total=f + 1, bounces=8, exposure=1.0)
        r = c.render(sc, u, acc_c, image=False, train_samples=4096, train_steps=4, disabled=f < 8,
                     mode=gbrt.NRC_MODE_PRIMARY_INDIRECT)
        if f >= 8:
            rays_c += int(r["stats"]["rays_total"])
            rays_p += int(sc.render(u, acc_p, image=False, mode=gbrt.MODE_WAVEFRONT)["stats"]["rays_total"])
        else:
            sc.render(u, acc_p, image=False, mode=gbrt.MODE_WAVEFRONT)
        if f == 15:
            e16 = _relmse(acc_c.download()[..., :3] / 16.0, ref)
    img_c = acc_c.download()[..., :3] / 64.0
    img_p = acc_p.download()[..., :3] / 64.0
    assert np.all(np.isfinite(img_c))
    e_c, e_p = _relmse(img_c, ref), _relmse(img_p, ref)
    assert e_c < 0.6 * e16, (e16, e_c)
    assert e_c < 1.5 * e_p, (e_c, e_p)
    assert rays_c < 0.7 * rays_p, (rays_c, rays_p)


def test_query_device_buffers(gpu_ctx):
    """gbrt_nrc_query_device on framework tensors gives the host-buffer query's result."""
    import torch
    rng = np.random.default_rng(13)
    c = _cache(gpu_ctx)
    mlp, grid = _random_params(rng)
    c.set_params(mlp, grid)
    pos = _points(rng, 3001)
    y = c.query(pos)
    p4 = torch.zeros(len(pos), 4, device="cuda")
    p4[:, :3] = torch.from_numpy(pos).cuda()
    out = torch.empty_like(p4)
    torch.cuda.synchronize()
    ms = c.query_device(p4.data_ptr(), len(pos), out.data_ptr())
    assert ms >= 0.0
    np.testing.assert_array_equal(out[:, :3].cpu().numpy(), y)
