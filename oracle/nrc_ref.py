"""CPU restatement of the radiance cache (test infrastructure only).

float64 numpy model of what rustracer_gb300/csrc/nrc.cu computes: the
multiresolution hash-grid encoding (16 levels, 2 features, trilinear) of a
position normalised to the cache box, the MLP 32 -> 5 x 64 (ReLU) -> 3
without biases, the relative L2 loss mean((y - t)^2 / (y^2 + 0.01)) with y
held constant in the denominator, and its exact gradients with respect to
the weights and the table (manual backpropagation; checked against finite
differences in tests).  The cache has no counterpart in the reference, so
there is nothing to pin it to beyond its own published definition
(Mueller et al. 2022 encoding, Mueller et al. 2021 loss): parity with the
GPU is the check.

loss_and_grads(..., bf16=True) follows the library's tensor-core training:
every matrix operand (encoding, activations, weights, dL/dy and the
pre-activation gradients) is rounded to BF16 (round to nearest even) where
the kernels round it, and the products are summed in float64.
"""
import numpy as np

LEVELS, FEAT, HIDDEN, LAYERS, OUT = 16, 2, 64, 5, 3
PRIMES = (1, 2654435761, 805459861)


def level_table(base, growth, log2_table):
    """(scale, dense resolution or 0) per level, rounded like the library:
    scale computed in double from the float32 growth factor, then stored as
    float32."""
    T = 1 << log2_table
    growth = float(np.float32(growth))  # the C ABI passes the growth factor as a float
    out = []
    for l in range(LEVELS):
        s = np.float32(base * growth ** l - 1.0)
        res = np.ceil(np.float64(s)) + 2.0
        out.append((s, int(res) if res ** 3 <= T else 0))
    return out


def encode_corners(p01, levels, log2_table):
    """Per point, level and corner: flat table entry index and weight.
    p01: (n, 3) float32 in [0, 1].  Returns idx (n, L, 8) int64, w (n, L, 8)."""
    T = 1 << log2_table
    n = len(p01)
    idx = np.zeros((n, LEVELS, 8), np.int64)
    w = np.zeros((n, LEVELS, 8), np.float64)
    p = p01.astype(np.float32)
    for l, (s, res) in enumerate(levels):
        # g = fmaf(p, s, 0.5): the float32 product is exact in float64, so one
        # rounding of the float64 sum reproduces the fused multiply-add
        g = (p.astype(np.float64) * np.float64(s) + 0.5).astype(np.float32)
        f = np.floor(g)
        t = (g - f).astype(np.float64)
        c0 = f.astype(np.int64)
        for c in range(8):
            b = np.array([(c >> 0) & 1, (c >> 1) & 1, (c >> 2) & 1])
            xyz = (c0 + b).astype(np.uint64)
            if res:
                k = xyz[:, 0] + xyz[:, 1] * res + xyz[:, 2] * res * res
            else:
                k = (xyz[:, 0] * np.uint64(PRIMES[0])) ^ (xyz[:, 1] * np.uint64(PRIMES[1]) & np.uint64(0xFFFFFFFF)) \
                    ^ (xyz[:, 2] * np.uint64(PRIMES[2]) & np.uint64(0xFFFFFFFF))
                k = k & np.uint64(T - 1)
            idx[:, l, c] = l * T + k.astype(np.int64)
            w[:, l, c] = np.prod(np.where(b == 1, t, 1.0 - t), axis=1)
    return idx, w


def unpack_mlp(flat):
    flat = np.asarray(flat, np.float64)
    Ws, off = [], 0
    for l in range(LAYERS + 1):
        i = 32 if l == 0 else HIDDEN
        o = OUT if l == LAYERS else HIDDEN
        Ws.append(flat[off:off + o * i].reshape(o, i))
        off += o * i
    return Ws


def forward(mlp_flat, grid, p01, levels, log2_table):
    """Returns y (n, 3) and the cache of intermediate values."""
    idx, w = encode_corners(p01, levels, log2_table)
    g2 = np.asarray(grid, np.float64).reshape(-1, 2)
    x = np.einsum("nlc,nlcf->nlf", w, g2[idx]).reshape(len(p01), 32)
    Ws = unpack_mlp(mlp_flat)
    hs = [x]
    h = x
    for l in range(LAYERS):
        h = np.maximum(h @ Ws[l].T, 0.0)
        hs.append(h)
    y = h @ Ws[LAYERS].T
    return y, (idx, w, hs, Ws)


def bf16(x):
    """Rounds to BF16 (nearest even) through float32, returned as float64."""
    f = np.asarray(x, np.float64).astype(np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def forward_bf16(mlp_flat, grid, p01, levels, log2_table):
    """The forward pass with BF16 operands: H_0 = bf16(encoding), H_{l+1} =
    bf16(relu(H_l bf16(W_l)^T)), y = H_5 bf16(W_5)^T."""
    idx, w = encode_corners(p01, levels, log2_table)
    g2 = np.asarray(grid, np.float64).reshape(-1, 2)
    x = np.einsum("nlc,nlcf->nlf", w, g2[idx]).reshape(len(p01), 32)
    Ws = [bf16(W) for W in unpack_mlp(mlp_flat)]
    hs = [bf16(x)]
    for l in range(LAYERS):
        hs.append(bf16(np.maximum(hs[-1] @ Ws[l].T, 0.0)))
    y = hs[LAYERS] @ Ws[LAYERS].T
    return y, (idx, w, hs, Ws)


def loss_and_grads(mlp_flat, grid, p01, target, levels, log2_table, bf16_ops=False):
    if bf16_ops:
        return _loss_and_grads_bf16(mlp_flat, grid, p01, target, levels, log2_table)
    y, (idx, w, hs, Ws) = forward(mlp_flat, grid, p01, levels, log2_table)
    n = len(p01)
    t = np.asarray(target, np.float64)[:, :3]
    d = y - t
    den = y * y + 0.01
    loss = float(np.sum(d * d / den) / (n * 3))
    dy = 2.0 * d / den / (3 * n)
    gW = [None] * (LAYERS + 1)
    gW[LAYERS] = dy.T @ hs[LAYERS]
    dz = (dy @ Ws[LAYERS]) * (hs[LAYERS] > 0)
    for l in range(LAYERS - 1, 0, -1):
        gW[l] = dz.T @ hs[l]
        dz = (dz @ Ws[l]) * (hs[l] > 0)
    gW[0] = dz.T @ hs[0]
    dx = (dz @ Ws[0]).reshape(n, LEVELS, 2)
    ggrid = np.zeros(np.asarray(grid).size, np.float64).reshape(-1, 2)
    np.add.at(ggrid, idx.reshape(-1), (w[..., None] * dx[:, :, None, :]).reshape(-1, 2))
    return loss, np.concatenate([g.reshape(-1) for g in gW]), ggrid.reshape(-1)


def _loss_and_grads_bf16(mlp_flat, grid, p01, target, levels, log2_table):
    y, (idx, w, hs, Ws) = forward_bf16(mlp_flat, grid, p01, levels, log2_table)
    n = len(p01)
    t = np.asarray(target, np.float64)[:, :3]
    d = y - t
    den = y * y + 0.01
    loss = float(np.sum(d * d / den) / (n * 3))
    dy = bf16(2.0 * d / den / (3 * n))
    gW = [None] * (LAYERS + 1)
    gW[LAYERS] = dy.T @ hs[LAYERS]
    dz = bf16((dy @ Ws[LAYERS]) * (hs[LAYERS] > 0))
    for l in range(LAYERS - 1, 0, -1):
        gW[l] = dz.T @ hs[l]
        dz = bf16((dz @ Ws[l]) * (hs[l] > 0))
    gW[0] = dz.T @ hs[0]
    dx = (dz @ Ws[0]).reshape(n, LEVELS, 2)
    ggrid = np.zeros(np.asarray(grid).size, np.float64).reshape(-1, 2)
    np.add.at(ggrid, idx.reshape(-1), (w[..., None] * dx[:, :, None, :]).reshape(-1, 2))
    return loss, np.concatenate([g.reshape(-1) for g in gW]), ggrid.reshape(-1)


def surrogate_loss(mlp_flat, grid, p01, target, levels, log2_table, y0):
    """The loss with the denominator's y fixed to y0: its exact derivative is
    the gradient loss_and_grads returns (for finite-difference checks)."""
    y, _ = forward(mlp_flat, grid, p01, levels, log2_table)
    t = np.asarray(target, np.float64)[:, :3]
    return float(np.sum((y - t) ** 2 / (y0 * y0 + 0.01)) / (len(p01) * 3))
