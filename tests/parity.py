"""The per-sample parity contract of the GPU render tests.

A GPU sample matches the oracle's when |a - b| <= 1e-4 * max(|a|, |b|) +
1e-6 in every channel.  A sample that does not match is EXPLAINED when the
oracle shows that its path is ill-conditioned at the ulp level:
  * a branch decision of the path sat within TAU_DECISION of its threshold
    (oracle margin[0]: Russian roulette, lobe choice, RIS acceptance, facing
    tests, TIR, MASK/BLEND opacity, sky face), or
  * a secondary hit lay within TAU_EDGE of a triangle edge (margin[1]), or
  * the oracle's own sample moves by more than 1e-4 (relative, with no
    absolute floor: a dark sample whose path changes under the nudges is as
    ill-conditioned as a bright one) when its transcendentals (sin, cos, pow,
    exp, log), shading divisions and square roots, dot products, lengths and
    normalised vectors are moved by a few ulps (CUDA's and libm's
    transcendentals, the shading kernels' approximate divisions and square
    roots, and fused against separate multiply-adds differ by that much);
    each nudge size and draw has its own signs, so several of each are
    tried (the oracle re-renders only the rows that hold candidates).
The contract: no unexplained mismatch, and at most FLIP_MAX of the samples
mismatched at all.
"""
import numpy as np

REL_TOL = 1e-4
ABS_TOL = 1e-6
FLIP_MAX = 2e-3
# Margins are in the decisions' own units (uniform random numbers,
# probabilities, cosines, barycentrics), all of unit scale.  2^-14 is 128
# float ulps at 1.0.
TAU_DECISION = 2.0 ** -14
TAU_EDGE = 2.0 ** -14
NUDGES = (1, 2, 3, 4, 6, 8)
NUDGE_DRAWS = 3


def mismatched(a, b, abs_tol=ABS_TOL):
    a, b = a.reshape(-1, 3).astype(np.float64), b.reshape(-1, 3).astype(np.float64)
    return ~np.all(np.abs(a - b) <= REL_TOL * np.maximum(np.abs(a), np.abs(b)) + abs_tol, axis=1)


def classify(gpu, ref, oracle, ubo, width, height, rows=None):
    """gpu: GPU samples of rows [r0, r1) ([pixel][sample][3]); ref: the
    oracle's render of the same rows with want_margins=True; oracle: its
    OracleScene (re-rendered with nudges where needed).  Returns counts."""
    r0, r1 = rows if rows is not None else (0, height)
    ns = int(np.asarray(ubo)["number_of_samples"])

    def band(x, c):
        return x.reshape(height, width, ns, c)[r0:r1].reshape(-1, c)
    g = np.asarray(gpu, np.float32).reshape(-1, 3)
    o = band(ref["samples"], 3)
    m = band(ref["margins"], 2)
    assert np.all(np.isfinite(g)), "non-finite GPU radiance"
    assert len(g) == len(o)
    bad = mismatched(g, o)
    near = (m[:, 0] < TAU_DECISION) | (m[:, 1] < TAU_EDGE)
    sens = np.zeros_like(bad)
    cand = np.nonzero(bad & ~near)[0]
    per_row = width * ns
    for row in np.unique(cand // per_row) + r0:
        sel = cand[cand // per_row == row - r0]
        for k in NUDGES:
            for draw in range(NUDGE_DRAWS):
                nb = oracle.render(ubo, width, height, rows=(int(row), int(row) + 1), want_samples=True, out=False,
                                   nudge_ulps=k, nudge_draw=draw)
                sens[sel] |= mismatched(band(nb["samples"], 3)[sel], o[sel], abs_tol=0.0)
    explained = bad & (near | sens)
    return dict(n=len(g), mismatched=int(bad.sum()), explained=int(explained.sum()),
                by_margin=int((bad & near).sum()), by_nudge=int((bad & ~near & sens).sum()),
                unexplained=int((bad & ~explained).sum()), share=float(bad.mean()),
                unexplained_idx=np.nonzero(bad & ~explained)[0][:10])


def assert_samples(gpu, ref, oracle, ubo, width, height, rows=None, flip_max=FLIP_MAX):
    """Asserts the contract; returns the counts."""
    c = classify(gpu, ref, oracle, ubo, width, height, rows)
    assert c["unexplained"] == 0, f"unexplained per-sample mismatches: {c}"
    assert c["share"] <= flip_max, f"too many explained flips: {c}"
    return c
