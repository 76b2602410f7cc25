"""Generates the golden fixtures in tests/golden/.

* golden_rng.json -- known-answer vectors of Random.glsl (TEA
  InitRandomSeed, the LCG RandomFloat, pcg4d and rand), computed by the
  pure-Python restatement below, which is independent of the C++ oracle.
* golden_cornell_32.npz / golden_ico2.npz / golden_trace_soup.npz -- small
  renders and ray queries of the CPU oracle (per-sample radiance, primary
  hits, tone-mapped image), used to detect regressions of the oracle and as
  fixed references for the GPU tests.

Run:  python tests/golden/make_golden.py
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [ROOT, os.path.join(ROOT, "oracle")]

M = 0xFFFFFFFF


def tea(v0, v1):  # crates/examples/gltf_viewer/shaders/lib/Random.glsl:12-25
    s0 = 0
    for _ in range(16):
        s0 = (s0 + 0x9E3779B9) & M
        v0 = (v0 + ((((v1 << 4) & M) + 0xA341316C) ^ ((v1 + s0) & M) ^ ((v1 >> 5) + 0xC8013EA4))) & M
        v1 = (v1 + ((((v0 << 4) & M) + 0xAD90777D) ^ ((v0 + s0) & M) ^ ((v0 >> 5) + 0x7E95761E))) & M
    return v0


def lcg_floats(seed, n):  # Random.glsl:27-42
    out = []
    for _ in range(n):
        seed = (1664525 * seed + 1013904223) & M
        out.append(np.float32(seed & 0x00FFFFFF) / np.float32(0x01000000))
    return [float(x) for x in out]


def pcg4d(v):  # Random.glsl:81-98
    x, y, z, w = [(c * 1664525 + 1013904223) & M for c in v]
    x = (x + y * w) & M
    y = (y + z * x) & M
    z = (z + x * y) & M
    w = (w + y * z) & M
    x ^= x >> 16
    y ^= y >> 16
    z ^= z >> 16
    w ^= w >> 16
    x = (x + y * w) & M
    y = (y + z * x) & M
    z = (z + x * y) & M
    w = (w + y * z) & M
    return [x, y, z, w]


def rand_seq(state, n):  # Random.glsl:70-72,102-105
    s = list(state)
    out = []
    for _ in range(n):
        s[3] = (s[3] + 1) & M
        bits = np.uint32(0x3F800000 | (pcg4d(s)[0] >> 9))
        out.append(float(bits.view(np.float32) - np.float32(1.0)))
    return out


def rng_vectors():
    tea_in = [(0, 0), (1, 2), (255, 255), (1919, 1079), (0x9E3779B9, 7), (M, M)]
    pcg_in = [(0, 0, 0, 0), (1, 2, 3, 4), (1919, 1079, 63, 5), (M, 0, M, 0)]
    rand_in = [(0, 0, 0, 0), (17, 23, 5, 0), (1919, 1079, tea(63, 0x9E3779B9), 0)]
    return {
        "tea": [[a, b, tea(a, b)] for a, b in tea_in],
        "pcg4d": [[list(v), pcg4d(v)] for v in pcg_in],
        "rand": [[list(s), rand_seq(s, 8)] for s in rand_in],
        "lcg": [[seed, lcg_floats(seed, 8)] for seed in (0, 1, 12345, tea(tea(3, 4), 0))],
    }


def main():
    from rustracer_gb300 import scenes, types as T
    import pyoracle as O

    with open(os.path.join(HERE, "golden_rng.json"), "w") as f:
        json.dump(rng_vectors(), f, indent=1)

    sc = scenes.cornell()
    o = O.OracleScene(sc)
    ubo = sc.ubo(32, 32, samples=4, bounces=8, exposure=1.0)
    r = o.render(ubo, 32, 32, want_samples=True, want_hits=True, threads=1)
    np.savez_compressed(os.path.join(HERE, "golden_cornell_32.npz"), samples=r["samples"], hits=r["hits"],
                        image=r["image"], ubo=np.frombuffer(ubo.tobytes(), np.uint8))

    sc = scenes.icosphere_scene(subdiv=2)
    o = O.OracleScene(sc)
    ubo = sc.ubo(24, 16, samples=2, bounces=8, exposure=1.0)
    r = o.render(ubo, 24, 16, want_samples=True, want_hits=True, threads=1)
    np.savez_compressed(os.path.join(HERE, "golden_ico2.npz"), samples=r["samples"], hits=r["hits"],
                        image=r["image"], ubo=np.frombuffer(ubo.tobytes(), np.uint8))

    sc = scenes.random_soup(500, seed=7)
    o = O.OracleScene(sc)
    rays = scenes.random_rays(2048, seed=8)
    hits, _ = o.trace(rays, threads=1)
    np.savez_compressed(os.path.join(HERE, "golden_trace_soup.npz"), rays=rays, hits=hits)
    print("written to", HERE)


if __name__ == "__main__":
    main()
