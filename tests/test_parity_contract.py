"""CPU checks of the per-sample parity contract (tests/parity.py) and of the
oracle's diagnostics build that it relies on.

* The diagnostics build renders the plain build's bits when no diagnostic
  is asked for, and its margins are finite where paths made decisions.
* Nudging transcendentals, shading divisions and square roots and dot
  products by ulps leaves most samples within 1e-4 (relative, no absolute
  floor, as the contract tests them): the "explained" class is small.
* A planted mistake -- the oracle re-rendered with every material's
  roughness off by 1%, standing in for a shading bug -- produces
  unexplained mismatches, so the contract does not explain real errors
  away.
"""
import numpy as np
import pytest

import parity
import pyoracle as O
from rustracer_gb300 import scenes


@pytest.fixture(scope="module")
def ico():
    sd = scenes.icosphere_scene(subdiv=3)
    ubo = sd.ubo(48, 32, samples=4, bounces=8, exposure=1.0)
    orc = O.OracleScene(sd, diag=True)
    ref = orc.render(ubo, 48, 32, want_samples=True, want_hits=True, want_margins=True)
    return sd, ubo, orc, ref


def test_diag_build_renders_the_plain_bits(ico):
    sd, ubo, orc, ref = ico
    plain = O.OracleScene(sd).render(ubo, 48, 32, want_samples=True, want_hits=True)
    assert np.array_equal(plain["samples"].view(np.uint32), ref["samples"].view(np.uint32))
    assert np.array_equal(plain["hits"], ref["hits"])
    m = ref["margins"].reshape(-1, 2)
    hit = ref["hits"].reshape(-1)["primitive_id"] != 0xFFFFFFFF
    assert np.all(np.isfinite(m[hit, 0]))  # every shaded path chose a lobe
    assert np.all((m[:, 0] >= 0) & (m[:, 1] >= 0))
    with pytest.raises(AssertionError):  # the plain build has no diagnostics
        O.OracleScene(sd).render(ubo, 48, 32, want_margins=True)


def test_nudged_oracle_mostly_in_band(ico):
    sd, ubo, orc, ref = ico
    for k in parity.NUDGES:
        nb = orc.render(ubo, 48, 32, want_samples=True, nudge_ulps=k)
        moved = parity.mismatched(nb["samples"], ref["samples"], abs_tol=0.0)
        assert moved.mean() < 0.01, (k, moved.mean())
    c = parity.classify(ref["samples"], ref, orc, ubo, 48, 32)
    assert c["mismatched"] == 0 and c["unexplained"] == 0


def test_planted_shading_mistake_is_unexplained(ico):
    sd, ubo, orc, ref = ico
    bad = scenes.icosphere_scene(subdiv=3)
    r = bad.materials["roughness_factor"]
    bad.materials["roughness_factor"] = np.where(r < 0.99, r * 1.01, r)
    wrong = O.OracleScene(bad).render(ubo, 48, 32, want_samples=True)["samples"]
    c = parity.classify(wrong, ref, orc, ubo, 48, 32)
    assert c["mismatched"] > 20 and c["unexplained"] > 0.5 * c["mismatched"], c
    with pytest.raises(AssertionError):
        parity.assert_samples(wrong, ref, orc, ubo, 48, 32)


def test_rows_band(ico):
    """classify on a band of rows reads the band out of full-image arrays."""
    sd, ubo, orc, ref = ico
    band = orc.render(ubo, 48, 32, rows=(8, 16), want_samples=True, want_margins=True)
    g = band["samples"].reshape(32, 48, 4, 3)[8:16]
    c = parity.classify(g, band, orc, ubo, 48, 32, rows=(8, 16))
    assert c["n"] == 8 * 48 * 4 and c["mismatched"] == 0


def test_nudge_draws_differ(ico):
    """Each draw index gives other nudge signs (the contract tries several
    per size); the oracle rejects sizes and draws outside 16 bits."""
    sd, ubo, orc, ref = ico
    a = orc.render(ubo, 48, 32, want_samples=True, nudge_ulps=2, nudge_draw=0)["samples"]
    b = orc.render(ubo, 48, 32, want_samples=True, nudge_ulps=2, nudge_draw=1)["samples"]
    again = orc.render(ubo, 48, 32, want_samples=True, nudge_ulps=2, nudge_draw=1)["samples"]
    assert np.array_equal(b.view(np.uint32), again.view(np.uint32))  # deterministic
    assert not np.array_equal(a.view(np.uint32), b.view(np.uint32))
    with pytest.raises(AssertionError):
        orc.render(ubo, 48, 32, want_samples=True, nudge_ulps=1, nudge_draw=1 << 16)
