"""Pins the CPU oracle against the reference's own kernels (no GPU needed).

tests/golden/*.npz hold seeded inputs, weights and the final activations /
categories produced by the reference's bf_inference, snig_inference and
identify kernels (compiled from the reference sources, run on a GB300 by
tests/golden/make_golden.py).  The FP64 oracle must reproduce them:
categories exactly, activations within 1e-5 relative (|a-b| / max(1,|b|);
the two reference kernels themselves differ by up to 8.5e-6 because their
shared-memory atomics sum in arbitrary order), per-layer live-row counts
exactly, and the reference identify's int-truncating sum exactly.
"""
import glob
import os

import numpy as np
import pytest

from oracle import oracle as orc

HERE = os.path.dirname(os.path.abspath(__file__))
FIXTURES = sorted(glob.glob(os.path.join(HERE, "golden", "*.npz")))
RTOL = 1e-5


def load(path):
    d = np.load(path)
    L = int(d["L"])
    layers = [(d["row_off"][l].astype(np.int32), d["cols"][l].astype(np.int32),
               d["vals"][l].astype(np.float32)) for l in range(L)]
    return d, layers


def rel(a, b):
    return float((np.abs(a.astype(np.float64) - b) / np.maximum(1.0, np.abs(b))).max())


def test_fixtures_present():
    assert len(FIXTURES) >= 4


@pytest.mark.parametrize("path", FIXTURES, ids=[os.path.basename(p) for p in FIXTURES])
def test_oracle_matches_reference_kernels(path):
    d, layers = load(path)
    N, L = int(d["N"]), int(d["L"])
    Y, alive, dead = orc.infer(layers, N, float(d["bias"]), d["Y0"], precision=64)
    for key in ("Y_bf", "Y_snig"):
        ref = d[key]
        assert np.array_equal(alive, (ref > 0).any(1).astype(np.int32)), key
        assert rel(ref, Y) <= RTOL, key
    # live rows after every layer, as BF's host compaction counted them
    assert [int((dead > l).sum()) for l in range(L)] == list(d["alive_bf"])


@pytest.mark.parametrize("path", FIXTURES, ids=[os.path.basename(p) for p in FIXTURES])
def test_identify_restatement(path):
    d, layers = load(path)
    N = int(d["N"])
    Y, alive, _ = orc.infer(layers, N, float(d["bias"]), d["Y0"], precision=64)
    # the reference identify (thrust int accumulation) on its own outputs and on the oracle's
    assert np.array_equal(orc.identify(d["Y_bf"].astype(np.float64), 1), d["identify_bf"])
    assert np.array_equal(orc.identify(d["Y_snig"].astype(np.float64), 1), d["identify_snig"])
    assert np.array_equal(orc.identify(Y, 1), d["identify_bf"])
    # the category definition used everywhere else: any activation > 0
    assert np.array_equal(orc.identify(Y, 0), alive)


def test_identify_int_rule_differs_below_one():
    """beyond-shaped net: activations stay below 1, so the reference identify
    reports no survivor although 97 rows are nonzero."""
    d, layers = load(os.path.join(HERE, "golden", "beyond_n256_l6.npz"))
    assert int(d["identify_bf"].sum()) == 0
    assert int((d["Y_bf"] > 0).any(1).sum()) == 97


@pytest.mark.parametrize("path", FIXTURES, ids=[os.path.basename(p) for p in FIXTURES])
def test_fp32_port_close_to_reference(path):
    d, layers = load(path)
    N = int(d["N"])
    Y32, alive32, _ = orc.infer(layers, N, float(d["bias"]), d["Y0"], precision=32)
    assert np.array_equal(alive32, (d["Y_bf"] > 0).any(1).astype(np.int32))
    assert rel(Y32, d["Y_bf"].astype(np.float64)) <= RTOL


def test_snicit_restatement_exact_on_fixture():
    """Residue form in FP64 with the reference's own centroid rule gives the same set."""
    d, layers = load(os.path.join(HERE, "golden", "sdgc_n128_l12.npz"))
    N, L = int(d["N"]), int(d["L"])
    bias = float(d["bias"])
    for T in (2, 4, 8):
        Yt, alive_t, _ = orc.infer(layers[:T], N, bias, d["Y0"], precision=64)
        live = np.flatnonzero(alive_t)
        cands = live[orc.ref_candidates(Yt[live].astype(np.float32))]
        Ys, flags, assign, nonempty = orc.snicit(layers, N, bias, d["Y0"], T, cands)
        assert np.array_equal(flags, (d["Y_bf"] > 0).any(1).astype(np.int32)), T
        assert rel(Ys.astype(np.float32), d["Y_bf"].astype(np.float64)) <= RTOL
        assert (assign[live] >= 0).all() and (assign[alive_t == 0] == -1).all()
