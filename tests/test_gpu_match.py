"""Descriptor matching on the device (zeroslam_gb300/csrc/ba_match.cu,
zs_find_matches) against feature::find_matches (source/feature.hpp:1190-1235):
the reference's matches in tests/golden/matches.npz, the known answers of
tests/feature.test.cpp, and the oracle's restatement on random sets, match
for match (lhs, rhs, score)."""

import numpy as np
import pytest

from conftest import known_answer_descriptors, load_npz
from zeroslam_gb300 import scenes

pytestmark = pytest.mark.gpu


def _ba():
    from zeroslam_gb300 import ba

    return ba.BundleAdjuster()


def _same(a, b):
    return (len(a) == len(b) and np.array_equal(a["lhs_index"], b["lhs_index"])
            and np.array_equal(a["rhs_index"], b["rhs_index"]) and np.array_equal(a["score"], b["score"]))


def test_find_matches_fixture(zs_lib):
    g = load_npz("matches.npz")
    with _ba() as h:
        for c, (thr, k, size) in enumerate(g["cases"]):
            m = h.find_matches(g["lhs"], g["rhs"], float(thr), int(k), int(size))
            assert np.array_equal(m["lhs_index"], g[f"case{c}_lhs"])
            assert np.array_equal(m["rhs_index"], g[f"case{c}_rhs"])
            assert np.array_equal(m["score"], g[f"case{c}_score"])


def test_find_matches_known_answers(zs_lib):
    onehot, (lhs, rhs, thr, k, size, want) = known_answer_descriptors()
    with _ba() as h:
        m = h.find_matches(onehot, np.zeros((1, 32), dtype=np.uint8), 2.0, 1, 256)
        assert len(m) == 256 and np.all(m["score"] == 1.0)
        assert len(h.find_matches(lhs, rhs, thr, k, size)) == want


@pytest.mark.parametrize("n_lhs,n_rhs", [(1, 1), (37, 1000), (2000, 2000), (5000, 3000), (300, 20000)])
def test_find_matches_random(zs_lib, oracle, n_lhs, n_rhs):
    lhs, rhs = scenes.descriptor_pair(n_lhs, n_rhs, seed=n_lhs + n_rhs)
    cases = [(32.0, 2, 2 * max(n_lhs, n_rhs)), (64.0, 1, n_lhs), (120.0, 5, 5 * n_lhs), (128.0, 8, 3 * n_lhs + 7)]
    with _ba() as h:
        for thr, k, size in cases:
            assert _same(h.find_matches(lhs, rhs, thr, k, size), oracle.find_matches(lhs, rhs, thr, k, size))


def test_find_matches_edges(zs_lib, oracle):
    from zeroslam_gb300 import ba

    lhs, rhs = scenes.descriptor_pair(200, 300, seed=5)
    with _ba() as h:
        for thr in (float("nan"), -1.0, 0.0, 1e9, 256.0, 256.5):
            assert _same(h.find_matches(lhs, rhs, thr, 3, 1000), oracle.find_matches(lhs, rhs, thr, 3, 1000))
        assert len(h.find_matches(lhs, rhs[:0], 32.0, 2, 100)) == 0
        assert len(h.find_matches(lhs[:0], rhs, 32.0, 2, 100)) == 0
        assert len(h.find_matches(lhs, rhs, 32.0, 0, 100)) == 0
        assert len(h.find_matches(lhs, rhs, 32.0, 2, 0)) == 0
        with pytest.raises(ba.ZsError) as ex:
            h.find_matches(lhs, rhs, 32.0, 9, 100)
        assert ex.value.status == ba.ZS_ERR_UNSUPPORTED
