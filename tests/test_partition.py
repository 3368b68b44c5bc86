"""Tree partition and landmark indices: the C ABI is bit-exact with the restated reference
(src/HODLR/src/indices.jl, src/HODLR/src/constructor.jl:31).  Host-only, no GPU needed."""
import itertools

import numpy as np
import pytest

from oracle import hodlr_oracle as O


def _c_partition(lib_mod, n, lvl):
    import kmhodlr
    return kmhodlr.HODLRindices(n, lvl)


def _levels():
    import kmhodlr
    for k in (0, 1, 2, 3, 5, 8, 9, 12, 40):
        yield O.FixedLevel(k), kmhodlr.FixedLevel(k)
    for k in (0, 1, 3, 7, 8, 10, 30):
        yield O.LogLevel(k), kmhodlr.LogLevel(k)


NS = [1, 2, 3, 5, 7, 8, 100, 255, 256, 257, 300, 511, 512, 513, 1000, 1023, 1024, 1025, 1500,
      4097, 65536, 65537, 262144, 100003]


@pytest.mark.parametrize("n", NS)
def test_partition_matches_reference(lib, n):
    import kmhodlr
    for olvl, clvl in _levels():
        lv_o, lf_o, nl_o = O.HODLRindices(n, olvl)
        lv_c, lf_c, nl_c = kmhodlr.HODLRindices(n, clvl)
        assert lv_o == lv_c
        assert lf_o == lf_c
        assert nl_o == nl_c


def test_partition_known_answers(lib):
    import kmhodlr
    # n = 1030, FixedLevel(2): leaves of 258, 258, 257, 257 (the remainder goes first)
    lv, lf, nl = kmhodlr.HODLRindices(1030, kmhodlr.FixedLevel(2))
    assert lv == 2
    assert lf == [(1, 258, 1, 258), (259, 516, 259, 516), (517, 773, 517, 773), (774, 1030, 774, 1030)]
    # rows a:b are the SECOND child, cols c:d the first
    assert nl == [[(259, 516, 1, 258), (774, 1030, 517, 773)], [(517, 1030, 1, 516)]]
    # LogLevel(8) at n = 1024 gives 2 levels of 256-point leaves
    lv, lf, nl = kmhodlr.HODLRindices(1024, kmhodlr.LogLevel(8))
    assert lv == 2 and all(b - a + 1 == 256 for a, b, _, _ in lf)
    # FixedLevel(8) at n = 2^16: 256 leaves of 256, 255 blocks
    lv, lf, nl = kmhodlr.HODLRindices(65536, kmhodlr.FixedLevel(8))
    assert lv == 8 and len(lf) == 256 and sum(len(x) for x in nl) == 255
    # level 0 keeps one empty non-leaf level, as the reference does
    lv, lf, nl = kmhodlr.HODLRindices(100, kmhodlr.LogLevel(8))
    assert lv == 0 and lf == [(1, 100, 1, 100)] and nl == [[]]


def test_partition_rejects_bad_input(lib):
    import kmhodlr
    with pytest.raises(kmhodlr.KMError):
        kmhodlr.HODLRindices(0, kmhodlr.LogLevel(8))
    with pytest.raises(kmhodlr.KMError):
        kmhodlr.HODLRindices(1024, kmhodlr.LogLevel(-1))


@pytest.mark.parametrize("n,r", [(1024, 72), (65536, 72), (262144, 72), (1500, 16), (4096, 2),
                                 (1000, 7), (32768, 72), (2048, 32)])
def test_landmarks_match_reference(lib, n, r):
    import kmhodlr
    assert np.array_equal(kmhodlr.nystrom_landmarks(n, r), O.nystrom_landmarks(n, r) + 1)


def test_landmark_rounding_has_no_ties_at_config_sizes():
    # round.(LinRange(1, n, r)) is insensitive to the interpolation formula at these sizes
    for n, r in itertools.product([2 ** k for k in range(10, 19)], [2, 72]):
        t = np.arange(r) / (r - 1)
        v1 = (1.0 - t) * 1.0 + t * n
        v2 = 1.0 + t * (n - 1)
        frac = np.abs(v1 - np.floor(v1) - 0.5)
        assert np.all(frac > 1e-6)
        assert np.array_equal(np.rint(v1), np.rint(v2))
