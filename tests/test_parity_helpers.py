"""The parity checker itself, on the CPU: the full byte comparison of large
states finds a changed byte anywhere, and ignores exactly the QCGD name
padding the reference never initialises."""
import numpy as np
import pytest

from quids_gb300 import workloads as W
from tests.parity import assert_all_bytes_equal


def _graphs():
    rng = W.Rng(3)
    gs = [W.random_graph(n, rng) for n in range(1, 30)]
    return gs, W.pack(gs, [1.0] * len(gs), 8)


@pytest.mark.parametrize("chunk", [64, 1 << 27])
def test_padding_is_ignored_and_pairs_follow_the_selection(chunk):
    gs, p = _graphs()
    q = (p[0].copy(), p[1], p[2], p[3])
    for i, g in enumerate(gs):
        b = int(p[1][i])
        q[0][b: b + len(g)][~W.graph_padding_mask(g)] = 0xAB
    perm = np.random.default_rng(0).permutation(len(gs))
    assert_all_bytes_equal(p, q, perm, perm, True, "padding", chunk_bytes=chunk)
    with pytest.raises(AssertionError):  # unmasked, the padding differs
        assert_all_bytes_equal(p, q, perm, perm, False, "no mask", chunk_bytes=chunk)
    with pytest.raises(AssertionError):  # a wrong pairing differs
        assert_all_bytes_equal(p, q, perm, np.roll(perm, 1), True, "pairs", chunk_bytes=chunk)


@pytest.mark.parametrize("obj", [0, 7, 28])
def test_any_changed_byte_is_found(obj):
    gs, p = _graphs()
    idx = np.arange(len(gs))
    mask = W.graph_padding_mask(gs[obj])
    for pos in np.nonzero(mask)[0][[0, len(np.nonzero(mask)[0]) // 2, -1]]:
        q = (p[0].copy(), p[1], p[2], p[3])
        q[0][int(p[1][obj]) + int(pos)] ^= 0x10
        with pytest.raises(AssertionError):
            assert_all_bytes_equal(p, q, idx, idx, True, "changed", chunk_bytes=100)
