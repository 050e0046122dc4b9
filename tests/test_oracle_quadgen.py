"""The oracle's quad generator (src/quad_generator.cpp restated): both greedy orders give a valid
quadization (every tri exactly once, pairs sharing an edge), and the parallel rounds (order 1)
leave about as few tris unpaired as the reference's sequential greedy (order 0)."""
import numpy as np
import pytest

from lucid_gb300 import scenes
from tests.quad_checks import check_quadization


@pytest.mark.parametrize("kind,shuffle", [("sphere", True), ("plane", False), ("plane", True)])
def test_quadgen_valid_both_orders(oracle, kind, shuffle):
    pos, tris = scenes.tri_mesh(kind, 40, 24, seed=3, shuffle=shuffle)
    res = {}
    for order in (0, 1):
        quads, nd = oracle.quadgen(pos, tris, 1.0, order)
        check_quadization(tris, quads, nd)
        res[order] = len(quads)
    # a grid of 2 tris per cell pairs almost everything, in both orders
    assert res[0] <= 0.505 * len(tris)
    assert res[1] <= res[0] * 1.005


def test_quadgen_grid_order_pairs_cells(oracle):
    """Grid order, unshuffled: the first tri of each quad comes first, so output order follows
    the input."""
    pos, tris = scenes.tri_mesh("plane", 8, 4, seed=1, noise=0.0, shuffle=False)
    quads, nd = oracle.quadgen(pos, tris, 1.0, 0)
    check_quadization(tris, quads, nd)
    assert nd <= 4


def test_quadgen_edge_cases(oracle):
    pos = np.zeros((4, 3), np.float32)
    pos[1, 0] = pos[2, 1] = pos[3, 2] = 1.0
    # two tris sharing all vertices (flipped duplicates) never pair; a lone tri is degenerate
    tris = np.array([[0, 1, 2], [0, 2, 1], [0, 1, 3]], np.int32)
    quads, nd = oracle.quadgen(pos, tris, 1.0, 0)
    check_quadization(tris, quads, nd)
    q0, nd0 = oracle.quadgen(pos, tris[:0], 1.0, 1)
    assert len(q0) == 0 and nd0 == 0
    with pytest.raises(RuntimeError):
        oracle.quadgen(pos, np.array([[0, 1, 9]], np.int32), 1.0, 0)
