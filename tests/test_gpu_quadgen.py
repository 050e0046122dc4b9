"""GPU quad generator (lucid_quad_generate) against the oracle's fixed-order greedy: the same
quads in the same order, a valid quadization, and argument errors."""
import numpy as np
import pytest

from lucid_gb300 import scenes
from tests.quad_checks import check_quadization

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("kind,nu,nv,shuffle,weight", [("sphere", 60, 30, True, 1.0), ("plane", 90, 40, False, 0.5),
                                                       ("plane", 128, 96, True, 1.0), ("sphere", 7, 5, True, 2.0)])
def test_quadgen_matches_oracle(gpu, oracle, kind, nu, nv, shuffle, weight):
    import torch
    from lucid_gb300.renderer import quad_generate
    pos, tris = scenes.tri_mesh(kind, nu, nv, seed=11, shuffle=shuffle)
    ref, ref_nd = oracle.quadgen(pos, tris, weight, 1)
    q, nd = quad_generate(torch.from_numpy(pos).cuda(), torch.from_numpy(tris).cuda(), weight)
    got = q.cpu().numpy().view(np.uint32)
    np.testing.assert_array_equal(got, ref)
    assert nd == ref_nd
    check_quadization(tris, got, nd)


def test_quadgen_meshes_and_errors(gpu):
    import torch
    from lucid_gb300 import _lib
    from lucid_gb300.renderer import quad_generate
    pos, tris = scenes.tri_mesh("sphere", 200, 100, seed=5)
    q, nd = quad_generate(torch.from_numpy(pos).cuda(), torch.from_numpy(tris).cuda())
    check_quadization(tris, q.cpu().numpy().view(np.uint32), nd)
    empty, nde = quad_generate(torch.from_numpy(pos).cuda(), torch.zeros((0, 3), dtype=torch.int32, device="cuda"))
    assert empty.shape[0] == 0 and nde == 0
    bad = torch.tensor([[0, 1, 10**6]], dtype=torch.int32, device="cuda")
    with pytest.raises(_lib.LucidError) as e:
        quad_generate(torch.from_numpy(pos).cuda(), bad)
    assert e.value.status == _lib.INVALID_ARG
