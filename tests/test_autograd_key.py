"""The refit cache key of the autograd binding (CPU): it follows the triangle array's contents,
not the array object, so equal contents share a key and any change of topology changes it."""
import numpy as np


def test_topology_key_follows_contents(pkg):
    import torch
    from illum_rt_gb300 import autograd
    g = np.random.default_rng(3)
    tris = g.integers(0, 1000, size=(5000, 4)).astype(np.uint32)
    k = autograd._topology_key(tris, 1000)
    assert k == autograd._topology_key(tris.copy(), 1000)
    assert k == autograd._topology_key(torch.from_numpy(tris.view(np.int32)), 1000)
    assert k != autograd._topology_key(tris, 1001)
    swapped = tris.copy()
    swapped[[10, 20]] = swapped[[20, 10]]
    assert k != autograd._topology_key(swapped, 1000)
    wound = tris.copy()
    wound[:, :3] = wound[:, [0, 2, 1]]
    assert k != autograd._topology_key(wound, 1000)
    edited = tris.copy()
    edited[4999, 2] ^= 1
    assert k != autograd._topology_key(edited, 1000)
    assert k != autograd._topology_key(tris[:-1], 1000)
