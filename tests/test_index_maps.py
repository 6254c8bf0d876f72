"""Bit-exact parity of the buffer index maps: product topology vs the oracle.

Each boundary record holds the sender/receiver gids, the sender-side neighbour slot,
the send and receive index boxes, the coarse-buffer flags, the 27-bit receive mask
and the element count (the reference's BndInfo ranges, bnd_info.cpp:273-340). The
product builds them with its own topology code (host only, no GPU needed).
"""
import numpy as np
import pytest

import oracle_lib as O
import parthenon_gb300 as pg
from meshes import INDEX_MAP_CASES


@pytest.mark.parametrize("name,nx,bnx,ng,leaves", INDEX_MAP_CASES, ids=[c[0] for c in INDEX_MAP_CASES])
def test_index_maps_match_oracle(name, nx, bnx, ng, leaves):
    o = O.OracleSim(nx, bnx, ng, leaves=leaves)
    m = pg.Mesh(nx, bnx, ng, leaves=leaves)
    assert o.nblocks == m.nblocks
    lo, go = o.block_info()
    lp, gp = m.block_info()
    assert np.array_equal(lo, lp), "gid order (Morton) differs"
    assert np.array_equal(go, gp), "block geometry differs"
    assert m.multilevel == o.multilevel
    bo, bp = o.boundaries(), m.boundaries()
    assert bo.shape == bp.shape
    assert np.array_equal(bo, bp)
    # every pair moves the same number of values on both sides
    assert (bp[:, 18] > 0).all()
    # every device access implied by the lowered tables stays inside the arrays
    from parthenon_gb300 import _native
    _native.check(_native.lib().pgb_mesh_validate(m.handle), "pgb_mesh_validate")


def test_c3_block_counts():
    """The static-refinement advection mesh: 128^3 root in 16^3 blocks, central 1/8 refined once -> 448 + 512."""
    from meshes import refined_cube
    m = pg.Mesh((128,) * 3, (16,) * 3, 4, leaves=refined_cube(3, 2, 6))
    locs, _ = m.block_info()
    assert m.nblocks == 960
    assert (locs[:, 0] == 3).sum() == 448 and (locs[:, 0] == 4).sum() == 512


def test_uniform_pairs_per_block():
    m = pg.Mesh((64,) * 3, (16,) * 3, 2)
    b = m.boundaries()
    assert m.npairs == 64 * 26
    # same-level uniform: every receive mask is full for cell-centred data
    assert (b[:, 17] == (1 << 27) - 1).all()
    # ghost values per block: (n+2g)^3 - n^3
    per_block = np.bincount(b[:, 1], weights=b[:, 18])
    assert np.all(per_block == 20 ** 3 - 16 ** 3)


def test_invalid_meshes_rejected():
    with pytest.raises(pg.NativeError):
        pg.Mesh((64, 64, 64), (24, 24, 24), 2)  # block size does not divide
    with pytest.raises(pg.NativeError):
        pg.Mesh((64, 64, 32), (16, 16, 16), 2)  # not one cubic tree
    with pytest.raises(pg.NativeError):
        pg.Mesh((64, 64, 64), (16, 16, 16), 3)  # odd ghost width
