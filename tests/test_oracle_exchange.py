"""Self-consistency of the oracle's exchange (reference pack -> buffer -> unpack)."""
import numpy as np

import oracle_lib as O
from meshes import refined_cube


def test_uniform_exchange_fills_periodic_ghosts():
    ng, n, nb = 2, 16, 4
    s = O.OracleSim((64,) * 3, (n,) * 3, ng)
    locs, _ = s.block_info()
    u = s.base()
    u[:] = np.nan
    idx = np.arange(n)
    for b in range(s.nblocks):
        gi = locs[b, 1] * n + idx
        gj = locs[b, 2] * n + idx
        gk = locs[b, 3] * n + idx
        u[b, 0, ng:ng + n, ng:ng + n, ng:ng + n] = (gi[None, None, :] + 64 * gj[None, :, None] +
                                                    4096 * gk[:, None, None])
    assert s.exchange() == 0
    full = np.arange(n + 2 * ng) - ng
    for b in range(s.nblocks):
        gi = (locs[b, 1] * n + full) % 64
        gj = (locs[b, 2] * n + full) % 64
        gk = (locs[b, 3] * n + full) % 64
        expect = gi[None, None, :] + 64 * gj[None, :, None] + 4096 * gk[:, None, None]
        assert np.array_equal(u[b, 0], expect)


def test_multilevel_exchange_sets_every_ghost_exactly_once_and_keeps_linear_fields():
    ng, n = 4, 16
    s = O.OracleSim((64,) * 3, (n,) * 3, ng, leaves=refined_cube(2, 1, 3))
    locs, geom = s.block_info()
    u = s.base()
    u[:] = np.nan

    def f(x, y, z):
        return 1.0 + 2.0 * x - 3.0 * y + 0.5 * z

    for b in range(s.nblocks):
        c = [geom[b, d] + (np.arange(n + 2 * ng) - ng + 0.5) * geom[b, 3 + d] for d in range(3)]
        Z, Y, X = np.meshgrid(c[2], c[1], c[0], indexing="ij")
        u[b, 0, ng:ng + n, ng:ng + n, ng:ng + n] = f(X, Y, Z)[ng:ng + n, ng:ng + n, ng:ng + n]
    assert s.exchange() == 0  # no overlapping active writes
    assert not np.isnan(u).any()
    for b in range(s.nblocks):
        c = [geom[b, d] + (np.arange(n + 2 * ng) - ng + 0.5) * geom[b, 3 + d] for d in range(3)]
        Z, Y, X = np.meshgrid(c[2], c[1], c[0], indexing="ij")
        inside = (X > 0) & (X < 1) & (Y > 0) & (Y < 1) & (Z > 0) & (Z < 1)
        assert np.abs(u[b, 0] - f(X, Y, Z))[inside].max() < 1e-13
