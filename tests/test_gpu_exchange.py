"""Ghost exchange on the GPU vs the oracle: bit-exact ghost copies, coarse buffers,
restriction and prolongation, in both the direct and the reference-buffer modes."""
import numpy as np
import pytest

import oracle_lib as O
import parthenon_gb300 as pg
from meshes import INDEX_MAP_CASES, refined_cube

pytestmark = pytest.mark.gpu

OPS = {"minmod": 0, "linear": 1, "constant": 2}


def _pair(nx, bnx, ng, leaves, ncomp, seed):
    o = O.OracleSim(nx, bnx, ng, leaves=leaves, ncomp=ncomp)
    m = pg.Mesh(nx, bnx, ng, leaves=leaves).upload()
    rng = np.random.default_rng(seed)
    u = o.base()
    u[:] = rng.standard_normal(u.shape)
    return o, m


def _run_product(m, o, ncomp, prolongate, op, buffered):
    import torch
    f = torch.tensor(np.array(o.base()), device="cuda")
    c = torch.tensor(np.array(o.coarse()), device="cuda") if m.multilevel else None
    m.exchange(f, c, prolongate=prolongate, op=op, buffered=buffered)
    torch.cuda.synchronize()
    return f.cpu().numpy(), (c.cpu().numpy() if c is not None else None)


@pytest.mark.parametrize("name,nx,bnx,ng,leaves", INDEX_MAP_CASES, ids=[c[0] for c in INDEX_MAP_CASES])
@pytest.mark.parametrize("buffered", [False, True], ids=["direct", "buffered"])
def test_exchange_bit_exact(name, nx, bnx, ng, leaves, buffered):
    ncomp = 3
    o, m = _pair(nx, bnx, ng, leaves, ncomp, seed=7)
    f, c = _run_product(m, o, ncomp, True, "minmod", buffered)
    assert o.exchange(True, OPS["minmod"]) == 0
    assert np.array_equal(f, o.base())
    if c is not None:
        assert np.array_equal(c, o.coarse())


@pytest.mark.parametrize("op", ["linear", "constant"])
def test_prolongation_ops_bit_exact(op):
    o, m = _pair((64,) * 3, (16,) * 3, 4, refined_cube(2, 1, 3), 2, seed=11)
    f, c = _run_product(m, o, 2, True, op, False)
    o.exchange(True, OPS[op])
    assert np.array_equal(f, o.base())
    assert np.array_equal(c, o.coarse())


def test_exchange_without_prolongation():
    o, m = _pair((64,) * 3, (16,) * 3, 4, refined_cube(2, 1, 3), 1, seed=12)
    f, c = _run_product(m, o, 1, False, "minmod", False)
    o.exchange(False, 0)
    assert np.array_equal(f, o.base())
    assert np.array_equal(c, o.coarse())


@pytest.mark.parametrize("name,nx,bnx,ng,leaves", INDEX_MAP_CASES[:4], ids=[c[0] for c in INDEX_MAP_CASES[:4]])
def test_packed_buffers_match_reference_layout(name, nx, bnx, ng, leaves):
    import torch
    ncomp = 2
    o, m = _pair(nx, bnx, ng, leaves, ncomp, seed=3)
    f = torch.tensor(np.array(o.base()), device="cuda")
    c = torch.tensor(np.array(o.coarse()), device="cuda") if m.multilevel else None
    buf = m.pack_buffers(f, c)
    torch.cuda.synchronize()
    ref = o.pack()
    assert np.array_equal(buf.cpu().numpy()[:ref.size], ref)


def test_large_uniform_exchange_periodic_identity():
    """A mesh of 32^3 blocks with 4 ghosts and 11 components at reduced block count: every ghost
    equals the periodic image of an interior cell."""
    import torch
    n, ng, nb = 32, 4, 4
    m = pg.Mesh((n * nb,) * 3, (n,) * 3, ng).upload()
    locs, _ = m.block_info()
    N = n + 2 * ng
    full = np.arange(N) - ng
    G = n * nb
    host = np.zeros((m.nblocks, 2, N, N, N))
    for b in range(m.nblocks):
        gi = (locs[b, 1] * n + full) % G
        gj = (locs[b, 2] * n + full) % G
        gk = (locs[b, 3] * n + full) % G
        gid = gi[None, None, :] + G * gj[None, :, None] + G * G * gk[:, None, None]
        host[b, 0] = gid
        host[b, 1] = -gid
    f = torch.tensor(host, device="cuda")
    f[:, :, :ng] = float("nan")
    f[:, :, -ng:] = float("nan")
    f[:, :, :, :ng] = float("nan")
    f[:, :, :, -ng:] = float("nan")
    f[:, :, :, :, :ng] = float("nan")
    f[:, :, :, :, -ng:] = float("nan")
    m.exchange(f)
    torch.cuda.synchronize()
    assert np.array_equal(f.cpu().numpy(), host)
