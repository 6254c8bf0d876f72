"""The allocation-free exchange entry point against the ordinary one.

Callers that cannot allocate device memory (their host framework owns the device
allocator, or their loop must never allocate) use pgb_exchange_static_buffer, whose
pack buffer is a fixed static array inside the library. It must move exactly the same
values as pgb_exchange with a caller-provided buffer, call after call. Ghost copies
are bit-exact, so the tolerance is zero. This file sorts last so that a run stopping
at its first failure has already run every other test.
"""
import ctypes

import numpy as np
import pytest

import parthenon_gb300 as pg
from parthenon_gb300 import _native as nat
from parthenon_gb300.mesh import _ptr, _stream
from meshes import refined_cube

pytestmark = pytest.mark.gpu


def _static_exchange(mesh, field, coarse, flags=1):
    import torch
    rc = nat.lib().pgb_exchange_static_buffer(mesh.handle, _ptr(field), _ptr(coarse), field.shape[1], flags,
                                              _stream(torch.cuda.current_stream()))
    nat.check(rc, "pgb_exchange_static_buffer")


@pytest.mark.parametrize("leaves", [None, refined_cube(2, 1, 3)], ids=["uniform", "refined"])
def test_static_buffer_exchange_matches_caller_buffer_twice(leaves):
    import torch
    mesh = pg.Mesh((64,) * 3, (16,) * 3, 4, leaves=leaves).upload()
    rng = np.random.default_rng(5)
    for call in range(2):
        host = rng.standard_normal((mesh.nblocks, 3) + tuple(mesh.N[::-1]))
        a = torch.tensor(host, device="cuda")
        b = torch.tensor(host, device="cuda")
        ca = mesh.new_coarse(3) if mesh.multilevel else None
        cb = mesh.new_coarse(3) if mesh.multilevel else None
        mesh.exchange(a, ca, prolongate=True, buffered=True)
        _static_exchange(mesh, b, cb)
        torch.cuda.synchronize()
        assert torch.equal(a, b), "call %d differs" % call
        if ca is not None:
            assert torch.equal(ca, cb), "call %d coarse buffers differ" % call


def test_static_buffer_rejects_oversized_requests():
    import torch
    mesh = pg.Mesh((64,) * 3, (16,) * 3, 4).upload()
    ncomp = 4194304 // mesh.buffer_elems + 1
    f = torch.zeros((mesh.nblocks, ncomp) + tuple(mesh.N[::-1]), dtype=torch.float64, device="cuda")
    rc = nat.lib().pgb_exchange_static_buffer(mesh.handle, _ptr(f), None, ncomp, 0,
                                              _stream(torch.cuda.current_stream()))
    assert rc == -1
    assert b"static buffer" in nat.lib().pgb_last_error()


def test_static_buffer_rejects_sparse_meshes():
    import torch
    mesh = pg.Mesh((32,) * 3, (16,) * 3, 2).upload()
    mesh.enable_sparse(2, 1e-5, 1e-6, dealloc_count=5)
    f = torch.zeros((mesh.nblocks, 2) + tuple(mesh.N[::-1]), dtype=torch.float64, device="cuda")
    rc = nat.lib().pgb_exchange_static_buffer(mesh.handle, _ptr(f), None, 2, 0,
                                              _stream(torch.cuda.current_stream()))
    assert rc == -3
    assert b"sparse" in nat.lib().pgb_last_error()
