"""Host-side mesh handle: the Python face of the native block topology.

Mirrors the parts of Parthenon's Mesh / MeshData that the hot path touches:
block list in gid (Morton) order, per-block geometry, boundary index maps, device
tables, and the ghost exchange (`AddBoundaryExchangeTasks` semantics). Field storage
is a torch CUDA tensor of shape (nblocks, ncomp, N3, N2, N1) in FP64 -- PyTorch only
provides the allocation and the stream; all work runs in the native library.
"""
import ctypes

import numpy as np

from . import _native as nat

PROLONG_OPS = {"minmod": 0, "linear": 2, "constant": 4}
CRITERIA = {"first": 0, "second": 1, "gradient": 2}


def _ptr(t):
    """Device pointer of a torch tensor (or None)."""
    if t is None:
        return None
    return ctypes.c_void_p(t.data_ptr())


def _stream(stream):
    import torch
    s = stream if stream is not None else torch.cuda.current_stream()
    return ctypes.c_void_p(s.cuda_stream)


class Mesh:
    """A single periodic octree of equal-size meshblocks.

    nx, block_nx: root-grid and block cell counts (x1, x2, x3); nghost: ghost width;
    leaves: optional list of (level, lx1, lx2, lx3) leaf locations (refined regions).
    """

    def __init__(self, nx, block_nx, nghost, xmin=(0.0, 0.0, 0.0), xmax=(1.0, 1.0, 1.0), leaves=None):
        L = nat.lib()
        spec = nat.MeshSpec()
        for d in range(3):
            spec.nx[d] = int(nx[d])
            spec.block_nx[d] = int(block_nx[d])
            spec.xmin[d] = float(xmin[d])
            spec.xmax[d] = float(xmax[d])
        spec.nghost = int(nghost)
        lv = np.zeros((0, 4), np.int64) if leaves is None else np.ascontiguousarray(leaves, np.int64).reshape(-1, 4)
        h = ctypes.c_void_p()
        nat.check(L.pgb_mesh_create(ctypes.byref(spec), int(lv.shape[0]), lv.ctypes.data_as(ctypes.c_void_p),
                                    ctypes.byref(h)), "pgb_mesh_create")
        self._h = h
        self._read_info(nghost, block_nx)

    @classmethod
    def _wrap(cls, handle, nghost, block_nx):
        m = cls.__new__(cls)
        m._h = handle
        m._read_info(nghost, block_nx)
        return m

    def _read_info(self, nghost, block_nx):
        L = nat.lib()
        self.nghost = int(nghost)
        self.block_nx = tuple(int(b) for b in block_nx)
        info = nat.MeshInfo()
        nat.check(L.pgb_mesh_get_info(self._h, ctypes.byref(info)), "pgb_mesh_get_info")
        self.nblocks = info.nblocks
        self.multilevel = bool(info.multilevel)
        self.root_level = info.root_level
        self.max_level = info.max_level
        self.N = tuple(info.N)
        self.Nc = tuple(info.Nc)
        self.npairs = info.npairs
        self.buffer_elems = info.buffer_elems
        self.nflux_corr = info.nflux_corr
        self._uploaded = False

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            nat.lib().pgb_mesh_destroy(h)
            self._h = None

    # ---------------------------------------------------------------- topology
    def block_info(self):
        locs = np.zeros((self.nblocks, 4), np.int64)
        geom = np.zeros((self.nblocks, 6), np.float64)
        nat.check(nat.lib().pgb_mesh_block_info(self._h, locs.ctypes.data_as(ctypes.c_void_p),
                                                geom.ctypes.data_as(ctypes.c_void_p)), "pgb_mesh_block_info")
        return locs, geom

    def boundaries(self):
        out = np.zeros((self.npairs, 23), np.int32)
        nat.check(nat.lib().pgb_mesh_boundaries(self._h, out.ctypes.data_as(ctypes.c_void_p), self.npairs),
                  "pgb_mesh_boundaries")
        return out

    def cell_centers(self):
        """Per-block cell-centre coordinates including ghosts: three arrays (nblocks, N)."""
        _, geom = self.block_info()
        out = []
        for d in range(3):
            idx = np.arange(self.N[d]) - self.nghost
            out.append(geom[:, d:d + 1] + (idx[None, :] + 0.5) * geom[:, 3 + d:4 + d])
        return out

    # ---------------------------------------------------------------- device
    def upload(self):
        nat.check(nat.lib().pgb_mesh_upload(self._h), "pgb_mesh_upload")
        self._uploaded = True
        return self

    def _ensure(self):
        if not self._uploaded:
            self.upload()

    def new_field(self, ncomp, fill=0.0):
        import torch
        return torch.full((self.nblocks, ncomp, self.N[2], self.N[1], self.N[0]), fill, dtype=torch.float64,
                          device="cuda")

    def new_coarse(self, ncomp, fill=0.0):
        import torch
        return torch.full((self.nblocks, ncomp, self.Nc[2], self.Nc[1], self.Nc[0]), fill, dtype=torch.float64,
                          device="cuda")

    def exchange(self, field, coarse=None, prolongate=True, op="minmod", buffered=False, stream=None):
        """SendBoundBufs -> ReceiveBoundBufs -> SetBounds [-> ProlongateBounds] on all blocks."""
        self._ensure()
        ncomp = field.shape[1]
        flags = (1 if prolongate else 0) | PROLONG_OPS[op]
        buf = None
        if buffered:
            import torch
            buf = torch.empty(max(1, self.buffer_elems * ncomp), dtype=torch.float64, device="cuda")
        nat.check(nat.lib().pgb_exchange(self._h, _ptr(field), _ptr(coarse), ncomp, flags, _ptr(buf),
                                         _stream(stream)), "pgb_exchange")
        return buf

    def pack_buffers(self, field, coarse=None, stream=None):
        import torch
        self._ensure()
        ncomp = field.shape[1]
        buf = torch.zeros(max(1, self.buffer_elems * ncomp), dtype=torch.float64, device="cuda")
        nat.check(nat.lib().pgb_pack_buffers(self._h, _ptr(field), _ptr(coarse), ncomp, _ptr(buf), _stream(stream)),
                  "pgb_pack_buffers")
        return buf

    def flux_correct(self, flux, ncomp, stream=None):
        self._ensure()
        nat.check(nat.lib().pgb_flux_correct(self._h, _ptr(flux), ncomp, _stream(stream)), "pgb_flux_correct")

    # ---------------------------------------------------------------- adaptive refinement
    def block_criterion(self, field, comp, method="first", stream=None):
        """Per-block refinement criterion of one component (device tensor, one value per block).

        method: "first" (FirstDerivative), "second" (SecondDerivative) or "gradient"
        (largest |grad q|). The field's ghosts must be current.
        """
        import torch
        self._ensure()
        out = torch.empty(self.nblocks, dtype=torch.float64, device="cuda")
        nat.check(nat.lib().pgb_amr_block_criterion(self._h, _ptr(field), field.shape[1], int(comp),
                                                    CRITERIA[method], _ptr(out), _stream(stream)),
                  "pgb_amr_block_criterion")
        return out

    def set_refinement(self, crit, refine_tol, derefine_tol, crit_max_level, mesh_max_level, derefine_count=10):
        """Refinement flags (+1/0/-1 per block) from host criterion values; updates the
        per-block derefinement counters kept with the mesh."""
        c = np.ascontiguousarray(crit, np.float64)
        if c.shape != (self.nblocks,):
            raise ValueError("one criterion value per block is required")
        flags = np.zeros(self.nblocks, np.int32)
        nat.check(nat.lib().pgb_amr_set_refinement(self._h, c.ctypes.data_as(ctypes.c_void_p), float(refine_tol),
                                                   float(derefine_tol), int(crit_max_level), int(mesh_max_level),
                                                   int(derefine_count), flags.ctypes.data_as(ctypes.c_void_p)),
                  "pgb_amr_set_refinement")
        return flags

    def remesh(self, flags):
        """The mesh after one adaptive step, or None when the leaf set is unchanged."""
        f = np.ascontiguousarray(flags, np.int32)
        if f.shape != (self.nblocks,):
            raise ValueError("one flag per block is required")
        h = ctypes.c_void_p()
        nat.check(nat.lib().pgb_amr_remesh(self._h, f.ctypes.data_as(ctypes.c_void_p), ctypes.byref(h)),
                  "pgb_amr_remesh")
        if not h:
            return None
        m = Mesh._wrap(h, self.nghost, self.block_nx)
        if self.sparse:
            # the native remesh carried the allocation flags to the new handle
            m.sparse_ncomp = self.sparse_ncomp
        return m

    def transfer(self, new_mesh, field, stream=None):
        """New field on new_mesh: same-level copies, prolongated new fine blocks,
        restricted new coarse blocks (ghosts to be filled by an exchange)."""
        import torch
        self._ensure()
        new_mesh._ensure()
        ncomp = field.shape[1]
        # allocate (and zero) on the stream the transfer runs on
        with torch.cuda.stream(stream if stream is not None else torch.cuda.current_stream()):
            out = new_mesh.new_field(ncomp)
        nat.check(nat.lib().pgb_amr_transfer(self._h, new_mesh._h, _ptr(field), _ptr(out), ncomp, _stream(stream)),
                  "pgb_amr_transfer")
        return out

    # ---------------------------------------------------------------- sparse variables
    def enable_sparse(self, ncomp, alloc_threshold=1e-12, dealloc_threshold=1e-14, dealloc_count=5,
                      default_value=0.0):
        """Every component of the fields on this mesh becomes a sparse variable
        (Metadata::Sparse) with these thresholds (scalars or one value per component);
        all start unallocated. Defaults: Globals::sparse_config (src/globals.hpp:33-35).
        Exchanges, stages, RK2 cycles and remeshes on this mesh then follow the
        reference's allocation rules."""
        def vec(x):
            return np.ascontiguousarray(np.broadcast_to(np.asarray(x, np.float64), (int(ncomp),)))
        self._sparse_keep = (vec(alloc_threshold), vec(dealloc_threshold), vec(default_value))
        p = nat.SparseParams()
        p.ncomp = int(ncomp)
        p.dealloc_count = int(dealloc_count)
        p.alloc_threshold, p.dealloc_threshold, p.default_value = (
            a.ctypes.data_as(nat.DP) for a in self._sparse_keep)
        nat.check(nat.lib().pgb_sparse_enable(self._h, ctypes.byref(p)), "pgb_sparse_enable")
        self.sparse_ncomp = int(ncomp)
        return self

    @property
    def sparse(self):
        return getattr(self, "sparse_ncomp", 0) > 0

    def set_sparse_alloc(self, alloc, counts=None):
        """Allocation flags (nblocks, ncomp) in {0, 1} and optional deallocation counters."""
        a = np.ascontiguousarray(alloc, np.uint8).reshape(self.nblocks, self.sparse_ncomp)
        c = None if counts is None else np.ascontiguousarray(counts, np.int32).reshape(a.shape)
        nat.check(nat.lib().pgb_sparse_set_alloc(self._h, a.ctypes.data_as(ctypes.c_void_p),
                                                 None if c is None else c.ctypes.data_as(ctypes.c_void_p)),
                  "pgb_sparse_set_alloc")

    def sparse_alloc(self, stream=None):
        """(allocation flags uint8 (nblocks, ncomp), deallocation counters int32) after
        synchronising the stream."""
        a = np.zeros((self.nblocks, self.sparse_ncomp), np.uint8)
        c = np.zeros((self.nblocks, self.sparse_ncomp), np.int32)
        nat.check(nat.lib().pgb_sparse_get_alloc(self._h, a.ctypes.data_as(ctypes.c_void_p),
                                                 c.ctypes.data_as(ctypes.c_void_p), _stream(stream)),
                  "pgb_sparse_get_alloc")
        return a, c

    def sparse_dealloc(self, field, cells=(), coarse=(), flux=None, stream=None):
        """SparseDealloc on `field`; deallocated variables are zeroed in `field`, the
        fields in `cells`, the coarse buffers in `coarse` and `flux`."""
        self._ensure()
        cl = [field] + [c for c in cells if c is not None and c is not field]
        cc = [c for c in coarse if c is not None]
        ca = (ctypes.c_void_p * max(1, len(cl)))(*[t.data_ptr() for t in cl])
        co = (ctypes.c_void_p * max(1, len(cc)))(*[t.data_ptr() for t in cc])
        nat.check(nat.lib().pgb_sparse_dealloc(self._h, _ptr(field), ca, len(cl), co, len(cc), _ptr(flux),
                                               _stream(stream)), "pgb_sparse_dealloc")

    def sparse_tag(self, field, refine_tol, derefine_tol, stream=None):
        """Per-block tag (-1/0/1, device tensor) of the sparse advection package's
        min/max CheckRefinement over allocated variables."""
        import torch
        self._ensure()
        out = torch.empty(self.nblocks, dtype=torch.float64, device="cuda")
        nat.check(nat.lib().pgb_sparse_tag(self._h, _ptr(field), float(refine_tol), float(derefine_tol), _ptr(out),
                                           _stream(stream)), "pgb_sparse_tag")
        return out

    @property
    def handle(self):
        return self._h
