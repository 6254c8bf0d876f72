"""Adaptive-refinement evolution driver on the GPU.

Mirrors EvolutionDriver::Execute with adaptive refinement (src/driver/driver.cpp:67-166):
RK2 cycles, then every `check_interval` cycles the refinement tags of the last stage
(Refinement::Tag, src/amr_criteria/refinement_package.cpp:51-91, 154-170) and
Mesh::LoadBalancingAndAdaptiveMeshRefinement (src/mesh/mesh-amr_loadbalance.cpp:324-351):
tree update, new block list, data movement, ghost fill, and a fresh dt vote. The
criterion reduction and the data movement run on the device (one launch each); the
tree update and the flag logic are host work on a few thousand blocks. The initial
refinement repeats problem generation and remeshing until the block count settles,
as Mesh::Initialize does (src/mesh/mesh.cpp:745-846).

With check_interval = 1 the tagging cadence is the reference's (every cycle).
"""
import ctypes

import numpy as np

from . import _native as nat
from .driver import RK2Driver
from .mesh import _ptr, _stream


class RefinementCriterion:
    """One refinement criterion on one or more components.

    method: "first" (derivative_order_1), "second" (derivative_order_2) or "gradient"
    (largest |grad q|); the per-block value is the maximum over `comps`. With
    relative=True the tolerances are fractions of the mesh-wide maximum of the
    criterion (refine above refine_tol * max, derefine below derefine_tol * max);
    otherwise they are absolute (the reference's AMRCriteria, amr_criteria.cpp:53-54).
    max_level: absolute level at or above which the criterion does not refine (None:
    the mesh's maximum level).
    """

    def __init__(self, comps=(0,), method="first", refine_tol=0.5, derefine_tol=0.05, relative=False,
                 max_level=None):
        self.comps = tuple(int(c) for c in comps)
        self.method = method
        self.refine_tol = float(refine_tol)
        self.derefine_tol = float(derefine_tol)
        self.relative = bool(relative)
        self.max_level = max_level

    def tolerances(self, crit):
        if not self.relative:
            return self.refine_tol, self.derefine_tol
        g = float(np.max(crit)) if crit.size else 0.0
        return self.refine_tol * g, self.derefine_tol * g


class SparseMinMaxCriterion:
    """The sparse advection package's CheckRefinement
    (example/sparse_advection/sparse_advection_package.cpp:94-123): over the allocated
    variables of a block, ghosts included, refine when max > refine_tol and min <
    derefine_tol, derefine when max < derefine_tol. Needs a mesh with sparse variables."""

    method = "sparse_minmax"
    comps = ()
    relative = False
    max_level = None

    def __init__(self, refine_tol=0.3, derefine_tol=0.03):
        self.refine_tol = float(refine_tol)
        self.derefine_tol = float(derefine_tol)

    def tolerances(self, crit):
        # the per-block values are the tags themselves
        return 0.5, -0.5


class AMRDriver:
    """RK2 evolution with adaptive refinement.

    numlevel: number of refinement levels (the mesh's maximum level is
    numlevel + root_level - 1, mesh.cpp:125,179); derefine_count: consecutive derefine
    tags a block needs before it is derefined (mesh_refinement.cpp:57).
    """

    def __init__(self, mesh, ncomp, config, criterion, numlevel=2, derefine_count=10, check_interval=1,
                 stream=None):
        self.rk = RK2Driver(mesh, ncomp, config, stream=stream)
        self.criterion = criterion
        self.mesh_max_level = int(numlevel) + mesh.root_level - 1
        self.crit_max_level = self.mesh_max_level if criterion.max_level is None else int(criterion.max_level)
        self.derefine_count = int(derefine_count)
        self.check_interval = max(1, int(check_interval))
        self.ncycle = 0
        self.nremesh = 0
        self.zone_cycles = 0
        self.block_history = [mesh.nblocks]

    @property
    def mesh(self):
        return self.rk.mesh

    @property
    def base(self):
        return self.rk.base

    @property
    def dt(self):
        return self.rk.dt

    @property
    def stream(self):
        return self.rk.stream

    def block_criterion(self):
        """Per-block criterion values of the current base field (host array)."""
        import torch
        m = self.mesh
        vals = None
        with torch.cuda.stream(self.stream):
            if self.criterion.method == "sparse_minmax":
                vals = m.sparse_tag(self.base, self.criterion.refine_tol, self.criterion.derefine_tol,
                                    stream=self.stream)
            for c in self.criterion.comps:
                v = m.block_criterion(self.base, c, self.criterion.method, stream=self.stream)
                vals = v if vals is None else torch.maximum(vals, v)
            host = vals.cpu()
        return host.numpy()

    def flags(self, crit):
        rt, dt = self.criterion.tolerances(crit)
        return self.mesh.set_refinement(crit, rt, dt, self.crit_max_level, self.mesh_max_level, self.derefine_count)

    def adapt(self):
        """Tag, update the tree and move the data; True when the mesh changed."""
        flags = self.flags(self.block_criterion())
        new = self.mesh.remesh(flags)
        if new is None:
            return False
        new.upload()
        # the old scratch goes first; the stream orders its last uses before the reuse
        self.rk.release_scratch()
        base = self.mesh.transfer(new, self.base, stream=self.stream)
        self.rk.rebind(new, base)
        self.nremesh += 1
        self.block_history.append(new.nblocks)
        return True

    def initialize(self, pgen, max_iterations=16):
        """Problem generation + initial refinement (Mesh::Initialize with adaptive
        refinement): pgen(mesh_or_geometry) -> host field; repeated on each new mesh
        until a remesh leaves the block count unchanged; then the first dt. With sparse
        variables pgen(mesh, current field, current allocation) -> (field, allocation):
        it sees what the previous mesh's data became on the new one."""
        for _ in range(max_iterations):
            if self.mesh.sparse:
                self.stream.synchronize()
                prev = self.base.cpu().numpy()
                alloc, _ = self.mesh.sparse_alloc(self.stream)
                state, alloc = pgen(self.mesh, prev, alloc)
                self.rk.set_state(state, alloc)
            else:
                self.rk.set_state(pgen(self.mesh))
            before = self.mesh.nblocks
            self.adapt()
            if self.mesh.nblocks == before:
                break
        self.first_dt()
        self.ncycle = 0

    def first_dt(self):
        import torch
        with torch.cuda.stream(self.stream):
            nat.check(nat.lib().pgb_estimate_dt(self.mesh.handle, ctypes.byref(self.rk.params), _ptr(self.base),
                                                self.rk.ncomp, _ptr(self.dt), 1, _stream(self.stream)),
                      "pgb_estimate_dt")

    def run(self, ncycles, graph=True, history=None):
        """ncycles RK2 cycles with a refinement check after every check_interval-th.
        history: written at cycle 0 and checked after each cycle's remesh and dt update
        (the order of EvolutionDriver::Execute, driver.cpp:109-144)."""
        done = 0
        nx = self.mesh.block_nx
        if history is not None and self.ncycle == 0:
            history.maybe_write(self.mesh, self.base, self.dt, 0, self.stream)
        while done < ncycles:
            k = min(ncycles - done, self.check_interval - self.ncycle % self.check_interval)
            if history is not None:
                k = 1
            self.rk.run(k, graph=graph)
            self.zone_cycles += k * self.mesh.nblocks * nx[0] * nx[1] * nx[2]
            self.ncycle += k
            done += k
            if self.ncycle % self.check_interval == 0:
                self.adapt()
            if history is not None:
                history.maybe_write(self.mesh, self.base, self.dt, self.ncycle, self.stream)
