"""RK2 evolution driver for the advection and Burgers packages on the GPU.

Mirrors EvolutionDriver::Execute + MultiStageDriverGeneric::Step
(src/driver/driver.cpp:67-166, src/driver/multistage.hpp:39-53) for the two task
collections on the hot path (example/advection/advection_driver.cpp:56-164 and
benchmarks/burgers/burgers_driver.cpp:53-148): per cycle two stages, each
fluxes -> [flux correction] -> flux divergence -> Average -> Update -> ghost exchange,
then EstimateTimestep + SetGlobalTimeStep. Every step runs on the device; dt lives in
device memory, so a cycle is one CUDA-graph launch.
"""
import ctypes

import numpy as np

from . import _native as nat
from .mesh import _ptr, _stream


class StageConfig:
    """physics: 'advection' or 'burgers'; recon: 'dc'/'plm' (advection) or
    'weno5'/'linear' (Burgers); exact: bitwise reference arithmetic instead of the
    FMA/shared-reciprocal kernels. comp_vel (advection): one (vx, vy, vz) per
    component instead of the common `vel` (the sparse advection package's velocities)."""

    def __init__(self, physics, recon, cfl, vel=(1.0, 1.0, 1.0), exact=False, comp_vel=None):
        self.physics = physics
        self.recon = recon
        self.cfl = float(cfl)
        self.vel = tuple(float(v) for v in vel)
        self.exact = bool(exact)
        self.comp_vel = None if comp_vel is None else np.ascontiguousarray(comp_vel, np.float64).reshape(-1, 3)

    def params(self):
        p = nat.StageParams()
        p.physics = {"advection": 0, "burgers": 1}[self.physics]
        rec = {"advection": {"dc": 0, "plm": 1}, "burgers": {"weno5": 0, "linear": 1}}[self.physics]
        p.recon = rec[self.recon]
        p.exact = 1 if self.exact else 0
        for d in range(3):
            p.vel[d] = self.vel[d]
        p.cfl = self.cfl
        if self.comp_vel is not None:
            p.ncomp_vel = self.comp_vel.shape[0]
            p.comp_vel = self.comp_vel.ctypes.data_as(nat.DP)  # kept alive by self.comp_vel
        return p


class RK2Driver:
    """Owns the device state of one run: base and stage fields, scratch, coarse
    buffers (multilevel), and the device dt."""

    def __init__(self, mesh, ncomp, config, stream=None):
        import torch
        self.ncomp = int(ncomp)
        self.cfg = config
        self.params = config.params()
        self.stream = stream if stream is not None else torch.cuda.Stream()
        self._allocate(mesh)
        with torch.cuda.stream(self.stream):
            # [current step, step the last update started from, simulation time]
            self.dt = torch.zeros(3, dtype=torch.float64, device="cuda")
        self.ncycle = 0

    def _allocate(self, mesh, base=None):
        import torch
        self.mesh = mesh.upload() if not mesh._uploaded else mesh
        ncomp = self.ncomp
        with torch.cuda.stream(self.stream):
            self.base = mesh.new_field(ncomp) if base is None else base
            self.stage = mesh.new_field(ncomp)
            if mesh.multilevel:
                self.dudt = None
                self.flux = torch.zeros((mesh.nblocks, 3) + tuple(self.base.shape[1:]), dtype=torch.float64,
                                        device="cuda")
                self.cbase = mesh.new_coarse(ncomp)
                self.cstage = mesh.new_coarse(ncomp)
            else:
                self.dudt = mesh.new_field(ncomp)
                self.flux = None
                self.cbase = self.cstage = None
            # Burgers: the package's "derived" field (one component), filled after every
            # stage's update (FillDerived, burgers_driver.cpp:121)
            self.derived = mesh.new_field(1) if self.cfg.physics == "burgers" else None
        nat.check(nat.lib().pgb_set_derived(self.mesh.handle, _ptr(self.derived)), "pgb_set_derived")

    def release_scratch(self):
        """Drops every buffer but the base field before a remesh, so that the new mesh's
        arena is allocated beside the old base alone (the transfer reads only the base)."""
        nat.check(nat.lib().pgb_set_derived(self.mesh.handle, None), "pgb_set_derived")
        self.stage = self.dudt = self.flux = self.cbase = self.cstage = self.derived = None

    def rebind(self, mesh, base):
        """Continue on a new mesh (after a remesh) with `base` already on it: fresh
        scratch and coarse buffers, ghosts filled with prolongation (the post-remesh
        CommunicateBoundaries of RedistributeAndRefineMeshBlocks), then every block of
        the new mesh votes again and the last dt update is repeated with those votes
        (InitializeBlockTimeSteps + SetGlobalTimeStep, driver.cpp:129-131). The cycle
        graph is captured again on the next run because the new mesh handle has an
        empty graph cache."""
        import torch
        self._allocate(mesh, base)
        with torch.cuda.stream(self.stream):
            self.mesh.exchange(self.base, self.cbase, prolongate=True, stream=self.stream)
            self.stage.copy_(self.base)
            nat.check(nat.lib().pgb_estimate_dt(self.mesh.handle, ctypes.byref(self.params), _ptr(self.base),
                                                self.ncomp, _ptr(self.dt), 2, _stream(self.stream)),
                      "pgb_estimate_dt")

    @property
    def prolongate(self):
        # The Burgers task list wires Send/Receive/Set without ProlongateBounds
        # (burgers_driver.cpp:108-120); the advection list prolongates.
        return self.cfg.physics != "burgers"

    def set_state(self, host_array, alloc=None):
        """Load the initial condition (numpy, field layout incl. ghosts), fill ghosts
        (Mesh::Initialize -> Mesh::CommunicateBoundaries, which prolongates on
        multilevel meshes for every package, mesh.cpp:640-706) and set the first dt.
        alloc (meshes with sparse variables): allocation flags (nblocks, ncomp); the
        values of unallocated variables are dropped (they hold zeros)."""
        import torch
        if alloc is not None:
            a = np.asarray(alloc, np.uint8).reshape(self.mesh.nblocks, self.ncomp)
            self.mesh.set_sparse_alloc(a)
            host_array = np.where(a[:, :, None, None, None] != 0, np.asarray(host_array, np.float64), 0.0)
        src = torch.as_tensor(host_array, dtype=torch.float64)
        if src.is_cuda:
            # produced on the caller's stream: order the copy after it
            self.stream.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(self.stream):
            self.base.copy_(src, non_blocking=False)
            self.dt.zero_()
            self.mesh.exchange(self.base, self.cbase, prolongate=True, stream=self.stream)
            self.stage.copy_(self.base)
            nat.check(nat.lib().pgb_estimate_dt(self.mesh.handle, ctypes.byref(self.params), _ptr(self.base),
                                                self.ncomp, _ptr(self.dt), 1, _stream(self.stream)),
                      "pgb_estimate_dt")
        self.ncycle = 0

    def run(self, ncycles, graph=True, history=None):
        """ncycles RK2 cycles. history (e.g. history.BurgersHistory): checked at cycle 0
        and after every cycle, as Outputs::MakeOutputs is in the driver loop; cycles then
        run one launch sequence at a time because the check reads the time."""
        if history is None:
            self._cycles(ncycles, graph)
            return
        if self.ncycle == 0:
            history.maybe_write(self.mesh, self.base, self.dt, 0, self.stream)
        for _ in range(ncycles):
            self._cycles(1, graph)
            history.maybe_write(self.mesh, self.base, self.dt, self.ncycle, self.stream)

    def _cycles(self, ncycles, graph):
        nat.check(nat.lib().pgb_rk2_cycles(self.mesh.handle, ctypes.byref(self.params), _ptr(self.base),
                                           _ptr(self.stage), _ptr(self.dudt), _ptr(self.flux), _ptr(self.cbase),
                                           _ptr(self.cstage), self.ncomp, _ptr(self.dt), int(ncycles),
                                           1 if graph else 0, _stream(self.stream)), "pgb_rk2_cycles")
        self.ncycle += ncycles

    def zone_cycles(self, ncycles):
        nx = self.mesh.block_nx
        return ncycles * self.mesh.nblocks * nx[0] * nx[1] * nx[2]
