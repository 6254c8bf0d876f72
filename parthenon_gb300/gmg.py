"""Host handle of the geometric-multigrid solver (native library, uniform periodic cube).

Mirrors MGSolver<u, rhs, PoissonEquation> (src/solvers/mg_solver.hpp:73-521) for the
Poisson equation div(grad u) = rhs: FAS V-cycles with SRJ or weighted-Jacobi
smoothing, solved in FP64 or as an FP32 V-cycle inside FP64 iterative refinement.
"""
import ctypes

from . import _native as nat
from .mesh import _ptr, _stream


class GmgSolver:
    def __init__(self, n, ncoarsen, stages=2, jacobi=False, weight=2.0 / 3.0, coarse_sweeps=0, exact=False,
                 xmin=0.0, xmax=1.0):
        p = nat.GmgParams()
        p.n, p.ncoarsen, p.stages, p.jacobi = int(n), int(ncoarsen), int(stages), int(bool(jacobi))
        p.weight, p.coarse_sweeps, p.exact = float(weight), int(coarse_sweeps), int(bool(exact))
        p.xmin, p.xmax = float(xmin), float(xmax)
        h = ctypes.c_void_p()
        nat.check(nat.lib().pgb_gmg_create(ctypes.byref(p), ctypes.byref(h)), "pgb_gmg_create")
        self._h = h
        self.n = int(n)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            nat.lib().pgb_gmg_destroy(h)
            self._h = None

    def vcycles(self, u, rhs, ncycles, stream=None):
        import numpy as np
        rms = np.zeros(max(1, ncycles))
        nat.check(nat.lib().pgb_gmg_vcycles(self._h, _ptr(u), _ptr(rhs), int(ncycles),
                                            rms.ctypes.data_as(ctypes.c_void_p), _stream(stream)),
                  "pgb_gmg_vcycles")
        return rms[:ncycles]

    def bicgstab(self, u, rhs, precondition="fp64", rtol=1e-10, relative=True, max_iters=1000, stream=None):
        """BiCGSTABSolver (bicgstab_solver.hpp) from u = 0 with a V-cycle preconditioner
        ("fp64", "fp32" or None); returns (iterations, final rms residual)."""
        import torch
        if stream is None:
            stream = self._stream = getattr(self, "_stream", None) or torch.cuda.Stream()
        stream.wait_stream(torch.cuda.current_stream())
        mode = {None: 0, "none": 0, "fp64": 1, "fp32": 2}[precondition]
        it = ctypes.c_int32(0)
        rms = ctypes.c_double(0.0)
        nat.check(nat.lib().pgb_gmg_bicgstab(self._h, _ptr(u), _ptr(rhs), mode, float(rtol), int(bool(relative)),
                                             int(max_iters), ctypes.byref(it), ctypes.byref(rms), _stream(stream)),
                  "pgb_gmg_bicgstab")
        torch.cuda.current_stream().wait_stream(stream)
        return it.value, rms.value

    METHODS = {"fp64": 0, "mixed": 1, "bicgstab-fp64": 2, "bicgstab-fp32": 3}

    def solve_blocks(self, mesh, u, rhs, comp_u=0, comp_rhs=0, method="fp64", rtol=1e-10, max_iters=200,
                     stream=None):
        """Solve on meshblock fields (Mesh.new_field layout): the right-hand side is
        component comp_rhs of rhs, the solution goes to the interior of component comp_u
        of u. Returns (iterations, relative residual)."""
        import torch
        if stream is None:
            stream = self._stream = getattr(self, "_stream", None) or torch.cuda.Stream()
        stream.wait_stream(torch.cuda.current_stream())
        mesh._ensure()
        it = ctypes.c_int32(0)
        rel = ctypes.c_double(0.0)
        nat.check(nat.lib().pgb_gmg_solve_blocks(self._h, mesh.handle, _ptr(u), _ptr(rhs), u.shape[1], int(comp_u),
                                                 int(comp_rhs), self.METHODS[method], float(rtol), int(max_iters),
                                                 ctypes.byref(it), ctypes.byref(rel), _stream(stream)),
                  "pgb_gmg_solve_blocks")
        torch.cuda.current_stream().wait_stream(stream)
        return it.value, rel.value

    def solve(self, u, rhs, mixed=False, rtol=1e-10, max_cycles=200, stream=None):
        cyc = ctypes.c_int32(0)
        rel = ctypes.c_double(0.0)
        nat.check(nat.lib().pgb_gmg_solve(self._h, _ptr(u), _ptr(rhs), int(bool(mixed)), float(rtol),
                                          int(max_cycles), ctypes.byref(cyc), ctypes.byref(rel), _stream(stream)),
                  "pgb_gmg_solve")
        return cyc.value, rel.value


class CompositeMultigrid:
    """MGSolver on the two-level composite grids of a (refined) mesh.

    Grid L holds every block of level L and the leaves of level L - 1 (mesh-gmg.cpp:
    103-201); FAS V-cycles smooth the level-L blocks, restrict to the parents and
    prolongate the correction back (mg_solver.hpp:375-520). Fields are the leaf blocks'
    arrays in the exchange layout with one component: (nblocks, N3, N2, N1) float64.
    The operator is div(D grad u) - alpha u with constant D. exact=True rounds every
    value as the reference does (bitwise against the oracle); the default fast build
    uses FMA and the 7-point form of the operator. The host part (grids, index maps)
    needs no GPU; device memory is taken on the first solve.
    """

    def __init__(self, mesh, stages=2, jacobi=False, weight=2.0 / 3.0, coarse_sweeps=0, max_coarsenings=30,
                 D=1.0, alpha=0.0, exact=False, flux_correct=False):
        p = nat.MgParams()
        p.exact = int(bool(exact))
        p.flux_correct = int(bool(flux_correct))
        p.stages, p.jacobi, p.weight = int(stages), int(bool(jacobi)), float(weight)
        p.coarse_sweeps, p.max_coarsenings = int(coarse_sweeps), int(max_coarsenings)
        p.D, p.alpha = float(D), float(alpha)
        self.mesh = mesh  # the solver reads the mesh's topology
        h = ctypes.c_void_p()
        nat.check(nat.lib().pgb_mg_create(mesh.handle, ctypes.byref(p), ctypes.byref(h)), "pgb_mg_create")
        self._h = h
        info = (ctypes.c_int32 * 5)()
        nat.check(nat.lib().pgb_mg_info(self._h, info), "pgb_mg_info")
        self.lmin, self.lmax, self.nslots, self.nleaf, self.ngrids = (int(x) for x in info)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            nat.lib().pgb_mg_destroy(h)
            self._h = None

    def boundaries(self, level):
        """gmg_same index maps of grid `level` (records as Mesh.boundaries)."""
        import numpy as np
        n = ctypes.c_int32(0)
        nat.check(nat.lib().pgb_mg_boundaries(self._h, int(level), None, 0, ctypes.byref(n)), "pgb_mg_boundaries")
        out = np.zeros((n.value, 23), np.int32)
        nat.check(nat.lib().pgb_mg_boundaries(self._h, int(level), out.ctypes.data_as(ctypes.c_void_p), n.value,
                                              ctypes.byref(n)), "pgb_mg_boundaries")
        return out

    def _check(self, *fields):
        n = self.nleaf * self.mesh.N[0] * self.mesh.N[1] * self.mesh.N[2]
        for f in fields:
            if not (f.is_cuda and f.dtype.is_floating_point and f.element_size() == 8 and f.is_contiguous()
                    and f.numel() == n):
                raise ValueError("fields must be contiguous float64 CUDA tensors of the leaf blocks, "
                                 "(nblocks, N3, N2, N1)")

    def _stream(self, stream):
        import torch
        if stream is None:
            stream = self._own_stream = getattr(self, "_own_stream", None) or torch.cuda.Stream()
        stream.wait_stream(torch.cuda.current_stream())
        return stream

    def set_coefficient(self, d, stream=None):
        """The face coefficient D of the leaves, (nblocks, 3, N3, N2, N1) float64 on the
        device (face i the low face of cell i); restricted to every grid."""
        n = self.nleaf * 3 * self.mesh.N[0] * self.mesh.N[1] * self.mesh.N[2]
        if not (d.is_cuda and d.element_size() == 8 and d.is_contiguous() and d.numel() == n):
            raise ValueError("D must be a contiguous float64 CUDA tensor (nblocks, 3, N3, N2, N1)")
        s = self._stream(stream)
        nat.check(nat.lib().pgb_mg_set_coefficient(self._h, _ptr(d), _stream(s)), "pgb_mg_set_coefficient")

    def vcycles(self, u, rhs, ncycles, stream=None):
        """ncycles V-cycles on u (in place); the rms leaf residual after each."""
        import numpy as np
        import torch
        self._check(u, rhs)
        s = self._stream(stream)
        rms = np.zeros(max(1, ncycles))
        nat.check(nat.lib().pgb_mg_vcycles(self._h, _ptr(u), _ptr(rhs), int(ncycles),
                                           rms.ctypes.data_as(ctypes.c_void_p), _stream(s)), "pgb_mg_vcycles")
        torch.cuda.current_stream().wait_stream(s)
        return rms[:ncycles]

    def solve(self, u, rhs, tol=1e-10, relative=True, max_cycles=200, mixed=False, stream=None):
        """Iterations until the rms leaf residual is below tol (times the initial one when
        relative); mixed: an FP32 V-cycle inside FP64 iterative refinement. Returns
        (iterations, final rms or relative rms)."""
        import torch
        self._check(u, rhs)
        s = self._stream(stream)
        cyc = ctypes.c_int32(0)
        r = ctypes.c_double(0.0)
        nat.check(nat.lib().pgb_mg_solve(self._h, _ptr(u), _ptr(rhs), float(tol), int(bool(relative)),
                                         int(bool(mixed)), int(max_cycles), ctypes.byref(cyc), ctypes.byref(r),
                                         _stream(s)),
                  "pgb_mg_solve")
        torch.cuda.current_stream().wait_stream(s)
        return cyc.value, r.value

    def bicgstab(self, u, rhs, precondition="fp64", rtol=1e-10, relative=True, max_iters=1000, stream=None):
        """BiCGSTABSolver on the leaf grid from u = 0 with one composite V-cycle per
        preconditioner application ("fp64", "fp32" or None); returns (iterations, final
        rms residual)."""
        import torch
        self._check(u, rhs)
        s = self._stream(stream)
        mode = {None: 0, "none": 0, "fp64": 1, "fp32": 2}[precondition]
        it = ctypes.c_int32(0)
        rms = ctypes.c_double(0.0)
        nat.check(nat.lib().pgb_mg_bicgstab(self._h, _ptr(u), _ptr(rhs), mode, float(rtol), int(bool(relative)),
                                            int(max_iters), ctypes.byref(it), ctypes.byref(rms), _stream(s)),
                  "pgb_mg_bicgstab")
        torch.cuda.current_stream().wait_stream(s)
        return it.value, rms.value
