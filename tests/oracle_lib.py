"""ctypes loader for the CPU oracle (test infrastructure).

Only tests, the smoke check and the CPU-baseline leg of bench.py load this module.
It builds oracle/liboracle.so on first use when the compiled library is missing.
"""
import ctypes
import os
import subprocess

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE_DIR = os.path.join(ROOT, "oracle")
LIB_PATH = os.path.join(ORACLE_DIR, "_build", "liboracle.so")

_lib = None

I32P = ctypes.POINTER(ctypes.c_int32)
I64P = ctypes.POINTER(ctypes.c_int64)
DP = ctypes.POINTER(ctypes.c_double)
U64P = ctypes.POINTER(ctypes.c_uint64)


def build():
    subprocess.check_call(["make", "-s", "-C", ORACLE_DIR])


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = ctypes.CDLL(LIB_PATH)
        L.orc_sim_create.restype = ctypes.c_void_p
        L.orc_sim_create.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
                                     ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
                                     ctypes.c_void_p, ctypes.c_int, ctypes.c_int,
                                     ctypes.c_int, ctypes.c_double, ctypes.c_void_p,
                                     ctypes.c_int]
        L.orc_sim_destroy.argtypes = [ctypes.c_void_p]
        for name in ["orc_nblocks", "orc_multilevel", "orc_num_boundaries"]:
            getattr(L, name).argtypes = [ctypes.c_void_p]
            getattr(L, name).restype = ctypes.c_int
        L.orc_block_info.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
        for name in ["orc_base", "orc_base_coarse", "orc_derived"]:
            getattr(L, name).argtypes = [ctypes.c_void_p]
            getattr(L, name).restype = DP
        for name in ["orc_field_size", "orc_coarse_size"]:
            getattr(L, name).argtypes = [ctypes.c_void_p]
            getattr(L, name).restype = ctypes.c_int64
        L.orc_boundaries.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
        L.orc_exchange.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int]
        L.orc_exchange.restype = ctypes.c_int64
        L.orc_init_dt.argtypes = [ctypes.c_void_p]
        L.orc_init_dt.restype = ctypes.c_double
        L.orc_dt.argtypes = [ctypes.c_void_p]
        L.orc_dt.restype = ctypes.c_double
        L.orc_run.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_void_p]
        L.orc_run.restype = ctypes.c_int
        L.orc_max_threads.restype = ctypes.c_int
        L.orc_pack.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
        L.orc_pack.restype = ctypes.c_int64
        L.orc_ownership.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]
        L.orc_ownership.restype = ctypes.c_uint32
        L.orc_range_mask.argtypes = [ctypes.c_int, ctypes.c_uint32, ctypes.c_int,
                                     ctypes.c_int, ctypes.c_int]
        L.orc_range_mask.restype = ctypes.c_uint32
        L.orc_morton.argtypes = [ctypes.c_int, ctypes.c_int64, ctypes.c_int64,
                                 ctypes.c_int64, ctypes.c_void_p]
        L.orc_block_criterion.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_void_p]
        L.orc_set_refinement.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_double, ctypes.c_double,
                                         ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_void_p]
        L.orc_remesh.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
        L.orc_remesh.restype = ctypes.c_int
        L.orc_remesh_dt.argtypes = [ctypes.c_void_p]
        L.orc_remesh_dt.restype = ctypes.c_double
        L.orc_time.argtypes = [ctypes.c_void_p]
        L.orc_time.restype = ctypes.c_double
        L.orc_ncycle.argtypes = [ctypes.c_void_p]
        L.orc_ncycle.restype = ctypes.c_int
        L.orc_history_mass.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_double,
                                       ctypes.c_void_p]
        L.orc_sparse_enable.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                        ctypes.c_int]
        L.orc_sparse_set.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
        L.orc_sparse_get.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
        L.orc_sparse_dealloc.argtypes = [ctypes.c_void_p]
        L.orc_sparse_tag.argtypes = [ctypes.c_void_p, ctypes.c_double, ctypes.c_double, ctypes.c_void_p]
        L.orc_set_comp_vel.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
        _lib = L
    return _lib


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p)


class OracleSim:
    """A Parthenon-semantics simulation on the CPU (one periodic tree)."""

    def __init__(self, nx, bnx, ng, xmin=(0.0, 0.0, 0.0), xmax=(1.0, 1.0, 1.0),
                 leaves=None, ncomp=1, physics="advection", recon=0, cfl=0.3,
                 vel=(1.0, 1.0, 1.0), prolong_in_stage=True):
        L = lib()
        nx = np.asarray(nx, np.int32)
        bnx = np.asarray(bnx, np.int32)
        xmin = np.asarray(xmin, np.float64)
        xmax = np.asarray(xmax, np.float64)
        lv = np.zeros((0, 4), np.int64) if leaves is None else np.asarray(leaves, np.int64)
        vel = np.asarray(vel, np.float64)
        self._keep = (nx, bnx, xmin, xmax, lv, vel)
        phys = {"advection": 0, "burgers": 1}[physics]
        self.h = L.orc_sim_create(_ptr(nx), _ptr(bnx), int(ng), _ptr(xmin), _ptr(xmax),
                                  int(lv.shape[0]), _ptr(lv), int(ncomp), phys, int(recon),
                                  float(cfl), _ptr(vel), int(bool(prolong_in_stage)))
        if not self.h:
            raise RuntimeError("oracle mesh construction failed")
        self.ng = int(ng)
        self.ncomp = int(ncomp)
        self.bnx = tuple(int(x) for x in bnx)
        self.nblocks = L.orc_nblocks(self.h)
        self.N = tuple(b + 2 * ng for b in self.bnx)
        self.Nc = tuple(max(1, b // 2) + 2 * ng for b in self.bnx)

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_sim_destroy(self.h)
            self.h = None

    @property
    def multilevel(self):
        return bool(lib().orc_multilevel(self.h))

    def block_info(self):
        locs = np.zeros((self.nblocks, 4), np.int64)
        geom = np.zeros((self.nblocks, 6), np.float64)
        lib().orc_block_info(self.h, _ptr(locs), _ptr(geom))
        return locs, geom

    def derived(self):
        """The Burgers "derived" field (nblocks, N3, N2, N1), filled after every stage."""
        p = lib().orc_derived(self.h)
        if not p:
            raise RuntimeError("no derived field (advection)")
        n = self.nblocks * self.N[0] * self.N[1] * self.N[2]
        return np.ctypeslib.as_array(p, shape=(n,)).reshape((self.nblocks,) + self.N[::-1])

    def base(self):
        n = lib().orc_field_size(self.h)
        p = lib().orc_base(self.h)
        a = np.ctypeslib.as_array(p, shape=(n,))
        return a.reshape(self.nblocks, self.ncomp, self.N[2], self.N[1], self.N[0])

    def coarse(self):
        n = lib().orc_coarse_size(self.h)
        p = lib().orc_base_coarse(self.h)
        a = np.ctypeslib.as_array(p, shape=(n,))
        return a.reshape(self.nblocks, self.ncomp, self.Nc[2], self.Nc[1], self.Nc[0])

    def boundaries(self):
        n = lib().orc_num_boundaries(self.h)
        out = np.zeros((n, 23), np.int32)
        lib().orc_boundaries(self.h, _ptr(out))
        return out

    def exchange(self, prolongate=True, op=0):
        return lib().orc_exchange(self.h, int(bool(prolongate)), int(op))

    def init_dt(self):
        return lib().orc_init_dt(self.h)

    def run(self, ncycles, nthreads=0):
        dts = np.zeros(max(ncycles, 1), np.float64)
        rc = lib().orc_run(self.h, int(ncycles), int(nthreads), _ptr(dts))
        if rc != 0:
            raise RuntimeError("oracle run failed")
        return dts[:ncycles]

    def dt(self):
        return lib().orc_dt(self.h)

    def pack(self):
        total = int(self.boundaries()[:, 18].sum()) * self.ncomp
        out = np.zeros(max(total, 1), np.float64)
        n = lib().orc_pack(self.h, _ptr(out))
        assert n == total
        return out[:total]

    # adaptive refinement
    def block_criterion(self, comp, method=0):
        out = np.zeros(self.nblocks, np.float64)
        lib().orc_block_criterion(self.h, int(comp), int(method), _ptr(out))
        return out

    def set_refinement(self, crit, rtol, dtol, crit_max_level, mesh_max_level, threshold=10):
        c = np.ascontiguousarray(crit, np.float64)
        flags = np.zeros(self.nblocks, np.int32)
        lib().orc_set_refinement(self.h, _ptr(c), float(rtol), float(dtol), int(crit_max_level),
                                 int(mesh_max_level), int(threshold), _ptr(flags))
        return flags

    def remesh(self, flags):
        """Tree update + data movement of the base field; True when the mesh changed."""
        f = np.ascontiguousarray(flags, np.int32)
        rc = lib().orc_remesh(self.h, _ptr(f))
        if rc < 0:
            raise RuntimeError("oracle remesh failed")
        self.nblocks = lib().orc_nblocks(self.h)
        return rc == 1

    def time(self):
        return lib().orc_time(self.h)

    def ncycle(self):
        return lib().orc_ncycle(self.h)

    def history_mass(self, regions, mesh_volume):
        r = np.ascontiguousarray(regions, np.float64).reshape(-1, 6)
        out = np.zeros(r.shape[0], np.float64)
        lib().orc_history_mass(self.h, _ptr(r), int(r.shape[0]), float(mesh_volume), _ptr(out))
        return out

    def remesh_dt(self):
        """Every block of the new mesh votes again; SetGlobalTimeStep from the previous step."""
        return lib().orc_remesh_dt(self.h)

    # sparse variables
    def sparse_enable(self, alloc_threshold, dealloc_threshold, dealloc_count=5, default_value=0.0):
        """Every component becomes a sparse variable; per-component thresholds (scalars
        broadcast). All variables start unallocated."""
        def vec(x):
            return np.ascontiguousarray(np.broadcast_to(np.asarray(x, np.float64), (self.ncomp,)))
        a, d, v = vec(alloc_threshold), vec(dealloc_threshold), vec(default_value)
        lib().orc_sparse_enable(self.h, _ptr(a), _ptr(d), _ptr(v), int(dealloc_count))

    def sparse_set(self, alloc, counts=None):
        a = np.ascontiguousarray(alloc, np.uint8).reshape(self.nblocks, self.ncomp)
        c = None if counts is None else np.ascontiguousarray(counts, np.int32).reshape(self.nblocks, self.ncomp)
        lib().orc_sparse_set(self.h, _ptr(a), None if c is None else _ptr(c))

    def sparse_alloc(self):
        """(alloc [nblocks, ncomp] uint8, dealloc counters [nblocks, ncomp] int32)"""
        a = np.zeros((self.nblocks, self.ncomp), np.uint8)
        c = np.zeros((self.nblocks, self.ncomp), np.int32)
        lib().orc_sparse_get(self.h, _ptr(a), _ptr(c))
        return a, c

    def sparse_dealloc(self):
        lib().orc_sparse_dealloc(self.h)

    def sparse_tag(self, refine_tol, derefine_tol):
        out = np.zeros(self.nblocks, np.float64)
        lib().orc_sparse_tag(self.h, float(refine_tol), float(derefine_tol), _ptr(out))
        return out

    def set_component_velocities(self, vel):
        v = np.ascontiguousarray(vel, np.float64).reshape(self.ncomp, 3)
        self._cvel = v
        lib().orc_set_comp_vel(self.h, _ptr(v))


def ownership(main, locs):
    locs = np.asarray(locs, np.int64).reshape(-1, 4)
    m = np.asarray(main, np.int64)
    return lib().orc_ownership(_ptr(m), int(locs.shape[0]), _ptr(locs))


def range_mask(el, own_bits, ox1, ox2, ox3):
    return lib().orc_range_mask(int(el), int(own_bits), int(ox1), int(ox2), int(ox3))


def morton(level, l1, l2, l3):
    out = np.zeros(3, np.uint64)
    lib().orc_morton(int(level), int(l1), int(l2), int(l3), _ptr(out))
    return out


def bit(a, b, c):
    return 1 << ((a + 1) + 3 * (b + 1) + 9 * (c + 1))


def _gmg_lib():
    L = lib()
    if not getattr(L, "_gmg_ready", False):
        L.orc_gmg_create.restype = ctypes.c_void_p
        L.orc_gmg_create.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                                     ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_int]
        L.orc_gmg_destroy.argtypes = [ctypes.c_void_p]
        for name in ["orc_gmg_u", "orc_gmg_rhs", "orc_gmg_res"]:
            getattr(L, name).argtypes = [ctypes.c_void_p]
            getattr(L, name).restype = DP
        L.orc_gmg_run.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]
        L.orc_gmg_residual.argtypes = [ctypes.c_void_p]
        L.orc_gmg_residual.restype = ctypes.c_double
        L.orc_bicgstab.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_double,
                                   ctypes.c_int, ctypes.c_int, ctypes.c_void_p]
        L.orc_bicgstab.restype = ctypes.c_int
        L._gmg_ready = True
    return L


class OracleGmg:
    """FP64 geometric multigrid (FAS V-cycle) on a uniform periodic grid."""

    def __init__(self, n, ncoarsen, xmin=0.0, xmax=1.0, stages=2, jacobi=False, weight=2.0 / 3.0,
                 coarse_sweeps=0):
        L = _gmg_lib()
        self.n = int(n)
        self.h = L.orc_gmg_create(self.n, int(ncoarsen), float(xmin), float(xmax), int(stages), int(bool(jacobi)),
                                  float(weight), int(coarse_sweeps))

    def __del__(self):
        if getattr(self, "h", None):
            _gmg_lib().orc_gmg_destroy(self.h)
            self.h = None

    def _view(self, fn):
        p = fn(self.h)
        return np.ctypeslib.as_array(p, shape=(self.n ** 3,)).reshape(self.n, self.n, self.n)

    def u(self):
        return self._view(_gmg_lib().orc_gmg_u)

    def rhs(self):
        return self._view(_gmg_lib().orc_gmg_rhs)

    def run(self, ncycles):
        rms = np.zeros(max(1, ncycles))
        _gmg_lib().orc_gmg_run(self.h, int(ncycles), _ptr(rms))
        return rms[:ncycles]

    def residual(self):
        return _gmg_lib().orc_gmg_residual(self.h)

    def bicgstab(self, rhs, precondition=True, rtol=1e-10, relative=True, max_iters=1000):
        """(solution, iterations, final rms residual) of the right-preconditioned BiCGSTAB."""
        b = np.ascontiguousarray(rhs, np.float64).reshape(-1)
        x = np.zeros_like(b)
        rms = np.zeros(1)
        it = _gmg_lib().orc_bicgstab(self.h, _ptr(b), _ptr(x), int(bool(precondition)), float(rtol),
                                     int(bool(relative)), int(max_iters), _ptr(rms))
        return x.reshape(self.n, self.n, self.n), it, float(rms[0])


def _mgb_lib():
    L = lib()
    if not getattr(L, "_mgb_ready", False):
        L.orc_mgb_create.restype = ctypes.c_void_p
        L.orc_mgb_create.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_int,
                                     ctypes.c_int, ctypes.c_double, ctypes.c_double]
        L.orc_mgb_destroy.argtypes = [ctypes.c_void_p]
        L.orc_mgb_info.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
        for name in ["orc_mgb_u", "orc_mgb_rhs", "orc_mgb_res"]:
            getattr(L, name).argtypes = [ctypes.c_void_p]
            getattr(L, name).restype = DP
        L.orc_mgb_run.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]
        L.orc_mgb_residual.argtypes = [ctypes.c_void_p]
        L.orc_mgb_residual.restype = ctypes.c_double
        L.orc_mgb_num_boundaries.argtypes = [ctypes.c_void_p, ctypes.c_int]
        L.orc_mgb_num_boundaries.restype = ctypes.c_int
        L.orc_mgb_boundaries.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]
        L.orc_mgb_bicgstab.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
                                       ctypes.c_double, ctypes.c_int, ctypes.c_int, ctypes.c_void_p]
        L.orc_mgb_bicgstab.restype = ctypes.c_int
        L.orc_mgb_set_coefficient.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
        L.orc_mgb_set_flux_correct.argtypes = [ctypes.c_void_p, ctypes.c_int]
        L._mgb_ready = True
    return L


class OracleMgBlocks:
    """FP64 FAS V-cycle on the two-level composite grids of a (refined) mesh.

    Fields u and rhs live on the leaf blocks in the exchange layout
    [block][k][j][i] with ghosts; the multigrid's internal blocks are private."""

    def __init__(self, sim, stages=2, jacobi=False, weight=2.0 / 3.0, coarse_sweeps=0, max_coarsenings=30,
                 D=1.0, alpha=0.0, flux_correct=False):
        L = _mgb_lib()
        self.sim = sim  # the mesh must outlive the solver
        self.h = L.orc_mgb_create(sim.h, int(stages), int(bool(jacobi)), float(weight), int(coarse_sweeps),
                                  int(max_coarsenings), float(D), float(alpha))
        if not self.h:
            raise RuntimeError("oracle multigrid construction failed")
        L.orc_mgb_set_flux_correct(self.h, int(bool(flux_correct)))
        info = np.zeros(4, np.int32)
        L.orc_mgb_info(self.h, _ptr(info))
        self.lmin, self.lmax, self.nslots, self.nleaf = (int(x) for x in info)

    def __del__(self):
        if getattr(self, "h", None):
            _mgb_lib().orc_mgb_destroy(self.h)
            self.h = None

    def _view(self, fn):
        N = self.sim.N
        p = fn(self.h)
        return np.ctypeslib.as_array(p, shape=(self.nleaf * N[0] * N[1] * N[2],)).reshape(
            self.nleaf, N[2], N[1], N[0])

    def u(self):
        return self._view(_mgb_lib().orc_mgb_u)

    def rhs(self):
        return self._view(_mgb_lib().orc_mgb_rhs)

    def res(self):
        return self._view(_mgb_lib().orc_mgb_res)

    def run(self, ncycles):
        rms = np.zeros(max(1, ncycles))
        _mgb_lib().orc_mgb_run(self.h, int(ncycles), _ptr(rms))
        return rms[:ncycles]

    def residual(self):
        return _mgb_lib().orc_mgb_residual(self.h)

    def boundaries(self, level):
        n = _mgb_lib().orc_mgb_num_boundaries(self.h, int(level))
        if n < 0:
            raise ValueError("no multigrid grid at that level")
        out = np.zeros((n, 23), np.int32)
        _mgb_lib().orc_mgb_boundaries(self.h, int(level), _ptr(out))
        return out

    def bicgstab(self, rhs, precondition=True, rtol=1e-10, relative=True, max_iters=1000):
        """(solution in the leaf layout, iterations, final rms residual) of BiCGSTAB with
        one composite V-cycle per preconditioner application."""
        b = np.ascontiguousarray(rhs, np.float64)
        x = np.zeros_like(b)
        rms = np.zeros(1)
        it = _mgb_lib().orc_mgb_bicgstab(self.h, _ptr(b), _ptr(x), int(bool(precondition)), float(rtol),
                                         int(bool(relative)), int(max_iters), _ptr(rms))
        return x, it, float(rms[0])

    def set_coefficient(self, d):
        """Face coefficient D of the leaves, (nleaf, 3, N3, N2, N1); face i is the low face
        of cell i. Restricted to the internal blocks as the setup tasks do."""
        d = np.ascontiguousarray(d, np.float64)
        self._d = d
        _mgb_lib().orc_mgb_set_coefficient(self.h, _ptr(d))
