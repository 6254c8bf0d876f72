"""Benchmark: zone-cycles/s of the 3-D Burgers WENO5/HLL RK2 cycle (256^3 periodic mesh,
512 meshblocks of 32^3, 4 ghost cells, 3 velocity components + 8 passive scalars,
FP64), plus ghost-exchange HBM GB/s on the same field.

One `step` is one full RK2 cycle over every block: two stages of fluxes, flux
divergence and update, a ghost exchange after each stage, and the device-side dt
update. Inputs stay resident in HBM between steps (each field is 2.9 GB, far larger
than the 129 MB L2). Prints one JSON line (rank 0).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

--impl reference times the CPU restatement of the reference algorithm (the oracle,
all host threads) on the same workload: the 256^3 mesh in 512 meshblocks of 32^3 with
the same ghosts, components, initial state and physics, one RK2 cycle per step. Its
mesh, block list and initial state come from the oracle and the problem generators'
numpy code; the GPU library is not loaded in that arm.

Extra legs in the same line: per-kernel rooflines, the end-to-end host-buffer run, the
multigrid solve (FP64 vs mixed precision, key "gmg") and the adaptive 3-level Burgers
run (key "amr", --amr-cycles cycles with remeshing inside the timed region).
"""
import argparse
import ctypes
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

MESH_N, BLOCK_N, NGHOST, NSCALARS, CFL = 256, 32, 4, 8, 0.8
NCOMP = 3 + NSCALARS
METRIC = "zone-cycles/s"
WORKLOAD = "burgers3d-weno5-hll-rk2-256^3-32^3blocks-ng4-11vars-fp64"


def workload_config(mesh_n=MESH_N):
    """The workload both arms run (identical `config` in both JSON lines)."""
    return {"workload": WORKLOAD if mesh_n == MESH_N else WORKLOAD.replace("256^3", "%d^3" % mesh_n),
            "mesh": [mesh_n] * 3, "block": [BLOCK_N] * 3, "nblocks": (mesh_n // BLOCK_N) ** 3, "nghost": NGHOST,
            "ncomp": NCOMP, "recon": "weno5", "riemann": "hll", "integrator": "rk2", "cfl": CFL,
            "fill_derived": True, "initial": "8 random-phase sinusoids per velocity component (k in 1..4, seed 2), "
                                             "8 scalars U(0,1)",
            "l2": "inputs larger than L2 (2.9 GB per field at 256^3)"}


def _problems_module():
    """The problem generators (plain numpy), loaded from their file without importing
    the package, so that the CPU arm never loads the GPU library."""
    import importlib.util
    spec = importlib.util.spec_from_file_location("_pgb_problems", os.path.join(ROOT, "parthenon_gb300", "problems.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


class _OracleBlocks:
    """The block geometry the problem generators read (block count, ghost width, block
    size, per-block cell centres), taken from the oracle's own block list."""

    def __init__(self, sim):
        self.locs, self.geom = sim.block_info()
        self.nblocks, self.nghost, self.block_nx, self.N = sim.nblocks, sim.ng, sim.bnx, sim.N

    def block_info(self):
        return self.locs, self.geom

    def cell_centers(self):
        out = []
        for d in range(3):
            idx = np.arange(self.N[d]) - self.nghost
            out.append(self.geom[:, d:d + 1] + (idx[None, :] + 0.5) * self.geom[:, 3 + d:4 + d])
        return out


def _oracle():
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import oracle_lib
    return oracle_lib


def oracle_burgers(mesh_n=MESH_N, state=None):
    """The oracle holding the benchmark's initial state with ghosts filled and the first
    dt set. state: the field (numpy, field layout) or None to generate it from the
    oracle's block list."""
    O = _oracle()
    o = O.OracleSim((mesh_n,) * 3, (BLOCK_N,) * 3, NGHOST, ncomp=NCOMP, physics="burgers", recon=0, cfl=CFL,
                    prolong_in_stage=False)
    if state is None:
        state = _problems_module().burgers_state(_OracleBlocks(o), nscalars=NSCALARS, nmodes=8, kmax=4, seed=2)
    o.base()[:] = state
    o.exchange(False, 0)
    o.init_dt()
    return o


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    return ws, rank


class ClockSampler:
    """Samples nvidia-smi clocks and throttle reasons during the timed region."""

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": float(np.median(sm)), "sm_min_mhz": min(sm), "sm_max_mhz": max(mx),
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except (OSError, ValueError):
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


def fp64_peak_tflops(torch):
    """cuBLAS DGEMM throughput on this GPU (the FP64 counterpart of the bf16 peak)."""
    n = 8192
    a = torch.randn(n, n, dtype=torch.float64, device="cuda")
    b = torch.randn(n, n, dtype=torch.float64, device="cuda")
    for _ in range(2):
        torch.matmul(a, b)
    torch.cuda.synchronize()
    best = 1e30
    for _ in range(3):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        torch.matmul(a, b)
        e1.record()
        e1.synchronize()
        best = min(best, e0.elapsed_time(e1))
    del a, b
    return 2.0 * n ** 3 / (best * 1e-3) / 1e12


# Algorithmic FP64 operations per cell per stage for the Burgers stencil, counted from
# the reference formulation (benchmarks/burgers/recon.hpp:42-99 WENO5Z, 2 per cell per
# direction on 34/32 of the cells; burgers_package.hpp:32-43 HLL; update.hpp:42-56 and
# 70-89 flux divergence and weighted sums). Divides count as one operation.
WENO5Z_OPS = 115   # adds/muls/divides/abs/min/max in one WENO5Z call (both sides)
HLL_VEL_OPS = 33   # wave speeds + 3 velocity fluxes
HLL_SCALAR_OPS = 10
DIVUPD_OPS = 12    # per component: 3 face differences, sum, /V, average, update


# From one ncu capture of the three directional launches of a stage on the 128^3 mesh
# (64 blocks of 32^3, 11 components): warp instructions executed (557.8 + 605.6 +
# 627.4 M) and DRAM bytes read + written (442.3 + 691.2 + 971.6 MB), and one direct
# exchange launch (319.6 MB). Instructions and traffic grow in proportion to the
# blocks processed.
STAGE_WARP_INSTR_PER_BLOCK = (557.8e6 + 605.6e6 + 627.4e6) / 64
STAGE_DRAM_BYTES_PER_BLOCK = (442.3e6 + 691.2e6 + 971.6e6) / 64
EXCHANGE_DRAM_BYTES_PER_BLOCK = 319.6e6 / 64
# instruction issue of a GB300: 152 SMs x 4 schedulers x one warp instruction per cycle
ISSUE_PER_SM_CYCLE = 4


def burgers_ops_per_cell_stage(n, nc):
    recon = 3 * nc * WENO5Z_OPS * (n + 2) / n
    faces = 3 * (n + 1) / n * (HLL_VEL_OPS + (nc - 3) * HLL_SCALAR_OPS)
    return recon + faces + nc * DIVUPD_OPS


def max_over_ranks(torch, value, ws):
    """The slowest rank's value (the job's time is its slowest replica's): an all-reduce
    on the device under NCCL, on the host under gloo."""
    if ws <= 1:
        return value
    dev = "cuda" if torch.distributed.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(value)], dtype=torch.float64, device=dev)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def run_ours(args, ws, rank):
    import torch
    import parthenon_gb300 as pg
    from parthenon_gb300 import _native as nat
    from parthenon_gb300.mesh import _ptr, _stream

    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    mesh = pg.Mesh((args.mesh,) * 3, (BLOCK_N,) * 3, NGHOST).upload()
    state = pg.problems.burgers_state(mesh, nscalars=NSCALARS, nmodes=8, kmax=4, seed=2)
    cfg = pg.StageConfig("burgers", "weno5", CFL)
    if not args.no_extras:
        zones = mesh.nblocks * BLOCK_N ** 3
        # --- end-to-end through the C ABI with host buffers ----------------------------
        # measured first, in a process that has run nothing else on the device: later in the
        # process (after the device-timed run and the per-kernel loops) single calls have
        # run up to 0.1 s slower, which a fresh process never showed
        L = nat.lib()
        p = cfg.params()
        host_in = torch.from_numpy(state).pin_memory()
        host_out = torch.empty_like(host_in).pin_memory()
        e2e_steps = args.steps
        dt_steps = (ctypes.c_double * max(e2e_steps, args.warmup))()
        # warm-up call: allocates the mesh's host-run workspace (device buffers kept between
        # calls) and runs W cycles; the timed call then copies the field in and out again
        dt_h = ctypes.c_double(0.0)
        nat.check(L.pgb_run_host_dt(mesh.handle, ctypes.byref(p), ctypes.c_void_p(host_in.data_ptr()),
                                    ctypes.c_void_p(host_out.data_ptr()), NCOMP, args.warmup, ctypes.byref(dt_h),
                                    dt_steps), "pgb_run_host_dt")
        # the median of five timed calls, with the clocks they ran at
        e2e_runs = []
        with ClockSampler(dev) as e2e_clk:
            for _ in range(5):
                dt_h = ctypes.c_double(0.0)
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                nat.check(L.pgb_run_host_dt(mesh.handle, ctypes.byref(p), ctypes.c_void_p(host_in.data_ptr()),
                                            ctypes.c_void_p(host_out.data_ptr()), NCOMP, e2e_steps, ctypes.byref(dt_h),
                                            dt_steps), "pgb_run_host_dt")
                e2e_runs.append(time.perf_counter() - t0)
        e2e_s = max_over_ranks(torch, sorted(e2e_runs)[len(e2e_runs) // 2], ws)
        nat.check(L.pgb_release_host_workspace(mesh.handle), "pgb_release_host_workspace")
        nbytes = state.nbytes
        e2e = {"value": ws * e2e_steps * zones / e2e_s, "unit": METRIC, "h2d_bytes_per_step": nbytes / e2e_steps,
               "d2h_bytes_per_step": nbytes / e2e_steps + 8, "steps": e2e_steps,
               "calls_s": [round(x, 4) for x in e2e_runs], "clocks": e2e_clk.summary(),
               "note": "pgb_run_host_dt with host buffers: H2D of the initial field (2.9 GB, pinned), ghost fill, "
                       "initial dt, K cycles (the mesh's cycle graph) each followed by a D2H of that step's dt, D2H of "
                       "the final field; the state stays resident between steps; the mesh's device workspace was "
                       "allocated by an untimed warm-up call of W cycles; the median of five timed calls, measured "
                       "first in the process"}
    drv = pg.RK2Driver(mesh, NCOMP, cfg)
    drv.set_state(state)
    s = drv.stream
    zones = mesh.nblocks * BLOCK_N ** 3

    drv.run(args.warmup, graph=True)
    s.synchronize()
    if ws > 1:
        torch.distributed.barrier()
    with ClockSampler(dev) as clk:
        torch.cuda.synchronize()
        if ws > 1:
            torch.distributed.barrier()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(s)
        drv.run(args.steps, graph=True)
        e1.record(s)
        e1.synchronize()
        torch.cuda.synchronize()
        if ws > 1:
            torch.distributed.barrier()
    ms = max_over_ranks(torch, e0.elapsed_time(e1), ws)
    value = ws * args.steps * zones / (ms * 1e-3)
    if args.no_extras:
        return {"metric": METRIC, "value": value, "unit": METRIC, "n_gpus": ws, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms / args.steps, "mesh": args.mesh}

    # --- per-kernel timing on the launching stream (CUDA events) -------------------
    L = nat.lib()
    p = cfg.params()

    def time_calls(fn, reps):
        fn()
        s.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(s)
        for _ in range(reps):
            fn()
        e1.record(s)
        e1.synchronize()
        return e0.elapsed_time(e1) / reps

    def one_stage():
        nat.check(L.pgb_stage(mesh.handle, ctypes.byref(p), _ptr(drv.base), _ptr(drv.base), _ptr(drv.stage),
                              _ptr(drv.dudt), None, _ptr(drv.dt), 1.0, 0.0, 1.0, NCOMP, _stream(s)), "pgb_stage")

    def one_exchange():
        mesh.exchange(drv.stage, None, prolongate=False, stream=s)

    # the reference-layout exchange: pack every boundary into one buffer, then unpack
    # (SendBoundBufs / SetBounds with their pack and unpack kernels)
    with torch.cuda.stream(s):
        xbuf = torch.empty(mesh.buffer_elems * NCOMP, dtype=torch.float64, device="cuda")

    def one_buffered_exchange():
        nat.check(L.pgb_exchange(mesh.handle, _ptr(drv.stage), None, NCOMP, 0, _ptr(xbuf), _stream(s)),
                  "pgb_exchange (buffered)")

    stage_ms = time_calls(one_stage, 3)
    xchg_ms = time_calls(one_exchange, 10)
    bxchg_ms = time_calls(one_buffered_exchange, 10)
    del xbuf
    ghost_values = NCOMP * mesh.nblocks * ((BLOCK_N + 2 * NGHOST) ** 3 - BLOCK_N ** 3)
    xchg_bytes = 16.0 * ghost_values  # read the sender cell, write the ghost
    xchg_gbs = xchg_bytes / (xchg_ms * 1e-3) / 1e9
    bxchg_gbs = 2.0 * xchg_bytes / (bxchg_ms * 1e-3) / 1e9  # pack and unpack: 32 B per ghost value
    # HBM bytes a stage must move at least: read u_in with ghosts, u_base (stage 2
    # only, here stage 1), write u_out -- per block and component
    stage_hbm_bytes = 8.0 * NCOMP * mesh.nblocks * ((BLOCK_N + 2 * NGHOST) ** 3 + BLOCK_N ** 3)
    ops_cell = burgers_ops_per_cell_stage(BLOCK_N, NCOMP)
    stage_flops = ops_cell * zones
    stage_tflops = stage_flops / (stage_ms * 1e-3) / 1e12
    fp64_peak = fp64_peak_tflops(torch)
    peaks, peak_src = measured_peaks()
    clk_summary = clk.summary()
    sm_mhz = clk_summary.get("sm_mhz") or peaks.get("sm_max_mhz", 2070.0)
    nsm = torch.cuda.get_device_properties(dev).multi_processor_count
    issue_peak = ISSUE_PER_SM_CYCLE * nsm * sm_mhz * 1e6  # warp instructions per second
    issue_achieved = STAGE_WARP_INSTR_PER_BLOCK * mesh.nblocks / (stage_ms * 1e-3)

    peak_hbm = peaks["hbm_gbs"]
    out = {
        "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "parallelism": "replicas" if ws > 1 else "single-gpu",
        "config": workload_config(args.mesh),
        "roofline": {"kernel": "k_burgers_dir (3 directional launches per stage)", "bound": "issue",
                     "achieved": issue_achieved, "peak": issue_peak, "unit": "warp instructions/s",
                     "frac": issue_achieved / issue_peak, "traffic": STAGE_DRAM_BYTES_PER_BLOCK * mesh.nblocks,
                     "traffic_unit": "DRAM bytes per stage (ncu, scaled by blocks)",
                     "peak_source": "4 warp instructions per SM cycle x SMs x sampled SM clock",
                     "instructions_source": "ncu warp instructions per launch on 64 blocks, scaled by blocks",
                     "stage_ms": stage_ms,
                     "hbm_achieved_gbs": stage_hbm_bytes / (stage_ms * 1e-3) / 1e9,
                     "hbm_frac": stage_hbm_bytes / (stage_ms * 1e-3) / 1e9 / peak_hbm,
                     "reference_fp64_ops_per_cell_stage": ops_cell,
                     "reference_fp64_tflops_equivalent": stage_tflops, "fp64_dgemm_tflops": fp64_peak},
        "exchange_roofline": {"kernel": "k_copy (direct ghost copy)", "bound": "hbm", "achieved": xchg_gbs,
                              "peak": peak_hbm, "unit": "GB/s", "frac": xchg_gbs / peak_hbm,
                              "traffic": EXCHANGE_DRAM_BYTES_PER_BLOCK * mesh.nblocks,
                              "bytes_per_launch": xchg_bytes, "ms": xchg_ms, "peak_source": peak_src},
        "buffered_exchange_roofline": {"kernel": "k_pack + k_unpack (reference buffer layout)", "bound": "hbm",
                                       "achieved": bxchg_gbs, "peak": peak_hbm, "unit": "GB/s",
                                       "frac": bxchg_gbs / peak_hbm, "bytes_per_exchange": 2.0 * xchg_bytes,
                                       "ms": bxchg_ms, "peak_source": peak_src},
        "e2e": e2e,
        "gpu_launches": 12 * args.steps,
        "clocks": clk_summary,
    }
    detail = {"autotune": {k: {"choice": c, "ms": t} for k, (c, t) in nat.tune_report().items()}}
    if rank == 0 and ws == 1:
        # the oracle on the full workload: one cycle from the same initial state
        o = oracle_burgers(args.mesh, state)
        out["cpu_baseline"] = cpu_baseline(o, cycles=1)
        del o
    del drv, state, host_in, host_out
    legs = {}
    if args.amr_cycles > 0:
        legs["amr"] = amr_bench(torch, args.amr_cycles, with_cpu=(rank == 0 and ws == 1), root=args.amr_root)
    if args.sparse_cycles > 0:
        legs["sparse"] = sparse_bench(torch, args.sparse_cycles, with_cpu=(rank == 0 and ws == 1))
    legs["smr"] = smr_bench(torch, with_cpu=(rank == 0 and ws == 1))
    legs["gmg"] = gmg_bench(torch)
    legs["gmg_composite"] = gmg_composite_bench(torch, with_cpu=(rank == 0 and ws == 1))
    # the full leg records go to stderr; the JSON line keeps a summary of each, the
    # multigrid legs last
    detail.update(legs)
    print(json.dumps({"detail": detail}), file=sys.stderr)
    out["legs"] = {k: leg_summary(k, v) for k, v in legs.items()}
    return out


def leg_summary(name, r):
    """The headline figures of one extra leg."""
    def rnd(x, n=4):
        return float("%.*g" % (n, x)) if isinstance(x, float) else x
    if name in ("amr", "sparse", "smr"):
        keep = {"value": rnd(r["value"]), "unit": "zone-cycles/s", "ms_per_cycle": rnd(r["ms_per_cycle"])}
        for k in ("blocks_min", "blocks_max", "remeshes", "peak_mem_gb"):
            if k in r:
                keep[k] = rnd(r[k])
        if "cpu_baseline" in r:
            cb = r["cpu_baseline"]
            keep["cpu"] = {"value": rnd(cb["value"]), "cores": cb["cores"], "kind": cb["kind"]}
            keep["x_cpu"] = rnd(r["value"] / cb["value"], 3)
        keep["workload"] = r.get("config", {}).get("workload", "")
        return keep
    if name == "gmg":
        return {"fp64_ms": rnd(1e3 * r["fp64"]["seconds"]), "fp64_vcycles": r["fp64"]["vcycles"],
                "mixed_ms": rnd(1e3 * r["mixed"]["seconds"]), "mixed_vcycles": r["mixed"]["vcycles"],
                "mixed_over_fp64": rnd(r["time_ratio_mixed_over_fp64"], 3),
                "mixed_vs_fp64_rel_err": rnd(r["mixed_vs_fp64_rel_err"], 2),
                "bicgstab_mg_fp32_ms": rnd(1e3 * r["bicgstab_mg_fp32"]["seconds"]),
                "blocks_fp64_ms": rnd(1e3 * r["blocks"]["fp64"]["seconds"]),
                "blocks_mixed_over_fp64": rnd(r["blocks"]["time_ratio_mixed_over_fp64"], 3),
                "workload": "poisson3d-128^3-periodic-vcycle-to-8^3-jacobi2/3-2+2"}
    keep = {"fp64_ms": rnd(1e3 * r["seconds"]), "fp64_vcycles": r["vcycles"],
            "mixed_ms": rnd(1e3 * r["mixed"]["seconds"]), "mixed_iterations": r["mixed"]["iterations"],
            "mixed_over_fp64": rnd(r["time_ratio_mixed_over_fp64"], 3),
            "bicgstab_mg_fp32_ms": rnd(1e3 * r["bicgstab_mg_fp32"]["seconds"])}
    if "cpu_baseline" in r:
        keep["cpu_s_to_tol"] = rnd(r["cpu_baseline"]["seconds_to_tolerance"])
    keep["workload"] = "poisson3d-composite-128^3root-16^3blocks-central-eighth-refined-srj2"
    return keep


GMG_N, GMG_COARSEN = 128, 4  # 128^3 periodic Poisson, levels down to 8^3


def gmg_bench(torch):
    """Time to a 1e-10 relative residual: FP64 V-cycles vs an FP32 V-cycle inside FP64
    iterative refinement (weighted Jacobi, omega 2/3, 2 pre + 2 post sweeps; coarsest
    level smoothed 16 more passes in FP64), and the mixed solution's error against the
    FP64 solution."""
    import parthenon_gb300 as pg
    rhs = torch.tensor(pg.problems.poisson_rhs(GMG_N, ngauss=32, sigma=0.03, seed=4), device="cuda")
    g = pg.GmgSolver(GMG_N, GMG_COARSEN, stages=2, jacobi=True, weight=2.0 / 3.0, coarse_sweeps=16)
    s = torch.cuda.Stream()
    res = {}
    sols = {}
    for mixed in (False, True):
        best = None
        for rep in range(3):
            u = torch.zeros((GMG_N,) * 3, dtype=torch.float64, device="cuda")
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            cyc, rel = g.solve(u, rhs, mixed=mixed, rtol=1e-10, max_cycles=400, stream=s)
            s.synchronize()
            dt = time.perf_counter() - t0
            if rep > 0 and (best is None or dt < best[0]):  # first solve builds the graph
                best = (dt, cyc, rel)
        sols[mixed] = u.cpu().double()
        res["mixed" if mixed else "fp64"] = {"seconds": best[0], "vcycles": best[1], "rel_residual": best[2]}
    a = sols[False] - sols[False].mean()
    b = sols[True] - sols[True].mean()
    res["mixed_vs_fp64_rel_err"] = float((a - b).abs().max() / a.abs().max())
    res["time_ratio_mixed_over_fp64"] = res["mixed"]["seconds"] / res["fp64"]["seconds"]
    # BiCGSTAB with one V-cycle as preconditioner (bicgstab_solver.hpp), same tolerance
    for prec in ("fp64", "fp32"):
        best = None
        for rep in range(3):
            u = torch.zeros((GMG_N,) * 3, dtype=torch.float64, device="cuda")
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            it, rms = g.bicgstab(u, rhs, precondition=prec, rtol=1e-10, relative=True, max_iters=400, stream=s)
            s.synchronize()
            dt = time.perf_counter() - t0
            if rep > 0 and (best is None or dt < best[0]):
                best = (dt, it, rms)
        x = u.cpu().double()
        x = x - x.mean()
        res["bicgstab_mg_" + prec] = {"seconds": best[0], "iterations": best[1], "rms_residual": best[2],
                                      "vs_fp64_vcycle_rel_err": float((x - a).abs().max() / a.abs().max())}
    res["config"] = {"n": GMG_N, "levels": GMG_COARSEN + 1, "smoother": "weighted Jacobi 2/3, 2+2",
                     "coarse": "+16 smoother passes, FP64", "rhs": "32 Gaussians sigma 0.03 seed 4, mean removed"}
    res["blocks"] = gmg_c4_blocks(torch, pg, a)
    return res


def gmg_c4_blocks(torch, pg, flat_fp64):
    """C4 through the block-structured solver (pgb_mg_*, the MGSolver path packages
    call): the same problem on the 128^3 periodic mesh in 16^3 blocks, grids down to one
    8^3 block (4 coarsenings), weighted Jacobi 2/3 with 2+2 sweeps and 16 more passes on
    the coarsest grid. FP64 V-cycles vs the FP32 V-cycle inside FP64 refinement, to a
    1e-10 relative residual; the FP64 solution against the flat solver's."""
    mesh = pg.Mesh((GMG_N,) * 3, (16,) * 3, 2)
    rhs_h = pg.problems.poisson_rhs_blocks(mesh, ngauss=32, sigma=0.03, seed=4)
    rhs = torch.tensor(rhs_h, device="cuda")
    mg = pg.CompositeMultigrid(mesh, stages=2, jacobi=True, weight=2.0 / 3.0, coarse_sweeps=16,
                               max_coarsenings=GMG_COARSEN, alpha=0.0)
    s = torch.cuda.Stream()
    out, sols = {}, {}
    for mixed in (False, True):
        best = None
        for rep in range(3):
            u = torch.zeros_like(rhs)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            cyc, rel = mg.solve(u, rhs, tol=1e-10, relative=True, max_cycles=400, mixed=mixed, stream=s)
            s.synchronize()
            dt = time.perf_counter() - t0
            if rep > 0 and (best is None or dt < best[0]):
                best = (dt, cyc, rel)
        sols[mixed] = u
        out["mixed" if mixed else "fp64"] = {"seconds": best[0], "vcycles": best[1], "rel_residual": best[2]}
    out["time_ratio_mixed_over_fp64"] = out["mixed"]["seconds"] / out["fp64"]["seconds"]
    # the block solution on the global grid, against the flat solver's (means removed)
    locs, geom = mesh.block_info()
    ng, b = 2, 16
    glob = torch.zeros((GMG_N,) * 3, dtype=torch.float64)
    ub = sols[False].cpu()
    for q in range(locs.shape[0]):
        lx = [int(x) for x in locs[q, 1:4]]
        glob[lx[2] * b:(lx[2] + 1) * b, lx[1] * b:(lx[1] + 1) * b, lx[0] * b:(lx[0] + 1) * b] = \
            ub[q, ng:ng + b, ng:ng + b, ng:ng + b]
    glob = glob - glob.mean()
    out["fp64_vs_flat_solver_rel_err"] = float((glob - flat_fp64).abs().max() / flat_fp64.abs().max())
    out["config"] = {"mesh": "128^3 periodic, 16^3 blocks (512)", "grids": mg.ngrids, "levels": [mg.lmin, mg.lmax]}
    return out


SMR_ROOT, SMR_BLOCK, SMR_NG, SMR_NSCALARS, SMR_CYCLES = 128, 16, 4, 4, 20


def _smr_leaves(pg):
    nb = SMR_ROOT // SMR_BLOCK
    return pg.problems.refined_region_leaves(nb.bit_length() - 1, nb // 4, 3 * nb // 4)


def smr_bench(torch, with_cpu):
    """The 2-level static-refinement advection workload: 128^3 root in 16^3 blocks with
    the central 1/8 refined once (448 + 512 blocks, 4 ghosts), a Gaussian plus 4 U(0,1)
    scalars, PLM, RK2, CFL 0.3, 20 cycles; prolongation/restriction at the fine/coarse
    faces and flux correction inside every stage (one CUDA graph per cycle)."""
    import parthenon_gb300 as pg
    mesh = pg.Mesh((SMR_ROOT,) * 3, (SMR_BLOCK,) * 3, SMR_NG, leaves=_smr_leaves(pg))
    ncomp = 1 + SMR_NSCALARS
    state = pg.problems.advection_state(mesh, nscalars=SMR_NSCALARS, seed=3)
    drv = pg.RK2Driver(mesh, ncomp, pg.StageConfig("advection", "plm", 0.3))
    drv.set_state(state)
    drv.run(3)  # warm-up: graph capture and tuning
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    ev0.record(drv.stream)
    drv.run(SMR_CYCLES)
    ev1.record(drv.stream)
    torch.cuda.synchronize()
    ms = ev0.elapsed_time(ev1)
    res = {"metric": "zone-cycles/s", "value": drv.zone_cycles(SMR_CYCLES) / (ms * 1e-3),
           "ms_per_cycle": ms / SMR_CYCLES,
           "config": {"workload": "advection3d-plm-rk2-smr-128^3-root-16^3blocks-central-eighth-refined",
                      "blocks": int(mesh.nblocks), "nghost": SMR_NG, "ncomp": ncomp, "cycles": SMR_CYCLES}}
    if with_cpu:
        sys.path.insert(0, os.path.join(ROOT, "tests"))
        import oracle_lib as O
        o = O.OracleSim((SMR_ROOT,) * 3, (SMR_BLOCK,) * 3, SMR_NG, leaves=_smr_leaves(pg), ncomp=ncomp,
                        physics="advection", recon=1, cfl=0.3)
        o.base()[:] = state
        o.exchange(True, 0)
        o.init_dt()
        threads = O.lib().orc_max_threads()
        t0 = time.perf_counter()
        o.run(1, nthreads=threads)
        dt = time.perf_counter() - t0
        res["cpu_baseline"] = {"value": drv.zone_cycles(1) / dt, "unit": "zone-cycles/s", "cores": threads,
                               "kind": "port", "sample": "1 RK2 cycle of the same mesh and state"}
    return res


GMGC_ROOT, GMGC_BLOCK, GMGC_NG, GMGC_ALPHA = 128, 16, 2, 10.0


def _gmgc_mesh(pg):
    # the statically refined mesh of the 2-level advection workload: 128^3 root in 16^3
    # blocks with the central 1/8 refined once (448 + 512 leaves)
    nb = GMGC_ROOT // GMGC_BLOCK
    root_level = nb.bit_length() - 1
    leaves = pg.problems.refined_region_leaves(root_level, nb // 4, 3 * nb // 4)
    return pg.Mesh((GMGC_ROOT,) * 3, (GMGC_BLOCK,) * 3, GMGC_NG, leaves=leaves)


def gmg_composite_bench(torch, with_cpu):
    """Multigrid on the two-level composite grids of the refined mesh: the reference's
    defaults (FAS, SRJ2, coarsening down to 1^3 blocks), div grad u - alpha u = rhs with
    alpha 10 (poisson/diagonal_alpha; the periodic refined operator without flux
    correction is singular and inconsistent at alpha 0), rhs the 32 Gaussians of the
    uniform leg. Time to a 1e-10 relative leaf residual, and the oracle's time per
    V-cycle on the host cores."""
    import parthenon_gb300 as pg
    mesh = _gmgc_mesh(pg)
    rhs_h = pg.problems.poisson_rhs_blocks(mesh, ngauss=32, sigma=0.03, seed=4)
    rhs = torch.tensor(rhs_h, device="cuda")
    mg = pg.CompositeMultigrid(mesh, stages=2, alpha=GMGC_ALPHA)
    s = torch.cuda.Stream()
    runs, sols = {}, {}
    for mixed in (False, True):
        best = None
        for rep in range(3):
            u = torch.zeros_like(rhs)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            cyc, rel = mg.solve(u, rhs, tol=1e-10, relative=True, max_cycles=200, mixed=mixed, stream=s)
            s.synchronize()
            dt = time.perf_counter() - t0
            if rep > 0 and (best is None or dt < best[0]):  # the first solve builds the graph
                best = (dt, cyc, rel)
        runs[mixed] = best
        sols[mixed] = u[:, GMGC_NG:-GMGC_NG, GMGC_NG:-GMGC_NG, GMGC_NG:-GMGC_NG].cpu()
    # BiCGSTAB with one composite V-cycle per preconditioner application (FP64, FP32)
    bicg = {}
    for prec in ("fp64", "fp32"):
        bb = None
        for rep in range(3):
            u = torch.zeros_like(rhs)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            it, rms = mg.bicgstab(u, rhs, precondition=prec, rtol=1e-10, relative=True, max_iters=200, stream=s)
            s.synchronize()
            dt = time.perf_counter() - t0
            if rep > 0 and (bb is None or dt < bb[0]):
                bb = (dt, it, rms)
        x = u[:, GMGC_NG:-GMGC_NG, GMGC_NG:-GMGC_NG, GMGC_NG:-GMGC_NG].cpu()
        bicg["bicgstab_mg_" + prec] = {"seconds": bb[0], "iterations": bb[1], "rms_residual": bb[2],
                                       "vs_fp64_vcycle_rel_err": float((x - sols[False]).abs().max() /
                                                                       sols[False].abs().max())}
    # the pure Poisson problem (alpha 0) on the refined mesh: conservative with flux
    # correction (poisson/flux_correct), solved by BiCGSTAB with the FP32 V-cycle
    mg0 = pg.CompositeMultigrid(mesh, stages=2, alpha=0.0, flux_correct=True)
    bb = None
    for rep in range(3):
        u = torch.zeros_like(rhs)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        it, rms = mg0.bicgstab(u, rhs, precondition="fp32", rtol=1e-10, relative=True, max_iters=200, stream=s)
        s.synchronize()
        dt = time.perf_counter() - t0
        if rep > 0 and (bb is None or dt < bb[0]):
            bb = (dt, it, rms)
    bicg["poisson_alpha0_flux_correct_bicgstab_mg_fp32"] = {"seconds": bb[0], "iterations": bb[1],
                                                             "rms_residual": bb[2]}
    best = runs[False]
    locs, _ = mesh.block_info()
    res = {"seconds": best[0], "vcycles": best[1], "rel_residual": best[2],
           "ms_per_vcycle": 1e3 * best[0] / max(1, best[1]),
           "mixed": {"seconds": runs[True][0], "iterations": runs[True][1], "rel_residual": runs[True][2],
                     "ms_per_iteration": 1e3 * runs[True][0] / max(1, runs[True][1])},
           "time_ratio_mixed_over_fp64": runs[True][0] / best[0],
           "mixed_vs_fp64_rel_err": float((sols[True] - sols[False]).abs().max() / sols[False].abs().max()),
           **bicg,
           "config": {"mesh": "128^3 root, 16^3 blocks, central 1/8 refined once", "leaves": int(mesh.nblocks),
                      "leaves_per_level": {str(int(l)): int((locs[:, 0] == l).sum()) for l in np.unique(locs[:, 0])},
                      "nghost": GMGC_NG, "grids": mg.ngrids, "levels": [mg.lmin, mg.lmax],
                      "storage_blocks": mg.nslots, "smoother": "SRJ2 (2+2)", "alpha": GMGC_ALPHA,
                      "rhs": "32 Gaussians sigma 0.03 seed 4, volume mean removed"}}
    if with_cpu:
        res["cpu_baseline"] = gmg_composite_cpu_baseline(mesh, rhs_h, best[1])
    return res


def gmg_composite_cpu_baseline(mesh, rhs_h, vcycles):
    """The oracle's composite V-cycle (oracle/gmg_blocks.hpp) on the same mesh and rhs,
    run to the same 1e-10 relative leaf residual (at most a few cycles past the GPU's
    count), all host threads."""
    O = _oracle()
    sim = O.OracleSim((GMGC_ROOT,) * 3, (GMGC_BLOCK,) * 3, GMGC_NG, leaves=_gmgc_leaves_of(mesh))
    om = O.OracleMgBlocks(sim, stages=2, alpha=GMGC_ALPHA)
    om.rhs()[:] = rhs_h
    t0 = time.perf_counter()
    r0 = om.residual()
    ncyc, rel = 0, 1.0
    while ncyc < vcycles + 5 and rel > 1e-10:
        rel = om.run(1)[0] / r0
        ncyc += 1
    el = time.perf_counter() - t0
    return {"seconds_to_tolerance": el, "vcycles": ncyc, "rel_residual": rel, "seconds_per_vcycle": el / ncyc,
            "kind": "port", "cores": int(O.lib().orc_max_threads()),
            "sample": "the whole solve to a 1e-10 relative leaf residual"}


def _gmgc_leaves_of(mesh):
    locs, _ = mesh.block_info()
    return [tuple(int(x) for x in r) for r in locs]


AMR_ROOT, AMR_BLOCK, AMR_NUMLEVEL, AMR_NSCALARS, AMR_CHECK = 128, 16, 3, 2, 5


def _amr_driver(pg, root):
    crit = pg.RefinementCriterion(comps=(0, 1, 2), method="gradient", refine_tol=0.5, derefine_tol=0.05,
                                  relative=True)
    mesh = pg.Mesh((root,) * 3, (AMR_BLOCK,) * 3, NGHOST)
    return pg.AMRDriver(mesh, 3 + AMR_NSCALARS, pg.StageConfig("burgers", "weno5", CFL), crit,
                        numlevel=AMR_NUMLEVEL, derefine_count=10, check_interval=AMR_CHECK)


def amr_bench(torch, cycles, with_cpu, root=AMR_ROOT):
    """Adaptive Burgers: 128^3 root in 16^3 blocks, 3 levels, refine above 0.5 and
    derefine below 0.05 of the mesh-wide max |grad u| (checked every 5 cycles, 10
    consecutive derefine tags needed), 16 random-phase sinusoids with wavenumbers 1-6,
    2 passive scalars, WENO5 + HLL, RK2, CFL 0.8. Zone-cycles/s over `cycles` cycles
    with every check, remesh, data movement and graph re-capture inside the timed
    region; the initial refinement (problem generation repeated on each new mesh) is
    timed separately."""
    import parthenon_gb300 as pg
    drv = _amr_driver(pg, root)
    adapt_s = []
    inner = drv.adapt

    def timed_adapt():
        torch.cuda.synchronize()
        t = time.perf_counter()
        changed = inner()
        torch.cuda.synchronize()
        adapt_s.append((time.perf_counter() - t, changed))
        return changed

    drv.adapt = timed_adapt
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    drv.initialize(lambda m: pg.problems.burgers_amr_state_device(m, nscalars=AMR_NSCALARS))
    torch.cuda.synchronize()
    init_s = time.perf_counter() - t0
    init_blocks = drv.mesh.nblocks
    adapt_s.clear()
    hist0 = len(drv.block_history)
    drv.run(2)  # warm-up: first graph capture on this mesh
    torch.cuda.synchronize()
    zc0 = drv.zone_cycles
    t0 = time.perf_counter()
    drv.run(cycles)
    torch.cuda.synchronize()
    el = time.perf_counter() - t0
    zc = drv.zone_cycles - zc0
    blocks = drv.block_history[hist0 - 1:]
    levels = np.bincount(drv.mesh.block_info()[0][:, 0])
    res = {
        "value": zc / el, "unit": METRIC, "cycles": cycles, "seconds": el, "ms_per_cycle": 1e3 * el / cycles,
        "zone_cycles": zc, "init_seconds": init_s, "blocks_after_init": init_blocks,
        "blocks_min": int(min(blocks)), "blocks_max": int(max(blocks)), "blocks_final": drv.mesh.nblocks,
        "levels_final": {str(l): int(c) for l, c in enumerate(levels) if c},
        "checks": len(adapt_s), "remeshes": int(sum(1 for _, c in adapt_s if c)),
        "check_seconds": float(sum(t for t, _ in adapt_s)),
        "remesh_seconds_max": float(max([t for t, c in adapt_s if c], default=0.0)),
        "peak_mem_gb": torch.cuda.max_memory_allocated() / 1e9,
        "config": {"workload": "burgers3d-amr-%d^3root-16^3blocks-3levels-ng4-5vars-fp64" % root,
                   "criterion": "|grad u| relative: refine > 0.5 max, derefine < 0.05 max (10 tags)",
                   "check_interval": AMR_CHECK, "initial": "16 sinusoids, k in 1..6, seed 5; 2 scalars"},
    }
    if with_cpu:
        res["cpu_baseline"] = amr_cpu_baseline(torch, pg, drv)
    del drv
    return res


def _host_mem_available():
    """Bytes of host memory this process may still use (the smaller of MemAvailable and
    the cgroup limit's headroom)."""
    avail = None
    try:
        with open("/proc/meminfo") as f:
            for line in f:
                if line.startswith("MemAvailable:"):
                    avail = int(line.split()[1]) * 1024
    except OSError:
        pass
    try:
        with open("/sys/fs/cgroup/memory.max") as f:
            lim = f.read().strip()
        with open("/sys/fs/cgroup/memory.current") as f:
            cur = int(f.read().strip())
        if lim != "max":
            head = int(lim) - cur
            avail = head if avail is None else min(avail, head)
    except (OSError, ValueError):
        pass
    return avail if avail is not None else 0


def _amr_oracle_cycle_and_check(O, root, locs, state, ncomp, mml):
    """The oracle on the given leaves and state: the time of one RK2 cycle and of one
    refinement check (criterion, flags, remesh with its data movement and ghost fill,
    dt vote) on the resulting state."""
    o = O.OracleSim((root,) * 3, (AMR_BLOCK,) * 3, NGHOST, leaves=locs, ncomp=ncomp, physics="burgers", recon=0,
                    cfl=CFL, prolong_in_stage=False)
    o.base()[:] = state
    o.exchange(True, 0)
    o.init_dt()
    threads = O.lib().orc_max_threads()
    nb = o.nblocks
    t0 = time.perf_counter()
    o.run(1, nthreads=threads)
    t_cycle = time.perf_counter() - t0
    t0 = time.perf_counter()
    crit = np.max([o.block_criterion(c, 2) for c in range(3)], axis=0)
    g = float(crit.max())
    flags = o.set_refinement(crit, 0.5 * g, 0.05 * g, mml, mml, 10)
    if o.remesh(flags):
        o.exchange(True, 0)
        o.remesh_dt()
    t_check = time.perf_counter() - t0
    return nb, t_cycle, t_check, threads


def amr_cpu_baseline(torch, pg, drv):
    """The oracle (all host threads) on the GPU run's final mesh and state: one RK2
    cycle plus one refinement check with its remesh, combined as the GPU run checks
    (one check per AMR_CHECK cycles). When the host cannot hold that mesh's oracle
    fields, the 64^3-root analogue of the workload (an eighth of the volume, same
    criterion, levels and physics) is timed the same way."""
    O = _oracle()
    ncomp = 3 + AMR_NSCALARS
    drv.stream.synchronize()
    locs, _ = drv.mesh.block_info()
    field_bytes = drv.base.numel() * 8
    # oracle: base, stage, dudt, three flux fields, coarse buffers, derived; plus the
    # host copy and the remesh's old/new fields
    need = 10 * field_bytes
    if _host_mem_available() > need:
        state = drv.base.cpu().numpy()
        nb, tc, tk, threads = _amr_oracle_cycle_and_check(O, AMR_ROOT, locs, state, ncomp,
                                                          drv.mesh_max_level)
        sample = "1 RK2 cycle + 1 refinement check with remesh on the GPU run's final mesh (%d meshblocks of 16^3)" % nb
    else:
        small = _amr_driver(pg, AMR_ROOT // 2)
        small.initialize(lambda m: pg.problems.burgers_amr_state_device(m, nscalars=AMR_NSCALARS))
        small.stream.synchronize()
        sl, _ = small.mesh.block_info()
        nb, tc, tk, threads = _amr_oracle_cycle_and_check(O, AMR_ROOT // 2, sl, small.base.cpu().numpy(), ncomp,
                                                          small.mesh_max_level)
        sample = ("1 RK2 cycle + 1 refinement check with remesh on the 64^3-root analogue (%d meshblocks of 16^3): "
                  "the final mesh's oracle fields exceed this host's memory" % nb)
    zones = nb * AMR_BLOCK ** 3
    return {"value": zones / (tc + tk / AMR_CHECK), "unit": METRIC, "cores": threads, "kind": "port",
            "cycle_seconds": tc, "check_seconds": tk, "sample": sample}


# Sparse advection (example/sparse_advection/parthinput.sparse_advection) in three
# dimensions: [-1,1]^3, 64^3 root in 8^3 blocks, 2 ghosts, 3 levels, four sparse fields
# (spheres of radius 0.1 moving diagonally at 1.5), donor cell, RK2, CFL 0.45;
# allocation threshold 1e-5, deallocation threshold 1e-6 after 5 checks; tagging every
# cycle (refine where max > 0.3 and min < 0.03, derefine where max < 0.03, 10 tags).
SPARSE_ROOT, SPARSE_BLOCK, SPARSE_NG, SPARSE_NUMLEVEL, SPARSE_NFIELDS = 64, 8, 2, 3, 4


def _sparse_driver(pg, root):
    mesh = pg.Mesh((root,) * 3, (SPARSE_BLOCK,) * 3, SPARSE_NG, xmin=(-1.0,) * 3, xmax=(1.0,) * 3)
    mesh.enable_sparse(SPARSE_NFIELDS, 1e-5, 1e-6, dealloc_count=5)
    cfg = pg.StageConfig("advection", "dc", 0.45, comp_vel=pg.problems.sparse_advection_velocities(1.5))
    return pg.AMRDriver(mesh, SPARSE_NFIELDS, cfg, pg.SparseMinMaxCriterion(0.3, 0.03), numlevel=SPARSE_NUMLEVEL,
                        derefine_count=10, check_interval=1)


def _sparse_pgen(pg):
    return lambda m, prev, a: pg.problems.sparse_advection_state(m, prev, a, init_size=0.1)


def sparse_bench(torch, cycles, with_cpu, root=SPARSE_ROOT, profile_range=False):
    """Adaptive sparse advection: zone-cycles/s over `cycles` cycles with the tagging
    of every cycle, the remeshes (allocation carried over), the allocation on receipt
    and the deallocation checks inside the timed region."""
    import parthenon_gb300 as pg
    drv = _sparse_driver(pg, root)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    drv.initialize(_sparse_pgen(pg))
    torch.cuda.synchronize()
    init_s = time.perf_counter() - t0
    init_blocks = drv.mesh.nblocks
    a0, _ = drv.mesh.sparse_alloc(drv.stream)
    drv.run(2)  # warm-up: first graph capture on this mesh
    torch.cuda.synchronize()
    zc0, nr0, hist0 = drv.zone_cycles, drv.nremesh, len(drv.block_history)
    if profile_range:  # launch lists of the timed cycles only (ncu --profile-from-start off)
        torch.cuda.profiler.start()
    t0 = time.perf_counter()
    drv.run(cycles)
    torch.cuda.synchronize()
    el = time.perf_counter() - t0
    if profile_range:
        torch.cuda.profiler.stop()
    zc = drv.zone_cycles - zc0
    a, _ = drv.mesh.sparse_alloc(drv.stream)
    blocks = drv.block_history[hist0 - 1:]
    res = {
        "value": zc / el, "unit": METRIC, "cycles": cycles, "seconds": el, "ms_per_cycle": 1e3 * el / cycles,
        "zone_cycles": zc, "init_seconds": init_s, "blocks_after_init": init_blocks,
        "blocks_min": int(min(blocks)), "blocks_max": int(max(blocks)), "blocks_final": drv.mesh.nblocks,
        "remeshes": drv.nremesh - nr0, "allocated_fraction_init": float(a0.mean()),
        "allocated_fraction_final": float(a.mean()),
        "config": {"workload": "sparse-advection3d-%d^3root-8^3blocks-3levels-ng2-4sparse-fp64" % root,
                   "sparse": "alloc 1e-5, dealloc 1e-6 after 5 checks, default 0",
                   "criterion": "min/max over allocated fields: refine max>0.3 & min<0.03, derefine max<0.03",
                   "check_interval": 1, "initial": "4 spheres r=0.1 at (+-0.8,+-0.8,0), speed 1.5 diagonal"},
    }
    if with_cpu:
        res["cpu_baseline"] = sparse_cpu_baseline(torch, pg, drv)
    del drv
    return res


def sparse_cpu_baseline(torch, pg, drv, cycles=8):
    """The oracle (all host threads) continuing the GPU run's mesh, fields and
    allocation for a few cycles, with the tagging and remesh of every cycle."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import oracle_lib as O
    drv.stream.synchronize()
    locs, _ = drv.mesh.block_info()
    o = O.OracleSim((SPARSE_ROOT,) * 3, (SPARSE_BLOCK,) * 3, SPARSE_NG, xmin=(-1.0,) * 3, xmax=(1.0,) * 3, leaves=locs,
                    ncomp=SPARSE_NFIELDS, physics="advection", recon=0, cfl=0.45)
    o.set_component_velocities(pg.problems.sparse_advection_velocities(1.5))
    o.sparse_enable(1e-5, 1e-6, dealloc_count=5)
    a, c = drv.mesh.sparse_alloc(drv.stream)
    o.sparse_set(a, c)
    o.base()[:] = drv.base.cpu().numpy()
    o.exchange(True, 0)
    o.init_dt()
    mml = SPARSE_NUMLEVEL + drv.mesh.root_level - 1
    threads = O.lib().orc_max_threads()
    zones = 0
    t0 = time.perf_counter()
    for _ in range(cycles):
        o.run(1, nthreads=threads)
        zones += o.nblocks * SPARSE_BLOCK ** 3
        t = o.sparse_tag(0.3, 0.03)
        flags = o.set_refinement(t, 0.5, -0.5, mml, mml, 10)
        if o.remesh(flags):
            o.exchange(True, 0)
            o.remesh_dt()
    el = time.perf_counter() - t0
    return {"value": zones / el, "unit": METRIC, "cores": threads, "kind": "port",
            "sample": "%d cycles (tag + remesh each) from the GPU run's final mesh of %d meshblocks of 8^3" %
                      (cycles, len(locs))}


def cpu_baseline(o, cycles=1):
    """The oracle (CPU restatement of the reference, all host threads) on the full
    workload: `cycles` RK2 cycles continuing from its current state."""
    O = _oracle()
    threads = O.lib().orc_max_threads()
    t0 = time.perf_counter()
    o.run(cycles, nthreads=threads)
    el = time.perf_counter() - t0
    zones = o.nblocks * BLOCK_N ** 3
    return {"value": cycles * zones / el, "unit": METRIC, "cores": threads, "kind": "port",
            "sample": "%d RK2 cycle(s) of the full workload (%d meshblocks of 32^3), same initial state" %
                      (cycles, o.nblocks)}


def run_reference(args, ws, rank):
    """The reference arm: the reference's algorithm on the host cores. The reference's
    own Kokkos-OpenMP build cannot be built (its Kokkos submodule is empty and there is
    no network), so its CPU restatement (oracle/, C++17 + OpenMP, -O3, no FMA
    contraction) stands in for it on the same workload."""
    if rank != 0:
        return None
    O = _oracle()
    threads = O.lib().orc_max_threads()
    o = oracle_burgers(args.mesh)
    zones = o.nblocks * BLOCK_N ** 3
    o.run(max(args.warmup, 0), nthreads=threads)  # untimed warm-up cycles on the same object
    t0 = time.perf_counter()
    o.run(max(args.steps, 1), nthreads=threads)
    el = time.perf_counter() - t0
    steps = max(args.steps, 1)
    value = steps * zones / el
    sample = "%d RK2 cycles of the full workload (%d meshblocks of 32^3) after %d warm-up cycles" % (
        steps, o.nblocks, max(args.warmup, 0))
    return {
        "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * el / steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic", "impl": "reference", "reference_kind": "port",
        "note": "CPU restatement of the reference (oracle/), not the reference's Kokkos build, which cannot be "
                "built here",
        "config": workload_config(args.mesh),
        "cpu_baseline": {"value": value, "unit": METRIC, "cores": threads, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--mesh", type=int, default=MESH_N, help="cells per direction (profiling runs use 128)")
    ap.add_argument("--no-extras", action="store_true",
                    help="skip the per-kernel timing, end-to-end and CPU-baseline legs (profiling runs)")
    ap.add_argument("--amr-cycles", type=int, default=100,
                    help="cycles of the adaptive Burgers leg (0 skips it)")
    ap.add_argument("--amr-root", type=int, default=AMR_ROOT, help="root cells per direction of the adaptive leg")
    ap.add_argument("--amr-only", action="store_true",
                    help="run only the adaptive leg (profiling runs), no CPU baseline")
    ap.add_argument("--gmg-only", action="store_true", help="run only the multigrid leg (profiling runs)")
    ap.add_argument("--smr-only", action="store_true",
                    help="run only the 2-level static-refinement advection leg (with its CPU baseline)")
    ap.add_argument("--gmg-composite-only", action="store_true",
                    help="run only the composite-grid multigrid leg, no CPU baseline (profiling runs)")
    ap.add_argument("--sparse-cycles", type=int, default=100,
                    help="cycles of the adaptive sparse-advection leg (0 skips it)")
    ap.add_argument("--sparse-only", action="store_true",
                    help="run only the sparse-advection leg (with its CPU baseline)")
    ap.add_argument("--profile-range", action="store_true",
                    help="bracket the sparse leg's timed cycles with cudaProfilerStart/Stop")
    args = ap.parse_args()
    ws, rank = _dist()
    if ws > 1:
        import torch
        torch.distributed.init_process_group("nccl" if args.impl == "ours" else "gloo")
    if args.amr_only:
        import torch
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        out = {"amr": amr_bench(torch, args.amr_cycles, with_cpu=False, root=args.amr_root)}
    elif args.gmg_only:
        import torch
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        out = {"gmg": gmg_bench(torch), "gmg_composite": gmg_composite_bench(torch, with_cpu=False)}
    elif args.smr_only:
        import torch
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        out = {"smr": smr_bench(torch, with_cpu=(rank == 0))}
    elif args.gmg_composite_only:
        import torch
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        out = {"gmg_composite": gmg_composite_bench(torch, with_cpu=False)}
    elif args.sparse_only:
        import torch
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        out = {"sparse": sparse_bench(torch, args.sparse_cycles, with_cpu=(rank == 0),
                                      profile_range=args.profile_range)}
    elif args.impl == "reference":
        out = run_reference(args, ws, rank)
    else:
        out = run_ours(args, ws, rank)
    if rank == 0 and out is not None:
        print(json.dumps(out))
    if ws > 1:
        import torch
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
