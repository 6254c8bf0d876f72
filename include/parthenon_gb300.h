/* C ABI of the GB300 block-AMR hot path (parthenon_gb300).
 *
 * One process, one GPU. Device arrays are plain pointers to device memory laid out
 * per block as [block][component][k][j][i] (cells with ghosts, FP64); coarse buffers
 * use the same layout with the coarse block size. Every call is stream-ordered on the
 * stream passed in (a cudaStream_t, or NULL for the legacy default stream) and does no
 * host synchronisation, so sequences of calls can be captured into a CUDA graph.
 *
 * Every function returns an int status: 0 success, < 0 failure (see PGB_ERR_*), and
 * never throws across the ABI; pgb_last_error() gives the message of the last failure
 * on the calling thread.
 *
 * Each entry point names the reference interface it replaces
 * (parthenon-hpc-lab/parthenon, file:line).
 */
#ifndef PARTHENON_GB300_H_
#define PARTHENON_GB300_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PGB_OK 0
#define PGB_ERR_INVALID (-1)
#define PGB_ERR_CUDA (-2)
#define PGB_ERR_UNSUPPORTED (-3)
#define PGB_ERR_STATE (-4)

/* exchange flags */
#define PGB_EXCHANGE_PROLONGATE 1   /* run ProlongateBounds after SetBounds          */
#define PGB_PROLONG_MINMOD 0        /* ProlongateSharedMinMod (default CC op)        */
#define PGB_PROLONG_LINEAR 2        /* ProlongateSharedLinear      (flags bits 1-2)  */
#define PGB_PROLONG_CONSTANT 4      /* ProlongatePiecewiseConstant                   */

typedef struct pgb_mesh pgb_mesh;

/* Root mesh and block shape; every direction periodic (the only boundary the hot
 * path supports). Mirrors <parthenon/mesh> nx1..3, x?min/x?max, nghost and
 * <parthenon/meshblock> nx1..3. */
typedef struct {
  int32_t nx[3];
  int32_t block_nx[3];
  int32_t nghost;
  double xmin[3];
  double xmax[3];
} pgb_mesh_spec;

typedef struct {
  int32_t nblocks;
  int32_t multilevel;
  int32_t root_level;
  int32_t max_level;
  int32_t N[3];        /* block array extents with ghosts */
  int32_t Nc[3];       /* coarse buffer extents with ghosts */
  int32_t npairs;      /* boundary sender/receiver pairs (index maps) */
  int64_t buffer_elems;/* packed buffer length per component (reference layout) */
  int32_t nflux_corr;  /* fine/coarse faces with flux correction */
} pgb_mesh_info;

/* Stage parameters. physics: 0 advection (constant velocity), 1 Burgers.
 * recon: advection 0 donor cell / 1 PLM; Burgers 0 WENO5 / 1 MC-linear.
 * exact: 1 = separately rounded arithmetic in the reference's order (bitwise path),
 *        0 = FMA-contracted kernels with shared reciprocals (within 1e-12 relative).
 * Advection velocities: ncomp_vel == 0 moves every component with vel; otherwise
 * comp_vel (host memory, read at each call) holds ncomp_vel == ncomp rows of three
 * velocities, one per component (at most PGB_MAX_COMP_VEL), as the sparse advection
 * package's vx/vy/vz (example/sparse_advection/sparse_advection_package.cpp:61-66). */
#define PGB_MAX_COMP_VEL 16
typedef struct {
  int32_t physics;
  int32_t recon;
  int32_t exact;
  int32_t ncomp_vel;
  double vel[3];
  double cfl;
  const double *comp_vel;
} pgb_stage_params;

const char *pgb_last_error(void);
int pgb_version(void);

/* Mesh topology from leaf logical locations (level, lx1, lx2, lx3 per leaf; nleaves
 * == 0 gives the uniform root grid). Host only: builds gids, neighbours, ownership
 * and every boundary index range.
 * Replaces Mesh::Mesh/BuildBlockList (src/mesh/mesh.cpp:311-370), Forest::HyperRectangular
 * (src/mesh/forest/forest.cpp:64-195), SetMeshBlockNeighbors (src/mesh/mesh-gmg.cpp:48-101)
 * and the BndInfo/ProResInfo construction (src/bvals/comms/bnd_info.cpp:105-448). */
int pgb_mesh_create(const pgb_mesh_spec *spec, int32_t nleaves, const int64_t *leaves, pgb_mesh **out);
int pgb_mesh_destroy(pgb_mesh *mesh);
int pgb_mesh_get_info(const pgb_mesh *mesh, pgb_mesh_info *info);
/* locs: nblocks x (level, lx1, lx2, lx3); geom: nblocks x (xmin[3], dx[3]) */
int pgb_mesh_block_info(const pgb_mesh *mesh, int64_t *locs, double *geom);
/* Buffer index maps, 23 int32 per pair: sender gid, receiver gid, sender-side slot,
 * send box (is,ie,js,je,ks,ke), send-from-coarse flag, receive box (6), receive-into-
 * coarse flag, 27-bit receive mask, values per component, 4 reserved.
 * Replaces the BndInfo index ranges (src/bvals/comms/bnd_info.cpp:273-340). */
int pgb_mesh_boundaries(const pgb_mesh *mesh, int32_t *out, int32_t capacity);

/* Host-only check that every device access the lowered tables imply (boundary
 * boxes, restriction reads, prolongation stencils, flux-correction faces) stays inside
 * the block arrays; pgb_mesh_upload runs the same check before any upload. */
int pgb_mesh_validate(const pgb_mesh *mesh);

/* Lower the topology to device tables (needs a GPU); call once per mesh/remesh.
 * Replaces RebuildBufferCache (src/bvals/comms/bvals_utils.hpp:212-245). */
int pgb_mesh_upload(pgb_mesh *mesh);

/* Full same-rank ghost exchange of a cell-centred field: send-side restriction,
 * boundary copies, receive-side restriction, optional prolongation.
 * buffer == NULL: direct sender->receiver copies; otherwise buffer (>= buffer_elems *
 * ncomp doubles) is packed and unpacked in the reference layout.
 * Replaces SendBoundBufs / ReceiveBoundBufs / SetBounds / ProlongateBounds<any>
 * (src/bvals/comms/boundary_communication.cpp:48-393) and AddBoundaryExchangeTasks
 * (boundary_communication.cpp:405-445). */
int pgb_exchange(pgb_mesh *mesh, double *data, double *coarse, int32_t ncomp, int32_t flags, double *buffer,
                 void *stream);

/* Same exchange as pgb_exchange with a packed buffer, but the buffer is a fixed
 * 32 MiB (4,194,304 doubles) array in static device memory owned by the library, so
 * the call allocates nothing; for callers that cannot allocate device memory (another
 * runtime owns the allocator, or the loop must never allocate). No counterpart in the
 * reference. Requests needing more than buffer_elems * ncomp = 4,194,304 doubles are
 * rejected (PGB_ERR_INVALID), and so is a mesh with sparse variables
 * (PGB_ERR_UNSUPPORTED: the packed-buffer exchange has no sparse form; such meshes
 * exchange through pgb_exchange with buffer == NULL). The first call on each device looks up the array's
 * device address (make that first call before any stream capture); all calls share
 * the array, so calls that overlap on the GPU race with each other. */
int pgb_exchange_static_buffer(pgb_mesh *mesh, double *data, double *coarse, int32_t ncomp, int32_t flags,
                               void *stream);

/* Pack every boundary into `buffer` in the reference's buffer layout (parity checks).
 * Replaces the pack kernel of SendBoundBufs (boundary_communication.cpp:95-140). */
int pgb_pack_buffers(pgb_mesh *mesh, const double *data, const double *coarse, int32_t ncomp, double *buffer,
                     void *stream);

/* Flux correction at fine/coarse faces on flux arrays [block][dir][comp][N3][N2][N1].
 * Replaces AddFluxCorrectionTasks (boundary_communication.cpp:454-461). */
int pgb_flux_correct(pgb_mesh *mesh, double *flux, int32_t ncomp, void *stream);

/* One RK stage: fluxes from u_in, flux divergence, u_out = (w_in u_in + w_base u_base)
 * + beta * dt * dudt on the interior. dt is a device scalar (dt[0]). Uniform meshes use the
 * fused path (dudt is scratch of the field's size); on multilevel meshes the blocks with a
 * fine/coarse face store fluxes in `flux` (3x the field's size), which are corrected at
 * those faces before the update, and the other blocks take the fused path with `dudt`
 * as scratch (dudt NULL: the flux array serves; on a mesh with sparse variables every
 * block then stores fluxes).
 * Replaces CalculateFluxes (benchmarks/burgers/burgers_package.cpp:202-404,
 * example/advection/advection_package.cpp:499-647), FluxDivergence
 * (src/interface/update.cpp:62-85), AverageIndependentData and UpdateIndependentData
 * (src/interface/update.hpp:121-136). */
int pgb_stage(pgb_mesh *mesh, const pgb_stage_params *p, const double *u_in, const double *u_base, double *u_out,
              double *dudt, double *flux, const double *dt, double w_in, double w_base, double beta, int32_t ncomp,
              void *stream);

/* dt <- SetGlobalTimeStep(cfl * EstimateTimestep(u)) on the device. dt points to three
 * device doubles: dt[0] the current step (what the stage kernels read), dt[1] the step
 * the last update started from, dt[2] the simulation time. first = 0: regular update
 * after a cycle taken with dt[0] (dt[2] += dt[0]; growth limited to 2x); 1: the initial
 * step; 2: repeat the last update with votes from u (after a remesh, where every block
 * of the new list votes again).
 * Replaces EstimateTimestep (src/interface/update.hpp:268-278),
 * EvolutionDriver::SetGlobalTimeStep (src/driver/driver.cpp:210-232) and
 * InitializeBlockTimeSteps after a remesh (driver.cpp:129-131,194-204). */
int pgb_estimate_dt(pgb_mesh *mesh, const pgb_stage_params *p, const double *u, int32_t ncomp, double *dt,
                    int32_t first, void *stream);

/* The Burgers package's FillDerived on the device: derived = 0.5 * U(3) * (U(0)^2 +
 * U(1)^2 + U(2)^2) on the interior cells of every block (derived: one component in the
 * field layout, ghosts untouched), separately rounded in the reference's order.
 * Replaces FillDerived<MeshData> (src/interface/update.hpp) with the package's
 * CalculateDerived (benchmarks/burgers/burgers_package.cpp:143-167). */
int pgb_fill_derived(pgb_mesh *mesh, const double *u, int32_t ncomp, double *derived, void *stream);
/* Attach the Burgers derived field to the mesh (NULL detaches): pgb_rk2_cycles then runs
 * pgb_fill_derived on each stage's output after its update, as the Burgers task list
 * does (benchmarks/burgers/burgers_driver.cpp:121). pgb_run_host* fill a derived field
 * of their own for Burgers. */
int pgb_set_derived(pgb_mesh *mesh, double *derived);

/* ncycles RK2 cycles (two stages with a ghost exchange after each, then the dt update)
 * on device arrays. base/stage: fields; dudt: scratch of the field's size; flux:
 * 3x field size (multilevel only, else may be NULL); coarse_*: coarse buffers
 * (multilevel only); dt: three device doubles as for pgb_estimate_dt. use_graph != 0
 * captures one cycle in a CUDA graph and replays it.
 * Replaces MultiStageDriverGeneric::Step (src/driver/multistage.hpp:39-53) with the
 * advection/Burgers task collections (example/advection/advection_driver.cpp:56-164,
 * benchmarks/burgers/burgers_driver.cpp:53-148). */
int pgb_rk2_cycles(pgb_mesh *mesh, const pgb_stage_params *p, double *base, double *stage, double *dudt, double *flux,
                   double *coarse_base, double *coarse_stage, int32_t ncomp, double *dt, int32_t ncycles,
                   int32_t use_graph, void *stream);

/* Host-buffer entry point: copies host_in (interior+ghosts, the field layout) to the
 * device, exchanges ghosts, runs ncycles RK2 cycles and copies the result back.
 * *dt_inout: in, the current dt (<= 0: estimate the initial dt); out, the next dt.
 * The device buffers it needs (two fields, the increment or flux scratch, the coarse
 * buffers, a stream) belong to the mesh handle and are kept between calls of the same
 * sizes; pgb_release_host_workspace or pgb_mesh_destroy frees them. */
int pgb_run_host(pgb_mesh *mesh, const pgb_stage_params *p, const double *host_in, double *host_out, int32_t ncomp,
                 int32_t ncycles, double *dt_inout);
/* The same, and dt_cycles (host, ncycles doubles; may be NULL) receives the dt of the
 * step after each cycle, read back from the device as that cycle ends (the per-step
 * scalar result a driver would log). */
int pgb_run_host_dt(pgb_mesh *mesh, const pgb_stage_params *p, const double *host_in, double *host_out,
                    int32_t ncomp, int32_t ncycles, double *dt_inout, double *dt_cycles);
/* Frees the device buffers that pgb_run_host* keep in the mesh handle (waits for their
 * stream first). The next pgb_run_host* call allocates them again. */
int pgb_release_host_workspace(pgb_mesh *mesh);

/* ---------------------------------------------------------------- multigrid
 * Geometric multigrid for div(grad u) = rhs on a uniform periodic cube of n^3 cells
 * (n a power of two), arrays of n^3 doubles with x fastest. Levels n, n/2, ...,
 * n >> ncoarsen. FAS V-cycle with SRJ (Yang-Mittal weights for `stages` 1..3) or
 * weighted-Jacobi smoothing, volume-average restriction and linear prolongation. */
typedef struct pgb_gmg pgb_gmg;
typedef struct {
  int32_t n;             /* finest cells per direction */
  int32_t ncoarsen;      /* coarser levels below the finest (max_coarsenings) */
  int32_t stages;        /* pre- and post-smoothing sweeps */
  int32_t jacobi;        /* 0: SRJ weights; 1: weighted Jacobi with `weight` */
  double weight;
  int32_t coarse_sweeps; /* extra smoother passes at the coarsest level (0 = reference) */
  int32_t exact;         /* 1: separately rounded reference-order arithmetic */
  double xmin, xmax;
} pgb_gmg_params;

/* Allocates every level (FP64 and FP32 hierarchies). Replaces MGSolver construction and
 * the multigrid block lists (src/solvers/mg_solver.hpp:80-117, src/mesh/mesh-gmg.cpp:103-201). */
int pgb_gmg_create(const pgb_gmg_params *params, pgb_gmg **out);
int pgb_gmg_destroy(pgb_gmg *gmg);
/* ncycles FP64 V-cycles on u (in/out) with right-hand side rhs; rms (host, may be NULL)
 * receives sqrt(sum r^2 / N) after each cycle. Replaces AddLinearOperatorTasks +
 * the residual check of MGSolver::AddTasks (mg_solver.hpp:119-186). Synchronises the
 * stream once per cycle to read the residual. */
int pgb_gmg_vcycles(pgb_gmg *gmg, double *u, const double *rhs, int32_t ncycles, double *rms, void *stream);
/* Solve to rms(rhs - A u) / rms(rhs - A u_initial) <= rtol. mixed = 0: FP64 V-cycles;
 * mixed = 1: FP32 V-cycle on the FP64 residual (iterative refinement, FP64 coarsest
 * level). Replaces MGSolver::AddTasks (mg_solver.hpp:119-161). */
int pgb_gmg_solve(pgb_gmg *gmg, double *u, const double *rhs, int32_t mixed, double rtol, int32_t max_cycles,
                  int32_t *cycles_out, double *relres_out, void *stream);
/* Right-preconditioned BiCGSTAB for A u = rhs from u = 0 (the result is written to u):
 * precondition 0: none; 1: one FP64 V-cycle from zero per application; 2: one FP32
 * V-cycle (FP64 coarsest level). Stops when sqrt((r,r)/N) < rtol (relative = 0) or
 * < rtol * sqrt((rhs,rhs)/N) (relative = 1), or after max_iters. One iteration is one
 * CUDA-graph launch (stream must not be the legacy default stream); the host reads one
 * double per iteration. Replaces BiCGSTABSolver::AddTasks
 * (src/solvers/bicgstab_solver.hpp:116-315) with MGSolver as its preconditioner. */
int pgb_gmg_bicgstab(pgb_gmg *gmg, double *u, const double *rhs, int32_t precondition, double rtol,
                     int32_t relative, int32_t max_iters, int32_t *iters_out, double *rms_out, void *stream);
/* The same solves on fields in the meshblock layout of pgb_exchange ([block][comp][k]
 * [j][i] with ghosts): component comp_rhs of rhs is the right-hand side, component
 * comp_u of u the initial guess (V-cycle methods) and the result (interior cells; run
 * an exchange for its ghosts). The mesh must be uniform, uploaded, with n cells per
 * direction and the solver's extent. method 0: FP64 V-cycles, 1: mixed V-cycles (rtol
 * relative to the initial residual); 2: BiCGSTAB + FP64 V-cycle, 3: BiCGSTAB + FP32
 * V-cycle (rtol relative to rms(rhs)). As MGSolver / BiCGSTABSolver on MeshData
 * (src/solvers/mg_solver.hpp:119-161, src/solvers/bicgstab_solver.hpp:116-315). */
int pgb_gmg_solve_blocks(pgb_gmg *gmg, pgb_mesh *mesh, double *u, const double *rhs, int32_t ncomp, int32_t comp_u,
                         int32_t comp_rhs, int32_t method, double rtol, int32_t max_iters, int32_t *iters_out,
                         double *relres_out, void *stream);

/* ---- multigrid on the composite grids of a refined mesh --------------------------
 * MGSolver<u, rhs, PoissonEquation> on a mesh with refinement: FAS V-cycles over the
 * two-level composite grids (grid L = every block of level L plus the leaves of level
 * L-1; the level-L blocks are smoothed, the coarser leaves lend boundary values), with
 * SRJ or weighted-Jacobi smoothing, volume-average restriction, linear prolongation and
 * the gmg_same ghost exchange (restriction/prolongation across coarse/fine faces) on
 * every grid; the outer residual is taken on the leaf grid. The operator is
 * div(D grad u) - alpha u with constant D (poisson_equation.hpp:41-210, flux correction
 * off as in the package default). FP64; the exact build is bitwise the reference's
 * arithmetic, the fast build within rounding of it.
 * Replaces MGSolver::AddTasks / AddSetupTasks (src/solvers/mg_solver.hpp:119-520) with
 * Mesh::BuildGMGBlockLists / SetGMGNeighbors (src/mesh/mesh-gmg.cpp:103-201). */
typedef struct pgb_mg pgb_mg;
typedef struct {
  int32_t stages;          /* SRJ stages 1..3, or weighted-Jacobi sweeps when jacobi */
  int32_t jacobi;          /* 0: SRJ (Yang-Mittal weights); 1: weighted Jacobi with weight */
  double weight;
  int32_t coarse_sweeps;   /* extra smoother passes on the coarsest grid (0 = reference) */
  int32_t max_coarsenings; /* MGParams::max_coarsenings: grids max .. max(max - this, min) */
  double D;                /* constant face coefficient (the poisson D field) */
  double alpha;            /* poisson/diagonal_alpha */
  int32_t exact;           /* 1: separately rounded reference-order arithmetic (bitwise);
                              0: FMA 7-point operator with the diagonal's reciprocal */
  int32_t flux_correct;    /* poisson/flux_correct: flux correction inside Ax on the leaf
                              grid (the outer residual and BiCGSTAB's operator); the
                              composite grids' operator has none, as in the reference */
} pgb_mg_params;
/* Host only: builds the composite grids of the mesh (which must outlive the solver);
 * device memory is taken on the first solve. */
int pgb_mg_create(pgb_mesh *mesh, const pgb_mg_params *params, pgb_mg **out);
int pgb_mg_destroy(pgb_mg *mg);
/* out[5]: coarsest and finest logical level, storage slots of full-size blocks, leaf
 * blocks, grids */
int pgb_mg_info(const pgb_mg *mg, int32_t *out);
/* gmg_same boundary index maps of grid `level` in the pgb_mesh_boundaries record
 * format; *count receives the number of records (out may be NULL to query it). */
int pgb_mg_boundaries(const pgb_mg *mg, int32_t level, int32_t *out, int32_t capacity, int32_t *count);
/* A spatially varying coefficient: the poisson_gmg package's face field D, D grad u on
 * every face. d: device array of the leaf blocks, [block][3][k][j][i] with the block
 * extents of the cell arrays (x1, x2, x3 faces; face i is the low face of cell i, the
 * block's last face sits at nghost + nx). Restricted to the internal blocks of every
 * grid as MGSolver::AddSetupTasks does (mg_solver.hpp:188-203, RestrictAverage on faces);
 * the constant D of the parameters is no longer used. Synchronises the stream. */
int pgb_mg_set_coefficient(pgb_mg *mg, const double *d, void *stream);
/* u, rhs: device arrays of the leaf blocks, [block][k][j][i] with ghosts (one
 * component). ncycles V-cycles on u (in/out: interior result, ghosts exchanged);
 * rms (host, may be NULL) receives sqrt(sum r^2 / N) of the leaf residual after each.
 * The stream must be a created stream (each iteration is one CUDA-graph launch). */
int pgb_mg_vcycles(pgb_mg *mg, double *u, const double *rhs, int32_t ncycles, double *rms, void *stream);
/* Iterations until rms(rhs - A u) <= tol (relative = 0, the reference's
 * residual_tolerance) or <= tol * the initial rms (relative = 1), or max_cycles.
 * mixed = 0: FP64 V-cycles on u. mixed = 1: iterative refinement, an FP32 V-cycle (the
 * fast build's arithmetic; the coarsest grid in FP64 when it lies below level 0) on
 * A e = r from e = 0 with r the FP64 leaf residual, then u += e. */
int pgb_mg_solve(pgb_mg *mg, double *u, const double *rhs, double tol, int32_t relative, int32_t mixed,
                 int32_t max_cycles, int32_t *cycles_out, double *rms_out, void *stream);
/* Right-preconditioned BiCGSTAB on the leaf grid from u = 0 (the result, with exchanged
 * ghosts, is written to u): precondition 0: none; 1: one FP64 V-cycle on the composite
 * grids from zero per application; 2: one FP32 V-cycle (the coarsest grid in FP64 below
 * level 0). Stops when sqrt((r,r)/N) < rtol (relative = 0) or < rtol * sqrt((rhs,rhs)/N)
 * (relative = 1), or after max_iters; one CUDA-graph launch per iteration, the host
 * reads one double. Replaces BiCGSTABSolver::AddTasks (src/solvers/bicgstab_solver.hpp:
 * 116-315) with MGSolver on the composite grids as its preconditioner. */
int pgb_mg_bicgstab(pgb_mg *mg, double *u, const double *rhs, int32_t precondition, double rtol, int32_t relative,
                    int32_t max_iters, int32_t *iters_out, double *rms_out, void *stream);

/* ---- the composite grids for a package-side solver --------------------------------
 * MGSolver<u, rhs, Eq> with a package's own equation (src/solvers/mg_solver.hpp:59-72:
 * the Eq supplies Ax and SetDiagonal) runs its V-cycle on fields it holds itself; these
 * calls give it the grids of a pgb_mg and move one such field between them. A field has
 * one device array per store, [slot][k][j][i] with ghosts, x fastest; store 0 holds the
 * full-size blocks (the leaves first in gid order, so its first slots are the leaf
 * layout of the mesh, then the internal blocks of levels >= 0), store L < 0 the blocks of
 * level L. A face field has three such arrays back to back (x1, x2, x3 faces; face i is
 * the low face of cell i).
 * Replaces the gmg_same / gmg_restrict / gmg_prolongate boundary tasks
 * (src/bvals/comms/bvals_in_one.hpp:41-93 on the grids of src/mesh/mesh-gmg.cpp:103-201). */
/* out[5]: coarsest and finest grid level, leaf blocks, stores, exact build (1) or not */
int pgb_mg_layout(pgb_mg *mg, int32_t *out);
/* out[8]: slots, nx[3], nghost, N[3] of store `store` (0, or a level below 0); geom
 * (may be NULL): 6 doubles per slot, the first interior cell's low corner and the cell
 * widths; levels (may be NULL): the logical level per slot. */
int pgb_mg_store_info(pgb_mg *mg, int32_t store, int32_t *out, double *geom, int32_t *levels);
/* out[4]: the grid's store, its fine blocks (level `level`, internal blocks first), its
 * coarser leaves (level - 1) and internal blocks among the fine ones; fine / coarse (may
 * be NULL) receive the slots. */
int pgb_mg_grid_info(pgb_mg *mg, int32_t level, int32_t *out, int32_t *fine, int32_t *coarse);
/* gmg_same ghost exchange of one field on grid `level` (field: the array of the grid's
 * store), with ProlongateSharedLinear across its coarse/fine faces. */
int pgb_mg_field_exchange(pgb_mg *mg, int32_t level, double *field, void *stream);
/* RestrictAverage of the fine blocks of grid `level` (fine: their store's array) into
 * their parents' octants on grid level - 1 (coarse: that grid's store array). */
int pgb_mg_field_restrict(pgb_mg *mg, int32_t level, const double *fine, double *coarse, void *stream);
/* ProlongateSharedLinear of the parents (coarse: grid level - 1's store array, ghosts
 * current) written into the interior of every fine block of grid `level`. */
int pgb_mg_field_prolongate(pgb_mg *mg, int32_t level, const double *coarse, double *fine, void *stream);
/* RestrictAverage on faces of a face field from the fine blocks of grid `level` into
 * their parents (the setup step's GMGRestrict of a face field). */
int pgb_mg_face_restrict(pgb_mg *mg, int32_t level, const double *fine, double *coarse, void *stream);

/* ---- launch-shape autotuner ------------------------------------------------------ */

/* The first pgb_rk2_cycles call on a mesh (before it captures the cycle graph) times a
 * few launch shapes of the hot kernels on the caller's data -- threads per CTA of the
 * ghost copy, persistent CTAs per SM of the WENO5/HLL sweep -- and keeps the fastest
 * per kernel and problem size for the process; PGB_TUNE=0 in the environment keeps the
 * defaults. Writes "key=choice (ms per candidate) ; ..." (NUL-terminated, truncated to
 * capacity). No counterpart in the reference (its launch shapes are fixed by Kokkos
 * policies). */
int pgb_tune_report(char *buf, int32_t capacity);

/* ---- history reductions ----------------------------------------------------------- */

/* out[r] (host) = sum over blocks, components and interior cells whose centre lies in
 * box r (inclusive bounds) of u * u * vol / (mesh_volume + 1e-20); regions holds
 * nregions (1..8) boxes as x1min, x1max, x2min, x2max, x3min, x3max. Deterministic
 * (fixed reduction order); synchronises the stream. Replaces MassHistory
 * (benchmarks/burgers/burgers_package.cpp:406-439) as registered per octant (:106-135)
 * for the history output (src/outputs/history.cpp:40-210). */
int pgb_history_mass(pgb_mesh *mesh, const double *u, int32_t ncomp, const double *regions, int32_t nregions,
                     double mesh_volume, double *out, void *stream);

/* ---- adaptive refinement ------------------------------------------------------- */

/* Per-block refinement criterion of component `comp` of u (ghosts must be current),
 * written to the device array out[nblocks]. method 0: FirstDerivative, max over the
 * interior of 0.5|q(i+1)-q(i-1)| / (|q| + 1e-20) along each axis; 1: SecondDerivative;
 * 2: largest central-difference |grad q|. One launch for all blocks. Replaces the
 * per-block reductions of Refinement::FirstDerivative / SecondDerivative
 * (src/amr_criteria/refinement_package.cpp:93-150) called from AMRFirstDerivative /
 * AMRSecondDerivative::operator() (src/amr_criteria/amr_criteria.cpp:87-105). */
int pgb_amr_block_criterion(pgb_mesh *mesh, const double *u, int32_t ncomp, int32_t comp, int32_t method,
                            double *out, void *stream);

/* Host: refinement flags (+1, 0, -1 per block in gid order) from the criterion values
 * crit[nblocks] (host memory): refine above refine_tol, derefine below derefine_tol,
 * no refinement at or above crit_max_level; then the mesh's per-block derefinement
 * counters (kept in the handle and carried across pgb_amr_remesh) turn derefine tags
 * into -1 only after derefine_count consecutive tags and only without a finer
 * neighbour; no refinement at mesh_max_level. Replaces CheckAllRefinement
 * (src/amr_criteria/refinement_package.cpp:51-91) + MeshRefinement::SetRefinement
 * (src/mesh/mesh_refinement.cpp:82-118). */
int pgb_amr_set_refinement(pgb_mesh *mesh, const double *crit, double refine_tol, double derefine_tol,
                           int32_t crit_max_level, int32_t mesh_max_level, int32_t derefine_count,
                           int32_t *flags);

/* Host: the mesh after one adaptive step with the given flags (proper nesting kept, a
 * parent derefined only when all eight children ask). *out is a new, not yet uploaded
 * handle, or NULL when the leaf set does not change. Replaces Mesh::UpdateMeshBlockTree
 * (src/mesh/mesh-amr_loadbalance.cpp:496-629) with Tree::Refine / Tree::Derefine
 * (src/mesh/forest/tree.cpp:82-137,221-267). */
int pgb_amr_remesh(pgb_mesh *mesh, const int32_t *flags, pgb_mesh **out);

/* Moves a field from the old mesh to the new one (both uploaded): same-level blocks are
 * copied, new fine blocks are minmod-prolongated from their parent over the whole
 * array, new coarse blocks get their children's interiors restricted (ghosts zero; run
 * an exchange with PGB_EXCHANGE_PROLONGATE afterwards). One launch; synchronises the
 * stream. Replaces the same-rank data movement of RedistributeAndRefineMeshBlocks
 * (src/mesh/mesh-amr_loadbalance.cpp:663-1010, amr_loadbalance.cpp:95-135,205-245). */
int pgb_amr_transfer(pgb_mesh *old_mesh, pgb_mesh *new_mesh, const double *old_data, double *new_data,
                     int32_t ncomp, void *stream);

/* ---- sparse variables ------------------------------------------------------------ */

/* Every component of the fields exchanged and evolved on this mesh becomes a sparse
 * variable (Metadata::Sparse): per block an allocation flag and a deallocation counter,
 * per variable an allocation threshold, a deallocation threshold and a default value
 * (host arrays of ncomp doubles). Afterwards, on this mesh:
 *  - pgb_exchange sends a null buffer for an unallocated sender or one whose sent
 *    values are all below the allocation threshold, allocates a receiver's variable when
 *    any of its buffers carries data, writes allocated receivers only and fills their
 *    ghosts behind a null buffer with the default value; restriction and prolongation
 *    skip unallocated variables (SendBoundBufs / ReceiveBoundBufs / SetBounds,
 *    src/bvals/comms/boundary_communication.cpp:95-140,216-232,267-330);
 *  - pgb_flux_correct: an allocated fine block always sends and its coarse neighbour
 *    allocates (boundary_communication.cpp:121);
 *  - pgb_stage computes, corrects and applies fluxes of allocated variables only
 *    (advection only);
 *  - pgb_rk2_cycles runs pgb_sparse_dealloc on base after the last stage's exchange
 *    (example/sparse_advection/sparse_advection_driver.cpp:120-123);
 *  - pgb_amr_remesh carries the flags to the new mesh (a new fine block allocates what
 *    its parent had, a new coarse block what any child had, counters of new blocks start
 *    at zero; src/mesh/mesh-amr_loadbalance.cpp:95-145,187-213).
 * An unallocated variable must hold zeros in every container (what a fresh allocation
 * gives); the library keeps it so. All variables start unallocated. dealloc_count: a
 * variable is deallocated after more than this many consecutive all-below checks
 * (Globals::sparse_config, src/globals.hpp:33-35). */
typedef struct {
  int32_t ncomp;
  int32_t dealloc_count;
  const double *alloc_threshold;
  const double *dealloc_threshold;
  const double *default_value;
} pgb_sparse_params;
int pgb_sparse_enable(pgb_mesh *mesh, const pgb_sparse_params *p);
/* Flags alloc[nblocks * ncomp] (0/1, block-major) and, if non-NULL, counters. */
int pgb_sparse_set_alloc(pgb_mesh *mesh, const uint8_t *alloc, const int32_t *counts);
/* Reads the flags and counters (either may be NULL) after synchronising the stream. */
int pgb_sparse_get_alloc(pgb_mesh *mesh, uint8_t *alloc, int32_t *counts, void *stream);
/* SparseDealloc (src/interface/update.cpp:143-216) on field u: a variable whose values
 * (ghosts included) all satisfy |q| <= its deallocation threshold counts one more check,
 * otherwise its counter restarts; past dealloc_count checks it is deallocated and its
 * slices in `cells` (ncells fields like u), `coarse` (ncoarse coarse buffers) and `flux`
 * (flux arrays, may be NULL) are zeroed. */
int pgb_sparse_dealloc(pgb_mesh *mesh, const double *u, double *const *cells, int32_t ncells, double *const *coarse,
                       int32_t ncoarse, double *flux, void *stream);
/* Per-block tag (device out[nblocks], as -1.0 / 0.0 / 1.0) of the sparse advection
 * package's CheckRefinement (example/sparse_advection/sparse_advection_package.cpp:
 * 94-123): min and max over the allocated variables, ghosts included; refine when
 * max > refine_tol and min < derefine_tol, derefine when max < derefine_tol. Feed it to
 * pgb_amr_set_refinement with refine_tol 0.5 and derefine_tol -0.5. */
int pgb_sparse_tag(pgb_mesh *mesh, const double *u, double refine_tol, double derefine_tol, double *out,
                   void *stream);

#ifdef __cplusplus
}
#endif

#endif /* PARTHENON_GB300_H_ */
