// Multigrid on the two-level composite grids of a refined mesh.
//
// MGSolver on a mesh with refinement (src/solvers/mg_solver.hpp:119-520) runs its FAS
// V-cycle over the grids of src/mesh/mesh-gmg.cpp:103-201: grid L holds every block of
// level L (leaves and internal blocks) and the leaves of level L-1; the level-L blocks
// are the active ones (packs of a composite grid hold the finer blocks only,
// src/interface/sparse_pack.hpp:69-109) and the coarser leaves lend their values across
// coarse/fine faces through the grid's ghost exchange.
//
// Layout. Every block of the full block size (the leaves first, in gid order, then the
// internal blocks of levels >= 0 by gid) owns one slot of a store of five arrays (u,
// res_err, rhs, temp, u0) with ghosts, one component, x fastest; the blocks below level
// 0 are smaller and have a store per level. A leaf in two grids is one slot, as the
// reference shares the MeshBlock between the two lists, so nothing moves between grids
// but the restriction and the prolongation. A grid with coarse/fine faces runs the
// leaf-grid exchange kernels (exchange.cu) on tables whose block indices are store
// slots; a grid of one level reads its blocks' face neighbours directly instead.
//
// Fused steps per level: Ax + Jacobi, Ax + residual, u0 copy + Ax + FAS right-hand
// side; the restriction of u and res_err writes the parent's octant directly (the
// child's coarse buffer and the message buffer hold the same values); the linear
// prolongation of res_err is added straight into u over the child's interior. The values
// the reference also prolongates into the child's ghosts, and the child's res_err after
// the update, are never read again and are not written. Every read of a ghost cell
// follows an exchange that writes it. One solver iteration (V-cycle plus leaf-grid
// residual, or one BiCGSTAB iteration) is one CUDA graph whose kernels use programmatic
// dependent launch.
//
// Builds: exact (reference expression order, separately rounded: this file is compiled
// with -fmad=false and divides by powers of two as exact multiplications, so interiors
// are bitwise those of the CPU restatement) and fast (FMA, the 7-point form, the
// diagonal's reciprocal). The mixed solve runs the V-cycle on FP32 copies of the stores
// inside FP64 iterative refinement. Also here: the package's face coefficient D
// (restricted by the setup step), flux correction inside the leaf-grid operator, and
// BiCGSTAB with the V-cycle as preconditioner (src/solvers/bicgstab_solver.hpp:116-315).
#include <cuda_runtime.h>

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstring>
#include <map>
#include <set>
#include <stdexcept>
#include <unordered_map>
#include <vector>

#include "../../include/parthenon_gb300.h"
#include "common.cuh"
#include "gmg_state.hpp"
#include "mesh_state.hpp"

namespace pgb {
MeshState *mesh_state(pgb_mesh *m);
int exchange_grid(GridTables &t, double *fine, double *coarse, int ncomp, int prolongate, int prolong_op,
                  double *buffer, cudaStream_t s, const SparseDev *sp);
int exchange_grid_f32(GridTables &t, float *fine, float *coarse, cudaStream_t s);
int flux_correct_grid(GridTables &t, double *flux, int ncomp, cudaStream_t s, const SparseDev *sp);
}  // namespace pgb

using namespace pgb;

namespace {

// One fine block of a grid and its parent in the next coarser grid: `lo` is the first
// interior cell of the parent's octant that the child covers (parent index space with
// ghosts), from the InteriorRecv range of bnd_info.cpp:105-252.
struct MgXfer {
  int32_t child, parent;
  int32_t lo[3];
  int32_t pnb[6];  // the parent's face neighbours when its grid reads them directly, else -1
  int32_t pad;
};

struct MgOp {
  double D, alpha;
};

// Operator constants of one grid (its fine blocks share one spacing) or of one leaf
// block, formed once on the host.
struct MgCoef {
  double dx[3];  // exact build: the spacings (fluxes formed and divided as the reference does)
  double c[3];   // fast build: D / dx_d^2
  double ic[3];  // fast build, face coefficient: 1 / dx_d^2
  double dg;     // SetDiagonal (poisson_equation.hpp:59-102)
  double den;    // robust::ratio denominator dg + sgn(dg) 10 DBL_MIN (utils/robust.hpp)
};
// One Jacobi sweep: weight, 1 - weight, weight / den
struct MgSweep {
  double w, omw, wd;
};

template <class T>
struct StoreView {
  T *u, *res, *rhs, *temp, *u0;
  Dims d;
};

__device__ __forceinline__ double fma_t(double a, double b, double c) { return fma(a, b, c); }
__device__ __forceinline__ float fma_t(float a, float b, float c) { return fmaf(a, b, c); }

__device__ __forceinline__ int64_t cell_of(const Dims &d, int slot, int k, int j, int i) {
  return ((int64_t)slot * d.N[2] + k) * ((int64_t)d.N[1] * d.N[0]) + (int64_t)j * d.N[0] + i;
}

// log2 of a power of two, else -1
__device__ __forceinline__ int pow2_log(int v) { return v > 0 && (v & (v - 1)) == 0 ? __ffs(v) - 1 : -1; }

// Flat index e over boxes of n0 x n1 x n2 cells -> (box, k, j, i), i fastest. Block
// extents are powers of two on every mesh of this path, and then the split is shifts and
// masks; the integer divisions it replaces were a third of the instructions of the
// FP32 grid kernels. The branch is uniform across the launch.
struct CellSplit {
  int n0, n1, per, l0, l1, lp;
  __device__ __forceinline__ CellSplit(int a, int b, int c)
      : n0(a), n1(b), per(a * b * c), l0(pow2_log(a)), l1(pow2_log(b)), lp(pow2_log(a * b * c)) {}
  __device__ __forceinline__ void operator()(int e, int &q, int &k, int &j, int &i) const {
    if ((l0 | l1 | lp) >= 0) {
      q = e >> lp;
      const int c = e & (per - 1);
      i = c & (n0 - 1);
      const int r = c >> l0;
      j = r & (n1 - 1);
      k = r >> l1;
    } else {
      q = e / per;
      const int c = e - q * per;
      const int r = c / n0;
      i = c - r * n0;
      k = r / n1;
      j = r - k * n1;
    }
  }
};

// Every interior cell of the listed blocks (list == null: slots 0 .. n-1), consecutive
// threads on consecutive i; f gets (position in the list, slot, k, j, i). The host keeps
// cells x blocks below 2^31.
template <class F>
__device__ __forceinline__ void for_interior(const int *__restrict__ list, int n, const Dims &d, F &&f) {
  const int ng = d.ng;
  const CellSplit sp(d.nx[0], d.nx[1], d.nx[2]);
  const int total = sp.per * n;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < total; e += gridDim.x * blockDim.x) {
    int q, k, j, i;
    sp(e, q, k, j, i);
    f(q, list ? list[q] : q, k + ng, j + ng, i + ng);
  }
}

// A cell and its six face neighbours. nb == null: the neighbours outside the block are
// its ghosts, filled by the grid's exchange. Otherwise nb holds the block's six
// face-neighbour slots (-x, +x, -y, +y, -z, +z): on a grid of one level (no coarse/fine
// faces) a ghost cell is a copy of the neighbour's interior cell, which is read instead,
// so those grids need no exchange before a stencil.
template <class T>
struct Faces {
  T c, xm, xp, ym, yp, zm, zp;
};
template <class T>
__device__ __forceinline__ Faces<T> faces(const T *__restrict__ u, const Dims &d, const int *__restrict__ nb, int b,
                                          int k, int j, int i) {
  const int64_t sj = d.N[0], sk = (int64_t)d.N[0] * d.N[1];
  const int64_t c = cell_of(d, b, k, j, i);
  Faces<T> f;
  f.c = u[c];
  if (!nb) {
    f.xm = u[c - 1];
    f.xp = u[c + 1];
    f.ym = u[c - sj];
    f.yp = u[c + sj];
    f.zm = u[c - sk];
    f.zp = u[c + sk];
    return f;
  }
  const int lo = d.ng, h0 = d.ng + d.nx[0] - 1, h1 = d.ng + d.nx[1] - 1, h2 = d.ng + d.nx[2] - 1;
  f.xm = i > lo ? u[c - 1] : u[cell_of(d, nb[0], k, j, h0)];
  f.xp = i < h0 ? u[c + 1] : u[cell_of(d, nb[1], k, j, lo)];
  f.ym = j > lo ? u[c - sj] : u[cell_of(d, nb[2], k, h1, i)];
  f.yp = j < h1 ? u[c + sj] : u[cell_of(d, nb[3], k, lo, i)];
  f.zm = k > lo ? u[c - sk] : u[cell_of(d, nb[4], h2, j, i)];
  f.zp = k < h2 ? u[c + sk] : u[cell_of(d, nb[5], lo, j, i)];
  return f;
}

// The face coefficient of the poisson_gmg package (a Face field D): per block arrays in
// the cell layout, face i the low face of cell i (the block's last face at ng + nx).
// Null pointers: the constant MgOp::D.
template <class T>
struct FaceD {
  const T *d0, *d1, *d2;
};
// D on the low and high x1, x2, x3 faces of cell c
__device__ __forceinline__ void face_d6(const FaceD<double> &fd, int64_t c, int64_t sj, int64_t sk, double D,
                                        double *D6) {
  if (fd.d0) {
    D6[0] = fd.d0[c];
    D6[1] = fd.d0[c + 1];
    D6[2] = fd.d1[c];
    D6[3] = fd.d1[c + sj];
    D6[4] = fd.d2[c];
    D6[5] = fd.d2[c + sk];
  } else {
    for (int q = 0; q < 6; ++q) D6[q] = D;
  }
}

// Exact build, poisson_equation.hpp:104-210: face fluxes D grad u, then their
// divergence, -alpha u + sum over directions of (F_left - F_right) / dx, in the
// reference's order
__device__ __forceinline__ double ax_exact(const Faces<double> &f, const double *dx, const MgOp &o,
                                          const double *D6) {
  const double dx1 = dx[0], dx2 = dx[1], dx3 = dx[2];
  const double uc = f.c;
  const double f1l = div_rn(D6[0], dx1) * (f.xm - uc);
  const double f1r = div_rn(D6[1], dx1) * (uc - f.xp);
  const double f2l = div_rn(D6[2] * (f.ym - uc), dx2);
  const double f2r = div_rn(D6[3] * (uc - f.yp), dx2);
  const double f3l = div_rn(D6[4] * (f.zm - uc), dx3);
  const double f3r = div_rn(D6[5] * (uc - f.zp), dx3);
  double out = -o.alpha * uc;
  out += div_rn(f1l - f1r, dx1);
  out += div_rn(f2l - f2r, dx2);
  out += div_rn(f3l - f3r, dx3);
  return out;
}

// Exact build, SetDiagonal (poisson_equation.hpp:59-102) from the faces
__device__ __forceinline__ double diag_exact(const double *dx, const MgOp &o, const double *D6) {
  double d = -div_rn(D6[0] + D6[1], dx[0] * dx[0]) - o.alpha;
  d -= div_rn(D6[2] + D6[3], dx[1] * dx[1]);
  d -= div_rn(D6[4] + D6[5], dx[2] * dx[2]);
  return d;
}

// Exact build: the operator, its diagonal and the robust::ratio denominator at cell c
// (the grid's host-formed constants when D is constant)
struct ExactOp {
  double ax, dg, den;
};
__device__ __forceinline__ ExactOp exact_op(const Faces<double> &f, const MgCoef &cf, const MgOp &o,
                                            const FaceD<double> &fd, int64_t c, int64_t sj, int64_t sk) {
  double D6[6];
  face_d6(fd, c, sj, sk, o.D, D6);
  ExactOp r;
  r.ax = ax_exact(f, cf.dx, o, D6);
  if (fd.d0) {
    r.dg = diag_exact(cf.dx, o, D6);
    r.den = r.dg + (r.dg >= 0 ? 1.0 : -1.0) * (10.0 * DBL_MIN);
  } else {
    r.dg = cf.dg;
    r.den = cf.den;
  }
  return r;
}

// Fast build: the constant-coefficient operator as a 7-point stencil, A u = off + dg u
// with off = sum_d (D/dx_d^2) (u_{-d} + u_{+d}): 3 adds, a multiply and 2 FMAs (the FP64
// pipe, not HBM, bounds these kernels on GB300)
template <class T>
__device__ __forceinline__ T off_fast(const Faces<T> &f, const MgCoef &cf) {
  return fma_t((T)cf.c[2], f.zm + f.zp, fma_t((T)cf.c[1], f.ym + f.yp, (T)cf.c[0] * (f.xm + f.xp)));
}
// Fast build with face coefficients: off = sum_d (D_low u_{-d} + D_high u_{+d}) / dx_d^2,
// dg = -sum_d (D_low + D_high) / dx_d^2 - alpha
template <class T>
__device__ __forceinline__ void fast_op(const Faces<T> &f, const MgCoef &cf, const MgOp &o, const FaceD<T> &fd,
                                        int64_t c, int64_t sj, int64_t sk, T &off, T &dg) {
  if (fd.d0) {
    const T a0 = fd.d0[c], a1 = fd.d0[c + 1], b0 = fd.d1[c], b1 = fd.d1[c + sj], e0 = fd.d2[c], e1 = fd.d2[c + sk];
    const T i1 = (T)cf.ic[0], i2 = (T)cf.ic[1], i3 = (T)cf.ic[2];
    off = fma_t(fma_t(e0, f.zm, e1 * f.zp), i3, fma_t(fma_t(b0, f.ym, b1 * f.yp), i2, fma_t(a0, f.xm, a1 * f.xp) * i1));
    dg = -fma_t(e0 + e1, i3, fma_t(b0 + b1, i2, (a0 + a1) * i1)) - (T)o.alpha;
  } else {
    off = off_fast(f, cf);
    dg = (T)cf.dg;
  }
}

// Jacobi sweep (mg_solver.hpp:222-297): dst = w ratio(rhs - (A src - dg src), dg) + (1 - w) src
// ---- per-cell steps, shared by the grid kernels below and the one-CTA coarse end

template <bool kFast, class T>
__device__ __forceinline__ void jacobi_cell_f(const Faces<T> &f, const T *__restrict__ rhs, T *__restrict__ dst,
                                              const Dims &d, const MgCoef &cf, const MgOp &o, const MgSweep &sw,
                                              const FaceD<T> &fd, int b, int k, int j, int i);

// Jacobi sweep (mg_solver.hpp:222-297): dst = w ratio(rhs - (A src - dg src), dg) + (1 - w) src
template <bool kFast, class T>
__device__ __forceinline__ void jacobi_cell(const T *__restrict__ src, const T *__restrict__ rhs, T *__restrict__ dst,
                                            const Dims &d, const int *__restrict__ nb, const MgCoef &cf,
                                            const MgOp &o, const MgSweep &sw, const FaceD<T> &fd, int b, int k,
                                            int j, int i) {
  jacobi_cell_f<kFast>(faces(src, d, nb, b, k, j, i), rhs, dst, d, cf, o, sw, fd, b, k, j, i);
}

// the swept value of cell c (global index) from its stencil values f and right-hand side
template <bool kFast, class T>
__device__ __forceinline__ T jacobi_value(const Faces<T> &f, T rhs_c, const Dims &d, const MgCoef &cf,
                                          const MgOp &o, const MgSweep &sw, const FaceD<T> &fd, int64_t c) {
  const int64_t sj = d.N[0], sk = (int64_t)d.N[0] * d.N[1];
  if constexpr (kFast) {
    T off, dg;
    fast_op(f, cf, o, fd, c, sj, sk, off, dg);
    if (fd.d0) {
      const T small = (T)10 * (sizeof(T) == 8 ? (T)DBL_MIN : (T)FLT_MIN);
      const T den = dg + (dg >= (T)0 ? (T)1 : (T)-1) * small;
      return fma_t((T)sw.w / den, rhs_c - off, (T)sw.omw * f.c);
    }
    return fma_t((T)sw.wd, rhs_c - off, (T)sw.omw * f.c);
  } else {
    const ExactOp e = exact_op(f, cf, o, fd, c, sj, sk);
    const double off = e.ax - e.dg * f.c;
    const double val = rhs_c - off;
    return sw.w * div_rn(val, e.den) + sw.omw * f.c;
  }
}

// the sweep of one cell from its stencil values f
template <bool kFast, class T>
__device__ __forceinline__ void jacobi_cell_f(const Faces<T> &f, const T *__restrict__ rhs, T *__restrict__ dst,
                                              const Dims &d, const MgCoef &cf, const MgOp &o, const MgSweep &sw,
                                              const FaceD<T> &fd, int b, int k, int j, int i) {
  const int64_t c = cell_of(d, b, k, j, i);
  dst[c] = jacobi_value<kFast>(f, rhs[c], d, cf, o, sw, fd, c);
}

// Ax + AddFieldsAndStoreInteriorSelect<rhs, temp, res_err>(1, -1): res = rhs - A u
template <bool kFast, class T>
__device__ __forceinline__ void residual_cell(const StoreView<T> &s, const int *__restrict__ nb, const MgCoef &cf,
                                              const MgOp &o, const FaceD<T> &fd, int b, int k, int j, int i) {
  const int64_t sj = s.d.N[0], sk = (int64_t)s.d.N[0] * s.d.N[1];
  const int64_t c = cell_of(s.d, b, k, j, i);
  const Faces<T> f = faces(s.u, s.d, nb, b, k, j, i);
  if constexpr (kFast) {
    T off, dg;
    fast_op(f, cf, o, fd, c, sj, sk, off, dg);
    s.res[c] = fma_t(-dg, f.c, s.rhs[c] - off);
  } else {
    s.res[c] = s.rhs[c] - exact_op(f, cf, o, fd, c, sj, sk).ax;
  }
}

// Start of a level below the finest (mg_solver.hpp:405-430): u0 = u and, on internal
// blocks, the FAS right-hand side rhs = A u + res_err
template <bool kFast, class T>
__device__ __forceinline__ void fas_cell(const StoreView<T> &s, bool internal, const int *__restrict__ nb,
                                         const MgCoef &cf, const MgOp &o, const FaceD<T> &fd, int b, int k, int j,
                                         int i) {
  const int64_t sj = s.d.N[0], sk = (int64_t)s.d.N[0] * s.d.N[1];
  const int64_t c = cell_of(s.d, b, k, j, i);
  const T uc = s.u[c];
  s.u0[c] = uc;
  if (!internal) return;
  const Faces<T> f = faces(s.u, s.d, nb, b, k, j, i);
  if constexpr (kFast) {
    T off, dg;
    fast_op(f, cf, o, fd, c, sj, sk, off, dg);
    s.rhs[c] = fma_t(dg, uc, off + s.res[c]);
  } else {
    s.rhs[c] = exact_op(f, cf, o, fd, c, sj, sk).ax + s.res[c];
  }
}

// RestrictAverage (pr_ops.hpp:105-164) of one field of the child's interior into the
// parent's octant, one parent cell (f, p: the first fine cell and the parent cell).
// FP64 children: the reference's volume-weighted form; FP32 children (the mixed
// V-cycle): the mean of the eight cells. TP is the parent's type.
template <class TC, class TP>
__device__ __forceinline__ void restrict_field_cell(const TC *__restrict__ a, TP *__restrict__ out, const Dims &d,
                                                    double vol, int64_t f, int64_t p) {
  const int64_t cj = d.N[0], ck = (int64_t)d.N[0] * d.N[1];
  if constexpr (sizeof(TC) == 8) {
    const double tv = ((vol + vol) + (vol + vol)) + ((vol + vol) + (vol + vol));
    // t[ok][oj][oi] = vol * fine(k + ok, j + oj, i + oi)
    const double t000 = vol * a[f], t001 = vol * a[f + 1];
    const double t010 = vol * a[f + cj], t011 = vol * a[f + cj + 1];
    const double t100 = vol * a[f + ck], t101 = vol * a[f + ck + 1];
    const double t110 = vol * a[f + ck + cj], t111 = vol * a[f + ck + cj + 1];
    const double num = ((t000 + t010) + (t001 + t011)) + ((t100 + t110) + (t101 + t111));
    out[p] = (TP)div_rn(num, tv);
  } else {
    const TC sum = ((a[f] + a[f + cj]) + (a[f + 1] + a[f + cj + 1])) +
                   ((a[f + ck] + a[f + ck + cj]) + (a[f + ck + 1] + a[f + ck + cj + 1]));
    out[p] = (TP)((TC)0.125 * sum);
  }
}

// u and res_err of one parent cell (gmg_restrict_send + gmg_restrict_recv)
template <class TC, class TP>
__device__ __forceinline__ void restrict_cell(const StoreView<TC> &cs, const StoreView<TP> &ps, const MgXfer &t,
                                              double vol, int ci, int cjj, int ckk) {
  const int ng = cs.d.ng;
  const int64_t f = cell_of(cs.d, t.child, 2 * ckk + ng, 2 * cjj + ng, 2 * ci + ng);
  const int64_t p = cell_of(ps.d, t.parent, t.lo[2] + ckk, t.lo[1] + cjj, t.lo[0] + ci);
  restrict_field_cell(cs.u, ps.u, cs.d, vol, f, p);
  restrict_field_cell(cs.res, ps.res, cs.d, vol, f, p);
}

// ProlongateSharedLinear (pr_ops.hpp:166-285) of a parent field (its octant with ghosts
// is the child's coarse buffer), one coarse cell of the child's interior: apply(offset,
// value) receives each of the eight fine values, offset relative to the first fine cell
// `fine`. The exact build forms the slopes from the cell-centre coordinates as the
// reference does (g: the child's geometry); the fast build uses the uniform-spacing value
// dx_fine / 2 / dx_coarse = 1/4 of each difference. TC is the child's type (the
// arithmetic), TP the parent's.
template <bool kFast, class TC, class TP, class F>
__device__ __forceinline__ void prolong_field_cell(const TP *__restrict__ pf, const Dims &pd, const Dims &cd,
                                                   const MgXfer &t, const DevBlockGeom *__restrict__ g, int c0, int c1,
                                                   int c2, int64_t &fine, F &&apply) {
  const int ng = cd.ng;
  const int64_t pj = pd.N[0], pk = (int64_t)pd.N[0] * pd.N[1];
  const int64_t N0 = cd.N[0], N01 = (int64_t)cd.N[0] * cd.N[1];
  const int c[3] = {c0 + ng, c1 + ng, c2 + ng};  // coarse-buffer index
  const int f[3] = {2 * c0 + ng, 2 * c1 + ng, 2 * c2 + ng};
  const int p[3] = {t.lo[0] + c0, t.lo[1] + c1, t.lo[2] + c2};
  const int64_t pe = cell_of(pd, t.parent, p[2], p[1], p[0]);
  const TC fc = (TC)pf[pe];
  // the parent's cells next to p along d: its ghosts, or on a grid read directly the
  // face neighbour's interior cell
  auto side = [&](int d, int s) -> TC {
    const int64_t st = d == 0 ? 1 : (d == 1 ? pj : pk);
    const int lo = pd.ng, hi = pd.ng + pd.nx[d] - 1;
    if (t.pnb[0] < 0 || (s < 0 ? p[d] > lo : p[d] < hi)) return (TC)pf[pe + s * st];
    int q[3] = {p[0], p[1], p[2]};
    q[d] = s < 0 ? hi : lo;
    return (TC)pf[cell_of(pd, t.pnb[2 * d + (s > 0)], q[2], q[1], q[0])];
  };
  TC mq[3], pq[3];
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    if constexpr (kFast) {
      mq[d] = (TC)0.25 * (fc - side(d, -1));
      pq[d] = (TC)0.25 * (side(d, 1) - fc);
    } else {
      auto xcc = [&](int idx) { return g->cxmin[d] + ((double)idx + 0.5) * g->cdx[d]; };
      auto xfc = [&](int idx) { return g->xmin[d] + ((double)idx + 0.5) * g->dx[d]; };
      const double xm = xcc(c[d] - 1), xc = xcc(c[d]), xp = xcc(c[d] + 1);
      const double dxm = xc - xm, dxp = xp - xc;
      const double dfm = xc - xfc(f[d]);
      const double dfp = xfc(f[d] + 1) - xc;
      mq[d] = div_rn(fc - side(d, -1), dxm) * dfm;
      pq[d] = div_rn(side(d, 1) - fc, dxp) * dfp;
    }
  }
  const TC m0 = mq[0], p0 = pq[0], m1 = mq[1], p1 = pq[1], m2 = mq[2], p2 = pq[2];
  fine = cell_of(cd, t.child, f[2], f[1], f[0]);
  apply((int64_t)0, fc - ((m0 + m1) + m2));
  apply((int64_t)1, fc + ((p0 - m1) - m2));
  apply(N0, fc - ((m0 - p1) + m2));
  apply(N0 + 1, fc + ((p0 + p1) - m2));
  apply(N01, fc - ((m0 + m1) - p2));
  apply(N01 + 1, fc + ((p0 - m1) + p2));
  apply(N01 + N0, fc - ((m0 - p1) - p2));
  apply(N01 + N0 + 1, fc + ((p0 + p1) + p2));
}

// The prolongation of the parent's res_err added into the child's u
// (AddFieldsAndStore<u, res_err, u>), one coarse cell of the child's interior
template <bool kFast, class TC, class TP>
__device__ __forceinline__ void prolong_add_cell(const StoreView<TC> &cs, const StoreView<TP> &ps, const MgXfer &t,
                                                 const DevBlockGeom *__restrict__ g, int c0, int c1, int c2) {
  int64_t fine = 0;
  TC *__restrict__ U = cs.u;
  prolong_field_cell<kFast, TC>(ps.res, ps.d, cs.d, t, g, c0, c1, c2, fine,
                                [&](int64_t o, TC v) { U[fine + o] = U[fine + o] + v; });
}

// ---- grid kernels: every interior cell of the listed blocks

template <bool kFast, class T>
__global__ void __launch_bounds__(256) k_mg_jacobi(const T *__restrict__ src, const T *__restrict__ rhs,
                                                   T *__restrict__ dst, const int *__restrict__ list, int n,
                                                   const int *__restrict__ nbr, Dims d, MgCoef cf, MgOp o,
                                                   MgSweep sw, FaceD<T> fd) {
  pdl_enter();
  for_interior(list, n, d, [&](int q, int b, int k, int j, int i) {
    jacobi_cell<kFast>(src, rhs, dst, d, nbr ? nbr + 6 * q : nullptr, cf, o, sw, fd, b, k, j, i);
  });
}

// The first sweep from a zero initial guess: every value of the stencil is zero (ghosts
// included -- the exchange of a zero field writes zeros), so no exchange precedes it and
// the sweep reads only the right-hand side.
// The coarser leaves of the grid (clist, nc) get dst = 0, their u, which the next sweep's
// exchange of dst reads.
template <bool kFast, class T>
__global__ void __launch_bounds__(256) k_mg_jacobi_zero(const T *__restrict__ rhs, T *__restrict__ dst,
                                                        const int *__restrict__ list, int n,
                                                        const int *__restrict__ clist, int nc, Dims d, MgCoef cf,
                                                        MgOp o, MgSweep sw, FaceD<T> fd) {
  pdl_enter();
  const Faces<T> zero{};
  for_interior(list, n, d, [&](int, int b, int k, int j, int i) {
    jacobi_cell_f<kFast>(zero, rhs, dst, d, cf, o, sw, fd, b, k, j, i);
  });
  if (nc) for_interior(clist, nc, d, [&](int, int b, int k, int j, int i) { dst[cell_of(d, b, k, j, i)] = (T)0; });
}

template <bool kFast, class T>
__global__ void __launch_bounds__(256) k_mg_residual(StoreView<T> s, const int *__restrict__ list, int n,
                                                     const int *__restrict__ nbr, MgCoef cf, MgOp o,
                                                     FaceD<T> fd) {
  pdl_enter();
  for_interior(list, n, s.d, [&](int q, int b, int k, int j, int i) {
    residual_cell<kFast>(s, nbr ? nbr + 6 * q : nullptr, cf, o, fd, b, k, j, i);
  });
}

// the first nint blocks of the list are the internal ones
template <bool kFast, class T>
__global__ void __launch_bounds__(256) k_mg_fas(StoreView<T> s, const int *__restrict__ list, int n, int nint,
                                                const int *__restrict__ nbr, MgCoef cf, MgOp o, FaceD<T> fd) {
  pdl_enter();
  for_interior(list, n, s.d, [&](int q, int b, int k, int j, int i) {
    fas_cell<kFast>(s, q < nint, nbr ? nbr + 6 * q : nullptr, cf, o, fd, b, k, j, i);
  });
}

// The FAS start of a level fused with the first Jacobi sweep of its pre-smoothing, on a
// grid that reads its face neighbours directly: u0 = u, rhs = A u + res_err (internal
// blocks), then temp = the sweep of u against that rhs. The sweep reads u and the cell's
// own rhs, both final when the cell's thread reaches it, so the values are those of the
// two separate launches.
template <bool kFast, class T>
__global__ void __launch_bounds__(256) k_mg_fas_jacobi(StoreView<T> s, const int *__restrict__ list, int n,
                                                       int nint, const int *__restrict__ nbr, MgCoef cf, MgOp o,
                                                       MgSweep sw, FaceD<T> fd) {
  pdl_enter();
  for_interior(list, n, s.d, [&](int q, int b, int k, int j, int i) {
    const int *nb = nbr ? nbr + 6 * q : nullptr;
    fas_cell<kFast>(s, q < nint, nb, cf, o, fd, b, k, j, i);
    jacobi_cell<kFast>(s.u, s.rhs, s.temp, s.d, nb, cf, o, sw, fd, b, k, j, i);
  });
}

// A level's residual fused with its restriction: one thread per parent cell forms the
// residual of its eight fine cells (res = rhs - A u) and restricts u and res_err into
// the parent. MgXfer::pad holds the child's position in the grid's block list (its
// face-neighbour row on a grid read directly).
template <bool kFast, class TC, class TP>
__global__ void __launch_bounds__(256) k_mg_residual_restrict(StoreView<TC> cs, StoreView<TP> ps,
                                                              const MgXfer *__restrict__ x, int n,
                                                              const int *__restrict__ nbr, MgCoef cf, MgOp o,
                                                              FaceD<TC> fd, const DevBlockGeom *__restrict__ cgeom) {
  pdl_enter();
  const CellSplit sp(cs.d.nx[0] / 2, cs.d.nx[1] / 2, cs.d.nx[2] / 2);
  const int total = sp.per * n, ng = cs.d.ng;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < total; e += gridDim.x * blockDim.x) {
    int q, ck, cj, ci;
    sp(e, q, ck, cj, ci);
    const MgXfer t = x[q];
    const int *nb = nbr ? nbr + 6 * t.pad : nullptr;
#pragma unroll
    for (int o8 = 0; o8 < 8; ++o8)
      residual_cell<kFast>(cs, nb, cf, o, fd, t.child, 2 * ck + ng + (o8 >> 2), 2 * cj + ng + ((o8 >> 1) & 1),
                           2 * ci + ng + (o8 & 1));
    restrict_cell(cs, ps, t, cgeom[t.child].vol, ci, cj, ck);
  }
}

// CopyData on the interiors of the listed blocks
template <class T>
__global__ void __launch_bounds__(256) k_mg_copy(T *__restrict__ dst, const T *__restrict__ src,
                                                 const int *__restrict__ list, int n, Dims d) {
  pdl_enter();
  for_interior(list, n, d, [&](int, int b, int k, int j, int i) {
    const int64_t c = cell_of(d, b, k, j, i);
    dst[c] = src[c];
  });
}

// AddFieldsAndStore<u, u0, res_err>(1, -1): res = u - u0
template <class T>
__global__ void __launch_bounds__(256) k_mg_error(StoreView<T> s, const int *__restrict__ list, int n) {
  pdl_enter();
  for_interior(list, n, s.d, [&](int, int b, int k, int j, int i) {
    const int64_t c = cell_of(s.d, b, k, j, i);
    s.res[c] = s.u[c] - s.u0[c];
  });
}

// restriction of every fine block of a grid into its parent: one thread per parent cell
template <class TC, class TP>
__global__ void __launch_bounds__(256) k_mg_restrict(StoreView<TC> cs, StoreView<TP> ps, const MgXfer *__restrict__ x,
                                                     int n, const DevBlockGeom *__restrict__ cgeom) {
  pdl_enter();
  const CellSplit sp(max(1, cs.d.nx[0] / 2), max(1, cs.d.nx[1] / 2), max(1, cs.d.nx[2] / 2));
  const int total = sp.per * n;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < total; e += gridDim.x * blockDim.x) {
    int q, ck, cj, ci;
    sp(e, q, ck, cj, ci);
    const MgXfer t = x[q];
    restrict_cell(cs, ps, t, cgeom[t.child].vol, ci, cj, ck);
  }
}

// prolongation into every fine block of a grid: one thread per coarse cell of a child
template <bool kFast, class TC, class TP>
__global__ void __launch_bounds__(256) k_mg_prolong_add(StoreView<TC> cs, StoreView<TP> ps,
                                                        const MgXfer *__restrict__ x, int n,
                                                        const DevBlockGeom *__restrict__ cgeom) {
  pdl_enter();
  const CellSplit sp(max(1, cs.d.nx[0] / 2), max(1, cs.d.nx[1] / 2), max(1, cs.d.nx[2] / 2));
  const int total = sp.per * n;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < total; e += gridDim.x * blockDim.x) {
    int q, ck, cj, ci;
    sp(e, q, ck, cj, ci);
    const MgXfer t = x[q];
    prolong_add_cell<kFast>(cs, ps, t, cgeom + t.child, ci, cj, ck);
  }
}

// ---- one field of a package-side solver (pgb_mg_field_*): the same transfers on a
// field held in the store layout by the caller

// RestrictAverage of every fine block of a grid into its parent's octant, one field
__global__ void __launch_bounds__(256) k_mgf_restrict(const double *__restrict__ cf, Dims cd, double *__restrict__ pf,
                                                      Dims pd, const MgXfer *__restrict__ x, int n,
                                                      const DevBlockGeom *__restrict__ cgeom) {
  const int h0 = max(1, cd.nx[0] / 2), h1 = max(1, cd.nx[1] / 2), h2 = max(1, cd.nx[2] / 2);
  const int per = h0 * h1 * h2, total = per * n;
  const int ng = cd.ng;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < total; e += gridDim.x * blockDim.x) {
    const int q = e / per;
    const int r = e - q * per;
    const MgXfer t = x[q];
    const int ci = r % h0, cj = (r / h0) % h1, ck = r / (h0 * h1);
    restrict_field_cell(cf, pf, cd, cgeom[t.child].vol, cell_of(cd, t.child, 2 * ck + ng, 2 * cj + ng, 2 * ci + ng),
                        cell_of(pd, t.parent, t.lo[2] + ck, t.lo[1] + cj, t.lo[0] + ci));
  }
}

// ProlongateSharedLinear of the parents' field into the interior of every fine block of
// a grid (the values written, not added), one thread per coarse cell of a child
template <bool kFast>
__global__ void __launch_bounds__(256) k_mgf_prolong(const double *__restrict__ pf, Dims pd, double *__restrict__ cf,
                                                     Dims cd, const MgXfer *__restrict__ x, int n,
                                                     const DevBlockGeom *__restrict__ cgeom) {
  const int h0 = max(1, cd.nx[0] / 2), h1 = max(1, cd.nx[1] / 2), h2 = max(1, cd.nx[2] / 2);
  const int per = h0 * h1 * h2, total = per * n;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < total; e += gridDim.x * blockDim.x) {
    const int q = e / per;
    const int r = e - q * per;
    const MgXfer t = x[q];
    int64_t fine = 0;
    prolong_field_cell<kFast, double>(pf, pd, cd, t, cgeom + t.child, r % h0, (r / h0) % h1, r / (h0 * h1), fine,
                                      [&](int64_t o, double v) { cf[fine + o] = v; });
  }
}

// ---- the coarse end of the V-cycle in one launch
// The trailing grids that hold one block each (a single tree's levels at and below 0)
// run their down and up steps in one CTA, the steps separated by CTA barriers, instead
// of about a dozen launches per grid. Fast build only, grids of at most 8^3 cells (the
// 16^3 grid in the CTA made the mixed iteration slower on the refined 128^3 mesh: 0.85
// ms against 0.82 ms). Measured there: the FP64 V-cycle 1.19 ms with it, 1.22 ms
// without. On the uniform 128^3 mesh the one 8^3 grid's 16 x 2 extra sweeps run from
// shared memory (tail_coarse_sweeps_smem): FP64 solve 11.9 -> 11.6 ms.
constexpr int kTailMax = 8;
constexpr int kTailThreads = 1024;
struct TailGrid {
  int slot;      // the grid's block
  int nb[6];     // its face neighbours (itself: one block tiles the periodic domain)
  int dbl;       // FP64 (else FP32)
  int internal;  // not a leaf: the FAS right-hand side is formed
  int top;       // the finest grid of the solve: no FAS, no error
  double vol;    // cell volume (restriction weights)
  MgCoef coef;
  MgSweep sw[3];
  StoreView<double> v64;
  StoreView<float> v32;
  FaceD<double> fd64;
  FaceD<float> fd32;
  MgXfer up;  // this block and its parent in the next entry (unused for the last)
};
struct TailArgs {
  int n, stages, coarse_sweeps, pad;
  MgOp o;
  TailGrid g[kTailMax];
};

template <class T>
__device__ __forceinline__ const StoreView<T> &tview(const TailGrid &g) {
  if constexpr (sizeof(T) == 8) return g.v64;
  else return g.v32;
}
template <class T>
__device__ __forceinline__ const FaceD<T> &tfd(const TailGrid &g) {
  if constexpr (sizeof(T) == 8) return g.fd64;
  else return g.fd32;
}

// every interior cell of one block, the whole CTA
template <class F>
__device__ __forceinline__ void for_block(const Dims &d, F &&f) {
  const CellSplit sp(d.nx[0], d.nx[1], d.nx[2]);
  for (int e = threadIdx.x; e < sp.per; e += blockDim.x) {
    int q, k, j, i;
    sp(e, q, k, j, i);
    f(k + d.ng, j + d.ng, i + d.ng);
  }
}

template <class T>
__device__ void tail_smooth(const TailArgs &a, const TailGrid &g, int stages) {
  const StoreView<T> &v = tview<T>(g);
  T *src = v.u, *dst = v.temp;
  for (int st = 0; st < stages; ++st) {
    for_block(v.d, [&](int k, int j, int i) {
      jacobi_cell<true>(src, v.rhs, dst, v.d, g.nb, g.coef, a.o, g.sw[st], tfd<T>(g), g.slot, k, j, i);
    });
    __syncthreads();
    T *tmp = src;
    src = dst;
    dst = tmp;
  }
  if (src != v.u) {
    for_block(v.d, [&](int k, int j, int i) {
      const int64_t c = cell_of(v.d, g.slot, k, j, i);
      v.u[c] = v.temp[c];
    });
    __syncthreads();
  }
}

// The coarsest grid's extra sweeps (coarse_sweeps x stages passes) when it is one block
// that tiles the periodic domain (its own face neighbour on all six sides) of at most
// kTailSmemCells cells: the block's values and right-hand side sit in shared memory for
// all the passes, so a pass costs a CTA barrier instead of a round trip to L2. Each
// cell's value is the same expression (jacobi_value) as in tail_smooth; u ends with the
// last pass's values, as there.
constexpr int kTailSmemCells = 512;
__shared__ double tail_sweep_smem[3 * kTailSmemCells];  // two sweep buffers and the rhs
template <class T>
__device__ bool tail_smem_fits(const TailGrid &g) {
  const Dims &d = tview<T>(g).d;
  for (int q = 0; q < 6; ++q)
    if (g.nb[q] != g.slot) return false;
  return d.nx[0] * d.nx[1] * d.nx[2] <= kTailSmemCells;
}
template <class T>
__device__ void tail_coarse_sweeps_smem(const TailArgs &a, const TailGrid &g, double *smem) {
  const StoreView<T> &v = tview<T>(g);
  const Dims &d = v.d;
  const int n0 = d.nx[0], n1 = d.nx[1], n2 = d.nx[2], per = n0 * n1 * n2, ng = d.ng;
  T *s0 = reinterpret_cast<T *>(smem), *s1 = s0 + kTailSmemCells, *sr = s1 + kTailSmemCells;
  for (int e = threadIdx.x; e < per; e += blockDim.x) {
    const int i = e % n0, j = (e / n0) % n1, k = e / (n0 * n1);
    const int64_t c = cell_of(d, g.slot, k + ng, j + ng, i + ng);
    s0[e] = v.u[c];
    sr[e] = v.rhs[c];
  }
  __syncthreads();
  T *cur = s0, *nxt = s1;
  for (int c = 0; c < a.coarse_sweeps; ++c)
    for (int st = 0; st < a.stages; ++st) {
      for (int e = threadIdx.x; e < per; e += blockDim.x) {
        const int i = e % n0, j = (e / n0) % n1, k = e / (n0 * n1);
        const int im = i > 0 ? i - 1 : n0 - 1, ip = i < n0 - 1 ? i + 1 : 0;
        const int jm = j > 0 ? j - 1 : n1 - 1, jp = j < n1 - 1 ? j + 1 : 0;
        const int km = k > 0 ? k - 1 : n2 - 1, kp = k < n2 - 1 ? k + 1 : 0;
        Faces<T> f;
        f.c = cur[e];
        f.xm = cur[(k * n1 + j) * n0 + im];
        f.xp = cur[(k * n1 + j) * n0 + ip];
        f.ym = cur[(k * n1 + jm) * n0 + i];
        f.yp = cur[(k * n1 + jp) * n0 + i];
        f.zm = cur[(km * n1 + j) * n0 + i];
        f.zp = cur[(kp * n1 + j) * n0 + i];
        nxt[e] = jacobi_value<true>(f, sr[e], d, g.coef, a.o, g.sw[st], tfd<T>(g),
                                    cell_of(d, g.slot, k + ng, j + ng, i + ng));
      }
      __syncthreads();
      T *tmp = cur;
      cur = nxt;
      nxt = tmp;
    }
  for (int e = threadIdx.x; e < per; e += blockDim.x) {
    const int i = e % n0, j = (e / n0) % n1, k = e / (n0 * n1);
    v.u[cell_of(d, g.slot, k + ng, j + ng, i + ng)] = cur[e];
  }
  __syncthreads();
}

template <class T>
__device__ void tail_error(const TailGrid &g) {
  const StoreView<T> &v = tview<T>(g);
  for_block(v.d, [&](int k, int j, int i) {
    const int64_t c = cell_of(v.d, g.slot, k, j, i);
    v.res[c] = v.u[c] - v.u0[c];
  });
  __syncthreads();
}

template <class T, class TP>
__device__ void tail_down(const TailArgs &a, int t) {
  const TailGrid &g = a.g[t];
  const StoreView<T> &v = tview<T>(g);
  for_block(v.d, [&](int k, int j, int i) {
    if (g.top) {
      const int64_t c = cell_of(v.d, g.slot, k, j, i);
      v.u0[c] = v.u[c];
    } else {
      fas_cell<true>(v, g.internal != 0, g.nb, g.coef, a.o, tfd<T>(g), g.slot, k, j, i);
    }
  });
  __syncthreads();
  tail_smooth<T>(a, g, a.stages);
  if (t < a.n - 1) {
    for_block(v.d, [&](int k, int j, int i) { residual_cell<true>(v, g.nb, g.coef, a.o, tfd<T>(g), g.slot, k, j, i); });
    __syncthreads();
    const int h0 = max(1, v.d.nx[0] / 2), h1 = max(1, v.d.nx[1] / 2), h2 = max(1, v.d.nx[2] / 2);
    for (int e = threadIdx.x; e < h0 * h1 * h2; e += blockDim.x)
      restrict_cell(v, tview<TP>(a.g[t + 1]), g.up, g.vol, e % h0, (e / h0) % h1, e / (h0 * h1));
    __syncthreads();
  } else {
    if (a.coarse_sweeps > 0 && tail_smem_fits<T>(g)) {
      tail_coarse_sweeps_smem<T>(a, g, tail_sweep_smem);
    } else {
      for (int c = 0; c < a.coarse_sweeps; ++c) tail_smooth<T>(a, g, a.stages);
    }
    // res = u (the coarsest level's post-smooth copy), then res = u - u0 below the top
    for_block(v.d, [&](int k, int j, int i) {
      const int64_t c = cell_of(v.d, g.slot, k, j, i);
      v.res[c] = g.top ? v.u[c] : v.u[c] - v.u0[c];
    });
    __syncthreads();
  }
}

template <class T, class TP>
__device__ void tail_up(const TailArgs &a, int t) {
  const TailGrid &g = a.g[t];
  const StoreView<T> &v = tview<T>(g);
  const int h0 = max(1, v.d.nx[0] / 2), h1 = max(1, v.d.nx[1] / 2), h2 = max(1, v.d.nx[2] / 2);
  for (int e = threadIdx.x; e < h0 * h1 * h2; e += blockDim.x)
    prolong_add_cell<true>(v, tview<TP>(a.g[t + 1]), g.up, nullptr, e % h0, (e / h0) % h1, e / (h0 * h1));
  __syncthreads();
  tail_smooth<T>(a, g, a.stages);
  if (!g.top) tail_error<T>(g);
}

__global__ void __launch_bounds__(kTailThreads) k_mg_tail(TailArgs args) {
  pdl_enter();
  __shared__ TailArgs a;
  {
    const int *src = reinterpret_cast<const int *>(&args);
    int *dst = reinterpret_cast<int *>(&a);
    for (int w = threadIdx.x; w < (int)(sizeof(TailArgs) / sizeof(int)); w += blockDim.x) dst[w] = src[w];
  }
  __syncthreads();
  // a grid in FP64 has FP64 grids below it (only the coarsest runs in FP64 in the mixed
  // solve), so the type pairs are (double, double), (float, double), (float, float)
  for (int t = 0; t < a.n; ++t) {
    const bool d = a.g[t].dbl, dp = t + 1 < a.n ? a.g[t + 1].dbl : d;
    if (d) tail_down<double, double>(a, t);
    else if (dp) tail_down<float, double>(a, t);
    else tail_down<float, float>(a, t);
  }
  for (int t = a.n - 2; t >= 0; --t) {
    const bool d = a.g[t].dbl, dp = a.g[t + 1].dbl;
    if (d) tail_up<double, double>(a, t);
    else if (dp) tail_up<float, double>(a, t);
    else tail_up<float, float>(a, t);
  }
}

// Leaf-grid residual of MGSolver::AddTasks (mg_solver.hpp:135-158): res = rhs - A u
// over every leaf interior (operator constants per leaf, levels differ) and one partial
// sum of r^2 per CTA (fixed tree order, so the host's fixed-order total is reproducible).
// Mixed solve: also the FP32 right-hand side of the next V-cycle (rhs32 = r) and its
// zero initial guess (u32 = 0) on the leaves.
constexpr int kResThreads = 256;
template <bool kFast>
__global__ void __launch_bounds__(kResThreads) k_mg_leaf_residual(StoreView<double> s, int nleaf,
                                                                  const MgCoef *__restrict__ lc, MgOp o,
                                                                  FaceD<double> fd, double *__restrict__ partial,
                                                                  float *__restrict__ rhs32, float *__restrict__ u32) {
  pdl_enter();
  __shared__ double sh[kResThreads / 32];
  const int64_t sj = s.d.N[0], sk = (int64_t)s.d.N[0] * s.d.N[1];
  double acc = 0.0;
  for_interior(nullptr, nleaf, s.d, [&](int, int b, int k, int j, int i) {
    const int64_t c = cell_of(s.d, b, k, j, i);
    const MgCoef &cf = lc[b];
    const Faces<double> f = faces<double>(s.u, s.d, nullptr, b, k, j, i);
    double r;
    if constexpr (kFast) {
      double off, dg;
      fast_op(f, cf, o, fd, c, sj, sk, off, dg);
      r = fma(-dg, f.c, s.rhs[c] - off);
    } else {
      r = s.rhs[c] - exact_op(f, cf, o, fd, c, sj, sk).ax;
    }
    s.res[c] = r;
    acc += r * r;
    if (rhs32) {
      rhs32[c] = (float)r;
      u32[c] = 0.0f;
    }
  });
  // warp-shuffle tree within each warp, then the warps' sums in order (fixed order)
  for (int w = 16; w > 0; w >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, w);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < kResThreads / 32; ++w) t += sh[w];
    partial[blockIdx.x] = t;
  }
}

// Iterative refinement: u += e on the leaf interiors (e the FP32 V-cycle's result)
__global__ void __launch_bounds__(256) k_mg_correct(double *__restrict__ u, const float *__restrict__ e, int nleaf,
                                                    Dims d) {
  pdl_enter();
  for_interior(nullptr, nleaf, d, [&](int, int b, int k, int j, int i) {
    const int64_t c = cell_of(d, b, k, j, i);
    u[c] = u[c] + (double)e[c];
  });
}

// ---- BiCGSTAB on the leaf grid (bicgstab_solver.hpp:116-315). Vectors live in the leaf
// layout; every kernel touches the leaf interiors only. Scalars stay on the device:
// ks[0] (rhat0, r), ks[1] its previous value, ks[2] (rhat0, v), ks[3] (t, s), ks[4] (t, t),
// ks[5] (r, r), ks[6] (rhs, rhs).
enum { kRr = 0, kRrOld, kRv, kTs, kTt, kRes, kRhs2, kNumScalars };

// partial sums of a.b (and c.e when c is not null) per CTA, in a fixed order
__global__ void __launch_bounds__(kResThreads) k_bi_dot2(const double *__restrict__ a, const double *__restrict__ b,
                                                         const double *__restrict__ c, const double *__restrict__ e,
                                                         int nleaf, Dims d, double *__restrict__ part) {
  pdl_enter();
  __shared__ double sh[2][kResThreads / 32];
  double s0 = 0.0, s1 = 0.0;
  for_interior(nullptr, nleaf, d, [&](int, int blk, int k, int j, int i) {
    const int64_t q = cell_of(d, blk, k, j, i);
    s0 = fma(a[q], b[q], s0);
    if (c) s1 = fma(c[q], e[q], s1);
  });
  for (int w = 16; w > 0; w >>= 1) {
    s0 += __shfl_down_sync(0xffffffffu, s0, w);
    s1 += __shfl_down_sync(0xffffffffu, s1, w);
  }
  if ((threadIdx.x & 31) == 0) {
    sh[0][threadIdx.x >> 5] = s0;
    sh[1][threadIdx.x >> 5] = s1;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double t0 = 0.0, t1 = 0.0;
    for (int w = 0; w < kResThreads / 32; ++w) {
      t0 += sh[0][w];
      t1 += sh[1][w];
    }
    part[blockIdx.x] = t0;
    part[gridDim.x + blockIdx.x] = t1;
  }
}

// the partial sums of k_bi_dot2 (np per dot) into ks[i0] and ks[i1] (i1 < 0: one dot);
// one CTA, fixed order
__global__ void __launch_bounds__(256) k_bi_final(const double *__restrict__ part, int np, double *__restrict__ ks,
                                                  int i0, int i1) {
  pdl_enter();
  __shared__ double sh[2][8];
  double s0 = 0.0, s1 = 0.0;
  for (int q = threadIdx.x; q < np; q += blockDim.x) {
    s0 += part[q];
    s1 += part[np + q];
  }
  for (int w = 16; w > 0; w >>= 1) {
    s0 += __shfl_down_sync(0xffffffffu, s0, w);
    s1 += __shfl_down_sync(0xffffffffu, s1, w);
  }
  if ((threadIdx.x & 31) == 0) {
    sh[0][threadIdx.x >> 5] = s0;
    sh[1][threadIdx.x >> 5] = s1;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double t0 = 0.0, t1 = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
      t0 += sh[0][w];
      t1 += sh[1][w];
    }
    ks[i0] = t0;
    if (i1 >= 0) ks[i1] = t1;
  }
}

// x = 0; r = rhat0 = p = rhs
__global__ void __launch_bounds__(256) k_bi_init(const double *__restrict__ rhs, double *__restrict__ x,
                                                 double *__restrict__ r, double *__restrict__ rhat0,
                                                 double *__restrict__ p, int nleaf, Dims d) {
  pdl_enter();
  for_interior(nullptr, nleaf, d, [&](int, int b, int k, int j, int i) {
    const int64_t q = cell_of(d, b, k, j, i);
    const double v = rhs[q];
    x[q] = 0.0;
    r[q] = v;
    rhat0[q] = v;
    p[q] = v;
  });
}

__global__ void k_bi_begin(double *__restrict__ ks) {
  pdl_enter();
  ks[kRrOld] = ks[kRr];
}

// the preconditioner's input: rhs <- src and u <- 0 on the leaves (FP64 or FP32 copies),
// or, without a preconditioner, u <- src
template <class T>
__global__ void __launch_bounds__(256) k_bi_in(const double *__restrict__ src, T *__restrict__ rhs,
                                               T *__restrict__ u, int nleaf, Dims d) {
  pdl_enter();
  for_interior(nullptr, nleaf, d, [&](int, int b, int k, int j, int i) {
    const int64_t q = cell_of(d, b, k, j, i);
    if (rhs) {
      rhs[q] = (T)src[q];
      u[q] = (T)0;
    } else {
      u[q] = (T)src[q];
    }
  });
}

// the FP32 preconditioner's output into the FP64 u
__global__ void __launch_bounds__(256) k_bi_out32(const float *__restrict__ e, double *__restrict__ u, int nleaf,
                                                  Dims d) {
  pdl_enter();
  for_interior(nullptr, nleaf, d, [&](int, int b, int k, int j, int i) {
    const int64_t q = cell_of(d, b, k, j, i);
    u[q] = (double)e[q];
  });
}

// out = A u on the leaves (u's ghosts exchanged before)
__global__ void __launch_bounds__(256) k_bi_apply(const double *__restrict__ u, double *__restrict__ out, int nleaf,
                                                  Dims d, const MgCoef *__restrict__ lc, MgOp o, FaceD<double> fd) {
  pdl_enter();
  const int64_t sj = d.N[0], sk = (int64_t)d.N[0] * d.N[1];
  for_interior(nullptr, nleaf, d, [&](int, int b, int k, int j, int i) {
    const int64_t q = cell_of(d, b, k, j, i);
    const MgCoef &cf = lc[b];
    const Faces<double> f = faces<double>(u, d, nullptr, b, k, j, i);
    double off, dg;
    fast_op(f, cf, o, fd, q, sj, sk, off, dg);
    out[q] = fma(dg, f.c, off);
  });
}

// Setup restriction of the face coefficient (AddSetupTasks, mg_solver.hpp:188-203, 347-370,
// of the GMGRestrict field D): RestrictAverage on the faces of direction dir, the
// area-weighted mean of the 2x2 fine faces in the face's plane in the reference's
// pairing order, into the parent's octant. One thread per parent face.
__global__ void __launch_bounds__(256) k_mg_restrict_faces(const double *__restrict__ cd, Dims cdims,
                                                           double *__restrict__ pd, Dims pdims,
                                                           const MgXfer *__restrict__ x, int n,
                                                           const DevBlockGeom *__restrict__ cgeom, int dir) {
  const int e0 = max(1, cdims.nx[0] / 2) + (dir == 0), e1 = max(1, cdims.nx[1] / 2) + (dir == 1);
  const int e2 = max(1, cdims.nx[2] / 2) + (dir == 2);
  const int per = e0 * e1 * e2, total = per * n;
  const int ng = cdims.ng;
  const int64_t sj = cdims.N[0], sk = (int64_t)cdims.N[0] * cdims.N[1];
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < total; e += gridDim.x * blockDim.x) {
    const int q = e / per;
    const int r = e - q * per;
    const int ci = r % e0, cj = (r / e0) % e1, ck = r / (e0 * e1);
    const MgXfer t = x[q];
    const double a = cgeom[t.child].area[dir];
    const int64_t f = cell_of(cdims, t.child, 2 * ck + ng, 2 * cj + ng, 2 * ci + ng);
    double v[2][2][2] = {}, tt[2][2][2] = {};
#pragma unroll
    for (int ok = 0; ok < 2; ++ok)
#pragma unroll
      for (int oj = 0; oj < 2; ++oj)
#pragma unroll
        for (int oi = 0; oi < 2; ++oi) {
          if ((dir == 2 && ok) || (dir == 1 && oj) || (dir == 0 && oi)) continue;
          v[ok][oj][oi] = a;
          tt[ok][oj][oi] = a * cd[f + ok * sk + oj * sj + oi];
        }
    const double tv = ((v[0][0][0] + v[0][1][0]) + (v[0][0][1] + v[0][1][1])) +
                      ((v[1][0][0] + v[1][1][0]) + (v[1][0][1] + v[1][1][1]));
    const double num = ((tt[0][0][0] + tt[0][1][0]) + (tt[0][0][1] + tt[0][1][1])) +
                       ((tt[1][0][0] + tt[1][1][0]) + (tt[1][0][1] + tt[1][1][1]));
    pd[cell_of(pdims, t.parent, t.lo[2] + ck, t.lo[1] + cj, t.lo[0] + ci)] = div_rn(num, tv);
  }
}

__global__ void __launch_bounds__(256) k_to_f32(const double *__restrict__ a, float *__restrict__ b, int64_t n) {
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x)
    b[q] = (float)a[q];
}

// alpha = (rhat0, r)_old / (rhat0, v); h = x + alpha u; s = r - alpha v
__global__ void __launch_bounds__(256) k_bi_hs(const double *__restrict__ x, const double *__restrict__ u,
                                               const double *__restrict__ r, const double *__restrict__ v,
                                               double *__restrict__ h, double *__restrict__ s,
                                               const double *__restrict__ ks, int nleaf, Dims d) {
  pdl_enter();
  const double alpha = ks[kRrOld] / ks[kRv];
  for_interior(nullptr, nleaf, d, [&](int, int b, int k, int j, int i) {
    const int64_t q = cell_of(d, b, k, j, i);
    h[q] = fma(alpha, u[q], x[q]);
    s[q] = fma(-alpha, v[q], r[q]);
  });
}

// omega = (t, s) / (t, t); x = h + omega u; r = s - omega t; partial sums of (r, r) and
// (rhat0, r)
__global__ void __launch_bounds__(kResThreads) k_bi_xr(const double *__restrict__ h, const double *__restrict__ u,
                                                       const double *__restrict__ s, const double *__restrict__ t,
                                                       const double *__restrict__ rhat0, double *__restrict__ x,
                                                       double *__restrict__ r, const double *__restrict__ ks,
                                                       int nleaf, Dims d, double *__restrict__ part) {
  pdl_enter();
  __shared__ double sh[2][kResThreads / 32];
  const double omega = ks[kTs] / ks[kTt];
  double s0 = 0.0, s1 = 0.0;
  for_interior(nullptr, nleaf, d, [&](int, int b, int k, int j, int i) {
    const int64_t q = cell_of(d, b, k, j, i);
    x[q] = fma(omega, u[q], h[q]);
    const double rq = fma(-omega, t[q], s[q]);
    r[q] = rq;
    s0 = fma(rq, rq, s0);
    s1 = fma(rhat0[q], rq, s1);
  });
  for (int w = 16; w > 0; w >>= 1) {
    s0 += __shfl_down_sync(0xffffffffu, s0, w);
    s1 += __shfl_down_sync(0xffffffffu, s1, w);
  }
  if ((threadIdx.x & 31) == 0) {
    sh[0][threadIdx.x >> 5] = s0;
    sh[1][threadIdx.x >> 5] = s1;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double t0 = 0.0, t1 = 0.0;
    for (int w = 0; w < kResThreads / 32; ++w) {
      t0 += sh[0][w];
      t1 += sh[1][w];
    }
    part[blockIdx.x] = t0;
    part[gridDim.x + blockIdx.x] = t1;
  }
}

// beta = (rhat0, r) / (rhat0, r)_old * alpha / omega; p = r + beta (p - omega v)
__global__ void __launch_bounds__(256) k_bi_p(const double *__restrict__ r, const double *__restrict__ v,
                                              double *__restrict__ p, const double *__restrict__ ks, int nleaf,
                                              Dims d) {
  pdl_enter();
  const double alpha = ks[kRrOld] / ks[kRv];
  const double omega = ks[kTs] / ks[kTt];
  const double beta = ks[kRr] / ks[kRrOld] * alpha / omega;
  for_interior(nullptr, nleaf, d, [&](int, int b, int k, int j, int i) {
    const int64_t q = cell_of(d, b, k, j, i);
    p[q] = fma(beta, fma(-omega, v[q], p[q]), r[q]);
  });
}

// ---- flux correction inside Ax on the leaf grid (poisson/flux_correct,
// poisson_equation.hpp:41-58): CalculateFluxes (each cell its low faces, the last cell of
// a row also its high face; fluxes [block][dir][N3][N2][N1], face i the low face of cell
// i), the flux-correction exchange (exchange.cu), then FluxMultiplyMatrix. The reference's
// order and divisions, in both builds.
__global__ void __launch_bounds__(256) k_mg_leaf_fluxes(const double *__restrict__ u, double *__restrict__ F,
                                                        int nleaf, Dims d, const MgCoef *__restrict__ lc, MgOp o,
                                                        FaceD<double> fd) {
  pdl_enter();
  const int64_t sj = d.N[0], sk = (int64_t)d.N[0] * d.N[1], cs = sk * d.N[2];
  const int hi0 = d.ng + d.nx[0] - 1, hi1 = d.ng + d.nx[1] - 1, hi2 = d.ng + d.nx[2] - 1;
  for_interior(nullptr, nleaf, d, [&](int, int b, int k, int j, int i) {
    const int64_t c = cell_of(d, b, k, j, i);
    const int64_t cf0 = ((int64_t)b * 3) * cs + (c - (int64_t)b * cs);
    double D6[6];
    face_d6(fd, c, sj, sk, o.D, D6);
    const double *dx = lc[b].dx;
    const double uc = u[c];
    F[cf0] = div_rn(D6[0], dx[0]) * (u[c - 1] - uc);
    if (i == hi0) F[cf0 + 1] = div_rn(D6[1], dx[0]) * (uc - u[c + 1]);
    F[cf0 + cs] = div_rn(D6[2] * (u[c - sj] - uc), dx[1]);
    if (j == hi1) F[cf0 + cs + sj] = div_rn(D6[3] * (uc - u[c + sj]), dx[1]);
    F[cf0 + 2 * cs] = div_rn(D6[4] * (u[c - sk] - uc), dx[2]);
    if (k == hi2) F[cf0 + 2 * cs + sk] = div_rn(D6[5] * (uc - u[c + sk]), dx[2]);
  });
}

// FluxMultiplyMatrix: A u = -alpha u + sum_d (F_low - F_high) / dx_d
__device__ __forceinline__ double flux_div(const double *__restrict__ F, const double *__restrict__ u, int64_t c,
                                          int b, const Dims &d, const double *dx, double alpha) {
  const int64_t sj = d.N[0], sk = (int64_t)d.N[0] * d.N[1], cs = sk * d.N[2];
  const int64_t f = ((int64_t)b * 3) * cs + (c - (int64_t)b * cs);
  double out = -alpha * u[c];
  out += div_rn(F[f] - F[f + 1], dx[0]);
  out += div_rn(F[f + cs] - F[f + cs + sj], dx[1]);
  out += div_rn(F[f + 2 * cs] - F[f + 2 * cs + sk], dx[2]);
  return out;
}

// the leaf residual (as k_mg_leaf_residual) from the corrected fluxes
__global__ void __launch_bounds__(kResThreads) k_mg_leaf_residual_flux(StoreView<double> s, int nleaf,
                                                                       const MgCoef *__restrict__ lc, MgOp o,
                                                                       const double *__restrict__ F,
                                                                       double *__restrict__ partial,
                                                                       float *__restrict__ rhs32,
                                                                       float *__restrict__ u32) {
  pdl_enter();
  __shared__ double sh[kResThreads / 32];
  double acc = 0.0;
  for_interior(nullptr, nleaf, s.d, [&](int, int b, int k, int j, int i) {
    const int64_t c = cell_of(s.d, b, k, j, i);
    const double r = s.rhs[c] - flux_div(F, s.u, c, b, s.d, lc[b].dx, o.alpha);
    s.res[c] = r;
    acc += r * r;
    if (rhs32) {
      rhs32[c] = (float)r;
      u32[c] = 0.0f;
    }
  });
  for (int w = 16; w > 0; w >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, w);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < kResThreads / 32; ++w) t += sh[w];
    partial[blockIdx.x] = t;
  }
}

// BiCGSTAB's A u from the corrected fluxes
__global__ void __launch_bounds__(256) k_bi_apply_flux(const double *__restrict__ u, double *__restrict__ out,
                                                       int nleaf, Dims d, const MgCoef *__restrict__ lc, MgOp o,
                                                       const double *__restrict__ F) {
  pdl_enter();
  for_interior(nullptr, nleaf, d, [&](int, int b, int k, int j, int i) {
    const int64_t c = cell_of(d, b, k, j, i);
    out[c] = flux_div(F, u, c, b, d, lc[b].dx, o.alpha);
  });
}

unsigned grid_for(int64_t work) {
  return (unsigned)std::max<int64_t>(1, std::min<int64_t>((work + 255) / 256, 152 * 16));
}

}  // namespace

// ---------------------------------------------------------------------------- handle
struct pgb_mg {
  pgb_mesh *mesh = nullptr;
  MeshTopology *topo = nullptr;
  GmgConfig cfg;
  bool exact = true;  // reference-order arithmetic (bitwise) or the FMA 7-point build
  bool flux_correct = false;   // poisson/flux_correct on the leaf grid
  double *lflux = nullptr;     // leaf face fluxes [nleaf][3][N3][N2][N1] (flux_correct)
  int max_coarsenings = 30;
  int lmin = 0, lmax = 0, nleaf = 0;
  struct Store {
    int nslots = 0;
    std::vector<BlockInfo> blocks;
    double *u = nullptr, *res = nullptr, *rhs = nullptr, *temp = nullptr, *u0 = nullptr, *coarse = nullptr;
    // the FP32 copies of the mixed solve (allocated on its first use)
    float *u32 = nullptr, *res32 = nullptr, *rhs32 = nullptr, *temp32 = nullptr, *u032 = nullptr,
          *coarse32 = nullptr;
    // face coefficient D per slot (pgb_mg_set_coefficient), FP64 and FP32
    double *d[3] = {nullptr, nullptr, nullptr};
    float *d32[3] = {nullptr, nullptr, nullptr};
    template <class T>
    FaceD<T> fd() const {
      if constexpr (sizeof(T) == 8) return FaceD<T>{d[0], d[1], d[2]};
      else return FaceD<T>{d32[0], d32[1], d32[2]};
    }
    Dims dims{};
    template <class T>
    StoreView<T> view() const {
      if constexpr (sizeof(T) == 8) return StoreView<T>{u, res, rhs, temp, u0, dims};
      else return StoreView<T>{u32, res32, rhs32, temp32, u032, dims};
    }
  };
  std::map<int, Store> stores;  // key 0: full-size blocks; key L < 0: the blocks of level L
  struct Grid {
    int level = 0, store = 0;
    GridTopology remap;  // the composite grid's exchange boxes over store slots
    GridTables tab;
    std::vector<int> fine_h;    // slots of the level-L blocks, internal blocks first
    std::vector<int> coarse_h;  // slots of the leaves of level L-1
    int nint = 0;               // internal blocks at the head of fine_h
    std::vector<MgXfer> xfer_h; // fine blocks and their parents (grids above the coarsest)
    MgCoef coef{};              // operator constants of the fine blocks
    bool halofree = false;      // one level: stencils read the face neighbours directly
    std::vector<int> nbr_h;     // 6 face-neighbour slots per entry of fine_h (halofree)
    int *fine = nullptr, *coarse = nullptr, *nbr = nullptr;
    MgXfer *xfer = nullptr;
    const int *nb() const { return halofree ? nbr : nullptr; }
  };
  std::map<int, Grid> grids;
  GridTables leaf_tab;
  std::vector<MgCoef> leaf_coef_h;  // per leaf block (levels differ)
  MgCoef *leaf_coef = nullptr;
  void *lists = nullptr;
  double *partial = nullptr, *partial_h = nullptr;
  int nparts = 0;
  // BiCGSTAB (allocated on first use): leaf-layout vectors x r rhat0 p v h s t, device
  // scalars, dot-product partials, pinned copies of (r, r) and (rhs, rhs)
  double *kv[8] = {};
  double *ks = nullptr, *kpart = nullptr, *kres_h = nullptr;
  cudaGraphExec_t kgraph[3] = {nullptr, nullptr, nullptr};  // per preconditioner
  bool uploaded = false, uploaded32 = false;
  cudaGraphExec_t graph[2] = {nullptr, nullptr};  // FP64 and mixed iterations
  std::vector<void *> allocs;

  static int key(int level) { return level >= 0 ? 0 : level; }
  Store &store_of(int level) { return stores.at(key(level)); }

  ~pgb_mg() {
    for (auto &gr : graph)
      if (gr) cudaGraphExecDestroy(gr);
    for (auto &gr : kgraph)
      if (gr) cudaGraphExecDestroy(gr);
    if (kres_h) cudaFreeHost(kres_h);
    for (auto &kv : grids) kv.second.tab.release();
    leaf_tab.release();
    for (void *p : allocs) cudaFree(p);
    if (lists) cudaFree(lists);
    if (partial_h) cudaFreeHost(partial_h);
  }
};

namespace {

// A zeroed device array of n elements, owned by g (recorded before anything can fail,
// so that pgb_mg_destroy frees it whatever happens after).
template <class T>
int dev_zeros(pgb_mg *g, T **p, int64_t n) {
  PGB_CUDA(cudaMalloc((void **)p, (size_t)n * sizeof(T)));
  g->allocs.push_back(*p);
  PGB_CUDA(cudaMemset(*p, 0, (size_t)n * sizeof(T)));
  return kOk;
}

// Operator constants for spacing dx, in the order of poisson_equation.hpp:59-102 and
// utils/robust.hpp (the exact build's values are bitwise those formed per cell there)
MgCoef make_coef(const double *dx, const GmgConfig &c) {
  MgCoef o;
  const double D = c.D;
  for (int d = 0; d < 3; ++d) {
    o.dx[d] = dx[d];
    o.c[d] = D / (dx[d] * dx[d]);
    o.ic[d] = 1.0 / (dx[d] * dx[d]);
  }
  double dg = -(D + D) / (dx[0] * dx[0]) - c.alpha;
  dg -= (D + D) / (dx[1] * dx[1]);
  dg -= (D + D) / (dx[2] * dx[2]);
  o.dg = dg;
  o.den = dg + (dg >= 0 ? 1.0 : -1.0) * (10 * DBL_MIN);
  return o;
}

// Composite grids, store slots and transfer records (host only).
int mg_build(pgb_mg *g) {
  MeshTopology &topo = *g->topo;
  const MeshSpec &spec = topo.spec();
  const int ng = spec.ng;
  topo.build_multigrid();
  g->lmax = topo.max_level();
  g->lmin = std::max(g->lmax - g->max_coarsenings, topo.mg_min_level());
  const auto &leaves = topo.leaf().blocks;
  g->nleaf = (int)leaves.size();
  const auto &mg = topo.mg_grids();
  // store 0: leaves (slot = leaf index = gid), then internal blocks of levels >= 0 by gid
  std::map<int, int> slot0;
  pgb_mg::Store &s0 = g->stores[0];
  for (int b = 0; b < g->nleaf; ++b) {
    slot0[leaves[b].gid] = b;
    s0.blocks.push_back(leaves[b]);
  }
  std::map<int, const BlockInfo *> internal0;
  for (int L = std::max(g->lmin, 0); L <= g->lmax; ++L)
    for (auto &b : mg.at(L).blocks)
      if (!slot0.count(b.gid)) internal0[b.gid] = &b;
  for (auto &kv : internal0) {
    slot0[kv.first] = (int)s0.blocks.size();
    s0.blocks.push_back(*kv.second);
  }
  for (auto &b : s0.blocks) {
    b.nbrs.clear();
    b.same_nbrs.clear();
  }
  for (int L = g->lmin; L <= g->lmax; ++L) {
    const GridTopology &src = mg.at(L);
    if (src.blocks.empty()) return fail(kErrInvalid, "empty multigrid level");
    for (auto &b : src.blocks)
      if (b.loc.level != L && (L == g->lmin || b.loc.level != L - 1))
        return fail(kErrUnsupported, "the coarsest multigrid grid holds leaves of a coarser level "
                                     "(max_coarsenings must reach the root grid)");
    pgb_mg::Grid &G = g->grids[L];
    G.level = L;
    G.store = pgb_mg::key(L);
    std::vector<int> slot(src.blocks.size());
    if (L >= 0) {
      for (size_t i = 0; i < src.blocks.size(); ++i) slot[i] = slot0.at(src.blocks[i].gid);
    } else {
      pgb_mg::Store &sl = g->stores[L];
      for (size_t i = 0; i < src.blocks.size(); ++i) {
        slot[i] = (int)i;
        sl.blocks.push_back(src.blocks[i]);
        sl.blocks.back().same_nbrs.clear();
      }
    }
    G.remap.logical_level = L;
    G.remap.multilevel = src.multilevel;
    G.remap.pairs = src.pairs;
    for (auto &p : G.remap.pairs) {
      p.sender = slot[p.sender];
      p.receiver = slot[p.receiver];
    }
    auto remap_regions = [&](const std::vector<CoarseRegion> &in, std::vector<CoarseRegion> &out) {
      out = in;
      for (auto &r : out) r.block = slot[r.block];
    };
    remap_regions(src.restrict_send, G.remap.restrict_send);
    remap_regions(src.restrict_recv, G.remap.restrict_recv);
    remap_regions(src.prolong, G.remap.prolong);
    std::vector<int> fine_idx, leaf_idx;  // block indices, internal blocks first
    const BlockInfo *fb = nullptr;
    for (size_t i = 0; i < src.blocks.size(); ++i) {
      const BlockInfo &b = src.blocks[i];
      if (b.loc.level != L) {
        G.coarse_h.push_back(slot[i]);
        continue;
      }
      if (fb && (b.dx[0] != fb->dx[0] || b.dx[1] != fb->dx[1] || b.dx[2] != fb->dx[2]))
        return fail(kErrUnsupported, "blocks of one level with different spacings");
      fb = &b;
      (topo.is_leaf(b.loc) ? leaf_idx : fine_idx).push_back((int)i);
    }
    G.nint = (int)fine_idx.size();
    fine_idx.insert(fine_idx.end(), leaf_idx.begin(), leaf_idx.end());
    for (int i : fine_idx) G.fine_h.push_back(slot[i]);
    G.coef = make_coef(fb->dx, g->cfg);
    // A grid without coarser leaves is one level tiling the periodic domain (2:1
    // balance leaves no gap), so every face neighbour of a block is a block of the grid
    G.halofree = G.coarse_h.empty();
    if (G.halofree) {
      std::unordered_map<int, int> pos;
      for (size_t i = 0; i < src.blocks.size(); ++i) pos[src.blocks[i].gid] = (int)i;
      const int64_t n = L >= 0 ? (int64_t)1 << L : 1;
      for (int i : fine_idx) {
        const LLoc &l = src.blocks[i].loc;
        for (int d = 0; d < 3; ++d)
          for (int sgn : {-1, 1}) {
            std::array<int64_t, 3> x = l.lx;
            x[d] = (x[d] + sgn + n) % n;
            const int gid = topo.gid_of(LLoc(L, x[0], x[1], x[2]));
            auto it = pos.find(gid);
            if (gid < 0 || it == pos.end()) return fail(kErrInvalid, "face neighbour outside a one-level grid");
            G.nbr_h.push_back(slot[it->second]);
          }
      }
    }
  }
  for (auto &b : leaves) g->leaf_coef_h.push_back(make_coef(b.dx, g->cfg));
  // transfers between grid L and L - 1, per fine block of grid L
  for (int L = g->lmin + 1; L <= g->lmax; ++L) {
    pgb_mg::Grid &G = g->grids[L];
    const GridTopology &src = mg.at(L), &par = mg.at(L - 1);
    std::map<int, int> pidx;
    for (size_t i = 0; i < par.blocks.size(); ++i) pidx[par.blocks[i].gid] = (int)i;
    for (size_t i = 0; i < src.blocks.size(); ++i) {
      const BlockInfo &c = src.blocks[i];
      if (c.loc.level != L) continue;
      if (c.coarser.empty()) return fail(kErrInvalid, "multigrid block without a parent");
      const Neighbor &up = c.coarser[0];
      const int pi = pidx.at(up.gid);
      const BlockInfo &p = par.blocks[pi];
      const Neighbor *down = nullptr;
      for (auto &n : p.finer)
        if (n.gid == c.gid) down = &n;
      if (!down) return fail(kErrInvalid, "parent does not list its child");
      // gmg_restrict: child's coarse interior -> parent's octant; gmg_prolongate: the
      // octant with ng ghosts -> the child's whole coarse buffer
      const IBox rs = boundary_box(up, c.loc, c.nx, ng, 0, RangeKind::InteriorSend, true, false);
      const IBox tr = boundary_box(*down, p.loc, p.nx, ng, 0, RangeKind::InteriorRecv, false, false);
      const IBox ps = boundary_box(*down, p.loc, p.nx, ng, 0, RangeKind::InteriorSend, false, false);
      const IBox pr = boundary_box(up, c.loc, c.nx, ng, 0, RangeKind::InteriorRecv, false, false);
      for (int d = 0; d < 3; ++d) {
        const int h = std::max(1, c.nx[d] / 2);
        if (rs.lo[d] != ng || rs.hi[d] != ng + h - 1 || tr.hi[d] - tr.lo[d] != h - 1 || ps.lo[d] != tr.lo[d] - ng ||
            ps.hi[d] != tr.hi[d] + ng || pr.lo[d] != 0 || pr.hi[d] != h + 2 * ng - 1)
          return fail(kErrUnsupported, "multigrid transfer ranges of unexpected shape");
      }
      MgXfer x;
      x.child = slot0.count(c.gid) && L >= 0 ? slot0.at(c.gid) : (int)i;
      x.parent = L - 1 >= 0 ? slot0.at(p.gid) : pi;
      for (int d = 0; d < 3; ++d) x.lo[d] = tr.lo[d];
      const pgb_mg::Grid &PG = g->grids.at(L - 1);
      for (int q = 0; q < 6; ++q) x.pnb[q] = -1;
      if (PG.halofree) {
        const auto it = std::find(PG.fine_h.begin(), PG.fine_h.end(), x.parent);
        if (it == PG.fine_h.end()) return fail(kErrInvalid, "parent outside its grid's block list");
        const size_t q0 = 6 * (size_t)(it - PG.fine_h.begin());
        for (int q = 0; q < 6; ++q) x.pnb[q] = PG.nbr_h[q0 + q];
      }
      {
        const auto it = std::find(G.fine_h.begin(), G.fine_h.end(), x.child);
        if (it == G.fine_h.end()) return fail(kErrInvalid, "child outside its grid's block list");
        x.pad = (int32_t)(it - G.fine_h.begin());  // the child's row in the grid's lists
      }
      G.xfer_h.push_back(x);
    }
  }
  for (auto &kv : g->stores) {
    pgb_mg::Store &S = kv.second;
    S.nslots = (int)S.blocks.size();
    for (auto &kv2 : g->grids)
      if (kv2.second.store == kv.first) kv2.second.remap.blocks = S.blocks;
  }
  // every table must keep its accesses inside the store arrays (checked before upload)
  for (auto &kv : g->grids) {
    GridTables scratch;
    int rc = lower_grid(kv.second.remap, spec, scratch, true);
    if (rc) return rc;
  }
  return kOk;
}

int mg_upload(pgb_mg *g) {
  if (g->uploaded) return kOk;
  const MeshSpec &spec = g->topo->spec();
  for (auto &kv : g->grids) {
    int rc = lower_grid(kv.second.remap, spec, kv.second.tab);
    if (rc) return rc;
  }
  int rc = lower_grid(g->topo->leaf(), spec, g->leaf_tab);
  if (rc) return rc;
  for (auto &kv : g->stores) {
    pgb_mg::Store &S = kv.second;
    const pgb_mg::Grid *G = nullptr;
    for (auto &kv2 : g->grids)
      if (kv2.second.store == kv.first) G = &kv2.second;
    S.dims = G->tab.dims;
    const int64_t n = (int64_t)S.nslots * S.dims.N[0] * S.dims.N[1] * S.dims.N[2];
    if (n >= (int64_t)1 << 31) return fail(kErrUnsupported, "multigrid store above 2^31 cells");
    const int64_t nc = (int64_t)S.nslots * S.dims.Nc[0] * S.dims.Nc[1] * S.dims.Nc[2];
    for (double **p : {&S.u, &S.res, &S.rhs, &S.temp, &S.u0}) {
      PGB_TRY(dev_zeros(g, p, n));
    }
    PGB_TRY(dev_zeros(g, &S.coarse, nc));
  }
  // block lists and transfers in one allocation
  size_t bytes = 0;
  auto room = [&](size_t n) {
    const size_t off = bytes;
    bytes = (bytes + n + 255) & ~size_t(255);
    return off;
  };
  struct Off {
    size_t fine, coarse, xfer, nbr;
  };
  std::map<int, Off> off;
  for (auto &kv : g->grids) {
    Off o;
    o.fine = room(kv.second.fine_h.size() * sizeof(int));
    o.coarse = room(kv.second.coarse_h.size() * sizeof(int));
    o.xfer = room(kv.second.xfer_h.size() * sizeof(MgXfer));
    o.nbr = room(kv.second.nbr_h.size() * sizeof(int));
    off[kv.first] = o;
  }
  const size_t lc_off = room(g->leaf_coef_h.size() * sizeof(MgCoef));
  std::vector<char> h(std::max<size_t>(bytes, 256), 0);
  std::memcpy(h.data() + lc_off, g->leaf_coef_h.data(), g->leaf_coef_h.size() * sizeof(MgCoef));
  for (auto &kv : g->grids) {
    const Off &o = off[kv.first];
    auto &G = kv.second;
    std::memcpy(h.data() + o.fine, G.fine_h.data(), G.fine_h.size() * sizeof(int));
    std::memcpy(h.data() + o.coarse, G.coarse_h.data(), G.coarse_h.size() * sizeof(int));
    std::memcpy(h.data() + o.xfer, G.xfer_h.data(), G.xfer_h.size() * sizeof(MgXfer));
    std::memcpy(h.data() + o.nbr, G.nbr_h.data(), G.nbr_h.size() * sizeof(int));
  }
  PGB_CUDA(cudaMalloc(&g->lists, h.size()));
  PGB_CUDA(cudaMemcpy(g->lists, h.data(), h.size(), cudaMemcpyHostToDevice));
  for (auto &kv : g->grids) {
    const Off &o = off[kv.first];
    char *base = static_cast<char *>(g->lists);
    kv.second.fine = reinterpret_cast<int *>(base + o.fine);
    kv.second.coarse = reinterpret_cast<int *>(base + o.coarse);
    kv.second.xfer = reinterpret_cast<MgXfer *>(base + o.xfer);
    kv.second.nbr = reinterpret_cast<int *>(base + o.nbr);
  }
  g->leaf_coef = reinterpret_cast<MgCoef *>(static_cast<char *>(g->lists) + lc_off);
  if (g->flux_correct) {
    const Dims &dl = g->stores.at(0).dims;
    const int64_t nf = (int64_t)g->nleaf * 3 * dl.N[0] * dl.N[1] * dl.N[2];
    PGB_TRY(dev_zeros(g, &g->lflux, nf));
  }
  const Dims &d0 = g->stores.at(0).dims;
  g->nparts = (int)grid_for((int64_t)g->nleaf * d0.nx[0] * d0.nx[1] * d0.nx[2]);
  PGB_TRY(dev_zeros(g, &g->partial, g->nparts));
  PGB_CUDA(cudaMallocHost((void **)&g->partial_h, g->nparts * sizeof(double)));
  g->uploaded = true;
  return kOk;
}

// FP32 copies of every store for the mixed solve
int mg_upload32(pgb_mg *g) {
  if (g->uploaded32) return kOk;
  for (auto &kv : g->stores) {
    pgb_mg::Store &S = kv.second;
    const int64_t n = (int64_t)S.nslots * S.dims.N[0] * S.dims.N[1] * S.dims.N[2];
    const int64_t nc = (int64_t)S.nslots * S.dims.Nc[0] * S.dims.Nc[1] * S.dims.Nc[2];
    for (float **p : {&S.u32, &S.res32, &S.rhs32, &S.temp32, &S.u032}) {
      PGB_TRY(dev_zeros(g, p, n));
    }
    PGB_TRY(dev_zeros(g, &S.coarse32, nc));
  }
  g->uploaded32 = true;
  return kOk;
}

double srj_weight(const GmgConfig &c, int s) {
  // mg_solver.hpp:312-345, 3D weights (Yang & Mittal)
  static const double m1[3] = {1.0, 0.0, 0.0};
  static const double m2[3] = {1.7319, 0.5695, 0.0};
  static const double m3[3] = {2.2473, 0.8571, 0.5296};
  if (c.jacobi) return c.weight;
  return c.stages == 1 ? m1[s] : (c.stages == 2 ? m2[s] : m3[s]);
}

// exchange_grid's prolongation op: ProlongateSharedLinear with the reference's
// coordinate arithmetic (exact build) or in its uniform-spacing form (fast build)
int prolong_op(const pgb_mg *g) { return g->exact ? 1 : 3; }

// gmg_same exchange of grid L (ProlongateSharedLinear across coarse/fine faces)
int exch(pgb_mg *g, int L, double *f, cudaStream_t s) {
  return exchange_grid(g->grids.at(L).tab, f, g->store_of(L).coarse, 1, 1, prolong_op(g), nullptr, s, nullptr);
}
int exch(pgb_mg *g, int L, float *f, cudaStream_t s) {
  return exchange_grid_f32(g->grids.at(L).tab, f, g->store_of(L).coarse32, s);
}

// One V-cycle (AddLinearOperatorTasks, mg_solver.hpp:163-186, and per level
// AddMultiGridTasksPartitionLevel, :375-520). Every grid runs in FP64, or, in the mixed
// solve, in FP32 except the coarsest grid when it has a store of its own (FP64).
template <bool kFast>
struct VCycle {
  pgb_mg *g;
  cudaStream_t s;
  bool mixed;
  MgOp o;
  // the finest grid's u is zero on entry, ghosts and the coarser leaves included
  // (iterative refinement and the preconditioners solve for a correction from zero)
  bool zero_guess = false;
  bool dbl(int L) const { return !mixed || (L == g->lmin && g->lmin < 0); }
  int64_t cells(int L) const {
    const Dims &d = g->store_of(L).dims;
    return (int64_t)d.nx[0] * d.nx[1] * d.nx[2];
  }

  // Sweeps first .. stages - 1 of the smoother (first = 1: sweep 0, u into temp, was
  // fused into the level's FAS launch)
  template <class T>
  int smooth(int L, int stages, int first = 0, bool zero_first = false) {
    if (stages == 0) return kOk;
    pgb_mg::Grid &G = g->grids.at(L);
    pgb_mg::Store &S = g->store_of(L);
    const StoreView<T> v = S.template view<T>();
    const int nf = (int)G.fine_h.size(), nc = (int)G.coarse_h.size();
    const int64_t cl = cells(L);
    // Sweeps alternate between u and temp (odd sweeps write temp). The reference copies
    // u into temp on every block first and each sweep's result back into u; the
    // exchange of the second sweep then runs on temp, whose coarser leaves must hold
    // their u.
    const bool zero = zero_first && first == 0;  // the coarser leaves' temp = u = 0 in the first sweep
    if (stages >= 2 && nc && !zero)
      PGB_TRY(launch_pdl(k_mg_copy<T>, grid_for(nc * cl), 256, s, v.temp, v.u, G.coarse, nc, v.d));
    T *src = first % 2 ? v.temp : v.u, *dst = first % 2 ? v.u : v.temp;
    for (int st = first; st < stages; ++st) {
      MgSweep sw;
      sw.w = srj_weight(g->cfg, st);
      sw.omw = 1.0 - sw.w;
      sw.wd = sw.w / G.coef.den;
      if (zero_first && st == 0) {
        PGB_TRY(launch_pdl(k_mg_jacobi_zero<kFast, T>, grid_for(nf * cl), 256, s, (const T *)v.rhs, dst, G.fine, nf,
                           (const int *)G.coarse, stages >= 2 ? nc : 0, v.d, G.coef, o, sw,
                           g->store_of(L).template fd<T>()));
      } else {
        int rc = G.halofree ? kOk : exch(g, L, src, s);
        if (rc) return rc;
        PGB_TRY(launch_pdl(k_mg_jacobi<kFast, T>, grid_for(nf * cl), 256, s, src, v.rhs, dst, G.fine, nf, G.nb(),
                           v.d, G.coef, o, sw, g->store_of(L).template fd<T>()));
      }
      std::swap(src, dst);
    }
    if (src != v.u) PGB_TRY(launch_pdl(k_mg_copy<T>, grid_for(nf * cl), 256, s, v.u, v.temp, G.fine, nf, v.d));
    PGB_CUDA(cudaGetLastError());
    return kOk;
  }

  // res_err = u - u0 on the fine blocks and its exchange (mg_solver.hpp:489-517)
  template <class T>
  int error_out(int L) {
    pgb_mg::Grid &G = g->grids.at(L);
    const StoreView<T> v = g->store_of(L).template view<T>();
    const int nf = (int)G.fine_h.size();
    PGB_TRY(launch_pdl(k_mg_error<T>, grid_for(nf * cells(L)), 256, s, v, G.fine, nf));
    PGB_CUDA(cudaGetLastError());
    // a one-level grid's res_err ghosts are read from the neighbours by the prolongation
    return G.halofree ? kOk : exch(g, L, v.res, s);
  }

  template <class T, class TP>
  int restrict_down(int L) {
    pgb_mg::Grid &G = g->grids.at(L);
    const int nx = (int)G.xfer_h.size();
    PGB_TRY(launch_pdl(k_mg_restrict<T, TP>, grid_for(nx * cells(L) / 8), 256, s, 
        g->store_of(L).template view<T>(), g->store_of(L - 1).template view<TP>(), G.xfer, nx, G.tab.geom));
    PGB_CUDA(cudaGetLastError());
    return kOk;
  }

  // the level's residual and its restriction into the next coarser grid: one fused
  // launch when every block has at least two cells along each direction
  template <class T, class TP>
  int residual_restrict(int L) {
    pgb_mg::Grid &G = g->grids.at(L);
    const StoreView<T> v = g->store_of(L).template view<T>();
    const int nf = (int)G.fine_h.size(), nx = (int)G.xfer_h.size();
    if (v.d.nx[0] >= 2 && v.d.nx[1] >= 2 && v.d.nx[2] >= 2 && nx == nf) {
      PGB_TRY(launch_pdl(k_mg_residual_restrict<kFast, T, TP>, grid_for(nx * cells(L) / 8), 256, s, v,
                         g->store_of(L - 1).template view<TP>(), G.xfer, nx, G.nb(), G.coef, o,
                         g->store_of(L).template fd<T>(), G.tab.geom));
      PGB_CUDA(cudaGetLastError());
      return kOk;
    }
    PGB_TRY(launch_pdl(k_mg_residual<kFast, T>, grid_for(nf * cells(L)), 256, s, v, G.fine, nf, G.nb(), G.coef, o,
                       g->store_of(L).template fd<T>()));
    return restrict_down<T, TP>(L);
  }

  template <class T>
  int down(int L) {
    pgb_mg::Grid &G = g->grids.at(L);
    const StoreView<T> v = g->store_of(L).template view<T>();
    const int nf = (int)G.fine_h.size();
    const int64_t cl = cells(L);
    int rc;
    int first = 0;
    if (L < g->lmax) {
      // FAS: exchange, u0 = u, rhs = A u + res_err on internal blocks; on a grid read
      // directly, fused with the first sweep of the smoother
      if (!G.halofree && (rc = exch(g, L, v.u, s))) return rc;
      if (G.halofree && g->cfg.stages > 0 && G.coarse_h.empty()) {
        MgSweep sw;
        sw.w = srj_weight(g->cfg, 0);
        sw.omw = 1.0 - sw.w;
        sw.wd = sw.w / G.coef.den;
        PGB_TRY(launch_pdl(k_mg_fas_jacobi<kFast, T>, grid_for(nf * cl), 256, s, v, G.fine, nf, G.nint, G.nb(),
                           G.coef, o, sw, g->store_of(L).template fd<T>()));
        first = 1;
      } else {
        PGB_TRY(launch_pdl(k_mg_fas<kFast, T>, grid_for(nf * cl), 256, s, v, G.fine, nf, G.nint, G.nb(), G.coef, o,
                           g->store_of(L).template fd<T>()));
      }
    } else {
      PGB_TRY(launch_pdl(k_mg_copy<T>, grid_for(nf * cl), 256, s, v.u0, v.u, G.fine, nf, v.d));
    }
    if ((rc = smooth<T>(L, g->cfg.stages, first, zero_guess && L == g->lmax))) return rc;
    if (L > g->lmin) {
      if (!G.halofree && (rc = exch(g, L, v.u, s))) return rc;
      if constexpr (kFast) rc = dbl(L - 1) ? residual_restrict<T, double>(L) : residual_restrict<T, float>(L);
      else rc = residual_restrict<T, double>(L);
      if (rc) return rc;
    } else {
      for (int c = 0; c < g->cfg.coarse_sweeps; ++c)
        if ((rc = smooth<T>(L, g->cfg.stages))) return rc;
      PGB_TRY(launch_pdl(k_mg_copy<T>, grid_for(nf * cl), 256, s, v.res, v.u, G.fine, nf, v.d));
      if (L < g->lmax && (rc = error_out<T>(L))) return rc;
    }
    PGB_CUDA(cudaGetLastError());
    return kOk;
  }

  template <class T, class TP>
  int prolong_add(int L) {
    pgb_mg::Grid &G = g->grids.at(L);
    const int nx = (int)G.xfer_h.size();
    PGB_TRY(launch_pdl(k_mg_prolong_add<kFast, T, TP>, grid_for(nx * cells(L) / 8), 256, s, 
        g->store_of(L).template view<T>(), g->store_of(L - 1).template view<TP>(), G.xfer, nx, G.tab.geom));
    PGB_CUDA(cudaGetLastError());
    return kOk;
  }

  template <class T>
  int up(int L) {
    int rc;
    if constexpr (kFast) rc = dbl(L - 1) ? prolong_add<T, double>(L) : prolong_add<T, float>(L);
    else rc = prolong_add<T, double>(L);
    if (rc) return rc;
    if ((rc = smooth<T>(L, g->cfg.stages))) return rc;
    if (L < g->lmax && (rc = error_out<T>(L))) return rc;
    return kOk;
  }

  // The highest level of the trailing one-block grids that k_mg_tail takes (the fast
  // build), or lmin - 1 when none qualifies. A single one takes it too: the coarsest
  // grid's smoothing passes (2 + 2 and the extra coarse sweeps, about 35 launches of a
  // few microseconds) then run in one launch.
  int tail_top() const {
    int top = g->lmin - 1;
    for (int L = g->lmin; L <= g->lmax; ++L) {
      const pgb_mg::Grid &G = g->grids.at(L);
      if (G.fine_h.size() != 1 || !G.coarse_h.empty() || !G.halofree) break;
      if (cells(L) > 512) break;
      top = L;
    }
    const int n = top - g->lmin + 1;
    return (n >= 1 && n <= kTailMax) ? top : g->lmin - 1;
  }

  int tail(int top) {
    TailArgs a;
    std::memset(&a, 0, sizeof(a));
    a.n = top - g->lmin + 1;
    a.stages = g->cfg.stages;
    a.coarse_sweeps = g->cfg.coarse_sweeps;
    a.o = o;
    for (int t = 0; t < a.n; ++t) {
      const int L = top - t;
      const pgb_mg::Grid &G = g->grids.at(L);
      const pgb_mg::Store &S = g->store_of(L);
      TailGrid &T = a.g[t];
      T.slot = G.fine_h[0];
      for (int q = 0; q < 6; ++q) T.nb[q] = G.nbr_h[q];
      T.dbl = dbl(L) ? 1 : 0;
      T.internal = G.nint > 0 ? 1 : 0;
      T.top = L == g->lmax ? 1 : 0;
      T.vol = G.tab.geom_h.at(T.slot).vol;
      T.coef = G.coef;
      for (int st = 0; st < 3; ++st) {
        T.sw[st].w = srj_weight(g->cfg, st);
        T.sw[st].omw = 1.0 - T.sw[st].w;
        T.sw[st].wd = T.sw[st].w / G.coef.den;
      }
      T.v64 = S.template view<double>();
      T.v32 = S.template view<float>();
      T.fd64 = S.template fd<double>();
      T.fd32 = S.template fd<float>();
      if (L > g->lmin) T.up = G.xfer_h.at(0);
    }
    return launch_pdl(k_mg_tail, 1u, (unsigned)kTailThreads, s, a);
  }

  int run() {
    int rc;
    const int top = kFast ? tail_top() : g->lmin - 1;
    const int last_down = top >= g->lmin ? top + 1 : g->lmin;
    for (int L = g->lmax; L >= last_down; --L) {
      if constexpr (kFast) rc = dbl(L) ? down<double>(L) : down<float>(L);
      else rc = down<double>(L);  // the exact build is FP64 only
      if (rc) return rc;
    }
    if (top >= g->lmin && (rc = tail(top))) return rc;
    for (int L = (top >= g->lmin ? top + 1 : g->lmin + 1); L <= g->lmax; ++L) {
      if constexpr (kFast) rc = dbl(L) ? up<double>(L) : up<float>(L);
      else rc = up<double>(L);
      if (rc) return rc;
    }
    return kOk;
  }
};

// Leaf residual (exchange and rhs - A u on the leaf grid, mg_solver.hpp:131-146) with
// its partial sums copied to pinned host memory; mixed: also the FP32 right-hand side
// and zero guess of the next V-cycle.
template <bool kFast>
int leaf_residual_t(pgb_mg *g, bool mixed, cudaStream_t s) {
  pgb_mg::Store &S = g->stores.at(0);
  int rc = exchange_grid(g->leaf_tab, S.u, S.coarse, 1, 1, prolong_op(g), nullptr, s, nullptr);
  if (rc) return rc;
  if (g->flux_correct) {
    const unsigned grid = grid_for((int64_t)g->nleaf * S.dims.nx[0] * S.dims.nx[1] * S.dims.nx[2]);
    const MgOp o{g->cfg.D, g->cfg.alpha};
    PGB_TRY(launch_pdl(k_mg_leaf_fluxes, grid, 256, s, (const double *)S.u, g->lflux, g->nleaf, S.dims,
                       (const MgCoef *)g->leaf_coef, o, S.template fd<double>()));
    PGB_TRY(flux_correct_grid(g->leaf_tab, g->lflux, 1, s, nullptr));
    PGB_TRY(launch_pdl(k_mg_leaf_residual_flux, g->nparts, kResThreads, s, S.template view<double>(), g->nleaf,
                       (const MgCoef *)g->leaf_coef, o, (const double *)g->lflux, g->partial,
                       mixed ? S.rhs32 : nullptr, mixed ? S.u32 : nullptr));
    PGB_CUDA(cudaMemcpyAsync(g->partial_h, g->partial, g->nparts * sizeof(double), cudaMemcpyDeviceToHost, s));
    return kOk;
  }
  PGB_TRY(launch_pdl(k_mg_leaf_residual<kFast>, g->nparts, kResThreads, s, S.template view<double>(), g->nleaf, g->leaf_coef,
                                                              MgOp{g->cfg.D, g->cfg.alpha}, S.template fd<double>(), g->partial,
                                                              mixed ? S.rhs32 : nullptr, mixed ? S.u32 : nullptr));
  PGB_CUDA(cudaGetLastError());
  PGB_CUDA(cudaMemcpyAsync(g->partial_h, g->partial, g->nparts * sizeof(double), cudaMemcpyDeviceToHost, s));
  return kOk;
}

int leaf_residual(pgb_mg *g, bool mixed, cudaStream_t s) {
  return g->exact ? leaf_residual_t<false>(g, mixed, s) : leaf_residual_t<true>(g, mixed, s);
}

// One iteration of the solve: the V-cycle then the leaf residual. FP64: V-cycle on u;
// mixed: FP32 V-cycle on A e = r from e = 0, u += e, residual (iterative refinement).
template <bool kFast>
int enqueue_iteration_t(pgb_mg *g, bool mixed, cudaStream_t s) {
  VCycle<kFast> vc{g, s, mixed, MgOp{g->cfg.D, g->cfg.alpha}};
  vc.zero_guess = mixed;  // the FP32 correction starts from e = 0 (k_mg_leaf_residual)
  int rc = vc.run();
  if (rc) return rc;
  if (mixed) {
    pgb_mg::Store &S = g->stores.at(0);
    PGB_TRY(launch_pdl(k_mg_correct, grid_for((int64_t)g->nleaf * vc.cells(g->lmax)), 256, s, S.u, S.u32, g->nleaf, S.dims));
    PGB_CUDA(cudaGetLastError());
  }
  return leaf_residual_t<kFast>(g, mixed, s);
}

int enqueue_iteration(pgb_mg *g, bool mixed, cudaStream_t s) {
  if (mixed) return enqueue_iteration_t<true>(g, true, s);
  return g->exact ? enqueue_iteration_t<false>(g, false, s) : enqueue_iteration_t<true>(g, false, s);
}

// ---- BiCGSTAB with the composite V-cycle as preconditioner
enum { kX = 0, kR, kRhat0, kP, kV, kH, kS, kT, kNumVectors };

int bicg_alloc(pgb_mg *g) {
  if (g->kres_h) return kOk;  // allocated last: set only when every step succeeded
  const Dims &d = g->stores.at(0).dims;
  const int64_t n = (int64_t)g->nleaf * d.N[0] * d.N[1] * d.N[2];
  for (int q = 0; q < kNumVectors; ++q) {
    PGB_TRY(dev_zeros(g, &g->kv[q], n));
  }
  PGB_TRY(dev_zeros(g, &g->ks, kNumScalars));
  PGB_TRY(dev_zeros(g, &g->kpart, 2 * (int64_t)g->nparts));
  PGB_CUDA(cudaMallocHost((void **)&g->kres_h, 2 * sizeof(double)));
  return kOk;
}

// u <- M src with u the leaves of store 0: mode 1 one FP64 V-cycle from u = 0, mode 2 one
// FP32 V-cycle (FP64 coarsest grid below level 0), mode 0 no preconditioner (u <- src)
int bicg_precond(pgb_mg *g, int mode, const double *src, cudaStream_t s) {
  pgb_mg::Store &S = g->stores.at(0);
  const unsigned grid = grid_for((int64_t)g->nleaf * S.dims.nx[0] * S.dims.nx[1] * S.dims.nx[2]);
  if (mode == 0) return launch_pdl(k_bi_in<double>, grid, 256, s, src, (double *)nullptr, S.u, g->nleaf, S.dims);
  if (mode == 1) {
    PGB_TRY(launch_pdl(k_bi_in<double>, grid, 256, s, src, S.rhs, S.u, g->nleaf, S.dims));
    VCycle<true> vc{g, s, false, MgOp{g->cfg.D, g->cfg.alpha}};
    vc.zero_guess = true;  // k_bi_in zeroed u
    return vc.run();
  }
  PGB_TRY(launch_pdl(k_bi_in<float>, grid, 256, s, src, S.rhs32, S.u32, g->nleaf, S.dims));
  VCycle<true> vc{g, s, true, MgOp{g->cfg.D, g->cfg.alpha}};
  vc.zero_guess = true;  // k_bi_in zeroed u32
  PGB_TRY(vc.run());
  return launch_pdl(k_bi_out32, grid, 256, s, (const float *)S.u32, S.u, g->nleaf, S.dims);
}

// out <- A u on the leaf grid (exchange, then the operator)
int bicg_apply(pgb_mg *g, double *out, cudaStream_t s) {
  pgb_mg::Store &S = g->stores.at(0);
  PGB_TRY(exchange_grid(g->leaf_tab, S.u, S.coarse, 1, 1, prolong_op(g), nullptr, s, nullptr));
  const unsigned grid = grid_for((int64_t)g->nleaf * S.dims.nx[0] * S.dims.nx[1] * S.dims.nx[2]);
  if (g->flux_correct) {
    const MgOp o{g->cfg.D, g->cfg.alpha};
    PGB_TRY(launch_pdl(k_mg_leaf_fluxes, grid, 256, s, (const double *)S.u, g->lflux, g->nleaf, S.dims,
                       (const MgCoef *)g->leaf_coef, o, S.template fd<double>()));
    PGB_TRY(flux_correct_grid(g->leaf_tab, g->lflux, 1, s, nullptr));
    return launch_pdl(k_bi_apply_flux, grid, 256, s, (const double *)S.u, out, g->nleaf, S.dims,
                      (const MgCoef *)g->leaf_coef, o, (const double *)g->lflux);
  }
  return launch_pdl(k_bi_apply, grid, 256, s, (const double *)S.u, out, g->nleaf, S.dims,
                    (const MgCoef *)g->leaf_coef, MgOp{g->cfg.D, g->cfg.alpha}, S.template fd<double>());
}

int bicg_dots(pgb_mg *g, const double *a, const double *b, const double *c, const double *e, int i0, int i1,
              cudaStream_t s) {
  const Dims &d = g->stores.at(0).dims;
  PGB_TRY(launch_pdl(k_bi_dot2, g->nparts, kResThreads, s, a, b, c, e, g->nleaf, d, g->kpart));
  return launch_pdl(k_bi_final, 1u, 256u, s, (const double *)g->kpart, g->nparts, g->ks, i0, i1);
}

// One BiCGSTAB iteration (bicgstab_solver.hpp:170-306); the host reads (r, r) after it.
int bicg_iteration(pgb_mg *g, int mode, cudaStream_t s) {
  pgb_mg::Store &S = g->stores.at(0);
  double *const *v = g->kv;
  const Dims &d = S.dims;
  const unsigned grid = grid_for((int64_t)g->nleaf * d.nx[0] * d.nx[1] * d.nx[2]);
  PGB_TRY(launch_pdl(k_bi_begin, 1u, 1u, s, g->ks));
  PGB_TRY(bicg_precond(g, mode, v[kP], s));                                      // 1. u <- M p
  PGB_TRY(bicg_apply(g, v[kV], s));                                              // 2. v <- A u
  PGB_TRY(bicg_dots(g, v[kRhat0], v[kV], nullptr, nullptr, kRv, -1, s));         // 3. (rhat0, v)
  PGB_TRY(launch_pdl(k_bi_hs, grid, 256, s, (const double *)v[kX], (const double *)S.u, (const double *)v[kR],
                     (const double *)v[kV], v[kH], v[kS], (const double *)g->ks, g->nleaf, d));  // 4, 5
  PGB_TRY(bicg_precond(g, mode, v[kS], s));                                      // 6. u <- M s
  PGB_TRY(bicg_apply(g, v[kT], s));                                              // 7. t <- A u
  PGB_TRY(bicg_dots(g, v[kT], v[kS], v[kT], v[kT], kTs, kTt, s));                // 8. (t, s), (t, t)
  PGB_TRY(launch_pdl(k_bi_xr, g->nparts, kResThreads, s, (const double *)v[kH], (const double *)S.u,
                     (const double *)v[kS], (const double *)v[kT], (const double *)v[kRhat0], v[kX], v[kR],
                     (const double *)g->ks, g->nleaf, d, g->kpart));            // 9, 10
  PGB_TRY(launch_pdl(k_bi_final, 1u, 256u, s, (const double *)g->kpart, g->nparts, g->ks, (int)kRes,
                     (int)kRr));                                                 // (r, r), 11. (rhat0, r)
  PGB_TRY(launch_pdl(k_bi_p, grid, 256, s, (const double *)v[kR], (const double *)v[kV], v[kP],
                     (const double *)g->ks, g->nleaf, d));                       // 12, 13
  PGB_CUDA(cudaMemcpyAsync(g->kres_h, g->ks + kRes, sizeof(double), cudaMemcpyDeviceToHost, s));
  return kOk;
}

int run_bicg_iteration(pgb_mg *g, int mode, cudaStream_t s) {
  cudaGraphExec_t &graph = g->kgraph[mode];
  if (!graph) {
    cudaGraph_t gr;
    PGB_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    int rc = bicg_iteration(g, mode, s);
    cudaError_t e = cudaStreamEndCapture(s, &gr);
    if (rc) {
      if (e == cudaSuccess) cudaGraphDestroy(gr);
      return rc;
    }
    PGB_CUDA(e);
    e = cudaGraphInstantiate(&graph, gr, 0);
    cudaGraphDestroy(gr);
    PGB_CUDA(e);
  }
  PGB_CUDA(cudaGraphLaunch(graph, s));
  return kOk;
}

double host_rms(pgb_mg *g) {
  double sum = 0.0;
  for (int i = 0; i < g->nparts; ++i) sum += g->partial_h[i];
  double ncell = 0.0;
  for (auto &b : g->topo->leaf().blocks) ncell += (double)b.nx[0] * b.nx[1] * b.nx[2];
  return std::sqrt(sum / ncell);
}

int run_iteration(pgb_mg *g, bool mixed, cudaStream_t s) {
  cudaGraphExec_t &graph = g->graph[mixed ? 1 : 0];
  if (!graph) {
    cudaGraph_t gr;
    PGB_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    int rc = enqueue_iteration(g, mixed, s);
    cudaError_t e = cudaStreamEndCapture(s, &gr);
    if (rc) {
      if (e == cudaSuccess) cudaGraphDestroy(gr);
      return rc;
    }
    PGB_CUDA(e);
    e = cudaGraphInstantiate(&graph, gr, 0);
    cudaGraphDestroy(gr);
    PGB_CUDA(e);
  }
  PGB_CUDA(cudaGraphLaunch(graph, s));
  return kOk;
}

int copy_in(pgb_mg *g, const double *u, const double *rhs, cudaStream_t s) {
  pgb_mg::Store &S = g->stores.at(0);
  const size_t n = (size_t)g->nleaf * S.dims.N[0] * S.dims.N[1] * S.dims.N[2] * sizeof(double);
  PGB_CUDA(cudaMemcpyAsync(S.u, u, n, cudaMemcpyDeviceToDevice, s));
  PGB_CUDA(cudaMemcpyAsync(S.rhs, rhs, n, cudaMemcpyDeviceToDevice, s));
  return kOk;
}

int copy_out(pgb_mg *g, double *u, cudaStream_t s) {
  pgb_mg::Store &S = g->stores.at(0);
  const size_t n = (size_t)g->nleaf * S.dims.N[0] * S.dims.N[1] * S.dims.N[2] * sizeof(double);
  PGB_CUDA(cudaMemcpyAsync(u, S.u, n, cudaMemcpyDeviceToDevice, s));
  return kOk;
}

int check_stream(cudaStream_t s) {
  if (s == nullptr || s == cudaStreamLegacy || s == cudaStreamPerThread)
    return fail(kErrInvalid, "the multigrid solve captures a CUDA graph: pass a created stream");
  return kOk;
}

}  // namespace

extern "C" {

int pgb_mg_create(pgb_mesh *mesh, const pgb_mg_params *p, pgb_mg **out) {
  if (!mesh || !p || !out) return fail(kErrInvalid, "null argument");
  *out = nullptr;
  if (p->stages < 0 || p->stages > 3) return fail(kErrInvalid, "stages must be 0..3");
  if (!p->jacobi && p->stages == 0) return fail(kErrInvalid, "SRJ needs 1..3 stages");
  if (p->coarse_sweeps < 0 || p->max_coarsenings < 0) return fail(kErrInvalid, "negative count");
  MeshState *st = mesh_state(mesh);
  if (!st || !st->topo) return fail(kErrInvalid, "mesh without topology");
  const MeshSpec &sp = st->topo->spec();
  if (sp.ng < 1) return fail(kErrUnsupported, "the operator needs one ghost layer");
  auto *g = new pgb_mg();
  g->mesh = mesh;
  g->topo = st->topo.get();
  g->cfg.stages = p->stages;
  g->cfg.jacobi = p->jacobi;
  g->cfg.weight = p->weight;
  g->cfg.coarse_sweeps = p->coarse_sweeps;
  g->cfg.D = p->D;
  g->cfg.alpha = p->alpha;
  g->exact = p->exact != 0;
  g->flux_correct = p->flux_correct != 0;
  g->max_coarsenings = p->max_coarsenings;
  int rc;
  try {
    rc = mg_build(g);
  } catch (std::exception &e) {
    rc = fail(kErrInvalid, std::string("multigrid grids: ") + e.what());
  }
  if (rc) {
    delete g;
    return rc;
  }
  *out = g;
  return kOk;
}

int pgb_mg_destroy(pgb_mg *g) {
  delete g;
  return kOk;
}

int pgb_mg_info(const pgb_mg *g, int32_t *out) {
  if (!g || !out) return fail(kErrInvalid, "null argument");
  out[0] = g->lmin;
  out[1] = g->lmax;
  out[2] = g->stores.at(0).nslots;
  out[3] = g->nleaf;
  out[4] = (int32_t)g->grids.size();
  return kOk;
}

int pgb_mg_boundaries(const pgb_mg *g, int32_t level, int32_t *out, int32_t capacity, int32_t *count) {
  if (!g || !count) return fail(kErrInvalid, "null argument");
  const auto &mg = g->topo->mg_grids();
  auto it = mg.find(level);
  if (it == mg.end() || level < g->lmin || level > g->lmax) return fail(kErrInvalid, "no multigrid grid at that level");
  const GridTopology &gr = it->second;
  *count = (int32_t)gr.pairs.size();
  if (!out) return kOk;
  if (capacity < (int)gr.pairs.size()) return fail(kErrInvalid, "capacity too small");
  int r = 0;
  for (auto &p : gr.pairs) {
    int32_t *o = out + 23 * r++;
    o[0] = gr.blocks[p.sender].gid;
    o[1] = gr.blocks[p.receiver].gid;
    o[2] = p.loc_index;
    for (int d = 0; d < 3; ++d) {
      o[3 + 2 * d] = p.send.lo[d];
      o[4 + 2 * d] = p.send.hi[d];
      o[10 + 2 * d] = p.recv.lo[d];
      o[11 + 2 * d] = p.recv.hi[d];
    }
    o[9] = p.send_coarse;
    o[16] = p.recv_coarse;
    o[17] = (int32_t)p.recv.mask;
    o[18] = (int32_t)p.send.count();
    o[19] = o[20] = o[21] = o[22] = 0;
  }
  return kOk;
}

int pgb_mg_vcycles(pgb_mg *g, double *u, const double *rhs, int32_t ncycles, double *rms, void *stream) {
  if (!g || !u || !rhs) return fail(kErrInvalid, "null argument");
  cudaStream_t s = (cudaStream_t)stream;
  int rc;
  if ((rc = check_stream(s)) || (rc = mg_upload(g)) || (rc = copy_in(g, u, rhs, s))) return rc;
  for (int c = 0; c < ncycles; ++c) {
    if ((rc = run_iteration(g, false, s))) return rc;
    PGB_CUDA(cudaStreamSynchronize(s));
    if (rms) rms[c] = host_rms(g);
  }
  if ((rc = copy_out(g, u, s))) return rc;
  PGB_CUDA(cudaStreamSynchronize(s));
  return kOk;
}

int pgb_mg_solve(pgb_mg *g, double *u, const double *rhs, double tol, int32_t relative, int32_t mixed,
                 int32_t max_cycles, int32_t *cycles_out, double *rms_out, void *stream) {
  if (!g || !u || !rhs) return fail(kErrInvalid, "null argument");
  cudaStream_t s = (cudaStream_t)stream;
  const bool mx = mixed != 0;
  int rc;
  if ((rc = check_stream(s)) || (rc = mg_upload(g)) || (mx && (rc = mg_upload32(g))) ||
      (rc = copy_in(g, u, rhs, s)))
    return rc;
  if ((rc = mx ? leaf_residual_t<true>(g, true, s) : leaf_residual(g, false, s))) return rc;
  PGB_CUDA(cudaStreamSynchronize(s));
  const double r0 = host_rms(g);
  const double target = relative ? tol * r0 : tol;
  double r = r0;
  int c = 0;
  // MGSolver::AddTasks: iterate while rms > tolerance (mg_solver.hpp:147-158)
  while (r > target && c < max_cycles) {
    if ((rc = run_iteration(g, mx, s))) return rc;
    PGB_CUDA(cudaStreamSynchronize(s));
    r = host_rms(g);
    ++c;
  }
  if ((rc = copy_out(g, u, s))) return rc;
  PGB_CUDA(cudaStreamSynchronize(s));
  if (cycles_out) *cycles_out = c;
  if (rms_out) *rms_out = relative ? (r0 > 0 ? r / r0 : 0.0) : r;
  return kOk;
}

int pgb_mg_set_coefficient(pgb_mg *g, const double *d, void *stream) {
  if (!g || !d) return fail(kErrInvalid, "null argument");
  cudaStream_t s = (cudaStream_t)stream;
  int rc;
  if ((rc = mg_upload(g))) return rc;
  for (auto &kv : g->stores) {
    pgb_mg::Store &S = kv.second;
    const int64_t n = (int64_t)S.nslots * S.dims.N[0] * S.dims.N[1] * S.dims.N[2];
    for (int q = 0; q < 3; ++q)
      if (!S.d32[q]) {  // allocated second: null unless both exist
        if (!S.d[q]) PGB_TRY(dev_zeros(g, &S.d[q], n));
        PGB_TRY(dev_zeros(g, &S.d32[q], n));
      }
  }
  // the leaves' faces: [nleaf][3][N3][N2][N1] into the three face arrays of store 0
  pgb_mg::Store &S0 = g->stores.at(0);
  const size_t cells = (size_t)S0.dims.N[0] * S0.dims.N[1] * S0.dims.N[2];
  for (int q = 0; q < 3; ++q)
    PGB_CUDA(cudaMemcpy2DAsync(S0.d[q], cells * sizeof(double), d + q * cells, 3 * cells * sizeof(double),
                               cells * sizeof(double), g->nleaf, cudaMemcpyDeviceToDevice, s));
  // AddSetupTasks: from the finest grid down, each level's faces restricted into the next
  for (int L = g->lmax; L > g->lmin; --L) {
    pgb_mg::Grid &G = g->grids.at(L);
    const pgb_mg::Store &C = g->store_of(L), &P = g->store_of(L - 1);
    const int nx = (int)G.xfer_h.size();
    const int64_t per = (int64_t)(C.dims.nx[0] / 2 + 1) * (C.dims.nx[1] / 2 + 1) * (C.dims.nx[2] / 2 + 1);
    for (int q = 0; q < 3; ++q)
      k_mg_restrict_faces<<<grid_for(nx * per), 256, 0, s>>>(C.d[q], C.dims, P.d[q], P.dims, G.xfer, nx, G.tab.geom,
                                                              q);
    PGB_CUDA(cudaGetLastError());
  }
  for (auto &kv : g->stores) {
    pgb_mg::Store &S = kv.second;
    const int64_t n = (int64_t)S.nslots * S.dims.N[0] * S.dims.N[1] * S.dims.N[2];
    for (int q = 0; q < 3; ++q) k_to_f32<<<grid_for(n), 256, 0, s>>>(S.d[q], S.d32[q], n);
  }
  PGB_CUDA(cudaGetLastError());
  PGB_CUDA(cudaStreamSynchronize(s));
  // graphs captured before hold the constant-coefficient kernels
  for (auto &gr : g->graph)
    if (gr) {
      cudaGraphExecDestroy(gr);
      gr = nullptr;
    }
  for (auto &gr : g->kgraph)
    if (gr) {
      cudaGraphExecDestroy(gr);
      gr = nullptr;
    }
  return kOk;
}

int pgb_mg_bicgstab(pgb_mg *g, double *u, const double *rhs, int32_t precondition, double rtol, int32_t relative,
                    int32_t max_iters, int32_t *iters_out, double *rms_out, void *stream) {
  if (!g || !u || !rhs) return fail(kErrInvalid, "null argument");
  if (precondition < 0 || precondition > 2) return fail(kErrInvalid, "precondition must be 0, 1 or 2");
  cudaStream_t s = (cudaStream_t)stream;
  int rc;
  if ((rc = check_stream(s)) || (rc = mg_upload(g)) || (precondition == 2 && (rc = mg_upload32(g))) ||
      (rc = bicg_alloc(g)))
    return rc;
  pgb_mg::Store &S = g->stores.at(0);
  const Dims &d = S.dims;
  const unsigned grid = grid_for((int64_t)g->nleaf * d.nx[0] * d.nx[1] * d.nx[2]);
  double *const *v = g->kv;
  // x <- 0, r, rhat0, p <- rhs; (rhat0, r) and (rhs, rhs) (bicgstab_solver.hpp:125-140)
  if ((rc = launch_pdl(k_bi_init, grid, 256, s, rhs, v[kX], v[kR], v[kRhat0], v[kP], g->nleaf, d)) ||
      (rc = bicg_dots(g, v[kRhat0], v[kR], rhs, rhs, kRr, kRhs2, s)))
    return rc;
  PGB_CUDA(cudaMemcpyAsync(g->kres_h + 1, g->ks + kRhs2, sizeof(double), cudaMemcpyDeviceToHost, s));
  PGB_CUDA(cudaStreamSynchronize(s));
  double ncell = 0.0;
  for (auto &b : g->topo->leaf().blocks) ncell += (double)b.nx[0] * b.nx[1] * b.nx[2];
  const double tol = relative ? rtol * std::sqrt(g->kres_h[1] / ncell) : rtol;
  int it = 0;
  double rms = 0.0;
  while (it < max_iters) {
    if ((rc = run_bicg_iteration(g, precondition, s))) return rc;
    PGB_CUDA(cudaStreamSynchronize(s));
    rms = std::sqrt(g->kres_h[0] / ncell);
    ++it;
    if (rms < tol) break;
  }
  // u <- x, with its ghosts exchanged on the leaf grid
  if ((rc = launch_pdl(k_bi_in<double>, grid, 256, s, (const double *)v[kX], (double *)nullptr, S.u, g->nleaf, d)) ||
      (rc = exchange_grid(g->leaf_tab, S.u, S.coarse, 1, 1, prolong_op(g), nullptr, s, nullptr)) ||
      (rc = copy_out(g, u, s)))
    return rc;
  PGB_CUDA(cudaStreamSynchronize(s));
  if (iters_out) *iters_out = it;
  if (rms_out) *rms_out = rms;
  return kOk;
}

/* ---- the composite grids for a package-side solver ---------------------------- */

int pgb_mg_layout(pgb_mg *g, int32_t *out) {
  if (!g || !out) return fail(kErrInvalid, "null argument");
  int rc;
  if ((rc = mg_upload(g))) return rc;
  out[0] = g->lmin;
  out[1] = g->lmax;
  out[2] = g->nleaf;
  out[3] = (int32_t)g->stores.size();
  out[4] = g->exact ? 1 : 0;
  return kOk;
}

int pgb_mg_store_info(pgb_mg *g, int32_t store, int32_t *out, double *geom, int32_t *levels) {
  if (!g || !out) return fail(kErrInvalid, "null argument");
  int rc;
  if ((rc = mg_upload(g))) return rc;
  auto it = g->stores.find(store);
  if (it == g->stores.end()) return fail(kErrInvalid, "no multigrid store with that key");
  const pgb_mg::Store &S = it->second;
  out[0] = S.nslots;
  for (int d = 0; d < 3; ++d) {
    out[1 + d] = S.dims.nx[d];
    out[5 + d] = S.dims.N[d];
  }
  out[4] = S.dims.ng;
  for (int b = 0; b < S.nslots; ++b) {
    const BlockInfo &bi = S.blocks[b];
    if (geom)
      for (int d = 0; d < 3; ++d) {
        geom[6 * b + d] = bi.xmin[d];
        geom[6 * b + 3 + d] = bi.dx[d];
      }
    if (levels) levels[b] = bi.loc.level;
  }
  return kOk;
}

int pgb_mg_grid_info(pgb_mg *g, int32_t level, int32_t *out, int32_t *fine, int32_t *coarse) {
  if (!g || !out) return fail(kErrInvalid, "null argument");
  int rc;
  if ((rc = mg_upload(g))) return rc;
  auto it = g->grids.find(level);
  if (it == g->grids.end()) return fail(kErrInvalid, "no multigrid grid at that level");
  const pgb_mg::Grid &G = it->second;
  out[0] = G.store;
  out[1] = (int32_t)G.fine_h.size();
  out[2] = (int32_t)G.coarse_h.size();
  out[3] = G.nint;
  if (fine) std::memcpy(fine, G.fine_h.data(), G.fine_h.size() * sizeof(int32_t));
  if (coarse) std::memcpy(coarse, G.coarse_h.data(), G.coarse_h.size() * sizeof(int32_t));
  return kOk;
}

int pgb_mg_field_exchange(pgb_mg *g, int32_t level, double *field, void *stream) {
  if (!g || !field) return fail(kErrInvalid, "null argument");
  int rc;
  if ((rc = mg_upload(g))) return rc;
  if (!g->grids.count(level)) return fail(kErrInvalid, "no multigrid grid at that level");
  return exch(g, level, field, (cudaStream_t)stream);
}

int pgb_mg_field_restrict(pgb_mg *g, int32_t level, const double *fine, double *coarse, void *stream) {
  if (!g || !fine || !coarse) return fail(kErrInvalid, "null argument");
  int rc;
  if ((rc = mg_upload(g))) return rc;
  if (!g->grids.count(level) || level <= g->lmin) return fail(kErrInvalid, "no coarser grid below that level");
  const pgb_mg::Grid &G = g->grids.at(level);
  const pgb_mg::Store &C = g->store_of(level), &P = g->store_of(level - 1);
  const int nx = (int)G.xfer_h.size();
  if (nx == 0) return kOk;
  const int64_t per = (int64_t)std::max(1, C.dims.nx[0] / 2) * std::max(1, C.dims.nx[1] / 2) *
                      std::max(1, C.dims.nx[2] / 2);
  k_mgf_restrict<<<grid_for(nx * per), 256, 0, (cudaStream_t)stream>>>(fine, C.dims, coarse, P.dims, G.xfer, nx,
                                                                        G.tab.geom);
  PGB_CUDA(cudaGetLastError());
  return kOk;
}

int pgb_mg_field_prolongate(pgb_mg *g, int32_t level, const double *coarse, double *fine, void *stream) {
  if (!g || !fine || !coarse) return fail(kErrInvalid, "null argument");
  int rc;
  if ((rc = mg_upload(g))) return rc;
  if (!g->grids.count(level) || level <= g->lmin) return fail(kErrInvalid, "no coarser grid below that level");
  const pgb_mg::Grid &G = g->grids.at(level);
  const pgb_mg::Store &C = g->store_of(level), &P = g->store_of(level - 1);
  const int nx = (int)G.xfer_h.size();
  if (nx == 0) return kOk;
  const int64_t per = (int64_t)std::max(1, C.dims.nx[0] / 2) * std::max(1, C.dims.nx[1] / 2) *
                      std::max(1, C.dims.nx[2] / 2);
  cudaStream_t s = (cudaStream_t)stream;
  if (g->exact)
    k_mgf_prolong<false><<<grid_for(nx * per), 256, 0, s>>>(coarse, P.dims, fine, C.dims, G.xfer, nx, G.tab.geom);
  else
    k_mgf_prolong<true><<<grid_for(nx * per), 256, 0, s>>>(coarse, P.dims, fine, C.dims, G.xfer, nx, G.tab.geom);
  PGB_CUDA(cudaGetLastError());
  return kOk;
}

int pgb_mg_face_restrict(pgb_mg *g, int32_t level, const double *fine, double *coarse, void *stream) {
  if (!g || !fine || !coarse) return fail(kErrInvalid, "null argument");
  int rc;
  if ((rc = mg_upload(g))) return rc;
  if (!g->grids.count(level) || level <= g->lmin) return fail(kErrInvalid, "no coarser grid below that level");
  const pgb_mg::Grid &G = g->grids.at(level);
  const pgb_mg::Store &C = g->store_of(level), &P = g->store_of(level - 1);
  const int nx = (int)G.xfer_h.size();
  if (nx == 0) return kOk;
  const int64_t per = (int64_t)(C.dims.nx[0] / 2 + 1) * (C.dims.nx[1] / 2 + 1) * (C.dims.nx[2] / 2 + 1);
  const int64_t cc = (int64_t)C.nslots * C.dims.N[0] * C.dims.N[1] * C.dims.N[2];
  const int64_t pc = (int64_t)P.nslots * P.dims.N[0] * P.dims.N[1] * P.dims.N[2];
  for (int q = 0; q < 3; ++q)
    k_mg_restrict_faces<<<grid_for(nx * per), 256, 0, (cudaStream_t)stream>>>(fine + q * cc, C.dims, coarse + q * pc,
                                                                               P.dims, G.xfer, nx, G.tab.geom, q);
  PGB_CUDA(cudaGetLastError());
  return kOk;
}

}  // extern "C"
