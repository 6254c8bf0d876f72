"""Seeded initial conditions (problem generators) for the benchmark workloads.

These stand in for the reference's ProblemGenerator functions
(example/advection/parthenon_app_inputs.cpp:40-124,
benchmarks/burgers/parthenon_app_inputs.cpp:40-78) with the synthetic fields the
benchmark configurations ask for. Arrays use the field layout
(nblocks, ncomp, N3, N2, N1); ghosts are left zero for the first exchange to fill.
"""
import numpy as np


def _centers(mesh):
    xs, ys, zs = mesh.cell_centers()
    return xs, ys, zs


def _interior(mesh):
    g = mesh.nghost
    n = mesh.block_nx
    return (slice(g, g + n[2]), slice(g, g + n[1]), slice(g, g + n[0]))


def gaussian(mesh, center=(0.5, 0.5, 0.5), sigma=0.1):
    """exp(-|x - c|^2 / (2 sigma^2)) on cell centres, shape (nblocks, N3, N2, N1)."""
    xs, ys, zs = _centers(mesh)
    dx2 = (xs - center[0]) ** 2
    dy2 = (ys - center[1]) ** 2
    dz2 = (zs - center[2]) ** 2
    r2 = dz2[:, :, None, None] + dy2[:, None, :, None] + dx2[:, None, None, :]
    return np.exp(-r2 / (2.0 * sigma * sigma))


def advection_state(mesh, nscalars=0, seed=3):
    """Advected Gaussian plus `nscalars` U(0,1) scalars (seeded), interior filled."""
    ncomp = 1 + nscalars
    out = np.zeros((mesh.nblocks, ncomp) + tuple(mesh.N[::-1]), np.float64)
    sk, sj, si = _interior(mesh)
    out[:, 0, sk, sj, si] = gaussian(mesh)[:, sk, sj, si]
    if nscalars:
        rng = np.random.default_rng(seed)
        n = mesh.block_nx
        out[:, 1:, sk, sj, si] = rng.random((mesh.nblocks, nscalars, n[2], n[1], n[0]))
    return out


def sinusoid_modes(nmodes, kmax, seed):
    """Per velocity component: wave vectors in {1..kmax}^3, amplitudes U(0,1), phases U(0,2pi)."""
    rng = np.random.default_rng(seed)
    modes = []
    for _ in range(3):
        k = rng.integers(1, kmax + 1, size=(nmodes, 3))
        a = rng.random(nmodes)
        phi = rng.random(nmodes) * 2.0 * np.pi
        modes.append((k, a, phi))
    return modes


def burgers_reference_state(mesh, nscalars=8, center=(0.0, 0.0, 0.0)):
    """The Burgers benchmark's own initial condition (ProblemGenerator,
    benchmarks/burgers/parthenon_app_inputs.cpp:34-70, with kx_fact = ky_fact = kz_fact
    = 1) about `center` (the reference's domain is [-0.5, 0.5]^3, centre 0): tanh fronts
    under Gaussian envelopes for the three velocity components, and scalars equal to 1
    with 10 added in a thin box -- exactly constant regions with jumps at the box."""
    ncomp = 3 + nscalars
    out = np.zeros((mesh.nblocks, ncomp) + tuple(mesh.N[::-1]), np.float64)
    sk, sj, si = _interior(mesh)
    xs, ys, zs = _centers(mesh)
    g = mesh.nghost
    n = mesh.block_nx
    x = (xs[:, g:g + n[0]] - center[0])[:, None, None, :]
    y = (ys[:, g:g + n[1]] - center[1])[:, None, :, None]
    z = (zs[:, g:g + n[2]] - center[2])[:, :, None, None]
    shape = (mesh.nblocks, n[2], n[1], n[0])
    out[:, 0, sk, sj, si] = np.broadcast_to(
        (np.tanh(-20.0 * x) * np.cos(np.pi * x) + 1.0) * np.exp(-30.0 * y * y) * np.exp(-30.0 * z * z), shape)
    out[:, 1, sk, sj, si] = np.broadcast_to(
        (np.sin(np.pi * y) + 0.2) * np.exp(-30.0 * x * x) * np.exp(-30.0 * z * z), shape)
    out[:, 2, sk, sj, si] = np.broadcast_to(
        (np.tanh(-20.0 * z) * np.cos(np.pi * z) + 0.5) * np.exp(-30.0 * x * x) * np.exp(-30.0 * y * y), shape)
    box = (np.abs(x) < 0.025) & (np.abs(y) < 0.15) & (np.abs(z) < 0.025)
    out[:, 3:, sk, sj, si] = np.broadcast_to(np.where(box, 11.0, 1.0), shape)[:, None]
    return out


def burgers_state(mesh, nscalars=8, nmodes=8, kmax=4, seed=2):
    """Burgers velocity as a sum of random-phase sinusoids per component plus
    `nscalars` U(0,1) passive scalars, all seeded; interior filled."""
    ncomp = 3 + nscalars
    out = np.zeros((mesh.nblocks, ncomp) + tuple(mesh.N[::-1]), np.float64)
    sk, sj, si = _interior(mesh)
    xs, ys, zs = _centers(mesh)
    g = mesh.nghost
    n = mesh.block_nx
    x = xs[:, g:g + n[0]]
    y = ys[:, g:g + n[1]]
    z = zs[:, g:g + n[2]]
    for c, (k, a, phi) in enumerate(sinusoid_modes(nmodes, kmax, seed)):
        acc = np.zeros((mesh.nblocks, n[2], n[1], n[0]))
        for m in range(nmodes):
            arg = (2.0 * np.pi * (k[m, 2] * z[:, :, None, None] + k[m, 1] * y[:, None, :, None] +
                                  k[m, 0] * x[:, None, None, :]) + phi[m])
            acc += a[m] * np.sin(arg)
        out[:, c, sk, sj, si] = acc
    if nscalars:
        rng = np.random.default_rng(seed + 1000)
        out[:, 3:, sk, sj, si] = rng.random((mesh.nblocks, nscalars, n[2], n[1], n[0]))
    return out


class BlockGeometry:
    """Cell-centre geometry of a block list given as (nblocks, 6) rows of
    (xmin1, xmin2, xmin3, dx1, dx2, dx3) -- the layout Mesh.block_info returns -- so the
    problem generators can run on any block list."""

    def __init__(self, geom, nghost, block_nx):
        self.geom = np.asarray(geom, np.float64)
        self.nblocks = self.geom.shape[0]
        self.nghost = int(nghost)
        self.block_nx = tuple(int(b) for b in block_nx)
        self.N = tuple(b + 2 * self.nghost for b in self.block_nx)

    def cell_centers(self):
        out = []
        for d in range(3):
            idx = np.arange(self.N[d]) - self.nghost
            out.append(self.geom[:, d:d + 1] + (idx[None, :] + 0.5) * self.geom[:, 3 + d:4 + d])
        return out


# The sparse advection example's fields (example/sparse_advection/
# sparse_advection_package.cpp:58-66): starting centres in the x-y plane, each field
# moving diagonally away from its corner. The example is two-dimensional; here the
# mesh is three-dimensional and the fields are spheres around z = 0 with vz = 0.
SPARSE_X0 = (0.8, -0.8, -0.8, 0.8)
SPARSE_Y0 = (0.8, 0.8, -0.8, -0.8)


def sparse_advection_velocities(speed=1.5):
    """(4, 3) velocities: field 0 moves along (-1,-1), 1 along (1,-1), 2 along (1,1),
    3 along (-1,1), each at `speed` (sparse_advection_package.cpp:61-66)."""
    s = speed / np.sqrt(2.0)
    return np.array([[-s, -s, 0.0], [s, -s, 0.0], [s, s, 0.0], [-s, s, 0.0]])


def sparse_advection_state(mesh, prev=None, prev_alloc=None, init_size=0.1, nfields=4):
    """ProblemGenerator of the sparse advection example
    (example/sparse_advection/parthenon_app_inputs.cpp:42-103) on the current block
    list: field f is allocated on every block where some interior cell centre lies
    within init_size of its centre, and there set to 1 inside and 0 outside; on other
    blocks the field keeps `prev` and its allocation `prev_alloc` (the previous mesh's
    data during the initial refinement). Returns (state, alloc)."""
    shape = (mesh.nblocks, nfields) + tuple(mesh.N[::-1])
    out = np.zeros(shape) if prev is None else np.array(prev, np.float64)
    alloc = np.zeros((mesh.nblocks, nfields), np.uint8) if prev_alloc is None else np.array(prev_alloc, np.uint8)
    xs, ys, zs = mesh.cell_centers()
    sk, sj, si = _interior(mesh)
    size = init_size * init_size
    for f in range(nfields):
        x = xs[:, si] - SPARSE_X0[f % 4]
        y = ys[:, sj] - SPARSE_Y0[f % 4]
        z = zs[:, sk]
        # x*x + y*y + z*z in the example's order
        r2 = (x[:, None, None, :] * x[:, None, None, :] + y[:, None, :, None] * y[:, None, :, None]) + \
            z[:, :, None, None] * z[:, :, None, None]
        inside = r2 < size
        hit = inside.reshape(mesh.nblocks, -1).any(axis=1)
        alloc[hit, f] = 1
        out[hit, f, sk, sj, si] = inside[hit].astype(np.float64)
    return out, alloc


def burgers_amr_state(mesh, nscalars=2, nmodes=16, kmax=6, seed=5):
    """Adaptive Burgers initial data, a pure function of position so that it can be
    evaluated again on every refined mesh (as Mesh::Initialize re-runs the problem
    generator while the initial refinement settles): velocity = sum of `nmodes`
    random-phase sinusoids per component with wave vectors in {1..kmax}^3 (seeded);
    scalar s (s = 0, 1, ...) = 1 + 0.5 sin(2 pi (s+1) x) sin(2 pi y) sin(2 pi z)."""
    ncomp = 3 + nscalars
    out = np.zeros((mesh.nblocks, ncomp) + tuple(mesh.N[::-1]), np.float64)
    sk, sj, si = _interior(mesh)
    xs, ys, zs = _centers(mesh)
    g = mesh.nghost
    n = mesh.block_nx
    x = xs[:, g:g + n[0]][:, None, None, :]
    y = ys[:, g:g + n[1]][:, None, :, None]
    z = zs[:, g:g + n[2]][:, :, None, None]
    for c, (k, a, phi) in enumerate(sinusoid_modes(nmodes, kmax, seed)):
        acc = np.zeros((mesh.nblocks, n[2], n[1], n[0]))
        for m in range(nmodes):
            acc += a[m] * np.sin(2.0 * np.pi * (k[m, 2] * z + k[m, 1] * y + k[m, 0] * x) + phi[m])
        out[:, c, sk, sj, si] = acc
    for s in range(nscalars):
        out[:, 3 + s, sk, sj, si] = 1.0 + 0.5 * (np.sin(2.0 * np.pi * (s + 1) * x) * np.sin(2.0 * np.pi * y) *
                                                 np.sin(2.0 * np.pi * z))
    return out


def burgers_amr_state_device(mesh, nscalars=2, nmodes=16, kmax=6, seed=5):
    """burgers_amr_state evaluated on the GPU (torch tensor in the field layout), for
    meshes of tens of thousands of blocks where the host evaluation would dominate."""
    import torch
    _, geom = mesh.block_info()
    geom = torch.as_tensor(geom, dtype=torch.float64, device="cuda")
    g = mesh.nghost
    n = mesh.block_nx
    ncomp = 3 + nscalars
    out = torch.zeros((mesh.nblocks, ncomp) + tuple(mesh.N[::-1]), dtype=torch.float64, device="cuda")
    c = [geom[:, d:d + 1] + (torch.arange(n[d], dtype=torch.float64, device="cuda")[None, :] + 0.5) *
         geom[:, 3 + d:4 + d] for d in range(3)]
    x = c[0][:, None, None, :]
    y = c[1][:, None, :, None]
    z = c[2][:, :, None, None]
    two_pi = 2.0 * np.pi
    for comp, (k, a, phi) in enumerate(sinusoid_modes(nmodes, kmax, seed)):
        acc = torch.zeros((mesh.nblocks, n[2], n[1], n[0]), dtype=torch.float64, device="cuda")
        for m in range(nmodes):
            arg = two_pi * (float(k[m, 2]) * z + float(k[m, 1]) * y + float(k[m, 0]) * x) + float(phi[m])
            acc += float(a[m]) * torch.sin(arg)
        out[:, comp, g:g + n[2], g:g + n[1], g:g + n[0]] = acc
    for s in range(nscalars):
        out[:, 3 + s, g:g + n[2], g:g + n[1], g:g + n[0]] = 1.0 + 0.5 * (
            torch.sin(two_pi * (s + 1) * x) * torch.sin(two_pi * y) * torch.sin(two_pi * z))
    return out


def poisson_rhs(n, ngauss=32, sigma=0.03, seed=4):
    """Sum of `ngauss` Gaussians (width sigma, centres U[0,1]^3, amplitudes N(0,1), seeded)
    with periodic-image distances on the unit cube, minus its mean; array (n, n, n),
    x fastest."""
    rng = np.random.default_rng(seed)
    centres = rng.random((ngauss, 3))
    amps = rng.standard_normal(ngauss)
    x = (np.arange(n) + 0.5) / n
    out = np.zeros((n, n, n))
    for c, a in zip(centres, amps):
        d = [x - c[q] for q in range(3)]
        d = [dd - np.round(dd) for dd in d]
        r2 = d[2][:, None, None] ** 2 + d[1][None, :, None] ** 2 + d[0][None, None, :] ** 2
        out += a * np.exp(-r2 / (2.0 * sigma * sigma))
    return out - out.mean()


def refined_region_leaves(root_level, lo, hi):
    """Leaves of a mesh whose root blocks lo..hi-1 (every direction) are refined once:
    (level, lx1, lx2, lx3) of the 8 children of each (static refinement of a cube)."""
    out = []
    for k in range(lo, hi):
        for j in range(lo, hi):
            for i in range(lo, hi):
                for dk in (0, 1):
                    for dj in (0, 1):
                        for di in (0, 1):
                            out.append((root_level + 1, 2 * i + di, 2 * j + dj, 2 * k + dk))
    return out


def poisson_rhs_blocks(mesh, ngauss=32, sigma=0.03, seed=4):
    """The right-hand side of poisson_rhs on the leaf blocks of `mesh`, (nblocks, N3, N2,
    N1) with zero ghosts: a sum of `ngauss` Gaussians (periodic images, centres U[0,1]^3,
    amplitudes N(0,1), seeded) minus its volume-weighted mean."""
    rng = np.random.default_rng(seed)
    centres = rng.random((ngauss, 3))
    amps = rng.standard_normal(ngauss)
    locs, geom = mesh.block_info()
    bnx, ng = mesh.block_nx, mesh.nghost
    out = np.zeros((mesh.nblocks, mesh.N[2], mesh.N[1], mesh.N[0]))
    vols = np.prod(geom[:, 3:], axis=1)
    total = 0.0
    for b in range(mesh.nblocks):
        x = [geom[b, q] + (np.arange(bnx[q]) + 0.5) * geom[b, 3 + q] for q in range(3)]
        val = np.zeros((bnx[2], bnx[1], bnx[0]))
        for c, a in zip(centres, amps):
            d = [x[q] - c[q] for q in range(3)]
            d = [dd - np.round(dd) for dd in d]
            r2 = d[2][:, None, None] ** 2 + d[1][None, :, None] ** 2 + d[0][None, None, :] ** 2
            val += a * np.exp(-r2 / (2.0 * sigma * sigma))
        out[b, ng:ng + bnx[2], ng:ng + bnx[1], ng:ng + bnx[0]] = val
        total += val.sum() * vols[b]
    volume = float(np.sum(vols)) * bnx[0] * bnx[1] * bnx[2]
    out[:, ng:ng + bnx[2], ng:ng + bnx[1], ng:ng + bnx[0]] -= total / volume
    return out
