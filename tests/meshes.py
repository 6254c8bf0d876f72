"""Mesh layouts shared by the parity tests."""


def refined_cube(root_level, lo, hi):
    """Leaves one level below `root_level` covering root blocks lo..hi-1 in every
    direction (a statically refined central region)."""
    out = []
    for k in range(lo, hi):
        for j in range(lo, hi):
            for i in range(lo, hi):
                for dk in (0, 1):
                    for dj in (0, 1):
                        for di in (0, 1):
                            out.append((root_level + 1, 2 * i + di, 2 * j + dj, 2 * k + dk))
    return out


def two_level_nested(root_level, lo, hi, inner_lo, inner_hi):
    """Refined cube with a further refined cube inside it (three levels)."""
    out = refined_cube(root_level, lo, hi)
    fine = root_level + 1
    for k in range(inner_lo, inner_hi):
        for j in range(inner_lo, inner_hi):
            for i in range(inner_lo, inner_hi):
                for dk in (0, 1):
                    for dj in (0, 1):
                        for di in (0, 1):
                            out.append((fine + 1, 2 * i + di, 2 * j + dj, 2 * k + dk))
    return out


# (name, nx, block_nx, nghost, leaves)
INDEX_MAP_CASES = [
    ("uniform-64-16cubed-ng2", (64, 64, 64), (16, 16, 16), 2, None),
    ("uniform-g4", (64, 64, 64), (16, 16, 16), 4, None),
    ("smr-small", (64, 64, 64), (16, 16, 16), 4, refined_cube(2, 1, 3)),
    ("smr-128root-16cubed-ng4", (128, 128, 128), (16, 16, 16), 4, refined_cube(3, 2, 6)),
    ("smr-corner", (64, 64, 64), (8, 8, 8), 2, refined_cube(3, 0, 2)),
    ("three-level", (64, 64, 64), (8, 8, 8), 4, two_level_nested(3, 2, 6, 6, 10)),
    # smallest meshes: one block that is its own neighbour in all 26 directions, and
    # 2x2x2 blocks that meet every neighbour across two periodic images
    ("single-block", (16, 16, 16), (16, 16, 16), 2, None),
    ("two-per-dim", (32, 32, 32), (16, 16, 16), 4, None),
    ("two-per-dim-refined", (16, 16, 16), (8, 8, 8), 2, refined_cube(1, 0, 1)),
]


def gaussian_rhs(locs, geom, bnx, ng, ngauss=8, sigma=0.05, seed=5):
    """Right-hand side on leaf blocks (nblocks, N3, N2, N1): a sum of `ngauss` Gaussians
    with centres U[0,1]^3 and N(0,1) amplitudes, minus its volume-weighted mean, on the
    interiors (ghosts zero). locs/geom as Mesh.block_info()."""
    import numpy as np
    rng = np.random.default_rng(seed)
    cen = rng.random((ngauss, 3))
    amp = rng.normal(size=ngauss)
    nb = locs.shape[0]
    N = [b + 2 * ng for b in bnx]
    out = np.zeros((nb, N[2], N[1], N[0]))
    vols = np.prod(geom[:, 3:], axis=1)
    total = 0.0
    for b in range(nb):
        x0, dx = geom[b, :3], geom[b, 3:]
        xs = [x0[d] + (np.arange(bnx[d]) + 0.5) * dx[d] for d in range(3)]
        Z, Y, X = np.meshgrid(xs[2], xs[1], xs[0], indexing="ij")
        val = np.zeros_like(X)
        for q in range(ngauss):
            r2 = (X - cen[q, 0]) ** 2 + (Y - cen[q, 1]) ** 2 + (Z - cen[q, 2]) ** 2
            val += amp[q] * np.exp(-r2 / (2 * sigma ** 2))
        out[b, ng:ng + bnx[2], ng:ng + bnx[1], ng:ng + bnx[0]] = val
        total += val.sum() * vols[b]
    volume = sum(vols[b] * bnx[0] * bnx[1] * bnx[2] for b in range(nb))
    out[:, ng:ng + bnx[2], ng:ng + bnx[1], ng:ng + bnx[0]] -= total / volume
    return out


# (name, nx, block_nx, nghost, leaves) of the composite-grid multigrid cases
MG_CASES = [
    ("uniform-32-b8", (32, 32, 32), (8, 8, 8), 2, None),
    ("smr-32-b8", (32, 32, 32), (8, 8, 8), 2, refined_cube(2, 1, 3)),
    ("smr-64-b16-g4", (64, 64, 64), (16, 16, 16), 4, refined_cube(2, 1, 3)),
    ("smr-corner-32-b8", (32, 32, 32), (8, 8, 8), 2, refined_cube(2, 0, 2)),
    ("three-level-32-b4", (32, 32, 32), (4, 4, 4), 2, two_level_nested(3, 2, 6, 6, 10)),
]


def region_coefficient(locs, geom, bnx, ng, inside=10.0, outside=1.0):
    """Face coefficient D on leaf blocks (nblocks, 3, N3, N2, N1), face i the low face of
    cell i: `inside` where the face centre lies in the union of two boxes (the shape of
    the poisson_gmg example's inside_region, moved into the unit cube), else `outside`."""
    import numpy as np
    nb = locs.shape[0]
    N = [b + 2 * ng for b in bnx]
    out = np.full((nb, 3, N[2], N[1], N[0]), outside)

    def inside_region(x, y, z):
        a = (x > 0.125) & (x < 0.375) & (y > 0.25) & (y < 0.75) & (z > 0.375) & (z < 0.625)
        b = (x > 0.125) & (x < 0.75) & (y > 0.125) & (y < 0.375) & (z > 0.375) & (z < 0.625)
        return a | b

    for b in range(nb):
        x0, dx = geom[b, :3], geom[b, 3:]
        idx = [np.arange(N[d]) - ng for d in range(3)]
        cc = [x0[d] + (idx[d] + 0.5) * dx[d] for d in range(3)]
        fc = [x0[d] + idx[d] * dx[d] for d in range(3)]
        for dirn in range(3):
            c = [fc[d] if d == dirn else cc[d] for d in range(3)]
            Z, Y, X = np.meshgrid(c[2], c[1], c[0], indexing="ij")
            out[b, dirn] = np.where(inside_region(X, Y, Z), inside, outside)
    return out
