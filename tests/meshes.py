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
    ("C1-uniform-64", (64, 64, 64), (16, 16, 16), 2, None),
    ("uniform-g4", (64, 64, 64), (16, 16, 16), 4, None),
    ("smr-small", (64, 64, 64), (16, 16, 16), 4, refined_cube(2, 1, 3)),
    ("C3-smr-128", (128, 128, 128), (16, 16, 16), 4, refined_cube(3, 2, 6)),
    ("smr-corner", (64, 64, 64), (8, 8, 8), 2, refined_cube(3, 0, 2)),
    ("three-level", (64, 64, 64), (8, 8, 8), 4, two_level_nested(3, 2, 6, 6, 10)),
    # smallest meshes: one block that is its own neighbour in all 26 directions, and
    # 2x2x2 blocks that meet every neighbour across two periodic images
    ("single-block", (16, 16, 16), (16, 16, 16), 2, None),
    ("two-per-dim", (32, 32, 32), (16, 16, 16), 4, None),
    ("two-per-dim-refined", (16, 16, 16), (8, 8, 8), 2, refined_cube(1, 0, 1)),
]
