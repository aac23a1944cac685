"""TEST INFRASTRUCTURE ONLY: lid-driven cavity meshes in the reference's file
format, generated with numpy alone.

The CPU legs of bench.py build their sample cavity here so that the process
timing the reference's arithmetic never loads the GPU library.  The layout is
that of the reference's shipped cases (``cases/coarse``, ``cases/medium``):
fluid cells i, j in [1, side], a solid ring, one extra solid row on top, the
unit square as the physical domain, the lid (type 2, ID 2) on top and
bounce-back walls west = 1, east = 3, south = 4 (type 1).  Node lines are
``i j x y fluid`` and link lines ``i j dir type x y id`` (serial/FileIO.c:39-44
and :116-133).  The links are those of ``lbm_mesh_cavity`` of the library, line
for line (``tests/test_oracle.py`` checks the two against each other).
"""
import numpy as np

# D2Q9 lattice directions of the reference (serial/CellFunctions.c:11-92)
MCX = (0, 1, 0, -1, 0, 1, -1, -1, 1)
MCY = (0, 0, 1, 0, -1, 1, 1, -1, -1)


def _box_exit(px, py, dx, dy):
    """First crossing of the ray (px, py) + t (dx, dy) with the unit square's
    sides; a tie between a vertical and a horizontal side goes to the
    horizontal one.  Returns (x, y, side) with side 0 west, 1 east, 2 south,
    3 north, the coordinate on the side snapped to it."""
    tx = ty = 1e300
    sx = sy = -1
    if dx < 0:
        tx, sx = (0.0 - px) / dx, 0
    if dx > 0:
        tx, sx = (1.0 - px) / dx, 1
    if dy < 0:
        ty, sy = (0.0 - py) / dy, 2
    if dy > 0:
        ty, sy = (1.0 - py) / dy, 3
    if ty <= tx + 1e-9:
        t, side = ty, sy
    else:
        t, side = tx, sx
    x, y = px + t * dx, py + t * dy
    if side == 0:
        x = 0.0
    elif side == 1:
        x = 1.0
    elif side == 2:
        y = 0.0
    elif side == 3:
        y = 1.0
    return x, y, side


def cavity(side):
    """(nodes [N, 5] float32, conns [C, 7] float32, (n, m)) of a side^2 cavity."""
    if side < 2:
        raise ValueError("cavity side must be >= 2")
    n, m = side + 2, side + 3
    d = 1.0 / side
    jj, ii = np.meshgrid(np.arange(m), np.arange(n), indexing="ij")
    fluid = (ii >= 1) & (ii <= side) & (jj >= 1) & (jj <= side)
    nodes = np.empty((m, n, 5), np.float32)
    nodes[..., 0] = ii
    nodes[..., 1] = jj
    nodes[..., 2] = ((ii - 0.5) * d).astype(np.float32)
    nodes[..., 3] = ((jj - 0.5) * d).astype(np.float32)
    nodes[..., 4] = fluid
    ids = (1, 3, 4, 2)  # west, east, south, north (lid)
    rows = []
    # only the fluid ring next to the walls has links to solid cells
    for j in range(1, side + 1):
        cols = range(1, side + 1) if j in (1, side) else (1, side)
        for i in cols:
            for k in range(1, 9):
                a, b = i + MCX[k], j + MCY[k]
                if 1 <= a <= side and 1 <= b <= side:
                    continue
                x, y, s = _box_exit((i - 0.5) * d, (j - 0.5) * d, MCX[k] * d, MCY[k] * d)
                rows.append((i, j, k, 2 if s == 3 else 1, np.float32(x), np.float32(y), ids[s]))
    conns = np.array(rows, np.float32).reshape(-1, 7)
    return nodes.reshape(-1, 5), conns, (n, m)
