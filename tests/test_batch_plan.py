"""A CPU model of the batched step's work queue (k_batch_step in
landslidehysea_gb300/csrc/lsh_queue.cuh): its tilings (16 x 4 edge lines
horizontal, 8 x 8 vertical, 16 x 4 cells), the cell rows each item waits for
(item_rows, producer_rows) and the pass chain the ensemble builds
(lsh_batch.cu build_plan), restated in Python.  Every pair of items that
touch one array cell, one of them writing, must be ordered by a chain of
waits, or belong to one pass and touch disjoint cells.

The arrays are those of a batch scenario: the state X, the stage-1 output Y,
the accumulators, and the slopes, which both stages of a second-order step
share (the stage-2 reconstruction overwrites what the stage-1 edge passes
read).  The single-grid step's overlapped launches follow the same rules with
taller cell blocks (the last test)."""
import itertools
from collections import defaultdict

HX, HY, VX, VY, CX, CY = 16, 4, 8, 8, 16, 4


def tiles(nx, ny, kind):
    """(tiles per row, tile rows) of a tiling: queue_tiles."""
    if kind in ("h0", "h1"):
        p = int(kind[1])
        return (nx + HX - 1) // HX, ((ny - p) // 2 + 1 + HY - 1) // HY
    if kind in ("v0", "v1"):
        p = int(kind[1])
        return ((nx - p) // 2 + 1 + VX - 1) // VX, (ny + VY - 1) // VY
    return (nx + CX - 1) // CX, (ny + CY - 1) // CY


def item_rows(op, kind, ty, ny):
    """Cell rows an item reads: item_rows."""
    if kind in ("h0", "h1"):
        y0 = int(kind[1]) + 2 * HY * ty
        r0, r1 = y0 - 1, y0 + 2 * (HY - 1)
    elif kind in ("v0", "v1"):
        r0, r1 = VY * ty, VY * ty + VY - 1
    elif op.startswith("recon"):
        r0, r1 = CY * ty - 1, CY * ty + CY
    else:
        r0, r1 = CY * ty, CY * ty + CY - 1
    return max(r0, 0), min(r1, ny - 1)


def producer_rows(kind, r0, r1):
    """Tile rows of a pass of `kind` that write cell rows [r0, r1]: producer_rows."""
    if kind in ("v0", "v1"):
        return r0 // VY, r1 // VY
    if kind == "cell":
        return r0 // CY, r1 // CY
    p = int(kind[1])
    return (max(r0 - p + 1, 0) // 2) // HY, (max(r1 + 1 - p, 0) // 2) // HY


def edges_of(kind, tx, ty, nx, ny):
    """Per edge of an edge tile, the cells it joins."""
    out = []
    p = int(kind[1])
    if kind[0] == "h":
        for w in range(HY):
            for u in range(HX):
                x, line = tx * HX + u, ty * HY + w
                if x < nx and line < (ny - p) // 2 + 1:
                    y = p + 2 * line
                    out.append([(x, yy) for yy in (y - 1, y) if 0 <= yy < ny])
    else:
        for w in range(VY):
            for u in range(VX):
                t, y = tx * VX + u, ty * VY + w
                x = p + 2 * t
                if x <= nx and y < ny:
                    out.append([(xx, y) for xx in (x - 1, x) if 0 <= xx < nx])
    return out


def cells_of(tx, ty, nx, ny):
    return [(tx * CX + u, ty * CY + w) for w in range(CY) for u in range(CX)
            if tx * CX + u < nx and ty * CY + w < ny]


def footprint(op, kind, tx, ty, nx, ny, order):
    """(reads, writes): sets of (array, i, j).  Stage s reads state W_s
    (X for stage 1, Y for stage 2); the volume of stage 1 writes Y, of stage 2
    (or of a first-order step) writes X."""
    R, W = set(), set()
    st = op[-1]
    w_in = "X" if st == "1" else "Y"
    if op.startswith("recon"):
        for i, j in cells_of(tx, ty, nx, ny):
            W.add(("slope", i, j))
            for di, dj in ((0, 0), (1, 0), (-1, 0), (0, 1), (0, -1)):
                if 0 <= i + di < nx and 0 <= j + dj < ny:
                    R.add((w_in, i + di, j + dj))
        return R, W
    if op.startswith("vol"):
        for i, j in cells_of(tx, ty, nx, ny):
            R.update({(w_in, i, j), ("acc", i, j)})
            if order == 2:
                R.add(("slope", i, j))
            if st == "1" and order == 2:
                W.add(("Y", i, j))
            else:
                R.add(("X", i, j))
                W.add(("X", i, j))
        return R, W
    first = op.startswith("h0")
    for cs in edges_of(kind, tx, ty, nx, ny):
        for i, j in cs:
            R.add((w_in, i, j))
            if order == 2:
                R.add(("slope", i, j))
            if not first:
                R.add(("acc", i, j))
            W.add(("acc", i, j))
    return R, W


def passes(order):
    """The chain of build_plan: per stage reconstruction (order 2), the four
    colour passes, the Euler stage; each waits for the pass before it."""
    out = []
    for st in ("1", "2") if order == 2 else ("1",):
        if order == 2:
            out.append(("recon" + st, "cell"))
        out += [("h0_" + st, "h0"), ("h1_" + st, "h1"), ("v0_" + st, "v0"), ("v1_" + st, "v1"), ("vol" + st, "cell")]
    return out


def check(nx, ny, order, rows=item_rows):
    P = passes(order)
    items = [(p, tx, ty) for p, (_, kind) in enumerate(P)
             for ty in range(tiles(nx, ny, kind)[1]) for tx in range(tiles(nx, ny, kind)[0])]
    idx = {it: k for k, it in enumerate(items)}
    anc = [0] * len(items)
    for k, (p, tx, ty) in enumerate(items):
        if p == 0:
            continue
        op, kind = P[p]
        pk = P[p - 1][1]
        r0, r1 = rows(op, kind, ty, ny)
        t0, t1 = producer_rows(pk, r0, r1)
        ptx, pty = tiles(nx, ny, pk)
        m = 0
        for r in range(max(t0, 0), min(t1, pty - 1) + 1):
            for x in range(ptx):
                d = idx[(p - 1, x, r)]
                m |= anc[d] | (1 << d)
        anc[k] = m
    fps = [footprint(P[p][0], P[p][1], tx, ty, nx, ny, order) for (p, tx, ty) in items]
    touch = defaultdict(list)
    for k, (R, W) in enumerate(fps):
        for c in R | W:
            touch[c].append(k)
    bad = 0
    for c, ks in touch.items():
        for a, b in itertools.combinations(ks, 2):
            Ra, Wa = fps[a]
            Rb, Wb = fps[b]
            if not ((c in Wa and (c in Rb or c in Wb)) or (c in Wb and c in Ra)):
                continue
            if items[a][0] == items[b][0]:
                bad += 1
                continue
            lo, hi = min(a, b), max(a, b)
            if not (anc[hi] >> lo) & 1:
                bad += 1
    return bad


SHAPES = [(37, 29), (19, 70), (40, 24), (1, 1), (1, 7), (9, 1), (33, 17)]


def test_second_order_step_orders_every_conflict():
    for nx, ny in SHAPES:
        assert check(nx, ny, 2) == 0, (nx, ny)


def test_first_order_step_orders_every_conflict():
    for nx, ny in SHAPES:
        assert check(nx, ny, 1) == 0, (nx, ny)


def test_model_flags_a_reconstruction_without_its_halo_rows():
    # without the reconstruction's rows above and below its tile, its stencil
    # reads of the previous stage's output are no longer ordered after it
    def narrow(op, kind, ty, ny):
        return item_rows("vol" if op.startswith("recon") else op, kind, ty, ny)
    assert check(37, 29, 2, rows=narrow) > 0


def test_single_grid_overlapped_step_orders_every_conflict(monkeypatch):
    """The single-grid step's overlapped launches (lsh_kernels.cuh: dep_begin
    in k_recon, k_edges_h/v, k_volume) use the same row rules and edge
    blocks, with cell blocks 16 rows high."""
    monkeypatch.setitem(globals(), "CY", 16)
    for nx, ny in [(40, 70), (37, 33), (1, 40), (20, 1)]:
        assert check(nx, ny, 2) == 0, (nx, ny)
        assert check(nx, ny, 1) == 0, (nx, ny)
