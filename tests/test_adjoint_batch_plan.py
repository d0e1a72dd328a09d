"""A CPU model of the batched adjoint's reverse queue (k_adjb_reverse in
landslidehysea_gb300/csrc/lsh_adjoint.cu): its tilings (the single adjoint
kernels' blocks), the cell rows each item waits for (r_item_rows,
r_producer_rows) and the pass plan of build_rplan, restated in Python.  Every
pair of items that touch one array cell, one of them writing, must be ordered
by a chain of waits, or belong to one pass and touch disjoint cells.  The
arrays are the adjoints the passes write: the new state adjoint (Xbn), the
stage-1 output's adjoint (Yb), the accumulator and slope adjoints, and the
rate selection."""
import itertools
from collections import defaultdict


def tiles(nx, ny, kind):
    """(tiles per row, tile rows) of a tiling: adj_tiles / adj_edge_grid / adj_cell_grid."""
    if kind == 'member': return 1, 1
    if kind == 'cell': return (nx + 15) // 16, (ny + 7) // 8
    par = int(kind[1])
    if kind[0] == 'h':
        nl = (ny - par) // 2 + 1
        return (nx + 15) // 16, (nl + 7) // 8
    nl = (nx - par) // 2 + 1
    return (nl + 7) // 8, (ny + 15) // 16


def item_rows(op, kind, ty, ny):
    """Cell rows an item reads or overwrites: r_item_rows."""
    if kind in ('h0', 'h1'):
        y0 = int(kind[1]) + 16 * ty; r0, r1 = y0 - 1, y0 + 14
    elif kind in ('v0', 'v1'):
        r0 = 16 * ty; r1 = r0 + 15
    elif op in ('recon', 'vol1'):
        r0, r1 = 8 * ty - 1, 8 * ty + 8
    else:
        r0, r1 = 8 * ty, 8 * ty + 7
    return max(r0, 0), min(r1, ny - 1)


def producer_rows(kind, r0, r1):
    """Tile rows of a pass of `kind` touching cell rows [r0, r1]: r_producer_rows."""
    if kind in ('v0', 'v1'): return r0 // 16, r1 // 16
    if kind == 'cell': return r0 // 8, r1 // 8
    if kind == 'member': return 0, 0
    p = int(kind[1])
    return (max(r0 - p + 1, 0) // 2) // 8, (max(r1 + 1 - p, 0) // 2) // 8


def cells_of(kind, tx, ty, nx, ny):
    """The cells of a cell tile, or per edge of an edge tile the cells it joins."""
    out = []
    if kind == 'cell':
        for w in range(8):
            for u in range(16):
                i, j = tx * 16 + u, ty * 8 + w
                if i < nx and j < ny: out.append(('c', i, j))
        return out
    par = int(kind[1])
    if kind[0] == 'h':
        for w in range(8):
            for u in range(16):
                x, line = tx * 16 + u, ty * 8 + w
                if x < nx and line < (ny - par) // 2 + 1:
                    y = par + 2 * line
                    cs = []
                    if y >= 1: cs.append((x, y - 1))
                    if y <= ny - 1: cs.append((x, y))
                    out.append(('e', cs))
    else:
        for w in range(16):
            for u in range(8):
                t, y = tx * 8 + u, ty * 16 + w
                if t < (nx - par) // 2 + 1 and y < ny:
                    x = par + 2 * t
                    cs = []
                    if x >= 1: cs.append((x - 1, y))
                    if x <= nx - 1: cs.append((x, y))
                    out.append(('e', cs))
    return out


def footprint(op, kind, tx, ty, nx, ny):
    """(reads, writes): sets of (array, i, j)."""
    R, W = set(), set()
    if op in ('ratemax', 'argmax', 'ratebar'):
        if op == 'ratemax': W.add(('rmax', 0, 0))
        if op == 'argmax': R.add(('rmax', 0, 0)); W.add(('argmax', 0, 0))
        if op == 'ratebar': R.update({('rmax', 0, 0), ('argmax', 0, 0)}); W.add(('rsel', 0, 0))
        return R, W
    if kind == 'cell':
        for _, i, j in cells_of(kind, tx, ty, nx, ny):
            if op == 'zero': W.update({('Yb', i, j), ('Xbn', i, j)})
            elif op == 'vol2':
                W.update({('accb', i, j), ('sb', i, j), ('Yb', i, j), ('Xbn', i, j)}); R.update({('Yb', i, j), ('Xbn', i, j)})
            elif op == 'vol1':
                R.update({('rsel', 0, 0), ('Yb', i, j), ('Xbn', i, j)}); W.update({('accb', i, j), ('sb', i, j), ('Xbn', i, j)})
            elif op in ('recon2', 'recon1'):
                tgt = 'Yb' if op == 'recon2' else 'Xbn'
                R.add((tgt, i, j)); W.add((tgt, i, j))
                for di, dj in ((0, 0), (1, 0), (-1, 0), (0, 1), (0, -1)):
                    if 0 <= i + di < nx and 0 <= j + dj < ny: R.add(('sb', i + di, j + dj))
        return R, W
    stage = op[-1]
    tgt = 'Yb' if stage == '2' else 'Xbn'
    for _, cs in cells_of(kind, tx, ty, nx, ny):
        for (i, j) in cs:
            R.update({('accb', i, j), (tgt, i, j), ('sb', i, j)}); W.update({(tgt, i, j), ('sb', i, j)})
            if stage == '1': R.add(('rsel', 0, 0))
    return R, W

PASSES2 = [  # op, kind, prod, fprod  (the plan of build_rplan, order 2)
    ('zero', 'cell', -1, -1), ('ratemax', 'cell', -1, -1), ('argmax', 'cell', -1, 1), ('ratebar', 'member', -1, 2),
    ('vol2', 'cell', 0, -1), ('ev1_2', 'v1', 4, -1), ('ev0_2', 'v0', 5, -1), ('eh1_2', 'h1', 6, -1), ('eh0_2', 'h0', 7, -1),
    ('recon2', 'cell', 8, -1), ('vol1', 'cell', 9, 3), ('ev1_1', 'v1', 10, -1), ('ev0_1', 'v0', 11, -1),
    ('eh1_1', 'h1', 12, -1), ('eh0_1', 'h0', 13, -1), ('recon1', 'cell', 14, -1)]


def check(nx, ny, passes):
    """Conflicting item pairs that no chain of waits orders, and the item count."""
    items = []  # (pass, tx, ty)
    for p, (op, kind, _, _) in enumerate(passes):
        tx_n, ty_n = tiles(nx, ny, kind)
        for ty in range(ty_n):
            for tx in range(tx_n):
                items.append((p, tx, ty))
    idx = {it: k for k, it in enumerate(items)}
    deps = defaultdict(set)
    for k, (p, tx, ty) in enumerate(items):
        op, kind, prod, fprod = passes[p]
        key_op = 'recon' if op.startswith('recon') else op
        if prod >= 0:
            pk = passes[prod][1]
            r0, r1 = item_rows(key_op, kind, ty, ny)
            t0, t1 = producer_rows(pk, r0, r1)
            ptx, pty = tiles(nx, ny, pk)
            t0, t1 = max(t0, 0), min(t1, pty - 1)
            for r in range(t0, t1 + 1):
                for x in range(ptx): deps[k].add(idx[(prod, x, r)])
        if fprod >= 0:
            pk = passes[fprod][1]
            ptx, pty = tiles(nx, ny, pk)
            for r in range(pty):
                for x in range(ptx): deps[k].add(idx[(fprod, x, r)])
        for d in deps[k]: assert d < k
    # transitive closure as bitsets
    anc = [0] * len(items)
    for k in range(len(items)):
        m = 0
        for d in deps[k]: m |= anc[d] | (1 << d)
        anc[k] = m
    fps = [footprint(passes[p][0], passes[p][1], tx, ty, nx, ny) for (p, tx, ty) in items]
    touch = defaultdict(list)
    for k, (R, W) in enumerate(fps):
        for c in R | W: touch[c].append(k)
    bad = 0
    for c, ks in touch.items():
        for a, b in itertools.combinations(ks, 2):
            Ra, Wa = fps[a]; Rb, Wb = fps[b]
            conflict = (c in Wa and (c in Rb or c in Wb)) or (c in Wb and c in Ra)
            if not conflict: continue
            if c[0] in ('rmax', 'argmax') and items[a][0] == items[b][0]: continue  # atomics within a pass
            if items[a][0] == items[b][0]:
                bad += 1
                continue
            lo, hi = (a, b) if a < b else (b, a)
            if not (anc[hi] >> lo) & 1:
                bad += 1
    return bad, len(items)


PASSES1 = [  # order 1: the step's volume adjoint reads the rate selection
    ('zero', 'cell', -1, -1), ('ratemax', 'cell', -1, -1), ('argmax', 'cell', -1, 1), ('ratebar', 'member', -1, 2),
    ('vol1', 'cell', 0, 3), ('ev1_1', 'v1', 4, -1), ('ev0_1', 'v0', 5, -1), ('eh1_1', 'h1', 6, -1),
    ('eh0_1', 'h0', 7, -1)]

SHAPES = [(37, 29), (16, 8), (23, 9), (40, 33), (1, 1), (5, 70)]


def test_second_order_plan_orders_every_conflict():
    for nx, ny in SHAPES:
        bad, n = check(nx, ny, PASSES2)
        assert bad == 0, (nx, ny)


def test_first_order_plan_orders_every_conflict(monkeypatch):
    # first order: the volume adjoint writes no slope adjoint a reconstruction reads,
    # and the kernel gives it no row extension (kRVol0)
    orig = item_rows
    monkeypatch.setitem(globals(), "item_rows", lambda op, kind, ty, ny: orig("vol0" if op == "vol1" else op, kind, ty, ny))
    for nx, ny in SHAPES[:4]:
        bad, n = check(nx, ny, PASSES1)
        assert bad == 0, (nx, ny)


def test_model_flags_a_missing_row_extension(monkeypatch):
    # without the stage-1 volume's extra row, the stage-2 reconstruction adjoint's
    # reads of slope adjoints one row away are no longer ordered before it
    orig = item_rows
    monkeypatch.setitem(globals(), "item_rows", lambda op, kind, ty, ny: orig("vol" if op == "vol1" else op, kind, ty, ny))
    bad, n = check(37, 29, PASSES2)
    assert bad > 0
