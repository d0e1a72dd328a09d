"""Writers of small data.dat / .bat / .ini / gauge cases for the tests."""
import numpy as np


def write_case(tmp, *, nx=6, ny=4, normalizar=1, gauges_line="0.85", extra_gauge_file=None, land=True):
    """A data.dat in the reference's field order (main.cxx:24-60) with its
    .bat (xmin xmax ymin ymax nx ny, then depths row by row) and .ini (six
    values per cell: h1 q1x q1y h2 q2x q2y) as text."""
    rng = np.random.default_rng(7)
    depth = rng.uniform(20.0, 80.0, (ny, nx))
    if land:
        depth[0, 0] = -12.5  # one land cell: the loader shifts H by Hmin
    h2 = np.where(depth > 30, 2.0, 0.0)
    h1 = np.maximum(depth - h2, 0.0)
    q = rng.uniform(-1, 1, (4, ny, nx))
    with open(tmp / "topo.bat", "w") as f:
        f.write(f"0 {nx * 50.0} 0 {ny * 40.0} {nx} {ny}\n")
        f.write("\n".join(f"{v:.6f}" for v in depth.ravel()) + "\n")
    with open(tmp / "state.ini", "w") as f:
        for c in range(nx * ny):
            j, i = divmod(c, nx)
            f.write(f"{h1[j, i]:.6f} {q[0, j, i]:.6f} {q[1, j, i]:.6f} {h2[j, i]:.6f} {q[2, j, i]:.6f} {q[3, j, i]:.6f}\n")
    lines = ["my_bathymetry", "1", "topo.bat", "state.ini", "-1", "1", "0", "1", "12.5", "2.0"]
    if extra_gauge_file:
        lines += ["1", extra_gauge_file]
    else:
        lines += [gauges_line]           # gauge flag read as int: "0.85" -> 0, ".85" left for CFL
    if extra_gauge_file:
        lines += ["0.8"]
    lines += ["0.45", "11", "0.01", "0.02", "0.03", "15", "25", str(normalizar)]
    if normalizar:
        lines += ["1000", "100"]
    lines += ["out/run1"]
    (tmp / "data.dat").write_text("\n".join(lines) + "\n")
    return depth, h1, h2, q
