"""bench.py's roofline arithmetic (no GPU): the step's algorithmic bytes,
the per-step sums of the ncu counters, and the source hash that keys them."""
import os
import shutil

import pytest


def test_algorithmic_bytes_per_cell_step():
    import bench
    # first order: read 6 state + H, write 6; TVD-RK2 adds stage 2's 6 + H + 6 read, 6 written
    assert bench.ALGO_BYTES_PER_CELL_STEP == {1: 13 * 8, 2: 13 * 8 + 19 * 8}


def test_step_counter_sums():
    import bench
    d = bench.FJORD2048_DRAM_BYTES_PER_LAUNCH
    edges = d["edge_h0"] + d["edge_h1"] + d["edge_v0"] + d["edge_v1"]
    assert bench.edge_dram_bytes() == pytest.approx(2 * edges)
    assert bench.step_dram_bytes() == pytest.approx(2 * (edges + d["recon"]) + d["volume1"] + d["volume2"])


def test_counters_follow_the_kernel_sources(tmp_path, monkeypatch):
    import bench
    h = bench.source_hash()
    assert len(h) == 16 and h == bench.source_hash()
    # a copy of the sources with one byte changed hashes differently
    root = tmp_path / "repo"
    for rel in bench.COUNTER_SOURCES:
        dst = root / rel
        dst.parent.mkdir(parents=True, exist_ok=True)
        shutil.copy(os.path.join(bench.ROOT, rel), dst)
    monkeypatch.setattr(bench, "ROOT", str(root))
    assert bench.source_hash() == h
    with open(root / bench.COUNTER_SOURCES[0], "a") as f:
        f.write(" ")
    assert bench.source_hash() != h
    assert not bench.counters_current() or bench.COUNTERS_SOURCE_HASH != h
