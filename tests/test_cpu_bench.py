"""CPU checks of bench.py's measurement arithmetic: the per-point byte
formulas behind the roofline, the bucket-tree size, the committed ncu
traffic figures it scales, and the clock record it attaches to every line
(parsed from an nvidia-smi CSV written here)."""
import os

import pytest

from conftest import ROOT


def test_boruvka_round_bytes_per_point():
    """Per round and point: k kNN edges of 12 bytes, coordinates + core +
    component + candidate (4d + 16), the relabel read and write (8); per
    component 8.  At the benchmark's k = 16, d = 3: 228 bytes per point."""
    from bench import boruvka_round_bytes

    n = 1_000_000
    assert boruvka_round_bytes(n, 16, 3, 0) == 228 * n
    assert boruvka_round_bytes(n, 16, 3, 1000) == 228 * n + 8 * 1000
    assert boruvka_round_bytes(10, 2, 5, 3) == 10 * (24 + 36 + 8) + 24


def test_knn_stage_bytes_per_point():
    from bench import knn_stage_bytes

    # 4d (read X) + 2 (4d + 8) (sort write + read) + 8k (rows) + 4 (core)
    assert knn_stage_bytes(1, 16, 3) == 12 + 40 + 128 + 4
    assert knn_stage_bytes(1000, 16, 3) == 184 * 1000


def test_tree_nodes_and_narrow_bytes():
    from bench import algorithmic_bytes, tree_nodes

    assert tree_nodes(32) == 1 and tree_nodes(33) == 3 and tree_nodes(1000) == 63
    n, k, p = 4096, 16, 4
    assert algorithmic_bytes("knn_kernel", n, k, p) == n * (16 + 4) + n * k * 8 + n * 15 * 4 + n
    assert algorithmic_bytes("search_kernel", n, k, p) == n * 21 + tree_nodes(n) * 8
    assert algorithmic_bytes("other_kernel", n, k, p) is None


def test_high_dimensional_gemm_depth():
    """Two bf16 terms make the candidate GEMM 3 x the padded width deep,
    rounded up to whole 64-element rows on the tcgen05 path."""
    from bench import hd_kernel_depth

    assert hd_kernel_depth(12) == 128 and hd_kernel_depth(32) == 128
    assert hd_kernel_depth(40) == 192 and hd_kernel_depth(64) == 192
    assert hd_kernel_depth(96) == 288


def test_traffic_per_point_reads_the_committed_summary():
    from bench import traffic_per_point

    path = os.path.join(ROOT, "profiles", "ncu_traffic_per_point.txt")
    kernels = [ln.split()[0] for ln in open(path) if len(ln.split()) == 2]
    assert kernels, "no '<kernel> <bytes>' lines"
    for name in kernels:
        assert traffic_per_point(name) > 0
    assert traffic_per_point("no_such_kernel") is None


class _Exited:
    def terminate(self):
        pass

    def wait(self, timeout=None):
        return 0


@pytest.mark.parametrize("rows,median,reasons", [
    (["0, 2070, 2070, 900.1, 0x0, Not Active, Not Active, Not Active, Not Active"] * 3,
     2070.0, []),
    (["0, 1980, 2070, 1390.0, 0x4, Not Active, Not Active, Not Active, Active",
      "0, 2070, 2070, 1200.0, 0x0, Not Active, Not Active, Not Active, Not Active",
      "0, 1900, 2070, 1400.0, 0x4, Not Active, Not Active, Not Active, Active"],
     1980.0, ["sw_power_cap"]),
    (["0, 1200, 2070, 700.0, 0x8, Active, Not Active, Active, Not Active",
      "garbage line",
      "0, [N/A], 2070, 700.0, 0x8, Active, Not Active, Active, Not Active",
      "0, 1300, 2070, 700.0, 0x8, Active, Not Active, Active, Not Active"],
     1250.0, ["hw_slowdown", "sw_thermal_slowdown"]),
])
def test_clock_record_from_nvidia_smi_csv(tmp_path, rows, median, reasons):
    """The clocks key: median SM clock under load, the maximum, and every
    throttle reason seen active in any sample (unparsable lines skipped)."""
    from bench import ClockSampler

    path = tmp_path / "clocks.csv"
    path.write_text("\n".join(rows) + "\n")
    cs = ClockSampler(0)
    cs.proc, cs.path = _Exited(), str(path)
    out = cs.summary()
    assert out["sm_mhz"] == median and out["sm_max_mhz"] == 2070.0
    assert out["reasons"] == reasons
    assert out["samples"] == sum(1 for r in rows if r.count(",") >= 8 and "[N/A]" not in r)


def test_clock_record_without_nvidia_smi():
    from bench import ClockSampler

    out = ClockSampler(0).summary()
    assert out["sm_mhz"] is None and out["reasons"] == ["nvidia-smi unavailable"]
