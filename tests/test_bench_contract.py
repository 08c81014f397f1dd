"""CPU checks of what bench.py reports beside its measurement: the DRAM
traffic of its roofline comes from the committed ncu summary of the kernel
the solver runs, and that summary's capture names the same kernel."""
import os
import re
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def test_roofline_traffic_is_the_product_kernels_capture():
    import bench
    traffic = bench.load_traffic()
    cells = 100 * 256 * 128
    # DRAM bytes per sweep of the 100x256x128 system: positive and below the
    # algorithmic 40 B per cell (its 131 MB about fill the L2)
    assert traffic is not None and 0 < traffic < bench.BYTES_FP32_SWEEP * cells
    summary = open(os.path.join(ROOT, "profiles", "sweeps32_local_shell256.md")).read()
    assert "-k regex:sweeps32_local" in summary
    assert re.search(r"^traffic_bytes_per_sweep: %d$" % traffic, summary, re.M)


def test_roofline_names_the_kernel_it_times():
    """The kernel bench.py names in its roofline is the one ttfld_time_sweeps
    runs for TTFLD_SOLVER_MIXED (the neighbour-flag kernel of sweep_form 0)."""
    src = open(os.path.join(ROOT, "bench.py")).read()
    named = set(re.findall(r'"kernel": "(\w+) \(one full sweep\)"', src))
    assert named == {"sweeps32_local"}
    cu = open(os.path.join(ROOT, "ttcode_gb300", "csrc", "ttfld_mixed.cu")).read()
    assert "sweeps32_local<POLES>, dim3(gr.local)" in cu
    assert re.search(r"solver == 6 \? kFormGrid", cu) and re.search(r":\s+kFormNeighbour;", cu)
