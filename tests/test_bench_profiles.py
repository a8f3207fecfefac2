"""bench.py reads two figures of its roofline object from the committed ncu
summary (profiles/ncu_traffic.txt): the dominant kernel's DRAM bytes per
launch and the FP64 pipe activity of the same capture."""
import bench


def test_traffic_and_pipe_figures_come_from_the_committed_summary():
    t = bench.traffic_from_profiles("beam98k_nh_newmark", "pcg_persistent_kernel")
    pct = bench.traffic_from_profiles("beam98k_nh_newmark", "pcg_persistent_kernel", "fp64_pipe_pct")
    assert t is not None and t > 1e6
    assert pct is not None and 0.0 < pct <= 100.0


def test_unknown_entries_read_as_missing():
    assert bench.traffic_from_profiles("no_such_workload", "pcg_persistent_kernel") is None
    assert bench.traffic_from_profiles("beam98k_nh_newmark", "invhyper_kernel", "fp64_pipe_pct") is None
