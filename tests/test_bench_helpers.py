"""bench.py's helpers that need no GPU: the roofline traffic read from the
committed ncu summaries (profiles/), and the workload builders' shapes."""
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def test_roofline_traffic_comes_from_the_committed_summaries():
    import bench
    for kernel, workload in (("k_pre5", "poisson_guided_2048x2048x3"), ("k_post5", "poisson_guided_2048x2048x3"),
                             ("k_spmv5", "poisson_guided_2048x2048x3"), ("k_amle_fused", "amle_2048x2048x1")):
        t = bench.ncu_traffic(kernel, workload)
        assert t is not None, kernel
        assert t["traffic"] > 1e6, (kernel, t)
        assert t["traffic_source"].startswith(f"profiles/{kernel}_{workload}.md")
    t = bench.ncu_traffic("k_pre5", "poisson_guided_2048x2048x3")
    assert t["traffic_algorithmic"] and 0.3 < t["traffic"] / t["traffic_algorithmic"] < 3
    assert bench.ncu_traffic("no_such_kernel", "nowhere") is None


def test_headline_workload_shape():
    import bench
    insts, name = bench.make_workload("c0", 0)
    assert insts[0].g.shape == (1, 512, 512) and "laplace-512x512x1" in name
