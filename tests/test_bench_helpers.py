"""bench.py's helpers that need no GPU: the roofline traffic read from the
committed ncu summaries (profiles/), and the workload builders' shapes."""
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def test_roofline_traffic_comes_from_the_committed_summaries():
    import bench
    for kernel, workload in (("k_pre5", "batched_256_uneven"), ("k_post5", "batched_256_uneven"),
                             ("k_spmv5", "batched_256_uneven"), ("k_amle_fused", "amle_2048x2048x1")):
        t = bench.ncu_traffic(kernel, workload)
        assert t is not None, kernel
        assert t["traffic"] > 1e6, (kernel, t)
        assert t["traffic_source"].startswith(f"profiles/{kernel}_{workload}.md")
    t = bench.ncu_traffic("k_pre5", bench.PROFILE_NAMES["c3"])
    assert t["traffic_algorithmic"] and 0.3 < t["traffic"] / t["traffic_algorithmic"] < 3
    assert bench.ncu_traffic("no_such_kernel", "nowhere") is None


def test_workload_shapes():
    import bench
    insts = bench.make_workload("c0", 0)
    assert insts[0].g.shape == (1, 512, 512) and "laplace-512x512x1" in bench.WORKLOADS["c0"]


def test_both_arms_print_the_same_config():
    """The reference arm and the GPU arm describe the same workload with the
    same dict (the same input sets, seeds and sizes)."""
    import argparse
    import bench
    from imscript_gb300 import synth
    args = argparse.Namespace(workload="c1s")
    sets = [bench.make_workload("c1s", sd) for sd in bench.input_seeds(0, 2)]
    cfg = bench.bench_config(args, sets)
    again = bench.bench_config(args, [bench.make_workload("c1s", sd) for sd in bench.input_seeds(0, 2)])
    assert cfg == again
    assert cfg["rtol"] == 1e-6 and cfg["instances_per_step"] == 1
    assert cfg["unknown_samples_per_step"] == round(sum(s[0].unknowns for s in sets) / 2)
    assert synth.config1(seed=0, size=512).unknowns == sets[0][0].unknowns


def test_cpu_sample_takes_whole_instances_in_parts():
    import bench
    from imscript_gb300 import synth
    insts = [synth.config0(seed=k, size=64) for k in range(5)]
    parts = [bench.cpu_sample(insts, p, 2) for p in range(2)]
    assert [len(p) for p in parts] == [3, 2]
    assert all(any(i is j for j in insts) for p in parts for i in p)
    chans = bench.channels_of(parts[0])
    assert len(chans) == 3 and chans[0][0].shape == (64, 64) and chans[0][2] == 0
