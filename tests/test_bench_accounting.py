"""The bench's accounting for the shared-matrix GLV's tensor-core cluster
sweeps (no GPU): the bf16 MMA FLOPs it charges to a launch and the kernels
it counts per gradient follow the kernels' structure (csrc/va_bundle_tc.cuh:
per tile and product 8 CTAs x 108 MMAs of M 128, N 64, K 16; the forward
f(y_0) plus 6 products per attempt, the backward 6 per accepted step; the
tiles the clusters run, the rest in the tail sweep)."""
import numpy as np

import bench

PER_PRODUCT = 8 * 108 * 2 * 128 * 64 * 16


def test_cluster_flops_follow_the_longest_instance_of_each_tile():
    attempts = np.full(128, 50)
    attempts[3] = 60   # tile 0's longest
    attempts[70] = 41  # shorter than its tile-mates: no effect
    fwd = bench.cluster_mma_flops(attempts, True, 2)
    assert fwd == PER_PRODUCT * ((1 + 6 * 60) + (1 + 6 * 50))
    bwd = bench.cluster_mma_flops(attempts, False, 2)
    assert bwd == PER_PRODUCT * (6 * 60 + 6 * 50)


def test_cluster_flops_leave_out_the_tail():
    attempts = np.full(1024, 50)
    attempts[1000] = 90  # in the 16th tile, which runs in the tail sweep
    assert bench.cluster_mma_flops(attempts, True, 15) == PER_PRODUCT * 15 * (1 + 6 * 50)
    assert bench.cluster_mma_flops(attempts, True, 16) == PER_PRODUCT * (15 * (1 + 6 * 50) + (1 + 6 * 90))


def test_launch_count_per_gradient():
    bundles = {"fwd_block": 256, "fwd_grid": 512, "bwd_block": 256, "bwd_grid": 512}
    assert bench.glv_shared_launches(bundles, 1024) == 6
    # both cluster sweeps with their tails (15 of 16 tiles in clusters)
    tc = {"fwd_block": 512, "fwd_grid": 120, "bwd_block": 512, "bwd_grid": 120}
    assert bench.glv_shared_launches(tc, 1024) == 12
    # every tile in clusters: no tail
    assert bench.glv_shared_launches(tc, 960) == 10
    # CK54: the bundle forward, the cluster backward
    ck = {"fwd_block": 256, "fwd_grid": 512, "bwd_block": 512, "bwd_grid": 120}
    assert bench.glv_shared_launches(ck, 1024) == 9
