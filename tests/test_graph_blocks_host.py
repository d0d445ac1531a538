"""The block-structure diagnostic of a side graph (no GPU)."""
import numpy as np

from streamsim_gb300 import graph_blocks


def test_morton_rank_is_a_permutation_along_the_curve():
    rng = np.random.default_rng(0)
    c = rng.uniform(0, 1, (1000, 3))
    r = graph_blocks.morton_rank(c)
    assert sorted(r.tolist()) == list(range(1000))
    # the two octants split: every centroid below the middle in all axes
    # comes before every one above it in all axes
    low = np.all(c < 0.45, axis=1)
    high = np.all(c > 0.55, axis=1)
    assert r[low].max() < r[high].min()


def test_block_counts_on_a_known_graph():
    # 4 facets = 8 sides in Morton order 0..3; block 2: side blocks {0,1}
    # {2,3} {4,5} {6,7}.  Edges: side 0 -> 1, 2 (blocks (0,0), (0,1));
    # side 5 -> 4 (block (2,2)); side 7 -> 0, 1 (block (3,0) twice).
    rows = np.array([0, 2, 2, 2, 2, 2, 3, 3, 5])
    nbrs = np.array([1, 2, 4, 0, 1])
    st = graph_blocks.block_stats(rows, nbrs, np.arange(4), block=2, panel=4)
    assert st["nonzeros"] == 5 and st["nonzero_blocks"] == 4
    assert st["fill_max"] == 0.5 and abs(st["fill_mean"] - 5 / 16) < 1e-12
    assert st["useful_flop_fraction"] == 5 / 16
    assert st["block_tensor_flops_per_sweep"] == 4 * 2 * 2 * 2 * 4
    assert st["csr_hbm_bytes_per_sweep"] == 5 * 4 + 9 * 4
