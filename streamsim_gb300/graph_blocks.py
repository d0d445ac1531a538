"""Block structure of a view-factor graph under a Morton order of facets.

A block-sparse tensor-core gather would renumber the facets along a Morton
curve of their centroids, cut the side x side matrix F into dense B x B
blocks (B = 128) and contract every block that holds a nonzero with a
B x P panel of the iterate (P right-hand sides) on the tensor cores.  This
module measures what that layout costs on a given graph:

  - the number of nonzero blocks and how full they are (nonzeros / B^2);
  - the bytes one sweep reads: every nonzero block in BF16 (B^2 x 2 B) and
    its B x P panel rows, against the packed CSR gather (4 B per edge and a
    P-byte int8 row per edge, the latter from L2);
  - the tensor-core work: 2 B^2 P flops per nonzero block, and the fraction
    of those flops that multiply a true nonzero.

Run on the 203,840-facet forest (the headline workload, hemisphere view
factors of 512 rays per side, top-K 256; needs a GPU for the graph):

    python -m streamsim_gb300.graph_blocks
"""
import json

import numpy as np


def morton_rank(centroids, bits=10):
    """Rank of every facet along a Morton curve of its centroid (bits per
    axis over the centroids' bounding box), ties in index order."""
    c = np.asarray(centroids, np.float64)
    lo, hi = c.min(0), c.max(0)
    q = np.floor((c - lo) / np.maximum(hi - lo, 1e-30) * ((1 << bits) - 1)).astype(np.uint64)
    code = np.zeros(len(c), np.uint64)
    for b in range(bits):
        for a in range(3):
            code |= ((q[:, a] >> np.uint64(b)) & np.uint64(1)) << np.uint64(3 * b + a)
    order = np.argsort(code, kind="stable")
    rank = np.empty(len(c), np.int64)
    rank[order] = np.arange(len(c))
    return rank


def block_stats(rows, neighbors, facet_rank, block=128, panel=64):
    """Statistics of the nonzero block x block tiles of a side graph (CSR
    rows over 2F sides, side s = 2f + k) renumbered by facet_rank."""
    rows = np.asarray(rows, np.int64)
    nb = np.asarray(neighbors, np.int64)
    S = len(rows) - 1
    side_rank = 2 * np.asarray(facet_rank, np.int64)[np.arange(S) // 2] + (np.arange(S) & 1)
    src = np.repeat(np.arange(S), np.diff(rows))
    rb = side_rank[src] // block
    cb = side_rank[nb] // block
    nblk_axis = (S + block - 1) // block
    keys = rb * nblk_axis + cb
    _, counts = np.unique(keys, return_counts=True)
    nnz = len(nb)
    blocks = len(counts)
    fill = counts / float(block * block)
    csr_bytes = nnz * 4 + (S + 1) * 4
    csr_gather = nnz * panel  # int8 rows from L2
    blk_bytes = blocks * block * block * 2 + blocks * 8
    blk_panel = blocks * block * panel * 2  # BF16 panel rows per block, from L2
    return {
        "sides": S, "nonzeros": nnz, "block": block, "panel_columns": panel,
        "nonzero_blocks": blocks,
        "blocks_per_block_row": blocks / nblk_axis,
        "fill_mean": float(fill.mean()),
        "fill_p50": float(np.median(fill)),
        "fill_p90": float(np.quantile(fill, 0.9)),
        "fill_max": float(fill.max()),
        "nonzeros_in_blocks_over_1pct_fill": float(counts[fill > 0.01].sum() / nnz),
        "csr_hbm_bytes_per_sweep": int(csr_bytes),
        "csr_l2_gather_bytes_per_sweep": int(csr_gather),
        "block_hbm_bytes_per_sweep": int(blk_bytes),
        "block_l2_panel_bytes_per_sweep": int(blk_panel),
        "block_over_csr_hbm_bytes": blk_bytes / csr_bytes,
        "block_tensor_flops_per_sweep": float(blocks) * 2 * block * block * panel,
        "useful_flop_fraction": nnz / float(blocks * block * block),
        # the hybrid layout: blocks above a fill threshold as dense BF16
        # tiles on the tensor cores, the rest as the int8 CSR gather
        "hybrid": {f"{t:g}": hybrid_split(counts, fill, t, block, panel, nnz)
                   for t in (0.01, 0.05, 0.10)},
    }


def hybrid_split(counts, fill, threshold, block, panel, nnz):
    """The blocks above `threshold` fill: how many, their share of the
    nonzeros, the HBM bytes of their dense BF16 tiles against the 4-byte
    CSR words of the same edges, and their tensor flops at `panel`
    columns."""
    sel = fill > threshold
    n = int(sel.sum())
    e = int(counts[sel].sum())
    return {
        "blocks": n,
        "nonzero_share": e / float(nnz),
        "tile_hbm_bytes": n * block * block * 2,
        "csr_hbm_bytes_of_same_edges": e * 4,
        "tensor_flops": float(n) * 2 * block * block * panel,
    }


def main():
    from . import facetcu, scenes
    sc = scenes.config2(seed=0)
    m = facetcu.FacetrtCuda()
    m.initialize(1024, 1024, 1024)
    m.setGeometry(sc.vertices)
    uv, dirs = scenes.hemisphere_samples(512, 32, seed=7)
    m.buildHemisphereGraph(uv, dirs, 512, 256, 32)
    rows, nbrs, _, _, _ = m.graph()
    m.close()
    centroids = sc.vertices.reshape(-1, 3, 6)[:, :, :3].mean(1)
    out = {"workload": f"config2 forest: {sc.facet_count:,} facets, hemisphere 512 rays, top-K 256"}
    rank = morton_rank(centroids)
    for block in (128, 64):
        out[f"block{block}"] = block_stats(rows, nbrs, rank, block=block)
    print(json.dumps(out))


if __name__ == "__main__":
    main()
