"""The oracle's BVH hemisphere caster (host threads) against its brute force
over all facets: identical graphs, dropped-ray counts and sun fractions, with
and without periodic tiles.  The BVH caster is what checks the GPU graph at
the bench's full size, where the brute force would take days."""
import numpy as np
import pytest

from streamsim_gb300 import scenes


@pytest.mark.parametrize("leaves,grid,rays,top_k,periodic", [
    (256, 8, 64, 16, (0, 1.0, 1.0)),
    (200, 6, 48, 64, (4, 10.0, 10.0)),
    (300, 6, 32, 8, (8, 10.0, 10.0)),
])
def test_bvh_caster_equals_brute_force(oracle, leaves, grid, rays, top_k, periodic):
    sc = scenes.config1(seed=1, leaves=leaves, grid=grid)
    uv, dirs = scenes.hemisphere_samples(rays, 8, seed=7)
    g1, d1 = oracle.hemisphere_graph(sc.vertices, uv, dirs, rays, 8, top_k, periodic=periodic)
    for threads in (1, 3):
        g2, d2 = oracle.hemisphere_graph_bvh(sc.vertices, uv, dirs, rays, 8, top_k,
                                             periodic=periodic, threads=threads)
        for a, b in ((g1.row_offsets, g2.row_offsets), (g1.neighbors, g2.neighbors),
                     (g1.counts, g2.counts), (g1.denominators, g2.denominators),
                     (g1.sky_counts, g2.sky_counts)):
            assert np.array_equal(a, b)
        assert d1 == d2
    suv, _ = scenes.hemisphere_samples(48, 8, seed=8)
    sun = scenes.sun_direction(40.0, 210.0)
    l1 = oracle.hemisphere_sunlit(sc.vertices, suv, 48, 8, sun, periodic=periodic)
    l2 = oracle.hemisphere_sunlit_bvh(sc.vertices, suv, 48, 8, sun, periodic=periodic,
                                      threads=2)
    assert np.array_equal(l1, l2)


def test_bvh_caster_empty_and_single_facet(oracle):
    uv, dirs = scenes.hemisphere_samples(32, 4, seed=7)
    one = scenes.config1(seed=1, leaves=1, grid=1).vertices[:3]
    g, d = oracle.hemisphere_graph_bvh(one, uv, dirs, 32, 4, 8)
    assert g.nnz == 0 and d == 0
    assert np.all(g.sky_counts == 32) and np.all(g.denominators == 32)
