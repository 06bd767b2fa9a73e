"""The native scatter-plan builder (host C++) against scipy's geometry on the same grids (CPU only).

scipy is used here only as the checker: Delaunay triangulation (qhull), point location and
nearest-neighbour queries of the interpolants that holodeck's add_scatter_to_masses builds
(holodeck/sams/sam.py:1365-1383).
"""

import numpy as np
import pytest
import scipy.spatial

from oracle import sam_oracle as O


@pytest.mark.parametrize("shape,scatter", [((10, 11), 0.28), ((14, 13), 0.28), ((30, 30), 0.28), ((25, 17), 0.6),
                                           ((91, 81), 0.28)])
def test_plan_matches_scipy_geometry(built_lib, shape, scatter):
    from holodeck_gb300.sams import scatter as S
    mtot, mrat, _ = O.grid_edges(shape + (3,))
    arrs, sz = S.host_plan(mtot, mrat, scatter)
    m1 = mtot[:, None] / (1.0 + mrat[None, :])
    m2 = mtot[:, None] - m1
    pts = np.column_stack([np.log10(m1.ravel()), np.log10(m2.ravel())])
    np.testing.assert_allclose(arrs["pts"], pts, rtol=1e-15, atol=0)
    tri = scipy.spatial.Delaunay(pts)
    assert sz.n_tri == len(tri.simplices)
    assert set(map(tuple, np.sort(arrs["tri"], axis=1))) == set(map(tuple, np.sort(tri.simplices, axis=1)))
    # neighbour lists are the triangulation's edges
    indptr, indices = tri.vertex_neighbor_vertices
    for ii in range(0, len(pts), max(1, len(pts) // 200)):
        mine = set(arrs["nbr_idx"][arrs["nbr_ptr"][ii]:arrs["nbr_ptr"][ii + 1]])
        assert mine == set(indices[indptr[ii]:indptr[ii + 1]])
    # wavefront levels: every point comes after all of its lower-indexed neighbours
    level = np.empty(len(pts), int)
    for lv in range(sz.n_levels):
        level[arrs["level_vtx"][arrs["level_ptr"][lv]:arrs["level_ptr"][lv + 1]]] = lv
    for ii in range(len(pts)):
        nb = arrs["nbr_idx"][arrs["nbr_ptr"][ii]:arrs["nbr_ptr"][ii + 1]]
        lower = nb[nb < ii]
        assert np.all(level[lower] < level[ii])
    # regular grid, point location, nearest points, redistribution weights
    N = 4 * shape[0]
    lo = 0.9 * mtot[0] * mrat[0] / (1.0 + mrat[0])
    hi = mtot[-1] * (1.0 + mrat[0]) / mrat[0]
    axis = np.log10(np.logspace(*np.log10([min(lo, hi), max(lo, hi)]), N))
    np.testing.assert_allclose(arrs["grid_axis"], axis, rtol=1e-15, atol=0)
    grid = np.meshgrid(axis, axis, indexing="ij")
    q = np.column_stack([grid[0].ravel(), grid[1].ravel()])
    s = tri.find_simplex(q)
    assert np.array_equal(s >= 0, arrs["grid_tri"] >= 0)
    inside = np.flatnonzero(s >= 0)
    mine = np.sort(arrs["tri"][arrs["grid_tri"][inside]], axis=1)
    theirs = np.sort(tri.simplices[s[inside]], axis=1)
    same = np.all(mine == theirs, axis=1)
    # nodes on a shared edge may be assigned to either triangle: check the barycentric of the others
    lam = arrs["grid_bary"][inside[~same]]
    assert np.all(np.min(np.abs(lam), axis=1) < 1e-12)
    near = scipy.spatial.cKDTree(pts).query(q)[1]
    assert np.array_equal(near, arrs["grid_near"])
    w = O.scatter_weights(axis, scatter)
    big = w > 1e-200
    np.testing.assert_allclose(arrs["weights"][big], w[big], rtol=1e-10, atol=0)
