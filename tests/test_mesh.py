"""TreeMesh connectivity (host side): every element face is covered exactly
once by an interface or a mortar, mortar geometry matches the conventions of
the reference containers, and coordinates/Jacobians are consistent."""
import numpy as np
import pytest

import trixicuda as T


def _face_cover(c, d):
    cover = np.zeros((c.nelements, 2 * d), dtype=int)
    for (l, r), o in zip(c.interface_neighbor_ids, c.interface_orientations):
        cover[l - 1, 2 * (o - 1) + 1] += 1
        cover[r - 1, 2 * (o - 1)] += 1
    nc = 2 ** (d - 1)
    for ids, ls, o in zip(c.mortar_neighbor_ids, c.mortar_large_sides, c.mortar_orientations):
        for s in ids[:nc]:
            cover[s - 1, 2 * (o - 1) + (ls - 1)] += 1
        cover[ids[nc] - 1, 2 * (o - 1) + (1 if ls == 1 else 0)] += 1
    return cover


@pytest.mark.parametrize("d,level,refined", [(1, 4, False), (2, 3, False), (2, 3, True), (3, 2, False), (3, 2, True)])
def test_faces_covered_once(d, level, refined):
    patches = [dict(type="box", coordinates_min=(0.0,) * d, coordinates_max=(1.0,) * d)] if refined else []
    mesh = T.TreeMesh((-1.0,) * d, (1.0,) * d, initial_refinement_level=level, refinement_patches=patches)
    c = mesh.build_containers(T.LobattoLegendreBasisGPU(3).nodes)
    assert np.all(_face_cover(c, d) == 1)
    E0 = 2 ** (d * level)
    if refined:
        assert c.nelements == E0 - E0 // 2**d + E0 // 2**d * 2**d
        assert c.nmortars > 0
    else:
        assert c.nelements == E0 and c.ninterfaces == d * E0 and c.nmortars == 0


def test_mortar_geometry_2d():
    mesh = T.TreeMesh((-1.0, -1.0), (1.0, 1.0), initial_refinement_level=2,
                      refinement_patches=[dict(type="box", coordinates_min=(0.0, -1.0), coordinates_max=(1.0, 1.0))])
    c = mesh.build_containers(T.LobattoLegendreBasisGPU(2).nodes)
    for ids, ls, o in zip(c.mortar_neighbor_ids, c.mortar_large_sides, c.mortar_orientations):
        small_lo, small_hi, large = (mesh.elements[i - 1] for i in ids)
        ax = o - 1
        t = 1 - ax
        cl = mesh.cell_center(large)
        cs0, cs1 = mesh.cell_center(small_lo), mesh.cell_center(small_hi)
        assert cs0[t] < cs1[t]                                # lower then upper along the tangent
        assert (cs0[ax] > cl[ax]) == (ls == 1) or abs(cs0[ax] - cl[ax]) > 1.0  # periodic wrap allowed


def test_coordinates_and_jacobian():
    mesh = T.TreeMesh((-2.0, -2.0), (2.0, 2.0), initial_refinement_level=3)
    b = T.LobattoLegendreBasisGPU(3)
    c = mesh.build_containers(b.nodes)
    assert np.allclose(c.inverse_jacobian, 2.0 / 0.5)
    xy = c.node_coordinates.reshape(-1, 2)
    assert xy.min() == -2.0 and xy.max() == 2.0
    # node (i, j) of element 0 sits at (x_i, y_j), x fastest in memory
    e0 = c.node_coordinates[0]
    assert np.allclose(e0[0, :, 0], -2 + 0.25 * (b.nodes + 1))
    assert np.allclose(e0[:, 0, 1], -2 + 0.25 * (b.nodes + 1))


def test_repeated_patches_are_balanced():
    """Two identical refinement boxes (test/tree_dgsem_2d/euler_blob_mortar.jl):
    the second level of refinement forces the coarse neighbours of the box
    up one level, so faces differ by at most one level."""
    import collections

    mesh = T.TreeMesh((-32.0, -32.0), (32.0, 32.0), initial_refinement_level=4,
                      refinement_patches=[dict(type="box", coordinates_min=(-40.0, -5.0),
                                               coordinates_max=(40.0, 5.0))] * 2)
    levels = collections.Counter(c[0] for c in mesh.elements)
    # 32 level-4 cells in the box -> 128 level 5 -> 512 level 6; the 32 level-4
    # rows next to it are refined once to keep the 2:1 balance
    assert levels == {4: 192, 5: 128, 6: 512}
    mesh._check_balance()
    cont = mesh.build_containers(np.array([-1.0, 1.0]))
    area = np.sum((1.0 / cont.inverse_jacobian) ** 2 * 4.0)  # J = h/2 per dimension, reference square of area 4
    assert np.isclose(area, 64.0 * 64.0)
