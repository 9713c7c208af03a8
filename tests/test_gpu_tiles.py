"""The fused kernel's tile (warps per element group, groups per block) is a
launch parameter picked by the tile tuner; every valid tile must give
bit-identical results, and the tuner must leave its input untouched."""
import numpy as np
import pytest

import trixicuda as T
from problems import make

pytestmark = pytest.mark.gpu

CASES = [("euler_fd", 2, 3, 3, False, "mixed"), ("euler_fd", 2, 3, 4, True, "fp64"),
         ("euler_sc", 3, 2, 3, False, "mixed"), ("adv_weak", 3, 2, 5, True, "fp64"),
         ("adv_weak", 1, 4, 3, False, "fp64")]


def _valid_tiles(epg_warps):
    return [(w, g) for w in range(epg_warps, 9) for g in (1, 2, 4, 8) if g * w <= 16]


@pytest.mark.parametrize("kind,d,lvl,p,refined,prec", CASES)
def test_every_tile_gives_identical_results(kind, d, lvl, p, refined, prec, cuda):
    mesh, eq, ic, solver, _ = make(kind, d, lvl, polydeg=p, refined=refined)
    semi = T.SemidiscretizationHyperbolicGPU(mesh, eq, ic, solver, precision=prec)
    u = semi.compute_coefficients()
    du_ref = cuda.empty_like(u)
    T.rhs_gpu(du_ref, u, semi, 0.0)
    u1_ref, k1_ref = u.clone(), cuda.zeros_like(u)
    T.rk_steps(u1_ref, k1_ref, 0.0, 1e-4, 2, semi)
    (epg, wpg0, gpb0), table = T.tile(semi)
    assert table == {}
    min_w = -(-epg * semi.nnodes ** d // 32)
    tiles = _valid_tiles(min_w)
    assert (wpg0, gpb0) in tiles
    for w, g in tiles:
        try:
            T.set_tile(semi, w, g)
        except T._lib.TrixiError:
            continue  # more shared memory than one block may hold
        du = cuda.empty_like(u)
        T.rhs_gpu(du, u, semi, 0.0)
        u1, k1 = u.clone(), cuda.zeros_like(u)
        T.rk_steps(u1, k1, 0.0, 1e-4, 2, semi)
        cuda.cuda.synchronize()
        assert cuda.equal(du, du_ref), (w, g)
        assert cuda.equal(u1, u1_ref) and cuda.equal(k1, k1_ref), (w, g)
    with pytest.raises(T._lib.TrixiError):
        T.set_tile(semi, 9, 1)
    T.set_tile(semi, 0, 0)
    assert T.tile(semi)[0] == (epg, wpg0, gpb0)
    # the tuner: input untouched, picks a measured tile, results unchanged
    u_before = u.clone()
    T.autotune(u, semi)
    cuda.cuda.synchronize()
    assert cuda.equal(u, u_before)
    (_, w, g), table = T.tile(semi)
    assert (w, g) in table and all(ms > 0 for ms in table.values())
    assert min(table.values()) == table[(w, g)]
    du = cuda.empty_like(u)
    T.rhs_gpu(du, u, semi, 0.0)
    cuda.cuda.synchronize()
    assert cuda.equal(du, du_ref)
