"""trixi_integrate_noalloc, the handle-free integral entry point whose scratch
is a static device array (for callers that cannot allocate device memory),
called through the C ABI and checked against trixi_integrate.

The file name sorts last so that it also runs after every other test in the
same process; it passes alone in a fresh process as well."""
import ctypes as C

import numpy as np
import pytest

import trixicuda as T
from trixicuda import _lib
from conftest import assert_rel
from problems import make

pytestmark = pytest.mark.gpu

RTOL64 = 1e-12          # the FP64 tolerance of the parity tests
MAX_PARTIALS = 1 << 20  # size of the static scratch array, in doubles


def _noalloc(lib, semi, u, du, inv_jac, which, out, stream):
    eq = semi.equations
    gamma = float(getattr(eq, "gamma", 1.4))
    code = 1 if eq.nvariables > 1 else 0
    return lib.trixi_integrate_noalloc(semi.mesh.ndims, semi.solver.polydeg, code, gamma,
                                       C.c_void_p(u.data_ptr()),
                                       C.c_void_p(du.data_ptr()) if du is not None else None,
                                       C.c_void_p(inv_jac.data_ptr()), semi.nelements, which,
                                       C.c_void_p(out.data_ptr()), C.c_void_p(stream))


def test_noalloc_integrate_matches_integrate_twice(cuda):
    torch = cuda
    lib = _lib.load()
    mesh, eq, ic, solver, precision = make("euler_fd", 2, 4, polydeg=3)
    semi = T.SemidiscretizationHyperbolicGPU(mesh, eq, ic, solver, precision=precision)
    u = semi.compute_coefficients()
    du = torch.empty_like(u)
    T.rhs_gpu(du, u, semi, 0.0)
    inv_jac = torch.from_numpy(np.ascontiguousarray(semi.containers.inverse_jacobian)).to(u.device)
    stream = torch.cuda.current_stream(u.device)
    out = torch.full((8,), np.nan, dtype=torch.float64, device=u.device)

    # two calls in a row; the second one follows a call that left 4 partial
    # sums per element in the shared scratch
    for which, name, nq in [(_lib.INTEGRAL_STATE, "state", 4),
                            (_lib.INTEGRAL_ENTROPY_PRODUCTION, "entropy_production", 1)]:
        ref = T.integrate(u, semi, name, du=du)[:nq]
        out.fill_(np.nan)
        st = _noalloc(lib, semi, u, du, inv_jac, which, out, stream.cuda_stream)
        assert st == _lib.TRIXI_OK, _lib.last_error()
        stream.synchronize()
        got = out[:nq].cpu().numpy()
        assert np.all(np.isfinite(got))
        assert np.all(np.isnan(out[nq:].cpu().numpy())), "wrote beyond its nq results"
        if name == "state":
            assert_rel(got, ref, RTOL64, f"noalloc {name}")
        else:
            # entropy production of flux_ranocha is zero up to round-off: compare
            # on the scale of the entropy integral's magnitude
            scale = abs(T.integrate(u, semi, "entropy")[0])
            assert abs(got[0] - ref[0]) <= RTOL64 * scale, (got[0], ref[0], scale)


def test_noalloc_integrate_rejects_oversize(cuda):
    torch = cuda
    lib = _lib.load()
    mesh, eq, ic, solver, precision = make("euler_fd", 2, 3, polydeg=3)
    semi = T.SemidiscretizationHyperbolicGPU(mesh, eq, ic, solver, precision=precision)
    u = semi.compute_coefficients()
    inv_jac = torch.ones(1, dtype=torch.float64, device=u.device)
    out = torch.zeros(8, dtype=torch.float64, device=u.device)
    # 4 results per element: MAX_PARTIALS // 4 + 1 elements do not fit; the size
    # is rejected before anything is launched, so the short buffers are never read
    st = lib.trixi_integrate_noalloc(2, 3, 1, 1.4, C.c_void_p(u.data_ptr()), None, C.c_void_p(inv_jac.data_ptr()),
                                     MAX_PARTIALS // 4 + 1, _lib.INTEGRAL_STATE, C.c_void_p(out.data_ptr()), None)
    assert st == 1  # TRIXI_ERR_INVALID_ARGUMENT
    assert "exceed" in _lib.last_error()


CASES = [("adv_weak", 1, 4), ("adv_weak", 2, 3), ("adv_weak", 3, 2), ("euler_fd", 1, 4), ("euler_fd", 3, 2),
         ("euler_sc", 3, 2)]
KINDS = [(_lib.INTEGRAL_STATE, "state"), (_lib.INTEGRAL_ENTROPY, "entropy"),
         (_lib.INTEGRAL_ENTROPY_PRODUCTION, "entropy_production"), (_lib.INTEGRAL_DU, "du")]


@pytest.mark.parametrize("kind,d,level", CASES, ids=[f"{k}-{d}d" for k, d, _ in CASES])
def test_noalloc_every_integral_kind(kind, d, level, cuda):
    """Every integral kind, for linear advection and Euler in 1D/2D/3D: two
    calls in a row through the C ABI, each against trixi_integrate."""
    torch = cuda
    lib = _lib.load()
    mesh, eq, ic, solver, precision = make(kind, d, level, polydeg=3)
    semi = T.SemidiscretizationHyperbolicGPU(mesh, eq, ic, solver, precision=precision)
    u = semi.compute_coefficients()
    du = torch.empty_like(u)
    T.rhs_gpu(du, u, semi, 0.0)
    inv_jac = torch.from_numpy(np.ascontiguousarray(semi.containers.inverse_jacobian)).to(u.device)
    stream = torch.cuda.current_stream(u.device)
    nv = eq.nvariables
    # magnitudes for the integrals that are zero up to round-off (conservation
    # of du, entropy production of entropy-conservative fluxes)
    du_scale = np.abs(T.integrate(du.abs(), semi, "state")[:nv])
    ent_scale = abs(T.integrate(u, semi, "entropy")[0])
    out = torch.full((16,), np.nan, dtype=torch.float64, device=u.device)
    for which, name in KINDS:
        nq = nv if name in ("state", "du") else 1
        ref = T.integrate(u, semi, name, du=du)[:nq]
        for call in range(2):
            out.fill_(np.nan)
            st = _noalloc(lib, semi, u, du, inv_jac, which, out, stream.cuda_stream)
            assert st == _lib.TRIXI_OK, _lib.last_error()
            stream.synchronize()
            got = out[:nq].cpu().numpy()
            assert np.all(np.isnan(out[nq:].cpu().numpy())), "wrote beyond its results"
            if name == "du":
                assert np.all(np.abs(got - ref) <= RTOL64 * np.maximum(du_scale, np.abs(ref))), (name, call, got, ref)
            elif name == "entropy_production":
                assert abs(got[0] - ref[0]) <= RTOL64 * max(ent_scale, abs(ref[0])), (name, call, got, ref)
            else:
                assert_rel(got, ref, RTOL64, f"noalloc {name}, call {call}")
