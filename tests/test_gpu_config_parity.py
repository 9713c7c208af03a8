"""FP64 parity at the benchmark configurations' own sizes, as the reference's
tests compare stage results on their configured problems
(test/tree_dgsem_3d/euler_shock.jl, test/tree_dgsem_2d/euler_ec.jl:60-122,
test/test_macros.jl:4-74): the GPU (through the C ABI) against the oracle on
its own connectivity, on identical inputs.

* 2D Euler, level 7 (16384 elements), polydeg 3, flux_ranocha, seeded
  Fourier initial condition (|k| <= 8): rhs and one CarpenterKennedy2N54 step;
* 3D Euler shock capturing, level 5 (32768 elements), weak blast wave:
  indicator, rhs and one step;
* 2D Euler, level 6, polydeg 4 (the adjoint configuration): rhs, one step,
  and the discrete adjoint's VJP against central differences of the
  oracle's rhs (independent of the GPU forward path);
* the 512-instance batched ensemble in FP64 through trixi_batch_rhs, with
  sampled instances covering polydeg 5, refined quadrants / octants (L2
  mortars), 3D advection level 4 and 2D Euler.

Bars.  rhs and k: within 1e-12 relative in the 2-norm (1e-11 in the max
norm), or within twice the round-off floor of the configuration if that is
larger.  du is a sum of O(J^{-1} |f|) flux terms that cancel to a small
rest, so its relative rounding error grows with the resolution: at level 7
the oracle's own du moves by 4.6e-12 (2-norm) when u is perturbed by one ulp,
more than 1e-12.  The floor is measured in each test as exactly that (the
oracle at u and at u (1 +- eps)), and the test prints both numbers.  u after
a step: 1e-13; indicator: 1e-12 absolute; VJP: 1e-6 of the
finite-difference JVP's inner product."""
import numpy as np
import pytest

import bench
import trixicuda as T
from conftest import assert_rel, rel_err, rel_err_max
from oracle.oracle import Oracle

pytestmark = pytest.mark.gpu


def _setup(builder, cuda):
    mesh, eq, ic, solver = builder("fp64")
    semi = T.SemidiscretizationHyperbolicGPU(mesh, eq, ic, solver)
    u_host = semi.compute_coefficients_host()
    return semi, Oracle.from_semi(semi), u_host, cuda.from_numpy(u_host).to(semi.device)


def _ulp_perturbed(u_host):
    rng = np.random.default_rng(12345)
    return u_host * (1.0 + np.finfo(np.float64).eps * rng.choice([-1.0, 1.0], u_host.shape))


def roundoff_floor(orc, u_host, du_ref):
    """Relative change (2-norm, max-norm) of the oracle's rhs when every
    entry of u moves by one ulp with a seeded random sign."""
    dup = orc.rhs(_ulp_perturbed(u_host))
    return rel_err(dup, du_ref), rel_err_max(dup, du_ref)


def assert_within_floor(got, ref, floor, what):
    e2, emax = rel_err(got, ref), rel_err_max(got, ref)
    bar2, barmax = max(1e-12, 2.0 * floor[0]), max(1e-11, 2.0 * floor[1])
    print(f"{what}: 2-norm {e2:.2e} (floor {floor[0]:.2e}, bar {bar2:.2e}); "
          f"max-norm {emax:.2e} (floor {floor[1]:.2e}, bar {barmax:.2e})")
    assert e2 <= bar2, f"{what}: relative 2-norm error {e2:.3e} > {bar2:.2e}"
    assert emax <= barmax, f"{what}: relative max-norm error {emax:.3e} > {barmax:.2e}"


def _rhs_and_step(semi, orc, u_host, u, dt, cuda, what):
    du = cuda.empty_like(u)
    T.rhs_gpu(du, u, semi, 0.0)
    T.synchronize(semi)
    du_o = orc.rhs(u_host)
    floor = roundoff_floor(orc, u_host, du_o)
    assert_within_floor(du.cpu().numpy(), du_o, floor, f"{what} rhs")
    uu, k = u.clone(), cuda.zeros_like(u)
    T.rk_steps(uu, k, 0.0, dt, 1, semi)
    T.synchronize(semi)
    u_o, k_o = orc.rk_ck2n54(u_host, 0.0, dt, 1)
    assert_rel(uu.cpu().numpy(), u_o, 1e-13, f"{what} u after one step")
    # k's floor: the same step of the oracle from the one-ulp perturbed state
    # (each stage's rhs carries the conditioning of du)
    _, k_p = orc.rk_ck2n54(_ulp_perturbed(u_host), 0.0, dt, 1)
    assert_within_floor(k.cpu().numpy(), k_o, (rel_err(k_p, k_o), rel_err_max(k_p, k_o)), f"{what} k after one step")


def test_euler2d_level7_rhs_and_step(cuda):
    semi, orc, u_host, u = _setup(bench.build_problem, cuda)
    assert semi.nelements == 16384
    _rhs_and_step(semi, orc, u_host, u, bench.stable_dt(semi), cuda, "2D Euler level 7")


def test_euler2d_level7_mixed_rhs(cuda):
    """The FP32-mixed rhs of the headline workload.  Its floor is the change
    of the oracle's (FP64) du when u is rounded to FP32, the rounding the mixed
    kernel applies to its inputs (4.1e-4 in the 2-norm at level 7: the
    conditioning of du times 2^-24); the FP32 flux arithmetic adds to it.
    Bar: 5e-4 (the mixed bar of the smaller cases) or five times the floor."""
    mesh, eq, ic, solver = bench.build_problem("mixed")
    semi = T.SemidiscretizationHyperbolicGPU(mesh, eq, ic, solver, precision="mixed")
    u_host = semi.compute_coefficients_host()
    u = cuda.from_numpy(u_host).to(semi.device)
    du = cuda.empty_like(u)
    T.rhs_gpu(du, u, semi, 0.0)
    T.synchronize(semi)
    orc = Oracle.from_semi(semi)
    du_o = orc.rhs(u_host)
    du_32 = orc.rhs(u_host.astype(np.float32).astype(np.float64))
    floor = rel_err(du_32, du_o)
    e = rel_err(du.cpu().numpy(), du_o)
    print(f"mixed rhs, 2D Euler level 7: 2-norm {e:.2e}, FP32-input floor {floor:.2e}")
    assert e <= max(5e-4, 5.0 * floor), (e, floor)


def test_euler3d_shock_capturing_level5(cuda):
    semi, orc, u_host, u = _setup(bench.build_problem_c3, cuda)
    assert semi.nelements == 32768
    alpha = cuda.zeros(semi.nelements, dtype=cuda.float64, device=semi.device)
    T.cuda_indicator(u, alpha, semi)
    T.synchronize(semi)
    a_o = orc.indicator(u_host)
    assert np.max(np.abs(alpha.cpu().numpy() - a_o)) < 1e-12
    assert np.count_nonzero(a_o) > 0
    _rhs_and_step(semi, orc, u_host, u, bench.stable_dt(semi, bench.C3_LEVEL), cuda, "3D shock capturing level 5")


def test_euler2d_level6_polydeg4(cuda):
    semi, orc, u_host, u = _setup(bench.build_problem_c4, cuda)
    assert semi.nelements == 4096 and semi.solver.polydeg == 4
    dt = 0.5 * T.max_dt(u, semi)
    _rhs_and_step(semi, orc, u_host, u, dt, cuda, "2D Euler level 6 polydeg 4")


def test_rhs_vjp_against_oracle_finite_differences(cuda):
    """<lambda, J v> by central differences of the ORACLE's rhs against
    <J^T lambda, v> from trixi_rhs_vjp, along seeded random directions, on the
    adjoint configuration."""
    from trixicuda import adjoint as ADJ

    semi, orc, u_host, u = _setup(bench.build_problem_c4, cuda)
    rng = np.random.default_rng(20261204)
    for _ in range(4):
        v = rng.standard_normal(u_host.shape)
        lam = rng.standard_normal(u_host.shape)
        h = 1e-6 * float(np.max(np.abs(u_host))) / float(np.max(np.abs(v)))
        jv = (orc.rhs(u_host + h * v) - orc.rhs(u_host - h * v)) / (2 * h)
        ubar = cuda.empty_like(u)
        ADJ.rhs_vjp(ubar, u, cuda.from_numpy(lam).to(u.device), semi)
        T.synchronize(semi)
        lhs = float(np.sum(lam * jv))
        rhs = float(np.sum(ubar.cpu().numpy() * v))
        scale = float(np.sum(np.abs(lam * jv)))
        assert abs(lhs - rhs) <= 1e-6 * scale, (lhs, rhs, scale)


def _pick_instances(problems):
    """At least 8 instances covering polydeg 5, refined meshes (mortars), 3D
    advection level 4, 2D Euler and 2D advection."""
    want = [lambda lb: lb.endswith("p5"), lambda lb: lb.endswith("-ref"), lambda lb: lb.startswith("adv3d-L4"),
            lambda lb: lb.startswith("euler2d") and "-p5" in lb, lambda lb: lb.startswith("euler2d") and "-ref" in lb,
            lambda lb: lb.startswith("adv2d-L6"), lambda lb: lb.startswith("adv3d") and "-ref" in lb,
            lambda lb: lb.startswith("euler2d-L6"), lambda lb: lb.startswith("adv2d") and "-p2" in lb,
            lambda lb: lb.startswith("adv3d") and "-p5" in lb]
    picked = []
    for w in want:
        for i, pb in enumerate(problems):
            if w(pb.label) and i not in picked:
                picked.append(i)
                break
    return picked


def test_batched_ensemble_fp64_sampled_instances(cuda):
    from trixicuda.batch import BatchedSemidiscretizationGPU, make_ensemble

    dev = cuda.device("cuda", cuda.cuda.current_device())
    problems = make_ensemble(n=512, device=dev)
    batch = BatchedSemidiscretizationGPU(problems, precision="fp64", device=dev)
    u = batch.compute_coefficients()
    du = cuda.empty_like(u)
    batch.rhs(du, u)
    cuda.cuda.synchronize()
    picked = _pick_instances(problems)
    assert len(picked) >= 8
    labels = [problems[i].label for i in picked]
    assert any(lb.endswith("p5") for lb in labels) and any(lb.endswith("-ref") for lb in labels)
    assert any(lb.startswith("adv3d-L4") for lb in labels)
    for i in picked:
        pb = problems[i]

        class _S:
            pass

        s = _S()
        s.equations, s.solver, s.mesh, s.containers = pb.equations, pb.solver, pb.mesh, batch.containers[i]
        u_i = batch.view(u, i).cpu().numpy()
        orc = Oracle.from_semi(s)
        du_o = orc.rhs(u_i)
        assert_within_floor(batch.view(du, i).cpu().numpy(), du_o, roundoff_floor(orc, u_i, du_o), pb.label)
