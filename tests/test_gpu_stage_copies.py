"""FP32 stage copies of trixi_rk_steps (FP32-mixed Euler and ideal GLM-MHD).

Inside one trixi_rk_steps call every stage after the first reads its flux
states (and the shock indicator its input) from the FP32 copy that the
previous stage wrote, instead of narrowing the FP64 state again.  Both are the
same round-to-nearest narrowing of the same FP64 values, so the steps must be
bit-identical to the same stages run one by one through trixi_rk_stage, which
never uses the copies."""
import numpy as np
import pytest

import trixicuda as T
from problems import semi_and_oracle
from trixicuda.time_integration import CK2N54_A, CK2N54_B, CK2N54_C

pytestmark = pytest.mark.gpu


def _stages(semi, u, k, t, dt, nsteps, cuda):
    """The CK2N54 steps as single stages (no FP32 copies)."""
    cur, nxt = u.clone(), cuda.empty_like(u)
    for _ in range(nsteps):
        for a, b, c in zip(CK2N54_A, CK2N54_B, CK2N54_C):
            T.rk_stage(nxt, cur, k, a, b, dt, t + c * dt, semi)
            cur, nxt = nxt, cur
        t += dt
    return cur


def _check(semi, u, dt, cuda, nsteps=2):
    k0 = cuda.zeros_like(u)
    u_steps, k_steps = u.clone(), k0.clone()
    T.rk_steps(u_steps, k_steps, 0.0, dt, nsteps, semi)
    k_stage = k0.clone()
    u_stage = _stages(semi, u, k_stage, 0.0, dt, nsteps, cuda)
    T.synchronize(semi)
    a, b = u_steps.cpu().numpy(), u_stage.cpu().numpy()
    assert np.isfinite(a).all()
    assert np.array_equal(a, b), f"u differs in {np.count_nonzero(a != b)} values"
    assert np.array_equal(k_steps.cpu().numpy(), k_stage.cpu().numpy())
    # and a second call continues from the caller's u (its first stage narrows u again)
    T.rk_steps(u_steps, k_steps, 0.0, dt, 1, semi)
    u_stage = _stages(semi, u_stage, k_stage, 0.0, dt, 1, cuda)
    T.synchronize(semi)
    assert np.array_equal(u_steps.cpu().numpy(), u_stage.cpu().numpy())


CASES = [
    ("euler_fd", 2, 3, 3, False),   # the 2D flux-differencing workload's physics
    ("euler_fd", 2, 3, 3, True),    # mortars
    ("euler_fd", 3, 2, 3, True),
    ("euler_fd", 1, 4, 3, False),
    ("euler_weak", 3, 2, 3, True),
    ("euler_sc", 3, 3, 3, False),   # the 3D shock-capturing workload's physics (indicator on the copy)
    ("euler_sc", 2, 3, 3, True),
    ("euler_fd", 2, 2, 5, False),   # odd N: 5-value records of 4 variables at odd offsets
    ("euler_sc", 3, 2, 2, False),
]


@pytest.mark.parametrize("case", CASES, ids=lambda c: f"{c[0]}-{c[1]}d-L{c[2]}-p{c[3]}{'-ref' if c[4] else ''}")
def test_rk_steps_with_copies_bit_identical(case, cuda):
    kind, d, level, p, refined = case
    semi, _ = semi_and_oracle(kind, d, level, polydeg=p, refined=refined, precision="mixed")
    u = cuda.from_numpy(semi.compute_coefficients_host()).to(semi.device)
    dt = 0.2 / float(np.max(semi.containers.inverse_jacobian)) / 4
    _check(semi, u, dt, cuda)


@pytest.mark.parametrize("setup,d", [("ec", 2), ("shock", 2), ("alfven", 3), ("shock", 3)])
def test_mhd_rk_steps_with_copies_bit_identical(setup, d, cuda):
    from test_gpu_mhd import _semi, _u

    semi, _ = _semi(setup, d, 2 if d == 3 else 3, precision="mixed")
    _, u = _u(semi, cuda)
    dt = 0.05 / float(np.max(semi.containers.inverse_jacobian)) / 4
    _check(semi, u, dt, cuda)


def test_boundaries_rk_steps_with_copies_bit_identical(cuda):
    from test_gpu_boundaries import _semi, _u

    for args in (("euler", 2, 3, 3, True, "weak"), ("euler", 3, 2, 3, False, "fd")):
        semi, _ = _semi(*args, precision="mixed")
        _, u = _u(semi, cuda)
        dt = 0.1 / float(np.max(semi.containers.inverse_jacobian)) / 4
        _check(semi, u, dt, cuda)


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_rk_steps_host_equals_device_path(precision, cuda):
    """trixi_rk_steps_host (host state in, host state out) gives the bits of
    trixi_rk_steps on the same state; u_out may be u_in; the ordering events
    are honoured."""
    semi, _ = semi_and_oracle("euler_fd", 2, 3, refined=True, precision=precision)
    u_host = semi.compute_coefficients_host()
    dt = 0.2 / float(np.max(semi.containers.inverse_jacobian)) / 4
    u = cuda.from_numpy(u_host).to(semi.device)
    k = cuda.zeros_like(u)
    T.rk_steps(u, k, 0.0, dt, 3, semi)
    pin_in = cuda.from_numpy(u_host.copy()).pin_memory()
    pin_out = cuda.empty_like(pin_in).pin_memory()
    wait, done = cuda.cuda.Event(), cuda.cuda.Event()
    wait.record()
    T.rk_steps_host(pin_in, pin_out, 0.0, dt, 3, semi, wait_event=wait, done_event=done)
    done.synchronize()
    cuda.cuda.synchronize()
    assert np.array_equal(pin_out.numpy(), u.cpu().numpy())
    # pageable numpy buffers, in place
    a = u_host.copy()
    T.rk_steps_host(a, a, 0.0, dt, 3, semi)
    T.synchronize(semi)
    assert np.array_equal(a, u.cpu().numpy())
