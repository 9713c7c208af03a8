"""The mixed-precision kernels convert with integer operations (the FP64
pipe of GB300 is ~64x slower than FP32); those conversions must equal the
hardware's bit for bit: double -> float round-to-nearest-even, float ->
double exact."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_integer_conversions_match_hardware(cuda):
    from trixicuda import _lib

    rng = np.random.default_rng(5)
    n = 1 << 20
    d = np.concatenate([
        rng.standard_normal(n // 4) * 10.0 ** rng.integers(-30, 30, n // 4),
        rng.uniform(0.5, 2.0, n // 4),
        # exact ties and near-ties in the discarded 29 bits
        (np.float64(1.0) + (np.arange(n // 4) % 4096) * 2.0**-52).astype(np.float64) * rng.choice([-1, 1], n // 4),
        np.array([0.0, -0.0, 1e-45, -1e-45, 1e-310, 3.4028234663852886e38, 3.4028235e38, 1e39, -1e39,
                  np.inf, -np.inf, 1.0 + 2.0**-24, 1.0 + 3 * 2.0**-24, 1.17549435e-38, 1.1754942e-38]),
    ])
    tied = np.float64(1.0) + np.arange(1, 4096) * 2.0**-29 + 2.0**-53
    d = np.concatenate([d, tied, -tied]).astype(np.float64)
    f = rng.standard_normal(d.size).astype(np.float32) * np.float32(10.0) ** rng.integers(-30, 30, d.size).astype(np.float32)
    f[:8] = np.array([0.0, -0.0, 1e-40, -1e-40, np.inf, -np.inf, 3.4e38, 1.2e-38], dtype=np.float32)
    dev = cuda.device("cuda")
    td = cuda.from_numpy(d).to(dev)
    tf = cuda.from_numpy(f).to(dev)
    of = cuda.empty(d.size, dtype=cuda.float32, device=dev)
    od = cuda.empty(d.size, dtype=cuda.float64, device=dev)
    st = _lib.load_diag().trixi_diag_convert(C.c_void_p(td.data_ptr()), C.c_void_p(of.data_ptr()),
                                            C.c_void_p(tf.data_ptr()), C.c_void_p(od.data_ptr()), d.size, None)
    assert st == 0
    cuda.cuda.synchronize()
    hw_f = td.float()
    hw_d = tf.double()
    assert cuda.equal(of.view(cuda.int32), hw_f.view(cuda.int32))
    assert cuda.equal(od.view(cuda.int64), hw_d.view(cuda.int64))
