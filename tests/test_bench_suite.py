"""The reference-benchmark set-ups of `bench.py --suite reference-benchmarks`
(no GPU): every set-up builds its containers and passes the library's
problem validation; only device allocation, which needs a GPU, is left."""
import ctypes as C
import sys
from pathlib import Path

import pytest

sys.path.insert(0, str(Path(__file__).resolve().parents[1]))
import bench  # noqa: E402


def test_suite_covers_the_reference_families():
    names = [n for n, _ in bench.reference_benchmark_problems()]
    assert len(names) == len(set(names)) == 19
    for fam, count in (("advection_", 5), ("euler_", 6), ("mhd_", 8)):
        assert sum(n.startswith(fam) for n in names) == count


@pytest.mark.parametrize("name", [n for n, _ in bench.reference_benchmark_problems()])
def test_suite_problem_passes_validation(name):
    import trixicuda as T
    from trixicuda import _lib
    from trixicuda.semidiscretization import build_problem_desc

    setup = dict(bench.reference_benchmark_problems())[name]
    d, keep, cont = build_problem_desc(setup.mesh, setup.equations, setup.solver)
    assert cont.nelements > 0
    if name.endswith("mortar_2d") or name.endswith("mortar_3d"):
        assert cont.nmortars > 0
    lib = _lib.load()
    h = C.c_void_p()
    st = lib.trixi_create(C.byref(d), C.byref(h))
    if st == 0:
        lib.trixi_destroy(h)
    # INVALID_ARGUMENT (1) / UNSUPPORTED (2) would mean the set-up is refused
    assert st not in (1, 2), _lib.last_error()


def test_nan_aware_error():
    import numpy as np

    ref = np.array([1.0, 2.0, np.nan, 4.0])
    r = bench._nan_aware_rel_err(np.array([1.0, 2.0, np.nan, 4.0 + 1e-12]), ref)
    assert r["nan_positions_match"] and r["nonfinite_entries"] == 1
    assert 0 < r["fp64_rel_err_vs_oracle"] < 1e-12
    r = bench._nan_aware_rel_err(np.array([1.0, np.nan, 3.0, 4.0]), ref)
    assert not r["nan_positions_match"]


def test_reference_arm_line(capsys, monkeypatch):
    """`bench.py --impl reference` prints one JSON line with the contract's
    keys, timed on the oracle alone (a shortened sample here)."""
    import json
    import types

    real = bench.cpu_baseline
    monkeypatch.setattr(bench, "cpu_baseline", lambda seconds_target=8.0, nthreads=None: real(0.2, nthreads))
    args = types.SimpleNamespace(steps=1, warmup=1, gpus=1)
    assert bench.run_reference(args) == 0
    line = json.loads(capsys.readouterr().out.strip().splitlines()[-1])
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "scaling", "dtype", "config", "impl", "cpu_baseline", "e2e"):
        assert key in line, key
    assert line["impl"] == "reference" and line["metric"] == bench.METRIC and line["value"] > 0
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["value"] == line["value"]
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["cores"] >= 1
