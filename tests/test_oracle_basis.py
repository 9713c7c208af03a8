"""Pins of the oracle's (and the library's) LGL basis against analytic known
answers -- the reference ships no golden vectors (its arithmetic lives in the
un-vendored Trixi.jl), so the basis is pinned by closed forms (Kopriva 2009)."""
import numpy as np
import pytest

from oracle import oracle as O


KNOWN = {
    # polydeg: (nodes, weights) in closed form
    1: ([-1.0, 1.0], [1.0, 1.0]),
    2: ([-1.0, 0.0, 1.0], [1 / 3, 4 / 3, 1 / 3]),
    3: ([-1.0, -np.sqrt(1 / 5), np.sqrt(1 / 5), 1.0], [1 / 6, 5 / 6, 5 / 6, 1 / 6]),
    4: ([-1.0, -np.sqrt(3 / 7), 0.0, np.sqrt(3 / 7), 1.0], [1 / 10, 49 / 90, 32 / 45, 49 / 90, 1 / 10]),
}


@pytest.mark.parametrize("p", sorted(KNOWN))
def test_lgl_nodes_weights_closed_form(p):
    b = O.basis(p)
    nodes, weights = KNOWN[p]
    np.testing.assert_allclose(b["nodes"], nodes, atol=1e-15)
    np.testing.assert_allclose(b["weights"], weights, atol=1e-15)


@pytest.mark.parametrize("p", [1, 2, 3, 4, 5, 6, 7])
def test_derivative_exact_and_sbp(p):
    b = O.basis(p)
    x, w, D = b["nodes"], b["weights"], b["dmat"]
    n = p + 1
    for k in range(n):
        np.testing.assert_allclose(D @ x**k, k * x ** max(k - 1, 0) if k else 0 * x, atol=2e-13)
    M = np.diag(w)
    B = np.zeros((n, n))
    B[0, 0], B[-1, -1] = -1, 1
    np.testing.assert_allclose(M @ D + (M @ D).T, B, atol=1e-13)   # SBP property
    np.testing.assert_allclose(b["dsplit"], 2 * D - np.linalg.inv(M) @ B, atol=1e-13)
    np.testing.assert_allclose(b["dhat"], -np.linalg.inv(M) @ D.T @ M, atol=1e-13)
    np.testing.assert_allclose(np.diag(b["dsplit"]), 0, atol=1e-13)  # LGL: split diagonal vanishes
    assert abs(np.sum(w) - 2) < 1e-14


@pytest.mark.parametrize("p", [1, 2, 3, 4, 5])
def test_mortar_operators(p):
    b = O.basis(p)
    x = b["nodes"]
    n = p + 1
    for k in range(n):
        f = lambda s: s**k  # noqa: E731
        np.testing.assert_allclose(b["fup"] @ f(x), f((x + 1) / 2), atol=1e-13)
        np.testing.assert_allclose(b["flo"] @ f(x), f((x - 1) / 2), atol=1e-13)
    # the L2 projection of the restriction of a P_{n-1} polynomial is itself
    np.testing.assert_allclose(b["rup"] @ b["fup"] + b["rlo"] @ b["flo"], np.eye(n), atol=1e-13)


@pytest.mark.parametrize("p", [1, 2, 3, 4, 5])
def test_inverse_vandermonde(p):
    from numpy.polynomial import legendre as L

    b = O.basis(p)
    x = b["nodes"]
    for j in range(p + 1):
        c = np.zeros(j + 1)
        c[j] = 1
        vals = L.legval(x, c) * np.sqrt(j + 0.5)
        e = b["ivdm"] @ vals
        np.testing.assert_allclose(e, np.eye(p + 1)[j], atol=1e-12)


@pytest.mark.parametrize("p", [1, 2, 3, 4, 5])
def test_library_basis_matches_oracle(p):
    """The product computes its own operators (host C++); they agree."""
    from trixicuda.solver import lgl_basis_item

    b = O.basis(p)
    pairs = [("nodes", "nodes"), ("weights", "weights"), ("derivative_split", "dsplit"), ("derivative_dhat", "dhat"),
             ("inverse_vandermonde_legendre", "ivdm"), ("forward_upper", "fup"), ("forward_lower", "flo"),
             ("reverse_upper", "rup"), ("reverse_lower", "rlo"), ("derivative_matrix", "dmat")]
    for lib_name, key in pairs:
        np.testing.assert_allclose(lgl_basis_item(p, lib_name), b[key], atol=2e-14, err_msg=lib_name)
