"""The oracle's restatement of deal.II's element arithmetic, against the
published definitions: QGauss<1>(n) (Gauss-Legendre on [0,1]) against the
closed-form nodes and weights and its degree of exactness; FE_DGQ(k)'s
Lagrange basis on equidistant support points (Kronecker property, partition
of unity, derivatives summing to zero); the tensor cell rule QGauss<2>(k+2)
the reference uses for its cell terms (SolarCell.cpp:402-403)."""
import math

import numpy as np
import pytest

import oracle


CLOSED_FORMS = {
    1: ([0.5], [1.0]),
    2: ([0.5 - 0.5 / math.sqrt(3), 0.5 + 0.5 / math.sqrt(3)], [0.5, 0.5]),
    3: ([0.5 - 0.5 * math.sqrt(0.6), 0.5, 0.5 + 0.5 * math.sqrt(0.6)], [5 / 18, 8 / 18, 5 / 18]),
    4: (sorted(0.5 + s * 0.5 * math.sqrt(3 / 7 + t * 2 / 7 * math.sqrt(6 / 5))
               for s in (-1, 1) for t in (-1, 1)), None),
}


@pytest.mark.parametrize("n", [1, 2, 3, 4])
def test_gauss_rule_closed_forms(n):
    x, w = oracle.gauss01(n)
    xs, ws = CLOSED_FORMS[n]
    np.testing.assert_allclose(np.sort(x), xs, rtol=0, atol=1e-15)
    if ws is not None:
        np.testing.assert_allclose(w[np.argsort(x)], ws, rtol=0, atol=1e-15)
    else:   # n = 4: (18 -+ sqrt 30)/72 on the outer/inner pairs
        wo, wi = (18 - math.sqrt(30)) / 72, (18 + math.sqrt(30)) / 72
        np.testing.assert_allclose(w[np.argsort(x)], [wo, wi, wi, wo], rtol=0, atol=1e-15)
    # exact up to degree 2n - 1, not beyond
    for d in range(2 * n):
        assert abs(np.dot(w, x ** d) - 1.0 / (d + 1)) < 1e-15
    assert abs(np.dot(w, x ** (2 * n)) - 1.0 / (2 * n + 1)) > 1e-6


@pytest.mark.parametrize("k", [1, 2, 3])
def test_dgq_lagrange_basis(k):
    nodes = oracle.dgq_nodes(k)
    np.testing.assert_allclose(nodes, np.linspace(0.0, 1.0, k + 1), rtol=0, atol=0)
    val, der = oracle.lagrange1d(nodes, nodes)
    np.testing.assert_allclose(val, np.eye(k + 1), rtol=0, atol=1e-14)
    x = np.linspace(-0.3, 1.3, 17)
    val, der = oracle.lagrange1d(nodes, x)
    np.testing.assert_allclose(val.sum(0), 1.0, rtol=0, atol=1e-13)
    np.testing.assert_allclose(der.sum(0), 0.0, rtol=0, atol=1e-12)
    # a degree-k polynomial is reproduced from its nodal values, derivative too
    p = np.polynomial.Polynomial(np.arange(1.0, k + 2))
    np.testing.assert_allclose(p(nodes) @ val, p(x), rtol=1e-13, atol=1e-13)
    np.testing.assert_allclose(p(nodes) @ der, p.deriv()(x), rtol=1e-12, atol=1e-12)


@pytest.mark.parametrize("k", [1, 2])
def test_cell_rule_integrates_the_cell_terms_exactly(k):
    """QGauss<2>(k+2) is exact for x^a y^b with a, b <= 2k+3: every product of
    two DGQ_k functions and a bilinear coefficient on a cell."""
    g, w = oracle.gauss01(k + 2)
    X, Y = np.tile(g, k + 2), np.repeat(g, k + 2)
    W = np.tile(w, k + 2) * np.repeat(w, k + 2)
    for a in range(2 * k + 4):
        for b in range(2 * k + 4):
            assert abs(np.dot(W, X ** a * Y ** b) - 1.0 / ((a + 1) * (b + 1))) < 1e-15
