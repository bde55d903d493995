"""GPU plain orderings vs their CPU restatement (bit-exact)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def oracle_graph(P, O, g):
    off, head, ln = g.csr(True)
    return O.OGraph.from_csr(g.get_n(), off, head, ln)


@pytest.mark.parametrize("seed", [1, 99])
def test_degree_order(P, O, seed):
    g = P.Graph.rmat(12, 8, seed=4)
    og = oracle_graph(P, O, g)
    assert np.array_equal(P.Order.degree(g, seed=seed), og.degree_order(seed))


def test_degree_order_grid(P, O):
    g = P.Graph.grid(50, 40, seed=3)
    og = oracle_graph(P, O, g)
    assert np.array_equal(P.Order.degree(g, seed=7), og.degree_order(7))


@pytest.mark.parametrize("sources", [1, 16, 64])
def test_betweenness_order(P, O, sources):
    g = P.Graph.grid(30, 30, highways=10, hw_steps=8, seed=5)
    og = oracle_graph(P, O, g)
    assert np.array_equal(P.Order.betweenness(g, sources, seed=11), og.betweenness_order(sources, 11))


def test_betweenness_is_a_permutation(P):
    g = P.Graph.rmat(10, 8, seed=2)
    o = P.Order.betweenness(g, 32, seed=3)
    assert sorted(o.tolist()) == list(range(g.get_n()))
