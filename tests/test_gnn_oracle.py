"""The ranking network's CPU restatement checked on its own (no GPU).

The FP64 backward is pinned by central finite differences; the BF16
rounding helper by exact values.
"""
import numpy as np
import pytest

from oracle import gnn_ref as R


def small_graph(n=23, arcs=70, seed=3, symmetric=False):
    rng = np.random.default_rng(seed)
    src = rng.integers(0, n, arcs)
    dst = rng.integers(0, n, arcs)
    keep = src != dst
    src, dst = src[keep], dst[keep]
    if symmetric:
        src, dst = np.concatenate([src, dst]), np.concatenate([dst, src])
    pairs = np.unique(np.stack([src, dst], 1), axis=0)

    def csr(a, b):
        order = np.lexsort((b, a))
        a, b = a[order], b[order]
        off = np.zeros(n + 1, np.uint64)
        np.add.at(off, a + 1, 1)
        return np.cumsum(off).astype(np.uint64), b.astype(np.uint32)

    off_out, head_out = csr(pairs[:, 0], pairs[:, 1])
    off_in, head_in = csr(pairs[:, 1], pairs[:, 0])
    return off_out, head_out, off_in, head_in


def test_bf16_rounding():
    v = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 2 ** -7, 1.0 + 3 * 2 ** -8, -2.5, 0.0, 3.0e38])
    q = R.bf16(v)
    # 1 + 2^-8 is halfway between 1 and 1 + 2^-7: ties to even -> 1
    assert q[0] == 1.0 and q[1] == 1.0 and q[2] == 1.0 + 2 ** -7
    # 1 + 3*2^-8 is halfway between 1 + 2^-7 and 1 + 2^-6: ties to even -> 1 + 2^-6
    assert q[3] == 1.0 + 2 ** -6
    assert q[4] == -2.5 and q[5] == 0.0
    assert np.isfinite(q[6])


def test_param_layout_round_trip():
    p = R.init_params(3, seed=5)
    assert p.size == R.param_count(3) == 3 * 64 + 64 + 3 * (128 * 64 + 64) + 64 + 1
    assert np.array_equal(R.pack(*R.unpack(p, 3)), p.astype(np.float64))


@pytest.mark.parametrize("symmetric", [False, True])
def test_fp64_gradient_matches_finite_differences(symmetric):
    layers = 2
    off_out, head_out, off_in, head_in = small_graph(symmetric=symmetric)
    csr = R.csr_of(off_out, head_out, off_in, head_in)
    x = R.features(off_out, head_out, off_in, seed=7).astype(np.float64)
    rng = np.random.default_rng(11)
    p = R.init_params(layers, seed=2).astype(np.float64)
    p += rng.normal(0, 0.05, p.size)       # non-zero biases
    y = rng.normal(0, 1, x.shape[0])
    loss, g = R.loss_and_grad(p, layers, x, csr, y, emulate=False)
    assert loss > 0
    idx = rng.choice(p.size, 80, replace=False)
    idx = np.concatenate([idx, [p.size - 1, p.size - 2, 0, 3 * 64 + 5]])
    eps = 1e-6
    for i in idx:
        d = np.zeros_like(p)
        d[i] = eps
        lp, _ = R.loss_and_grad(p + d, layers, x, csr, y, emulate=False)
        lm, _ = R.loss_and_grad(p - d, layers, x, csr, y, emulate=False)
        fd = (lp - lm) / (2 * eps)
        assert abs(fd - g[i]) <= 1e-6 + 1e-5 * abs(fd), (i, fd, g[i])


def test_features_definition():
    # path 0 -> 1 -> 2 and 1 -> 0: degrees (out + in) 2, 3, 1
    off_out = np.array([0, 1, 3, 3], np.uint64)
    head_out = np.array([1, 0, 2], np.uint32)
    off_in = np.array([0, 1, 2, 3], np.uint64)
    raw = R.raw_features(off_out, head_out, off_in, seed=1)
    assert np.allclose(raw[:, 0], np.log1p([2, 3, 1]).astype(np.float32))
    # 2-hop sums: 0 -> {1}: 3;  1 -> {0, 2}: 2 + 1;  2 -> {}: 0
    assert np.allclose(raw[:, 1], np.log1p([3, 3, 0]).astype(np.float32))
    # clustering: only vertex 1 has two out-neighbours (0, 2); 0's out-arcs {1}
    # contain neither 2 nor 0; 2 has none: no closed pair
    assert np.all(raw[:, 2] == 0)
    z = R.standardise(raw)
    assert np.allclose(z[:, 0].mean(), 0, atol=1e-6) and np.allclose(z[:, 2], 0)


def test_shipped_parameters_have_the_layout():
    import os
    p = np.load(os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                             "plant_gb300", "ranknet_l3.npy"))
    assert p.dtype == np.float32 and p.size == R.param_count(3)
    assert np.all(np.isfinite(p))
