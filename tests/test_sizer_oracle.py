"""CPU checks of the sizer's numpy oracle (the checker of the device kernels)
and of the training-data helpers: gradients against central finite
differences, BF16 rounding, and the complement used for erosion-chain inputs."""
from __future__ import annotations

import numpy as np

from oracle import sizer_oracle as S


def _params(seed=0):
    rng = np.random.default_rng(seed)
    p = np.zeros(S.NPARAM, np.float64)
    o = 0
    for name, shape in S.SHAPES:
        n = int(np.prod(shape))
        fan_in = shape[0] if len(shape) == 2 else 1
        p[o:o + n] = rng.uniform(-1, 1, n) * np.sqrt(6.0 / max(fan_in, 1)) * (1.0 if len(shape) == 2 else 0.1)
        o += n
    return p


def test_gradients_match_finite_differences():
    rng = np.random.default_rng(1)
    X = rng.normal(size=(37, S.NF))
    T = rng.normal(size=(37, S.NUSED))
    p = _params()
    loss, g = S.loss_and_gradients(p, X, T, quantize=False)
    # FP64 evaluation of an FP32-parameter network: perturb in FP64 directly
    def f(q):
        P = {k: v for k, v in S.unpack(q).items()}
        h1 = np.maximum(X @ P["W1"] + P["b1"], 0)
        h2 = np.maximum(h1 @ P["W2"] + P["b2"], 0)
        out = h2 @ P["W3"] + P["b3"]
        e = out[:, :S.NUSED] - T
        w = np.ones_like(e)
        w[:, 0] = np.where(e[:, 0] < 0, S.UNDER_WEIGHT, 1.0)
        return float((w * e ** 2).sum() / (len(X) * S.NUSED))
    assert abs(f(p.astype(np.float32).astype(np.float64)) - loss) < 1e-9
    idx = rng.choice(S.NPARAM, 200, replace=False)
    q = p.astype(np.float32).astype(np.float64)
    for i in idx:
        e = 1e-6
        a, b = q.copy(), q.copy()
        a[i] += e
        b[i] -= e
        fd = (f(a) - f(b)) / (2 * e)
        assert abs(fd - g[i]) <= 1e-6 + 1e-4 * abs(fd), (i, fd, g[i])
    # the unused fourth output has no gradient
    P = S.unpack(g)
    assert np.all(P["W3"][:, 3] == 0) and P["b3"][3] == 0


def test_bf16_round_to_nearest_even():
    x = np.array([1.0, 1.00390625, 1.005859375, 1.0078125 + 2 ** -9, -3.14159, 0.0], np.float32)
    r = S.bf16_round(x)
    # 1 + 2^-8 is a tie between 1 and 1 + 2^-7: even mantissa (1.0) wins
    assert r[0] == 1.0 and r[1] == 1.0
    assert r[2] == np.float32(1.0078125)
    assert np.all(np.abs(r[:-1] - x[:-1]) <= np.abs(x[:-1]) * 2 ** -8)
    assert np.all(r.view(np.uint32) & 0xFFFF == 0)


def test_complement_shape_and_order(vo):
    from voroffset_gb300.train_sizer import complement
    g, offs, z = vo.synth_volume(vo.SynthSpec(24, n_spheres=6, s_rmin=2, s_rmax=6, seed=4))
    g2, o2, z2 = complement(g, offs, z)
    assert (g2.nx, g2.ny) == (g.nx + 2, g.ny + 2)
    zmin = g.origin[2] / g.spacing - 1
    zmax = g.origin[2] / g.spacing + 2 * g.padding + g.extent[2] / g.spacing + 1
    for c in range(g2.nx * g2.ny):
        s = z2[2 * o2[c]:2 * o2[c + 1]]
        assert s.size >= 2 and np.all(np.diff(s) >= 0)
        assert s[0] >= zmin and s[-1] <= zmax
    # an empty input column becomes one full segment; the border is full
    x, y = 0, 0
    assert list(z2[2 * o2[0]:2 * o2[1]]) == [zmin, zmax]
    for c in range(g.nx * g.ny):
        if offs[c + 1] == offs[c]:
            cx, cy = c % g.nx + 1, c // g.nx + 1
            c2 = cx + g2.nx * cy
            assert list(z2[2 * o2[c2]:2 * o2[c2 + 1]]) == [zmin, zmax]
            break
