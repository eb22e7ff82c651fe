"""The CPU oracle of the charging network: its backward pass against finite differences of its
forward pass (FP64, no BF16 rounding), and the BF16 rounding it applies to the GEMM operands."""
import numpy as np

from oracle import mlp_oracle as M


def _blob(seed=0):
    rng = np.random.default_rng(seed)
    b = np.zeros(M.NBLOB)
    b[M.OFF_W1:M.OFF_B1] = (rng.standard_normal((M.H, M.KIN)) * 0.4 * (np.arange(M.KIN) < M.F)).reshape(-1)
    b[M.OFF_B1:M.OFF_W2] = rng.standard_normal(M.H) * 0.1
    b[M.OFF_W2:M.OFF_B2] = rng.standard_normal(M.H * M.H) * 0.15
    b[M.OFF_B2:M.OFF_W3] = rng.standard_normal(M.H) * 0.1
    b[M.OFF_W3:M.OFF_B3] = rng.standard_normal(M.H) * 0.2
    b[M.OFF_B3] = 0.05
    b[M.OFF_XMU:M.OFF_XSD] = rng.standard_normal(M.F)
    b[M.OFF_XSD:M.OFF_TMU] = 1.0 + rng.random(M.F)
    b[M.OFF_TMU], b[M.OFF_TSD] = 0.3, 2.0
    return b


def test_bf16_rounding_is_nearest_even():
    x = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -9, 1.0 + 2 ** -9, -2.5, 3.0e-39], np.float32)
    r = M.bf16(x)
    assert r[0] == 1.0
    assert r[1] == 1.0                                   # halfway between 1 and 1 + 2^-7: tie -> even
    assert r[3] == 1.0                                   # below halfway -> down
    assert r[2] == np.float32(1.0 + 2 ** -7)              # above halfway -> up
    assert r[4] == -2.5
    # bf16 keeps 8 significant bits
    y = M.bf16(np.float32(np.pi))
    assert abs(y - np.pi) / np.pi < 2 ** -8


def test_backward_matches_finite_differences():
    rng = np.random.default_rng(3)
    blob = _blob(1)
    feat = rng.standard_normal((40, M.F)) * 1.5 + blob[M.OFF_XMU:M.OFF_XSD]
    target = rng.standard_normal(40)
    g, _ = M.gradient(blob, feat, target, exact=True)

    def loss(b):
        t, c = M.forward(b, feat, exact=True)
        yn = (target - b[M.OFF_TMU]) / b[M.OFF_TSD]
        return np.mean((c["y"] - yn) ** 2)

    for p in list(rng.choice(M.NPARAM, 60, replace=False)) + [M.OFF_B3, M.OFF_W1 + 3, M.OFF_W2 + 77]:
        if p < M.OFF_B1 and (p % M.KIN) >= M.F:
            continue
        h = 1e-6
        bp, bm = blob.copy(), blob.copy()
        bp[p] += h
        bm[p] -= h
        fd = (loss(bp) - loss(bm)) / (2 * h)
        assert abs(fd - g[p]) <= 1e-6 * max(1.0, abs(fd)) + 1e-8, (p, fd, g[p])
