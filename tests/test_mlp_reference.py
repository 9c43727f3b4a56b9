"""The CPU checker of the warm-start network: its analytic backward pass against central
finite differences of its own FP64 forward pass."""
import numpy as np

from oracle import mlp_reference as R


def random_params(rng):
    p = {"w1": rng.normal(0, 0.4, (R.HID, R.IN_PAD)), "b1": rng.normal(0, 0.1, R.HID),
         "w2": rng.normal(0, 0.2, (R.HID, R.HID)), "b2": rng.normal(0, 0.1, R.HID),
         "w3": rng.normal(0, 0.2, (R.OUT_PAD, R.HID)), "b3": rng.normal(0, 0.1, R.OUT_PAD),
         "in_mu": rng.normal(0, 1, 8), "in_sig": rng.uniform(0.5, 2, 8), "out_mu": rng.normal(0, 1, 4),
         "out_sig": rng.uniform(0.5, 2, 4)}
    p["w1"][:, R.IN:] = 0.0
    p["w3"][R.OUT:] = 0.0
    p["b3"][R.OUT:] = 0.0
    return p


def test_backward_matches_finite_differences():
    rng = np.random.default_rng(1)
    p = random_params(rng)
    n = 17
    x = rng.normal(0, 2, (n, 8))
    t = np.zeros((n, 4))
    t[:, :3] = rng.normal(0, 1, (n, 3))
    t[:, 3] = rng.integers(1, 8, n)
    _, _, g = R.forward_backward(p, x, t, emulate_bf16=False)
    h = 1e-6
    for name, picks in (("w1", [(0, 0), (5, 3), (63, 5)]), ("b1", [(7,), (40,)]), ("w2", [(0, 0), (12, 31), (63, 63)]),
                        ("b2", [(3,), (60,)]), ("w3", [(0, 0), (1, 17), (2, 63)]), ("b3", [(0,), (2,)])):
        for idx in picks:
            q = {k: v.copy() for k, v in p.items()}
            q[name][idx] += h
            up = R.mean_loss(q, x, t)
            q[name][idx] -= 2 * h
            dn = R.mean_loss(q, x, t)
            fd = (up - dn) / (2 * h)
            assert abs(fd - g[name][idx]) <= 1e-6 * max(1.0, abs(fd)), (name, idx, fd, g[name][idx])


def test_bf16_rounding_is_nearest_even():
    assert R.bf16(np.float32(1.0)) == 1.0
    assert R.bf16(np.float32(1.0 + 2 ** -8)) == 1.0            # tie -> even
    assert R.bf16(np.float32(1.0 + 3 * 2 ** -8)) == 1.0 + 2 ** -6
    assert R.bf16(np.float32(-2.5)) == -2.5
