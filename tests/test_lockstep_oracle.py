"""The batched (lock-step) schedule against the reference's sequential model,
on the CPU oracle: the batched result must be a statistically faithful
erosion of the same terrain -- the same height budget identity and
hypsometry / slope / discharge distributions within the spread that the
sequential model itself shows between two random seeds."""
import numpy as np
import pytest


def hists(m):
    h = m.height.astype(np.float64)
    gx = np.zeros_like(h)
    gy = np.zeros_like(h)
    gx[1:-1] = (h[2:] - h[:-2]) / 2
    gy[:, 1:-1] = (h[:, 2:] - h[:, :-2]) / 2
    slope = np.hypot(gx, gy)
    return (np.histogram(h, 40, (0, 1))[0] / h.size,
            np.histogram(slope, 40, (0, 0.03))[0] / h.size,
            np.histogram(np.log1p(m.discharge), 40, (0, 7))[0] / h.size)


def l1(a, b):
    return [0.5 * np.abs(x - y).sum() for x, y in zip(a, b)]


@pytest.mark.parametrize("n,drops,cycles", [(256, 250, 200), (128, 1024, 40)])
def test_batched_matches_sequential_distributions(po, n, drops, cycles):
    H = po.value_noise(n, n, 1)
    seq = []
    for seed in (1, 2):
        m = po.Maps(n, n, height=H)
        sp = po.rand_spawns(seed, drops * cycles, n, n, 1)
        for c in range(cycles):
            po.erode_seq(m, sp[c * drops:(c + 1) * drops])
        seq.append(hists(m))
    spread = l1(seq[0], seq[1])
    mb = po.Maps(n, n, height=H)
    acc = po.erode_batched(mb, 7, 0, drops, cycles)
    dist = l1(seq[0], hists(mb))
    for d, s in zip(dist, spread):
        assert d < max(2.5 * s, 0.03), (dist, spread)
    dH = mb.height.astype(np.float64).sum() - H.astype(np.float64).sum()
    assert abs(dH - (acc.gain_q - acc.loss_q) / 2**32) < 1e-3 * max(1.0, abs(dH))
    assert np.isfinite(mb.height).all()


def test_batched_is_deterministic_and_cycle_keyed(po):
    n = 96
    H = po.value_noise(n, n, 8)
    a = po.Maps(n, n, height=H)
    b = po.Maps(n, n, height=H)
    po.erode_batched(a, 3, 0, 700, 3)
    hq = np.zeros((n, n), np.int64)      # the fixed-point heights carry over
    po.erode_batched(b, 3, 0, 700, 1, hq=hq)
    po.erode_batched(b, 3, 1, 700, 2, hq=hq)  # the cycle index keys the spawns
    for k in range(8):
        assert np.array_equal(a.f[k].view(np.uint32), b.f[k].view(np.uint32))


def test_one_drop_batched_equals_reference_step_rule(po):
    """With a single drop per cycle nothing is shared: the lock-step schedule
    reduces to the reference's Drop::descend + World::cascade, except that the
    cascade sees the step's erosion through fixed-point sums."""
    n = 64
    H = po.value_noise(n, n, 2)
    mb = po.Maps(n, n, height=H)
    acc = po.erode_batched(mb, 11, 0, 1, 1)
    assert acc.drops + acc.skipped == 1
    if acc.drops:
        assert acc.steps >= 1
