"""The large-scale configuration on the GPU: an 8192^2 value-noise terrain
(67 M cells, about 9 GB of maps), 4,194,304 drops per cycle, per-cell
vegetation coupled to erosion (spawn probability 1e-4 per cell per cycle).
At this size the oracle is too slow, so the checks are size-independent:
two runs from the same state give the same bits (integer sums make the
schedule independent of thread timing, here with the drops in spawn-cell
order and their slots in global memory), the FP64 height budget holds, and
the vegetation grows and couples (finite, bounded root density)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

N, DROPS, CYCLES, SEED = 8192, 4194304, 2, 5


def run(shy, torch):
    p = shy.default_params()
    p.plant_spawn_prob = 1e-4
    w = shy.World(N, N, params=p, seed=SEED)
    w.generate(SEED, 8)
    h0 = w.get_state_device()["height"].double().sum().item()
    for _ in range(CYCLES):
        w.erode(DROPS, 1)
        w.vegetation_step(1)
    st = w.stats()
    state = w.get_state_device()
    root = w.get_field("root_density")
    plant = w.get_field("plant_size")
    w.close()
    return h0, st, state, root, plant


def test_large_scale_with_vegetation_is_reproducible_and_keeps_the_budget(shy):
    torch = pytest.importorskip("torch")
    h0, st, a, root, plant = run(shy, torch)
    assert st.drop_steps > 0.5 * DROPS * CYCLES * 100  # drops live hundreds of steps
    dh = a["height"].double().sum().item() - h0
    assert abs(dh - (st.evap_gain - st.boundary_loss)) < 1e-4 * st.evap_gain
    assert (plant > 0).sum() > 1000 and np.isfinite(root).all() and root.min() >= -1e-6
    h0b, stb, b, rootb, plantb = run(shy, torch)
    assert stb.drop_steps == st.drop_steps and h0b == h0
    for f in a:
        assert torch.equal(a[f].view(torch.int32), b[f].view(torch.int32)), f
    assert np.array_equal(root.view(np.uint32), rootb.view(np.uint32))
    assert np.array_equal(plant.view(np.uint32), plantb.view(np.uint32))
