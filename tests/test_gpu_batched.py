"""GPU parity and properties of the batched (lock-step) mode.

At sizes the oracle finishes in seconds the engine must reproduce the
oracle's Lockstep restatement bit for bit (integer fixed-point sums make the
schedule deterministic).  At the full 1024^2 / 65,536-drop size the checks
are size-independent properties: run-to-run bit identity, the height budget
(sum of height changes = evaporation gain - boundary loss, FP64), finite and
bounded maps.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


def compare_all(get, m, po, what):
    for k, name in enumerate(po.FIELDS):
        got = get(name)
        if not np.array_equal(bits(got), bits(m.f[k])):
            d = np.abs(got.astype(np.float64) - m.f[k]).max()
            raise AssertionError(f"{what}: field {name} differs (max |diff| {d:.3g})")


@pytest.mark.parametrize("nx,ny,drops,cycles", [(128, 128, 512, 3), (96, 200, 2000, 2), (64, 64, 4096, 2)])
def test_batched_bitwise_vs_oracle(shy, po, nx, ny, drops, cycles):
    H = po.value_noise(nx, ny, 21)
    w = shy.World(nx, ny, seed=77)
    w.set_field("height", H)
    w.erode(drops, cycles)
    m = po.Maps(nx, ny, height=H)
    acc = po.erode_batched(m, 77, 0, drops, cycles)
    compare_all(w.get_field, m, po, f"{nx}x{ny}")
    st = w.stats()
    assert st.drop_steps == acc.steps
    assert st.drops == acc.drops and st.drops_skipped == acc.skipped and st.drops_oob == acc.oob
    assert st.evap_gain == pytest.approx(acc.gain_q / 2**32, abs=1e-9)
    assert st.boundary_loss == pytest.approx(acc.loss_q / 2**32, abs=1e-9)
    assert st.cycles == cycles
    w.close()


def test_relax_passes_bitwise(shy, po):
    nx, ny = 80, 72
    H = po.value_noise(nx, ny, 4)
    p = shy.default_params()
    p.cascade_passes = 2
    w = shy.World(nx, ny, params=p, seed=5)
    w.set_field("height", H)
    w.erode(800, 2)
    pp = po.default_params()
    pp.cascade_passes = 2
    m = po.Maps(nx, ny, height=H)
    po.erode_batched(m, 5, 0, 800, 2, pp)
    compare_all(w.get_field, m, po, "relax")


def test_other_evaporation_rates_bitwise(shy, po):
    # the batched kernel's float evaporation division off the default rate
    nx, ny = 90, 64
    H = po.value_noise(nx, ny, 6)
    for evap in (0.01, 0.0005):
        p = shy.default_params()
        p.evap_rate = evap
        w = shy.World(nx, ny, params=p, seed=8)
        w.set_field("height", H)
        w.erode(900, 2)
        pp = po.default_params()
        pp.evap_rate = evap
        m = po.Maps(nx, ny, height=H)
        po.erode_batched(m, 8, 0, 900, 2, pp)
        compare_all(w.get_field, m, po, f"evap {evap}")
        w.close()


def test_batch_of_terrains_matches_each_alone(shy, po):
    sizes = [(64, 96), (128, 128), (100, 37), (130, 70)]
    drops = [1536, 4096, 925, 2275]
    seeds = [1000, 1001, 1002, 1003]
    b = shy.Batch(sizes, drops, seeds)
    Hs = []
    for t, (nx, ny) in enumerate(sizes):
        b.generate(t, seeds[t], 8)
        Hs.append(po.value_noise(nx, ny, seeds[t]))
        assert np.array_equal(bits(b.get_field(t, "height")), bits(Hs[t]))
    b.erode(2)
    for t, (nx, ny) in enumerate(sizes):
        m = po.Maps(nx, ny, height=Hs[t])
        po.erode_batched(m, seeds[t], 0, drops[t], 2)
        compare_all(lambda f: b.get_field(t, f), m, po, f"terrain {t}")
    b.close()


def test_empty_and_degenerate(shy, po):
    # no drops: a cycle still blends (tracks are zero)
    w = shy.World(16, 16)
    H = po.value_noise(16, 16, 3)
    w.set_field("height", H)
    w.set_field("discharge", np.full((16, 16), 2.0, np.float32))
    w.erode(0, 1)
    m = po.Maps(16, 16, height=H)
    m.discharge[...] = 2.0
    po.erode_batched(m, 1, 0, 0, 1)
    # heights only pass through the 32.32 fixed point of the batched mode
    assert np.array_equal(bits(w.get_field("height")), bits(m.height))
    assert np.abs(m.height - H).max() < 2.0 ** -32
    assert np.allclose(w.get_field("discharge"), 1.8)
    # all spawns below 0.1 are skipped
    w.set_field("height", np.full((16, 16), 0.05, np.float32))
    w.reset_stats()
    w.erode(100, 1)
    st = w.stats()
    assert st.drops == 0 and st.drops_skipped == 100 and st.drop_steps == 0
    w.close()
    # a 1 x 1 map: every drop leaves at once
    w = shy.World(1, 1)
    w.set_field("height", np.ones((1, 1), np.float32))
    w.erode(50, 1)
    m = po.Maps(1, 1, height=np.ones((1, 1), np.float32))
    acc = po.erode_batched(m, 1, 0, 50, 1)
    assert w.stats().drop_steps == acc.steps
    compare_all(w.get_field, m, po, "1x1")
    w.close()


def test_full_size_properties(shy):
    """1024^2, 65,536 drops per cycle: bit-reproducible, budget holds."""
    n, drops, cycles = 1024, 65536, 4
    outs = []
    for rep in range(2):
        w = shy.World(n, n, seed=2)
        w.generate(2, 8)
        h0 = w.get_field("height").astype(np.float64)
        w.erode(drops, cycles)
        st = w.stats()
        h = w.get_field("height")
        outs.append((h, w.get_field("discharge"), w.get_field("momentum_x"), st.drop_steps))
        assert np.isfinite(h).all() and h.min() > -1.0 and h.max() < 2.0
        dH = h.astype(np.float64).sum() - h0.sum()
        budget = st.evap_gain - st.boundary_loss
        # float rounding of one height update per touched cell and step
        assert abs(dH - budget) < 1e-3 * max(1.0, abs(budget)), (dH, budget)
        assert st.drop_steps > drops * cycles * 50
        w.close()
    for a, b in zip(outs[0][:3], outs[1][:3]):
        assert np.array_equal(bits(a), bits(b))
    assert outs[0][3] == outs[1][3]


def test_consecutive_calls_carry_fixed_point_state(shy, po):
    """Three shy_erode calls of one cycle each == the oracle carrying its
    fixed-point heights between calls; a height upload restarts from floats."""
    nx, ny = 90, 110
    H = po.value_noise(nx, ny, 31)
    w = shy.World(nx, ny, seed=8)
    w.set_field("height", H)
    m = po.Maps(nx, ny, height=H)
    hq = np.zeros((nx, ny), np.int64)
    for c in range(3):
        w.erode(1500, 1)
        po.erode_batched(m, 8, c, 1500, 1, hq=hq)
    compare_all(w.get_field, m, po, "3 calls")
    # uploading heights makes the float map the state again
    h2 = w.get_field("height")
    w.set_field("height", h2)
    m.f[0][...] = h2
    m.hq_valid = False
    w.erode(1500, 1)
    po.erode_batched(m, 8, 3, 1500, 1, hq=hq)
    compare_all(w.get_field, m, po, "after upload")
    w.close()


@pytest.mark.parametrize("grid,order", [(1, 0), (7, 0), (0, 1), (1, 1)])
def test_launch_shape_does_not_change_results(shy, po, grid, order):
    """Few CTAs put the drop slots in global memory (4096 drops on one CTA
    need 640 KiB), and slots may be in spawn-cell order; the results equal
    the default launch's and the oracle's."""
    nx, ny, drops = 128, 96, 4096
    H = po.value_noise(nx, ny, 13)
    outs = []
    for g, o in ((0, 0), (grid, order)):
        w = shy.World(nx, ny, seed=6)
        w.set_launch(g, o)
        w.set_field("height", H)
        w.erode(drops, 2)
        outs.append([w.get_field(f) for f in po.FIELDS])
        steps = w.stats().drop_steps
        w.close()
    m = po.Maps(nx, ny, height=H)
    acc = po.erode_batched(m, 6, 0, drops, 2)
    assert steps == acc.steps
    for k, f in enumerate(po.FIELDS):
        assert np.array_equal(bits(outs[0][k]), bits(outs[1][k])), f
        assert np.array_equal(bits(outs[1][k]), bits(m.f[k])), f


def test_state_calls_equal_field_calls(shy, po):
    """shy_terrain_set_state / get_state: the same bits as four set_field /
    get_field calls, and the same erosion afterwards."""
    nx, ny = 70, 90
    rng = np.random.default_rng(3)
    st = {"height": po.value_noise(nx, ny, 5), "discharge": rng.gamma(0.5, 2.0, (nx, ny)).astype(np.float32),
          "momentum_x": rng.normal(0, 1, (nx, ny)).astype(np.float32),
          "momentum_y": rng.normal(0, 1, (nx, ny)).astype(np.float32)}
    a, b = shy.World(nx, ny, seed=4), shy.World(nx, ny, seed=4)
    for f, v in st.items():
        a.set_field(f, v)
    b.set_state(0, **st)
    got = b.get_state(0)
    for f in st:
        assert np.array_equal(bits(got[f]), bits(a.get_field(f))), f
    a.erode(1500, 2)
    b.erode(1500, 2)
    got = b.get_state(0)
    for f in st:
        assert np.array_equal(bits(got[f]), bits(a.get_field(f))), f
    # partial update leaves the other fields alone
    b.set_state(0, momentum_x=np.zeros((nx, ny), np.float32))
    assert np.array_equal(bits(b.get_field("discharge")), bits(got["discharge"]))
    assert not b.get_field("momentum_x").any()
    a.close()
    b.close()


def test_batch_beyond_shared_terrain_table(shy, po):
    """More terrains than the kernel's shared-memory terrain table (128): the
    table is read from global memory; every terrain still equals the oracle."""
    n = 130
    rng = np.random.default_rng(11)
    sizes = [(int(rng.integers(4, 20)), int(rng.integers(4, 20))) for _ in range(n)]
    drops = [int(rng.integers(0, 40)) for _ in range(n)]
    seeds = [500 + i for i in range(n)]
    b = shy.Batch(sizes, drops, seeds)
    for t in range(n):
        b.generate(t, seeds[t], 4)
    b.erode(2)
    for t in (0, 1, 64, 127, 128, 129):
        nx, ny = sizes[t]
        m = po.Maps(nx, ny, height=po.value_noise(nx, ny, seeds[t], 4))
        po.erode_batched(m, seeds[t], 0, drops[t], 2)
        compare_all(lambda f: b.get_field(t, f), m, po, f"terrain {t}")
    b.close()


def test_every_launch_shape_gives_the_oracle_bits(shy, po):
    """Every candidate of the autotuner's search space -- CTA size 64, 128 or
    256, every resident CTA or one per SM (and a small grid, so that CTAs
    hold several slots per thread), drop or spawn-cell order, drop slots in
    shared or global memory -- runs the same schedule: the oracle's bits."""
    from simplehydrology_gb300 import autotune
    nx, ny, drops = 96, 80, 3000
    H = po.value_noise(nx, ny, 21)
    m = po.Maps(nx, ny, height=H)
    acc = po.erode_batched(m, 3, 0, drops, 2)
    shapes = autotune.candidates() + [(7, 1, 64, 1), (5, 0, 128, 0), (3, -1, 256, 1)]
    for shape in shapes:
        w = shy.World(nx, ny, seed=3)
        w.set_field("height", H)
        autotune.apply(w, shape)
        w.erode(drops, 2)
        compare_all(w.get_field, m, po, f"shape {shape}")
        assert w.stats().drop_steps == acc.steps, shape
        w.close()


@pytest.mark.parametrize("settle", [0, 1])
@pytest.mark.parametrize("block,grid,order,resort", [(256, 0, 1, 1), (256, 0, 1, 2), (128, 5, 1, 3),
                                                     (64, 0, 0, 7), (256, 3, -1, 16), (64, 7, 1, 1)])
def test_redeal_gives_the_oracle_bits(shy, po, block, grid, order, resort, settle):
    """Live drops re-sorted by their cell and dealt to the CTAs again every
    `resort` steps (slots in global memory), after spawn in drop or
    spawn-cell order, with one or several slots per thread, each drop
    settling its own change or the first drop in a cell the cell's: the
    oracle's bits, on one terrain and on a batch of three (the sort key
    crosses terrain boundaries)."""
    nx, ny, drops = 96, 80, 3000
    H = po.value_noise(nx, ny, 21)
    m = po.Maps(nx, ny, height=H)
    acc = po.erode_batched(m, 3, 0, drops, 2)
    w = shy.World(nx, ny, seed=3)
    w.set_field("height", H)
    w.set_launch(grid, order)
    w.set_block(block, 0)
    w.set_resort(resort)
    w.set_settle(settle)
    w.erode(drops, 2)
    compare_all(w.get_field, m, po, f"re-deal every {resort}, settle {settle}")
    assert w.stats().drop_steps == acc.steps
    w.close()

    sizes = [(64, 48), (40, 72), (56, 56)]
    seeds = [11, 12, 13]
    b = shy.Batch(sizes, [900, 1500, 700], seeds)
    hs = [po.value_noise(x, y, 30 + t) for t, (x, y) in enumerate(sizes)]
    for t, h in enumerate(hs):
        b.set_field(t, "height", h)
    b.set_launch(grid, order)
    b.set_block(block, 0)
    b.set_resort(resort)
    b.set_settle(settle)
    b.erode(2)
    for t, ((x, y), h) in enumerate(zip(sizes, hs)):
        mt = po.Maps(x, y, height=h)
        po.erode_batched(mt, seeds[t], 0, [900, 1500, 700][t], 2)
        compare_all(lambda f: b.get_field(t, f), mt, po, f"batch terrain {t}, re-deal every {resort}")
    b.close()


def test_redeal_in_cuda_graphs_gives_the_oracle_bits(shy, po):
    """The re-deal interval is part of what a captured graph is keyed on:
    changing it between calls captures again, and the bits stay the
    oracle's."""
    nx, ny = 96, 80
    H = po.value_noise(nx, ny, 21)
    w = shy.World(nx, ny, seed=3)
    w.set_field("height", H)
    w.set_launch(0, 1)
    w.set_block(256, 0)
    w.set_graph(2)
    w.set_resort(4)
    w.set_settle(1)
    w.erode(2000, 2)
    w.set_resort(0)
    w.erode(2000, 2)
    m = po.Maps(nx, ny, height=H)
    po.erode_batched(m, 3, 0, 2000, 4)
    compare_all(w.get_field, m, po, "graphs with re-deals")
    w.close()


def test_autotune_applies_a_shape_and_keeps_results(shy, po):
    from simplehydrology_gb300 import autotune
    nx, ny, drops = 96, 80, 2000
    H = po.value_noise(nx, ny, 21)
    w = shy.World(nx, ny, seed=3)
    w.set_field("height", H)
    best, times = autotune.autotune(w, drops, cycles=3)
    assert best in times and len(times) == len(autotune.candidates()) == 36
    assert all(t > 0 for t in times.values())
    graph, gtimes = autotune.autotune.last_graphs
    assert graph in gtimes and sorted(gtimes) == sorted(autotune.GRAPHS)
    resort, rtimes = autotune.autotune.last_resorts
    assert resort in rtimes and sorted(rtimes) == sorted(autotune.RESORTS)
    w.erode(drops, 2)  # with the chosen shape
    m = po.Maps(nx, ny, height=H)
    po.erode_batched(m, 3, 0, drops, 2)
    compare_all(w.get_field, m, po, "after autotune")
    w.close()


def test_autotune_counts_the_sms():
    torch = pytest.importorskip("torch")
    from simplehydrology_gb300 import autotune
    assert autotune.sm_count() == torch.cuda.get_device_properties(0).multi_processor_count


def test_cycles_as_cuda_graphs_give_the_oracle_bits(shy, po):
    """Cycles replayed from CUDA graphs (7 cycles in graphs of 3: two
    replays and one cycle launched alone), a new capture after the drops per
    cycle change, and per-kernel timing (no graphs) all give the oracle's
    bits."""
    nx, ny = 96, 80
    H = po.value_noise(nx, ny, 21)
    w = shy.World(nx, ny, seed=3)
    w.set_field("height", H)
    w.set_graph(3)
    w.erode(2000, 7)
    w.erode(1500, 4)  # another drop count: captured again
    w.enable_timing(True)
    w.erode(1500, 2)  # timed kernels: launched one by one
    w.enable_timing(False)
    m = po.Maps(nx, ny, height=H)
    hq = np.zeros((nx, ny), np.int64)
    po.erode_batched(m, 3, 0, 2000, 7, hq=hq)
    po.erode_batched(m, 3, 7, 1500, 6, hq=hq)
    compare_all(w.get_field, m, po, "graphs")
    assert w.cycle() == 13
    w.close()


def test_whole_world_state_equals_per_terrain_state(shy, po):
    """shy_world_set_state / shy_world_get_state move every terrain's state
    in one call each way, laid out terrain after terrain; the result equals
    the per-terrain state calls' bit for bit, and a batch uploaded either way
    erodes to the same bits."""
    sizes = [(64, 48), (40, 72), (56, 56)]
    seeds = [21, 22, 23]
    drops = [900, 1500, 700]
    rng = np.random.default_rng(5)
    hs = [po.value_noise(x, y, 40 + t) for t, (x, y) in enumerate(sizes)]
    ds = [rng.random((x, y), dtype=np.float32) * 3 for x, y in sizes]
    mxs = [rng.standard_normal((x, y)).astype(np.float32) for x, y in sizes]
    mys = [rng.standard_normal((x, y)).astype(np.float32) for x, y in sizes]
    outs = []
    for whole in (False, True):
        b = shy.Batch(sizes, drops, seeds)
        if whole:
            cat = lambda arrs: np.concatenate([a.reshape(-1) for a in arrs])
            b.set_state_all(height=cat(hs), discharge=cat(ds), momentum_x=cat(mxs), momentum_y=cat(mys))
        else:
            for t in range(len(sizes)):
                b.set_state(t, height=hs[t], discharge=ds[t], momentum_x=mxs[t], momentum_y=mys[t])
        st = b.get_state_all()
        b.erode(2)
        st2 = b.get_state_all()
        per = [b.get_state(t) for t in range(len(sizes))]
        outs.append((st, st2, per))
        b.close()
    for k in outs[0][0]:
        assert np.array_equal(bits(outs[0][0][k]), bits(outs[1][0][k])), k
        assert np.array_equal(bits(outs[0][1][k]), bits(outs[1][1][k])), k
    # the flat layout is the per-terrain arrays back to back
    for k in outs[1][1]:
        flat = np.concatenate([p[k].reshape(-1) for p in outs[1][2]])
        assert np.array_equal(bits(outs[1][1][k]), bits(flat)), k
