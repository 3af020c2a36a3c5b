"""GPU parity of the exact (sequential, live) mode against the CPU oracle.

The oracle's float instance is pinned bit for bit to the compiled reference
(test_oracle_reference.py); here the engine, called through the C ABI, must
give the oracle's bits:
  * with the library's erf on both sides (SHY_ERF_DEVICE vs ORC_ERF_SHY), and
  * with the host C library's erff on both sides (SHY_ERF_HOST_LIBM vs
    ORC_ERF_LIBM), which is what the reference itself calls.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

NX, NY = 160, 128


def bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


def assert_maps_equal(w, m, po, what=""):
    for k, name in enumerate(po.FIELDS):
        got = w.get_field(name)
        if not np.array_equal(bits(got), bits(m.f[k])):
            d = np.abs(got.astype(np.float64) - m.f[k]).max()
            raise AssertionError(f"{what}: field {name} differs (max |diff| {d:.3g})")


@pytest.fixture(scope="module")
def terrain(po):
    return po.value_noise(NX, NY, 11)


def test_terrain_generator_matches_oracle(shy, po):
    for (nx, ny, seed) in [(NX, NY, 11), (1024, 1024, 2), (37, 300, 7)]:
        w = shy.World(nx, ny)
        w.generate(seed, 8)
        assert np.array_equal(bits(w.get_field("height")), bits(po.value_noise(nx, ny, seed)))
        w.close()


def test_field_roundtrip(shy, terrain):
    w = shy.World(NX, NY)
    rng = np.random.default_rng(0)
    for f in shy.FIELD_NAMES:
        a = rng.random((NX, NY), dtype=np.float32)
        w.set_field(f, a)
        assert np.array_equal(w.get_field(f), a), f
    w.close()


@pytest.mark.parametrize("erf", ["device", "libm"])
def test_erode_exact_bitwise(shy, po, terrain, erf):
    """Several World::erode calls; discharge becomes nonzero after the first."""
    w = shy.World(NX, NY)
    w.set_field("height", terrain)
    m = po.Maps(NX, NY, height=terrain)
    if erf == "libm":
        w.set_erf_source(shy.ERF_HOST_LIBM)
    mode = po.ERF_LIBM if erf == "libm" else po.ERF_SHY
    spawns = po.rand_spawns(1, 5 * 120, NX, NY, 1)
    st_o = []
    for c in range(5):
        sp = spawns[c * 120:(c + 1) * 120]
        w.erode_exact(sp)
        st_o.append(po.erode_seq(m, sp, erf_mode=mode))
        assert_maps_equal(w, m, po, f"erode call {c}")
    st = w.stats()
    assert st.drop_steps == sum(a.steps for a in st_o)
    assert st.drops == sum(a.drops for a in st_o)
    assert st.drops_skipped == sum(a.skipped for a in st_o)
    assert st.evap_gain == pytest.approx(sum(a.gain for a in st_o), rel=1e-12)
    w.close()


def test_drop_trace_bitwise(shy, po, terrain):
    """Single-drop mode: every step of Drop::descend, on an eroded map."""
    w = shy.World(NX, NY)
    w.set_field("height", terrain)
    m = po.Maps(NX, NY, height=terrain)
    sp = po.rand_spawns(4, 300, NX, NY, 1)
    w.erode_exact(sp)
    po.erode_seq(m, sp, erf_mode=po.ERF_SHY)
    rng = np.random.default_rng(3)
    n_checked = 0
    for _ in range(12):
        x, y = rng.integers(0, NX), rng.integers(0, NY)
        tr = w.drop_run(float(x) + 0.25, float(y) + 0.5)
        to, _ = po.drop_run(m, float(x) + 0.25, float(y) + 0.5, erf_mode=po.ERF_SHY)
        assert tr.shape == to.shape
        assert np.array_equal(bits(tr), bits(to))
        n_checked += len(tr)
    assert_maps_equal(w, m, po, "after traces")
    assert n_checked > 100


def test_drop_descend_stepwise(shy, po, terrain):
    """Drop(pos); while (drop.descend()) one ABI call per step == one-shot run."""
    w = shy.World(NX, NY)
    w.set_field("height", terrain)
    m = po.Maps(NX, NY, height=terrain)
    d = shy.Drop(w, (40.0, 70.0))
    recs = []
    while True:
        more = d.descend()
        recs.append([1.0 if more else 0.0, d.age, *d.pos, *d.speed, d.volume, d.sediment])
        if not more:
            break
    to, _ = po.drop_run(m, 40.0, 70.0, erf_mode=po.ERF_SHY)
    assert np.array_equal(bits(np.array(recs, np.float32)), bits(to))
    assert_maps_equal(w, m, po, "stepwise")


def test_cascade_and_normals(shy, po):
    rng = np.random.default_rng(5)
    h = (rng.random((64, 48)) ** 3).astype(np.float32)  # rough: many steep pairs
    w = shy.World(64, 48)
    w.set_field("height", h)
    m = po.Maps(64, 48, height=h)
    for (x, y) in [(0.5, 0.5), (63.9, 47.2), (10.0, 20.0), (31.7, 0.0), (-0.5, 3.0)]:
        w.cascade((x, y))
        po.cascade(m, x, y)
    assert np.array_equal(bits(w.get_field("height")), bits(m.height))
    assert np.array_equal(bits(w.normals()), bits(po.normals(m)))


def test_invalid_spawn_rejected(shy):
    w = shy.World(32, 32)
    with pytest.raises(shy.ShyError) as e:
        w.erode_exact([[0, 0], [32, 1]])
    assert e.value.code == -1
    w.close()
