"""The CPU oracle pinned against the reference (no GPU).

* against the golden fixtures made from the reference's own build
  (tests/golden/make_golden.py): per-step drop traces, World::erode outputs,
  World::cascade, quad::map::normal -- bit for bit;
* directly against the compiled reference where oracle/_ref exists;
* the budget identity of the sequential model;
* the library's erf (used by the GPU) against math.erf.
"""
import hashlib
import json
import math
import os

import numpy as np
import pytest

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
N = 512


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a, np.float32).tobytes()).hexdigest()


def load(name):
    with open(os.path.join(GOLD, name)) as f:
        return json.load(f)


@pytest.fixture(scope="module")
def terrain(po):
    return po.value_noise(N, N, 1)


def test_golden_traces_fresh(po, terrain):
    tr = np.load(os.path.join(GOLD, "ref_traces.npz"))
    post = load("ref_traces_post.json")["post_height_sha"]
    for i, (x, y) in enumerate(tr["spawns_fresh"]):
        m = po.Maps(N, N, height=terrain)
        got, _ = po.drop_run(m, float(x), float(y))
        want = tr[f"fresh_{i}"]
        assert got.shape == want.shape, i
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), i
        assert sha(m.height) == post[f"fresh_{i}"], i


@pytest.fixture(scope="module")
def eroded(po, terrain):
    """srand(1); World::erode(512) x 4 through the oracle, checked per call."""
    gold = load("ref_erode.json")
    m = po.Maps(N, N, height=terrain)
    sp = po.rand_spawns(1, 4 * 512, N, N, gold["order"])
    for c in range(4):
        po.erode_seq(m, sp[c * 512:(c + 1) * 512])
        for k, f in enumerate(po.FIELDS):
            assert sha(m.f[k]) == gold["calls"][c]["sha"][f], (c, f)
    return m


def test_golden_erode(eroded):
    assert eroded is not None


def test_golden_traces_eroded(po, eroded):
    tr = np.load(os.path.join(GOLD, "ref_traces.npz"))
    post = load("ref_traces_post.json")["post_height_sha"]
    for i, (x, y) in enumerate(tr["spawns_eroded"]):
        m = eroded.copy()
        got, _ = po.drop_run(m, float(x), float(y))
        want = tr[f"eroded_{i}"]
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), i
        assert sha(m.height) == post[f"eroded_{i}"], i


def test_golden_cascade_and_normals(po, terrain):
    gold = load("ref_cascade.json")
    rough = (np.random.default_rng(gold["rough_seed"]).random((N, N)) ** 3).astype(np.float32)
    m = po.Maps(N, N, height=rough)
    for x, y in gold["points"]:
        po.cascade(m, x, y)
    assert sha(m.height) == gold["height_sha"]
    m = po.Maps(N, N, height=terrain)
    assert sha(po.normals(m)) == load("ref_normals.json")["sha"]


def test_sequential_budget_identity(po, terrain):
    """sum(H_final) - sum(H_init) = evaporation gain - boundary loss."""
    m = po.Maps(N, N, height=terrain)
    sp = po.rand_spawns(3, 1024, N, N, 1)
    acc = po.erode_seq(m, sp)
    dH = m.height.astype(np.float64).sum() - terrain.astype(np.float64).sum()
    assert abs(dH - (acc.gain - acc.loss)) < 1e-3
    assert acc.steps > 100000


def test_fp64_oracle_close_to_fp32(po, terrain):
    """The FP64 instance is the error reference: single drops agree early on."""
    m32 = po.Maps(N, N, height=terrain)
    m64 = m32.copy(np.float64)
    t32, _ = po.drop_run(m32, 100.5, 200.25)
    t64, _ = po.drop_run(m64, 100.5, 200.25)
    k = min(len(t32), len(t64), 20)
    rel = np.abs(t32[:k, 2:4] - t64[:k, 2:4]) / np.maximum(1.0, np.abs(t64[:k, 2:4]))
    assert rel.max() < 1e-5


@pytest.mark.skipif(not os.path.exists(os.path.join(os.path.dirname(GOLD), "..", "oracle", "_ref",
                                                    "libshyref.so")),
                    reason="reference harness not built (no reference checkout here)")
def test_live_reference_random_drops(po, terrain):
    rng = np.random.default_rng(123)
    base = po.Maps(N, N, height=terrain)
    for _ in range(10):
        x, y = rng.uniform(0, N, 2)
        po.ref_set_maps(base)
        want = po.ref_drop_run(float(x), float(y))
        m = base.copy()
        got, _ = po.drop_run(m, float(x), float(y))
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
        ref_after = po.ref_get_maps()
        for k in range(8):
            assert np.array_equal(ref_after.f[k].view(np.uint32), m.f[k].view(np.uint32))


def test_library_erf(po):
    xs = np.concatenate([np.linspace(0, 4.5, 20001), np.geomspace(1e-30, 1.0, 2001)]).astype(np.float32)
    for x in xs:
        got = po.lib().orc_erff_shy(float(x))
        want = np.float32(math.erf(float(x)))
        # within one float ulp of the exact value rounded to float
        assert abs(got - want) <= np.spacing(np.float32(abs(want))), (x, got, want)
        assert po.lib().orc_erff_shy(float(-x)) == -got
    assert po.lib().orc_erff_shy(0.0) == 0.0
    assert po.lib().orc_erff_shy(10.0) == 1.0
