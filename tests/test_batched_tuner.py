"""CPU: the batched solver's panel-width autotuner (keys, choice, JSON cache) and its size buckets."""
import json

import pytest

from updes_gb300.batched import PanelTuner, size_bucket


def test_tuner_picks_the_fastest_and_caches(tmp_path):
    path = str(tmp_path / "widths.json")
    calls = []

    def measure(w):
        calls.append(w)
        return {16: 3.0, 32: 1.5, 64: 2.0}[w]

    t = PanelTuner(cache_path=path)
    key = PanelTuner.key("GB300", 0, "fp32", 1024)
    assert t.width(key, measure) == 32
    assert calls == [16, 32, 64]
    assert t.width(key, measure) == 32 and calls == [16, 32, 64]  # cached: no new measurement
    assert json.load(open(path)) == {key: 32}
    t2 = PanelTuner(cache_path=path)  # a new process reads the file
    assert t2.width(key, lambda w: pytest.fail("should not measure")) == 32


def test_tuner_ties_prefer_the_narrower_panel_and_memory_only_cache():
    t = PanelTuner(cache_path=None)
    assert t.width(PanelTuner.key("g", 1, "fp64", 256), lambda w: 1.0) == 16


def test_size_buckets():
    assert size_bucket(106) == 256 and size_bucket(257) == 512 and size_bucket(2031) == 2048
    with pytest.raises(ValueError):
        size_bucket(4097)


def test_pack_layout_aligns_and_separates_every_array():
    import numpy as np

    from updes_gb300.batched import _pack_layout
    rng = np.random.default_rng(5)
    sizes = []
    for _ in range(200):
        N = int(rng.integers(1, 2100))
        Ni = int(rng.integers(0, N + 1))
        sizes.append((N, Ni, N + int(rng.choice([1, 3, 6, 10]))))
    f_off, i_off, o_off, (fl, il, ol) = _pack_layout(sizes)
    fr, ir, orr = [], [], []
    for (N, Ni, n), fo, io, oo in zip(sizes, f_off, i_off, o_off):
        Nb = N - Ni
        fr += [(fo[0], 2 * N), (fo[1], 5 * Ni), (fo[2], 8 * Nb), (fo[3], N)]
        ir += [(io[0], Nb), (io[1], 2 * Nb)]
        orr += [(oo[0], n), (oo[1], N)]
        assert all(o % 32 == 0 for o in fo) and all(o % 64 == 0 for o in io) and all(o % 32 == 0 for o in oo)
    for regions, length in ((fr, fl), (ir, il), (orr, ol)):
        regions = sorted(r for r in regions if r[1] > 0)
        for (a, la), (b, _) in zip(regions, regions[1:]):
            assert a + la <= b
        assert regions[-1][0] + regions[-1][1] <= length
