"""CPU checks of the autotuner's search and cache (no GPU)."""
import itertools
import json

from acqgb300 import autotune as T


def test_coordinate_descent_finds_separable_minimum():
    space = {"a": [1, 2, 3, 4], "b": [8, 16, 32], "c": ["x", "y"]}
    target = {"a": 3, "b": 16, "c": "y"}
    cost = lambda s: (s["a"] - 3) ** 2 + abs(s["b"] - 16) / 8 + (0 if s["c"] == "y" else 1) + 1.0
    best, c, trials = T.coordinate_descent(cost, {"a": 1, "b": 32, "c": "x"}, space)
    assert best == target and c == 1.0
    full = len(list(itertools.product(*space.values())))
    assert len(trials) < full


def test_coordinate_descent_keeps_start_when_nothing_improves():
    best, c, trials = T.coordinate_descent(lambda s: 5.0, {"a": 1}, {"a": [1, 2, 3]})
    assert best == {"a": 1} and c == 5.0 and len(trials) == 3


def test_cache_round_trip(tmp_path):
    p = str(tmp_path / "sub" / "cache.json")
    assert T.load_cache(p) == {}
    T.save_cache({"k": {"settings": {"tile_threads": 128}, "ms": 1.5}}, p)
    assert T.load_cache(p)["k"]["settings"]["tile_threads"] == 128
    (tmp_path / "bad.json").write_text("{not json")
    assert T.load_cache(str(tmp_path / "bad.json")) == {}
    json.loads(open(p).read())


class _FakePlan:
    """Records set_option calls; every option is accepted as given."""

    def __init__(self):
        self.calls = []

    def set_option(self, opt, value):
        self.calls.append((opt, value))
        return value

    def set_form(self, form):
        return form


def test_apply_passes_zero_only_for_knobs_where_zero_is_a_setting():
    # tile_mma = 0 selects the FP32 FFT tile; a zero launch shape means "the plan lacks that kernel"
    plan = _FakePlan()
    eff = T.apply(plan, {"tile_mma": 0, "tile_threads": 0, "column_width": 64})
    assert (T.KNOBS["tile_mma"], 0) in plan.calls
    assert (T.KNOBS["column_width"], 64) in plan.calls
    assert all(opt != T.KNOBS["tile_threads"] for opt, _ in plan.calls)
    assert eff == {"tile_mma": 0, "column_width": 64}


def test_tile_mma_is_a_candidate_knob():
    class G:
        num_blocks = 20
        num_coherently_integrated_code_periods = 10

    class P:
        geometry = G()

    cands = T.candidates(P())
    assert cands["tile_mma"] == [1, 0]


class _KeepingPlan(_FakePlan):
    """Search widths other than 4 and 8 have no instantiation: the option keeps the old value."""

    def __init__(self):
        super().__init__()
        self.width = 4

    def set_option(self, opt, value):
        self.calls.append((opt, value))
        if opt == T.KNOBS["search_width"]:
            if value in (4, 8):
                self.width = value
            return self.width
        return value


def test_shapes_without_an_instantiation_are_skipped():
    plan = _KeepingPlan()
    ok = {"search_width": 8, "column_width": 64}
    assert not T.unavailable(ok, T.apply(plan, ok))
    missing = {"search_width": 2, "column_width": 64}
    assert T.unavailable(missing, T.apply(plan, missing))
    assert T.unavailable({"tile_threads": 64}, {"tile_threads": None})
    # tile_mma = 0 is a setting, read back as 0
    assert not T.unavailable({"tile_mma": 0}, T.apply(plan, {"tile_mma": 0}))
    # coordinate descent never keeps an unavailable shape
    def cost(sh):
        return float("inf") if T.unavailable(sh, T.apply(plan, sh)) else {4: 2.0, 8: 1.5}[sh["search_width"]]
    best, c, _ = T.coordinate_descent(cost, {"search_width": 4}, {"search_width": [2, 4, 8, 16]})
    assert best == {"search_width": 8} and c == 1.5


def test_search_knobs_are_candidates():
    class G:
        num_blocks = 20
        num_coherently_integrated_code_periods = 40

    class P:
        geometry = G()

    cands = T.candidates(P())
    assert set(cands["search_width"]) >= {2, 4, 8} and set(cands["search_split"]) >= {25, 32, 40}
