"""The GWHT schedule autotuner's host logic on CPU: the library lists the valid
schedules of a shape and keeps the selection (host-side table, no GPU), the
tuner picks the fastest of a timing, selects it, caches it per shape and does
not time a cached shape again; QSFT_GWHT_AUTOTUNE=0 turns it off.  A fake
timer stands in for the device timing."""
import pytest

from qsft_gb300 import _lib, autotune

ROW, ROWC, CLUSTER, PASSES, SMALL = 1, 2, 3, 4, 5


@pytest.fixture(autouse=True)
def fresh():
    autotune.clear()
    yield
    autotune.clear()


def test_valid_schedules_per_shape():
    assert autotune.schedules(4, 7, "fp32") == [ROW, ROWC, CLUSTER, PASSES, SMALL]   # 16384 values
    assert ROWC not in autotune.schedules(4, 6, "fp32")                                # 4096: one CTA per row
    assert autotune.schedules(2, 15, "fp32")[0] == ROWC and ROW not in autotune.schedules(2, 15, "fp32")
    assert ROW not in autotune.schedules(4, 7, "fp64")                                  # 256 KB: no longer fits
    s = autotune.schedules(20, 3, "fp32")
    assert ROW not in s and ROWC not in s and PASSES in s
    assert autotune.schedules(4, 11, "fp32") == [PASSES, SMALL]                         # 2^22 values


def test_select_and_builtin_rule():
    assert autotune.selected(4, 7, "fp32") == ROWC                                      # the built-in rule
    autotune.select(4, 7, "fp32", PASSES)
    assert autotune.selected(4, 7, "fp32") == PASSES
    assert autotune.selected(4, 7, "fp64") != PASSES                                    # per precision
    with pytest.raises(_lib.QsftError):
        autotune.select(20, 3, "fp32", ROW)                                             # not valid for q=20
    autotune.select(4, 7, "fp32", 0)
    assert autotune.selected(4, 7, "fp32") == ROWC


def test_tune_picks_the_fastest_and_caches():
    calls = []

    def timer(s):
        calls.append(s)
        return {ROW: 0.30, ROWC: 0.20, CLUSTER: 0.50, PASSES: 0.15, SMALL: 0.40}[s]
    rec = autotune.ensure(4, 7, "fp32", timer=timer)
    assert rec["schedule"] == PASSES and rec["name"] == "passes"
    assert sorted(calls) == [ROW, ROWC, CLUSTER, PASSES, SMALL]
    assert autotune.selected(4, 7, "fp32") == PASSES
    assert autotune.ensure(4, 7, "fp32", timer=timer) is rec and len(calls) == 5       # cached: no new timing
    assert "fp32 q=4 b=7" in autotune.table()


def test_ties_go_to_the_lower_id():
    assert autotune.pick({PASSES: 1.0, ROW: 1.0, CLUSTER: 2.0}) == ROW


def test_disabled(monkeypatch):
    monkeypatch.setenv("QSFT_GWHT_AUTOTUNE", "0")
    assert autotune.ensure(4, 7, "fp32", timer=lambda s: pytest.fail("timed while disabled")) is None
    assert autotune.selected(4, 7, "fp32") == ROWC


def test_single_schedule_shapes_are_not_timed():
    single = [(q, b) for q, b in [(2, 3), (3, 2), (5, 2), (20, 2)] if len(autotune.schedules(q, b, "fp32")) == 1]
    assert single
    for q, b in single:
        rec = autotune.ensure(q, b, "fp32", timer=lambda s: pytest.fail("a single schedule was timed"))
        assert rec["schedule"] == autotune.schedules(q, b, "fp32")[0]
