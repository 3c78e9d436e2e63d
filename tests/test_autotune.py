"""The launch-shape autotuner's coordinate descent (superscanner_gb300/autotune.py)
with fake timers on the CPU: it keeps the fastest value of each knob, times
each knob with the earlier knobs' winners, and caches the result."""
import json

import pytest

from superscanner_gb300 import autotune as at

GRID_KW = dict(c=int(1e9), trunc=0.016, voxlength=0.004, resi_=480, resj_=640, storage="f16")
FASTEST = {"raycast_rows": 4, "collect_rows": 2, "fuse_ctas_per_sm": 16, "track_ctas_per_sm": 1,
           "refuse_ctas_per_sm": 4}


def _fake(seen):
    def stage(cfg):
        seen.append(dict(cfg))
        # each stage is fastest at its FASTEST value; the raycast also depends on the
        # collection tile (a cross term), so the order of the descent matters
        t = {st: 1.0 for st in at.STAGE.values()}
        for k, st in at.STAGE.items():
            t[st] += abs(cfg[k] - FASTEST[k])
        t["raycast"] += 0.5 * cfg["collect_rows"]
        return t

    def refuse(cfg):
        seen.append(dict(cfg))
        return 2.0 + abs(cfg["refuse_ctas_per_sm"] - FASTEST["refuse_ctas_per_sm"])
    return stage, refuse


def test_coordinate_descent_picks_each_knobs_fastest_value(tmp_path):
    seen = []
    stage, refuse = _fake(seen)
    cache = tmp_path / "tune.json"
    best = at.autotune(None, None, GRID_KW, (525.0, 525.0, 319.5, 239.5), cache=cache, stage_timer=stage,
                       refuse_timer=refuse)
    timings = best.pop("_ms")
    assert best == FASTEST
    assert len(seen) == sum(len(v) for v in at.CANDIDATES.values())
    # knob order: every timing of a knob carries the winners of the knobs before it
    order = list(at.CANDIDATES)
    i = 0
    for q, knob in enumerate(order):
        for v in at.CANDIDATES[knob]:
            cfg = seen[i]
            i += 1
            assert cfg[knob] == v
            for earlier in order[:q]:
                assert cfg[earlier] == FASTEST[earlier]
            for later in order[q + 1:]:
                assert cfg[later] == at.DEFAULT[later]
    assert set(timings) == set(order)
    assert timings["raycast_rows"]["4"] == pytest.approx(1.0 + 0.5 * at.DEFAULT["collect_rows"])

    # the cache holds the result under this GPU / size / storage key and is used next time
    stored = json.loads(cache.read_text())
    (key, entry), = stored.items()
    assert key.endswith("|480x640|f16") and entry["config"] == FASTEST
    seen.clear()
    again = at.autotune(None, None, GRID_KW, (525.0, 525.0, 319.5, 239.5), cache=cache, stage_timer=stage,
                        refuse_timer=refuse)
    assert again == FASTEST and seen == []


def test_ties_keep_the_first_candidate():
    flat = lambda cfg: {st: 1.0 for st in at.STAGE.values()}  # noqa: E731
    best = at.autotune(None, None, GRID_KW, (525.0, 525.0, 319.5, 239.5), stage_timer=flat,
                       refuse_timer=lambda cfg: 1.0)
    best.pop("_ms")
    assert best == {k: v[0] for k, v in at.CANDIDATES.items()}
