"""Host-side checks of the autotuner (no GPU): its defaults are the
planner's, its search space names real tunables, and the coordinate descent
keeps the fastest tuning it timed."""
import re
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]


def _planner_defaults() -> dict:
    src = (ROOT / "bendy2d_gb300" / "csrc" / "engine.hpp").read_text()
    body = src[src.index("struct PlanTuning {"):src.index("bool set(const std::string& key")]
    out = {}
    for m in re.finditer(r"(?:float|uint32_t)\s+([^;]+);", body):
        for part in m.group(1).split(","):
            if "=" in part:
                k, v = (x.strip() for x in part.split("="))
                out[k] = float(eval(v.rstrip("f").replace("u", "")))
    return out


def test_defaults_match_the_planner():
    from bendy2d_gb300.autotune import DEFAULTS, RING_SPACE, SPACE
    planner = _planner_defaults()
    for k, v in DEFAULTS.items():
        assert planner[k] == float(v), k
    assert set(SPACE) <= set(DEFAULTS) and set(RING_SPACE) <= set(DEFAULTS)


class _FakeRunner:
    """Times a tuning by a made-up cost; records what was applied."""

    def __init__(self):
        self.applied = []
        self.cur = {}

    def set_tuning(self, **kv):
        self.cur = dict(kv)
        self.applied.append(dict(kv))


def test_coordinate_descent_keeps_the_fastest():
    from bendy2d_gb300.autotune import DEFAULTS, tune_runner
    space = {"stage_frac": [0.4, 0.67, 1.01], "serial_width": [1.5, 2.0, 4.0]}

    def cost(r):
        c = r.cur
        return 10.0 - 3.0 * (c["stage_frac"] == 0.4) - 2.0 * (c["serial_width"] == 4.0)

    r = _FakeRunner()
    log = []
    best = tune_runner(r, cost, space, log)
    assert best["stage_frac"] == 0.4 and best["serial_width"] == 4.0
    assert best["_ms_per_step"] == 5.0
    assert r.cur == {"stage_frac": 0.4, "serial_width": 4.0}  # left tuned to the best
    assert log[0] == ({}, 10.0)
    # every applied tuning sets every tunable of the space (defaults filled in)
    assert all(set(a) == set(space) for a in r.applied)
    assert r.applied[0] == {k: DEFAULTS[k] for k in space}
