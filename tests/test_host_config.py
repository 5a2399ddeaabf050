"""The host-side configuration the benchmark and the batched planner read:
the autotuner's table (prrtc_gb300/tuning.json) and lookup, and the named
workloads (seeded, deterministic, optionally cached).  CPU only."""
import json

import numpy as np


def test_tuning_table_entries_are_valid():
    """Every entry names a known robot/workload pair; its `best` sets every
    knob to a value the sweep searches; a hand-set entry says why."""
    from prrtc_gb300 import autotune, workloads
    table = json.loads(autotune.TUNING.read_text())
    assert table
    for key, entry in table.items():
        robot, name = key.split("/")
        assert workloads.WORKLOADS[name][0] == robot, key
        assert set(entry["best"]) == set(autotune.KNOBS), key
        for k, v in entry["best"].items():
            assert v in autotune.SPACE[k], (key, k, v)
        assert entry["source"] in ("sweep", "hand-set"), key
        if entry["source"] == "hand-set":
            assert entry.get("note"), key
        for row in entry.get("sweep", []):
            assert row["solved"] >= 0 and row["ms_median"] > 0, key


def test_autotune_load_falls_back_to_robot_then_defaults():
    from prrtc_gb300 import autotune
    table = json.loads(autotune.TUNING.read_text())
    key = next(iter(table))
    robot, name = key.split("/")
    assert autotune.load(robot, name) == table[key]["best"]
    first_of_robot = next(v["best"] for k, v in table.items() if k.startswith(robot + "/"))
    assert autotune.load(robot, "no_such_workload") == first_of_robot
    assert autotune.load("no_such_robot") == autotune.DEFAULT


def test_workload_settings_are_planner_settings():
    from prrtc_gb300 import api, workloads
    assert set(workloads.SETTINGS) == set(workloads.WORKLOADS)
    for name, s in workloads.SETTINGS.items():
        api.Settings(**s)   # every key is a pRRTC_settings field


def _same(a, b):
    assert len(a) == len(b)
    for x, y in zip(a, b):
        assert (x.seed, x.kind) == (y.seed, y.kind)
        np.testing.assert_array_equal(x.start, y.start)
        np.testing.assert_array_equal(x.goal, y.goal)
        for k in ("spheres", "capsules", "z_aligned_capsules", "cuboids", "z_aligned_cuboids"):
            np.testing.assert_array_equal(getattr(x.env, k), getattr(y.env, k))


def test_workloads_are_deterministic_and_cache_round_trips(tmp_path, monkeypatch):
    from prrtc_gb300 import workloads
    monkeypatch.delenv("PRRTC_CACHE", raising=False)
    a = workloads.make("panda_tabletop", 3, seed0=11, procs=1)
    b = workloads.make("panda_tabletop", 3, seed0=11, procs=1)
    _same(a, b)
    assert [q.seed for q in a] == [11, 12, 13]
    assert not any(tmp_path.iterdir())
    monkeypatch.setenv("PRRTC_CACHE", str(tmp_path))
    c = workloads.make("panda_tabletop", 3, seed0=11, procs=1)      # built, then written
    assert (tmp_path / "panda_tabletop_3_11.pkl").exists()
    d = workloads.make("panda_tabletop", 3, seed0=11, procs=1)      # read back
    _same(a, c)
    _same(a, d)
