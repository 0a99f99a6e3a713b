"""Host side of the launch-shape tuner (CPU only)."""


def test_tuning_table_round_trip(tmp_path):
    """The tuning table's host side: save/load, apply/reset through
    pz_tune_set (host only), and the gain of each tuned knob over its
    built-in default."""
    from pizza_gb300 import autotune
    table = {"k_fast_G": 8, "k_rloop_rg": {"96": 3, "192": 2}, "lanes": 2,
             "ms": {"k_fast": {"4": 0.75, "8": 0.63}, "k_rloop": {"96": {"3": 0.16, "default": 0.17},
                                                                   "192": {"2": 0.25, "default": 0.27}},
                    "lanes": {"1": 1.25, "2": 1.21}}}
    path = tmp_path / "t.json"
    autotune.save(table, str(path))
    assert autotune.load(str(path)) == table
    autotune.apply(table)
    autotune.reset(table)
    g = autotune.gain(table)
    assert g["k_fast"] == 1.0 and g["lanes"] == 1.0 and abs(g["k_rloop"] - 0.44 / 0.41) < 1e-3
