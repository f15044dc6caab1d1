"""The tuning table behind cbk_cuda_autotune (CPU: no device work).

The table is the library's only global state: set / get / reset of single
entries, argument checks in order, and a save -> reset -> load round trip
through the text file that CBK_CUDA_TUNE_FILE can name.
"""
import os

import pytest


@pytest.fixture
def tune():
    import cbk_gb300
    cbk_gb300.tune_reset()
    yield cbk_gb300
    cbk_gb300.tune_reset()


def test_set_get_reset(tune):
    assert tune.tune_get("posv", "d", 48)[1] == {"threads": 0, "variant": 0, "vlen": 0}
    assert tune.tune_set("posv", "d", 48, threads=256, vlen=64) == 0
    assert tune.tune_get("posv", "d", 48)[1] == {"threads": 256, "variant": 0, "vlen": 64}
    assert tune.tune_get("posv", "s", 48)[1]["threads"] == 0      # per precision
    assert tune.tune_get("posv", "d", 47)[1]["threads"] == 0      # per order
    assert tune.tune_set("posv_refined", "d", 48, variant=1) == 0
    assert tune.tune_get("posv_refined", "d", 48)[1]["variant"] == 1
    # the least squares' kernel choice (0: a warp per matrix, 1: a lane per matrix)
    assert tune.tune_set("gels_refined", "d", 16, variant=1) == 0
    assert tune.tune_get("gels_refined", "d", 16)[1]["variant"] == 1
    assert tune.tune_get("gels_refined", "d", 8)[1]["variant"] == 0
    assert tune.tune_set("sysvnp_bucketed", "d", 48, variant=3) == 0
    assert tune.tune_get("sysvnp_bucketed", "d", 48)[1]["variant"] == 3
    assert tune.tune_get("posv_bucketed", "d", 48)[1]["variant"] == 0
    # orders past 64 share one entry
    assert tune.tune_set("geqrf", "s", 100, threads=64) == 0
    assert tune.tune_get("geqrf", "s", 300)[1]["threads"] == 64
    tune.tune_reset()
    assert tune.tune_get("posv", "d", 48)[1] == {"threads": 0, "variant": 0, "vlen": 0}


def test_argument_checks(tune):
    assert tune.tune_set("nope", "d", 8) == -1
    assert tune.tune_set("posv", "z", 8) == -2
    assert tune.tune_set("posv", "d", -1) == -3
    assert tune.tune_set("posv", "d", 8, threads=96) == -4
    assert tune.tune_set("posv", "d", 8, variant=4) == -5
    assert tune.tune_set("posv", "d", 8, vlen=48) == -6
    assert tune.tune_get("nope", "d", 8)[0] == -1
    # autotune validates before touching the device
    assert tune.autotune("nope", "d", 8, 8, 1, 64)[0] == -1
    assert tune.autotune("posv", "q", 8, 8, 1, 64)[0] == -2
    assert tune.autotune("geqrf", "d", 4, 8, 0, 64)[0] == -3     # m < n
    assert tune.autotune("posv", "d", 8, 0, 1, 64)[0] == -4
    assert tune.autotune("posv", "d", 8, 8, 0, 64)[0] == -5
    assert tune.autotune("posv", "d", 8, 8, 1, 0)[0] == -6
    assert tune.autotune("posv_refined", "s", 8, 8, 1, 64)[0] == -2
    # the least squares' variant is set, not measured
    assert tune.autotune("gels_refined", "d", 64, 16, 8, 64)[0] == -1
    assert tune.autotune_at("posv", "d", 8, 8, 1, 64, 48)[0] == -7
    assert tune.autotune_at("nope", "d", 8, 8, 1, 64, 32)[0] == -1


def test_save_load_round_trip(tune, tmp_path):
    entries = [("posv", "d", 8, 64, 0, 32), ("posv_refined", "d", 48, 0, 1, 64),
               ("gels", "s", 16, 256, 0, 128), ("sysvnp", "d", 64, 128, 0, 0),
               ("gels_refined", "d", 16, 0, 1, 0)]
    for e in entries:
        assert tune.tune_set(*e) == 0
    path = str(tmp_path / "tune.txt")
    assert tune.tune_save(path) == 0
    text = open(path).read().splitlines()
    assert text[0].startswith("#") and len(text) == 1 + len(entries)
    tune.tune_reset()
    assert tune.tune_load(path) == len(entries)
    for r, p, n, t, v, w in entries:
        assert tune.tune_get(r, p, n)[1] == {"threads": t, "variant": v, "vlen": w}
    # a malformed line stops the load and names itself
    with open(path, "a") as f:
        f.write("posv d 8 96 0 0\n")
    tune.tune_reset()
    assert tune.tune_load(path) == -(len(entries) + 2)
    assert tune.tune_load(str(tmp_path / "missing.txt")) == -1
    assert not os.path.exists(str(tmp_path / "missing.txt"))
