"""The tuning sweep's header handling (no GPU): the TUNED block of
csrc/tg_tuning.h is read back as the settings compiled in now, and applying
a candidate (one change from those settings) keeps the rest."""
import shutil

from tetragpu_gb300 import tune


def test_tuned_block_round_trip(tmp_path):
    path = tmp_path / "tg_tuning.h"
    shutil.copy(tune.TUNING_H, path)
    now = tune.tuned_defines(str(path))
    assert all(k.startswith("TG_") and isinstance(v, int) for k, v in now.items())
    tune.write_header({**now, "TG_EFA_LANES": 1}, str(path))
    after = tune.tuned_defines(str(path))
    assert after == {**now, "TG_EFA_LANES": 1}
    # the defaults below the block are untouched
    text = path.read_text()
    assert text.count("// BEGIN TUNED") == 1 and text.count("// END TUNED") == 1
    assert "#define TG_STAR_WIN 256" in text


def test_default_selection_keeps_current_settings(tmp_path):
    path = tmp_path / "tg_tuning.h"
    shutil.copy(tune.TUNING_H, path)
    now = tune.tuned_defines(str(path))
    # "default" selects no change: applying it leaves the block as it was
    tune.write_header({**now, **{}}, str(path))
    assert tune.tuned_defines(str(path)) == now
