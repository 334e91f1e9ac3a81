"""The launch-shape cache of the autotuner (host logic, no GPU).

The library keeps tuned shapes in a process-wide table keyed by code,
settings and device; sicc_tune_save / sicc_tune_load carry it as text lines
"key value...".  Loading merges entries, rejects malformed lines without
touching the table, and save writes every entry back.
"""
import os

import pytest

from sicc_gb300 import _lib, tune


def test_cache_file_round_trip(tmp_path):
    tune.clear()
    src = tmp_path / "shapes.txt"
    src.write_text("# tuned on one GB300\n"
                   "fec:00000000000000ab@NVIDIA_GB300/152 8 4 0 2 0\n"
                   "engine-code:00000000000000cd@NVIDIA_GB300/152 2\n")
    tune.load(str(src))
    assert tune.entries() == 2
    out = tmp_path / "again.txt"
    tune.save(str(out))
    assert sorted(out.read_text().splitlines()) == [
        "engine-code:00000000000000cd@NVIDIA_GB300/152 2",
        "fec:00000000000000ab@NVIDIA_GB300/152 8 4 0 2 0"]
    tune.clear()
    assert tune.entries() == 0


@pytest.mark.parametrize("line", ["no-colon-key 1 2", "fec:ab@x/1", "fec:ab@x/1 1 two", "fec:ab@x/1 99999999"])
def test_malformed_cache_lines_are_rejected(tmp_path, line):
    tune.clear()
    good = tmp_path / "good.txt"
    good.write_text("fec:01@NVIDIA_GB300/152 8 0 0 0 0\n")
    tune.load(str(good))
    bad = tmp_path / "bad.txt"
    bad.write_text(line + "\n")
    with pytest.raises(_lib.SiccError):
        tune.load(str(bad))
    assert tune.entries() == 1  # the table is unchanged
    tune.clear()


def test_missing_file_is_an_error(tmp_path):
    with pytest.raises(_lib.SiccError):
        tune.load(os.path.join(str(tmp_path), "absent.txt"))
