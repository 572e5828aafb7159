"""The batched solver's tuning table on disk (bola_batch_tuning_save/_load,
batch.Tuning), host only: a table written is read back unchanged, and files
that are not tables or hold values the kernel does not support are refused."""
import json

import pytest


@pytest.fixture(scope="module")
def Tuning():
    from bola_gb300 import _lib
    if not __import__("os").path.exists(_lib.LIB_PATH):
        from bola_gb300 import build
        build.build()
    from bola_gb300.batch import Tuning
    return Tuning


def test_round_trip(tmp_path, Tuning):
    t = Tuning([32, 64, 64, 128, 128, 256, 256, 256], [8, 12, 16, 16, 12, 8, 16, 12], 2)
    p = tmp_path / "tuning.json"
    t.save(p)
    data = json.loads(p.read_text())  # plain JSON
    assert data["group_size"] == t.group_size and data["panel_width"] == t.panel_width and data["tile_rows"] == 2
    u, sms = Tuning.load(p)
    assert u.as_dict() == t.as_dict()
    assert sms == data["sms"]


def test_refuses_bad_tables(tmp_path, Tuning):
    p = tmp_path / "bad.json"
    p.write_text('{"group_size": [32, 32], "panel_width": [8], "tile_rows": 4}')
    with pytest.raises(ValueError):
        Tuning.load(p)
    p.write_text(json.dumps({"group_size": [32, 48, 64, 64, 128, 128, 256, 256], "panel_width": [8] * 8,
                             "tile_rows": 4}))
    with pytest.raises(ValueError):  # 48 threads per system is not a group size
        Tuning.load(p)
    p.write_text(json.dumps({"group_size": [32] * 8, "panel_width": [8] * 7 + [10], "tile_rows": 4}))
    with pytest.raises(ValueError):  # panel width 10 is not built
        Tuning.load(p)
    p.write_text(json.dumps({"group_size": [32] * 8, "panel_width": [8] * 8, "tile_rows": 3}))
    with pytest.raises(ValueError):
        Tuning.load(p)
    with pytest.raises(ValueError):
        Tuning.load(tmp_path / "missing.json")
