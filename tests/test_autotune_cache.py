"""The autotuner's cache on CPU: defaults without an entry, per-device entries, and a damaged file read as empty."""

import json

import pytest


@pytest.fixture()
def tune(tmp_path, monkeypatch):
    from pamo_gb300 import autotune

    path = tmp_path / "tune" / "autotune.json"
    monkeypatch.setenv("PAMO_GB300_TUNE", str(path))
    monkeypatch.setattr(autotune.torch.cuda, "is_available", lambda: True)
    monkeypatch.setattr(autotune.torch.cuda, "get_device_name", lambda *a: "GPU A")
    return autotune, path


def test_defaults_without_a_cache(tune):
    autotune, path = tune
    assert not path.exists()
    assert autotune.best_workers() == autotune.DEFAULT_WORKERS
    assert autotune.best_workers(7) == 7
    assert autotune.best_cg_mode() == 0


def test_entries_are_kept_per_device(tune, monkeypatch):
    autotune, path = tune
    autotune._store("batch_workers", 12)
    autotune._store("stage3_cg_mode", 3)
    assert autotune.best_workers() == 12 and autotune.best_cg_mode() == 3
    monkeypatch.setattr(autotune.torch.cuda, "get_device_name", lambda *a: "GPU B")
    assert autotune.best_workers() == autotune.DEFAULT_WORKERS  # another model: nothing tuned yet
    autotune._store("batch_workers", 24)
    data = json.loads(path.read_text())
    assert data == {"GPU A": {"batch_workers": 12, "stage3_cg_mode": 3}, "GPU B": {"batch_workers": 24}}


def test_damaged_cache_reads_as_empty(tune):
    autotune, path = tune
    path.parent.mkdir(parents=True)
    path.write_text("{not json")
    assert autotune.best_workers() == autotune.DEFAULT_WORKERS
    autotune._store("batch_workers", 8)  # rewritten whole
    assert autotune.best_workers() == 8
