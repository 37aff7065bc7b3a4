"""The autotuner's cache file (CPU): entries written by several processes at
the same time (replicas tuning on their own GPUs) are all kept, and an
unreadable or missing file means an empty cache."""
import json
import multiprocessing as mp

from gisapr_gb300.autotune import Autotuner


def _writer(path, tag, n):
    t = Autotuner(cache_path=path)
    for i in range(n):
        t._save(f"{tag}|{i}", {"size": i, "tag": tag})


def test_concurrent_writers_keep_every_entry(tmp_path):
    path = tmp_path / "tuning.json"
    ctx = mp.get_context("spawn")
    procs = [ctx.Process(target=_writer, args=(str(path), f"w{k}", 25)) for k in range(3)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    data = json.loads(path.read_text())
    assert sorted(data) == sorted(f"w{k}|{i}" for k in range(3) for i in range(25))
    assert not list(tmp_path.glob("*.tmp"))


def test_unreadable_cache_is_empty(tmp_path):
    path = tmp_path / "tuning.json"
    t = Autotuner(cache_path=path)
    assert t._load() == {}
    path.write_text("{not json")
    assert t._load() == {}
    t._save("k", {"size": 1})
    assert json.loads(path.read_text()) == {"k": {"size": 1}}
