"""The tuning caches (autotune.tune_direct, ensemble.autotune) are written by every rank
of a job that tunes at the same time: a write is a private file renamed over the
cache, so a reader always sees a whole cache, never a torn one."""
import json
import multiprocessing as mp
import os


def _writer(path, tag, count):
    from gravhopper_gb300.autotune import save_cache
    for k in range(count):
        save_cache(path, {"writer": tag, "k": k, "ms": {str(s): float(s) for s in range(2000)}})


def test_concurrent_cache_writes_stay_whole(tmp_path):
    path = str(tmp_path / "cache" / "autotune.json")
    ctx = mp.get_context("spawn")
    procs = [ctx.Process(target=_writer, args=(path, t, 150)) for t in range(2)]
    for p in procs:
        p.start()
    reads = 0
    while any(p.is_alive() for p in procs):
        if os.path.exists(path):
            with open(path) as f:
                d = json.load(f)  # a torn file would not parse
            assert len(d["ms"]) == 2000
            reads += 1
    for p in procs:
        p.join()
        assert p.exitcode == 0
    with open(path) as f:
        assert json.load(f)["k"] == 149
    assert reads > 0
    assert os.listdir(os.path.dirname(path)) == ["autotune.json"]  # no private files left
