"""The batch autotuner's host logic on the CPU: the workload signature, the JSON cache,
the candidate set, how a configuration is applied, and that a cached choice is reused
without a search (no GPU needed: a fake backend records the options it is given)."""
import json
from types import SimpleNamespace

from portablert_gb300 import autotune


class FakeBackend:
    def __init__(self):
        self.options = {}

    def set_option(self, key, value):
        self.options[key] = value

    def device_name(self):
        return "fake-gb300"


def _queries(n_rays):
    return [SimpleNamespace(scene=i, field_mask=31, n_rays=n, rec_size=32)
            for i, n in enumerate(n_rays)]


def test_signature_is_stable_and_tells_workloads_apart():
    a = autotune.signature([0, 10, 30], _queries([5, 7]))
    assert a == autotune.signature([0, 10, 30], _queries([5, 7]))
    assert a.startswith("S2-T30-R12-")
    assert a != autotune.signature([0, 10, 31], _queries([5, 7]))
    assert a != autotune.signature([0, 10, 30], _queries([5, 8]))


def test_cache_round_trip(tmp_path):
    path = str(tmp_path / "sub" / "autotune.json")
    assert autotune._load(path) == {}
    autotune._store(path, {"k": {"ms": 1.5}})
    assert autotune._load(path) == {"k": {"ms": 1.5}}
    with open(path, "w") as f:
        f.write("not json")
    assert autotune._load(path) == {}


def test_candidates_cover_every_knob_combination():
    c = list(autotune.candidates())
    assert len(c) == 2 * 4 * 2
    assert {(x["node_format"], x["leaf_size"], x["block"]) for x in c} == {
        (f, l, b) for f in (0, 1) for l in (1, 2, 4, 8) for b in (64, 128)}


def test_apply_sets_every_knob_and_the_compressed_build():
    be = FakeBackend()
    autotune.apply(be, {"node_format": 1, "leaf_size": 4, "block": 64, "pool_depth": 9})
    assert be.options == {"build_compressed": 1, "node_format": 1, "leaf_size": 4,
                          "block": 64, "pool_depth": 9}
    autotune.apply(be, {"node_format": 0, "leaf_size": 1, "block": 128, "pool_depth": 0})
    assert be.options["build_compressed"] == 0


def test_cached_choice_is_reused_without_a_search(tmp_path):
    be = FakeBackend()
    tri_off, qs = [0, 100, 250], _queries([64, 32])
    key = f"fake-gb300|{autotune.signature(tri_off, qs)}|0,1"
    best = {"config": {"node_format": 0, "leaf_size": 2, "block": 128, "pool_depth": 7},
            "ms": 3.25, "tried": []}
    path = tmp_path / "autotune.json"
    path.write_text(json.dumps({key: best}))
    got = autotune.tune_batch(be, 0, tri_off, qs, cache=str(path))
    assert got["cached"] is True and got["config"] == best["config"]
    assert be.options["leaf_size"] == 2 and be.options["pool_depth"] == 7
