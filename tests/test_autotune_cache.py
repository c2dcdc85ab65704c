"""The autotuner's JSON cache (starpolymersmd_gb300/autotune.py), with a fake
context standing in for the C ABI (no GPU needed): a miss measures and
stores the chosen launch shapes, a hit applies them without measuring,
entries written before the periodic-MD shapes existed still apply, and an
unreadable cache counts as empty."""
import json
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

from starpolymersmd_gb300 import autotune  # noqa: E402


class FakeContext:
    def __init__(self, tuned=(1, 5, 2), pmd=3):
        self.variants = (0, 0, 0)
        self.pmd = 0
        self.tuned = tuned
        self.tuned_pmd = pmd
        self.calls = []

    def autotune(self, cycles):
        self.calls.append(("autotune", cycles))
        self.variants, self.pmd = self.tuned, self.tuned_pmd
        return {"collide": {"chosen": "128t 64c cap704 cp.async", "index": self.tuned[1]}}

    def set_variants(self, bin, collide, md):
        self.calls.append(("set_variants", (bin, collide, md)))
        self.variants = (bin, collide, md)

    def get_variants(self):
        return self.variants

    def set_pmd_variant(self, pmd):
        self.calls.append(("set_pmd_variant", pmd))
        self.pmd = pmd

    def get_pmd_variant(self):
        return self.pmd


def test_miss_measures_and_hit_applies(tmp_path):
    path = str(tmp_path / "cache.json")
    a = FakeContext()
    first = autotune.tune(a, "gpu|rep=1", cycles=4, cache_path=path)
    assert first["cached"] is False
    assert a.calls == [("autotune", 4)]
    assert first["index"] == [1, 5, 2, 3]
    assert json.load(open(path))["gpu|rep=1"]["index"] == [1, 5, 2, 3]

    b = FakeContext()
    second = autotune.tune(b, "gpu|rep=1", cache_path=path)
    assert second["cached"] is True
    assert ("autotune", 3) not in b.calls
    assert b.get_variants() == (1, 5, 2) and b.get_pmd_variant() == 3

    # another workload signature is measured on its own
    c = FakeContext(tuned=(2, 9, 4), pmd=1)
    assert autotune.tune(c, "gpu|rep=256", cache_path=path)["cached"] is False
    cache = json.load(open(path))
    assert set(cache) == {"gpu|rep=1", "gpu|rep=256"}


def test_entries_without_the_periodic_shape_and_force(tmp_path):
    path = str(tmp_path / "cache.json")
    with open(path, "w") as f:
        json.dump({"k": {"index": [3, 7, 1], "report": {}}}, f)
    a = FakeContext()
    out = autotune.tune(a, "k", cache_path=path)
    assert out["cached"] is True
    assert a.calls == [("set_variants", (3, 7, 1))]  # no periodic-MD shape stored: left alone
    assert a.get_pmd_variant() == 0

    b = FakeContext(tuned=(0, 11, 4), pmd=2)
    out = autotune.tune(b, "k", cache_path=path, force=True)
    assert out["cached"] is False and b.calls[0][0] == "autotune"
    assert json.load(open(path))["k"]["index"] == [0, 11, 4, 2]


def test_unreadable_cache_counts_as_empty(tmp_path):
    path = str(tmp_path / "cache.json")
    with open(path, "w") as f:
        f.write("{not json")
    a = FakeContext()
    assert autotune.tune(a, "k", cache_path=path)["cached"] is False
    assert json.load(open(path))["k"]["index"] == [1, 5, 2, 3]
    assert not [p for p in os.listdir(tmp_path) if ".tmp" in p]  # written atomically
