"""The committed tile-shape table of the serving stream (luxum_gb300/serve_tile_shapes.json,
written by `bench.py --config serve-tune`) is well formed: one entry per class, every field in
the range lx_batch_set_tune_table accepts, for the stream's precision (FP32)."""
import json
import os

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PATH = os.path.join(ROOT, "luxum_gb300", "serve_tile_shapes.json")


def test_serve_table_is_well_formed():
    with open(PATH) as f:
        doc = json.load(f)
    table = doc["table"]
    assert table, "empty table"
    keys = set()
    for e in table:
        assert set(e) == {"planar", "size_class", "precision", "slab_class", "march"}
        assert e["planar"] in (0, 1)
        assert 0 <= e["size_class"] <= 15
        assert e["precision"] == 1  # the serving stream runs FP32
        assert 0 <= e["slab_class"] <= 3
        assert e["march"] in (1, 2, 4, 8)
        keys.add((e["planar"], e["size_class"], e["precision"], e["slab_class"]))
    assert len(keys) == len(table)  # one entry per class


def test_bench_loads_the_committed_table():
    import sys

    sys.path.insert(0, ROOT)
    import bench

    assert bench.SERVE_TABLE == PATH
    assert bench.load_serve_table() == json.load(open(PATH))["table"]
