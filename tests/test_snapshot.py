"""FLSHVEC1 snapshot files (persistence.rs) without a GPU: the library's
reader against files laid out as the reference writes them."""
from __future__ import annotations

import numpy as np
import pytest

from flshvec1 import EMPTY_GRAPH_SECTIONS, write_snapshot


def small_file(path, n=100, dim=8):
    rng = np.random.default_rng(1)
    x = rng.standard_normal((n, dim)).astype(np.float32)
    cfg = {"dim": dim, "max_elements": n, "m": 32, "ef_construction": 128, "nlist": 0, "m_pq": 0, "metric": 0}
    write_snapshot(path, cfg, n, [("vectors", x), ("logical_ids", np.arange(n, dtype=np.uint32)),
                                  ("main_valid_words", np.full((n + 31) // 32, 0xFFFFFFFF, np.uint32))]
                   + EMPTY_GRAPH_SECTIONS, next_logical_id=n)
    return x


def test_manifest_and_sections_are_read(built_lib, tmp_path):
    from fvgb300.index import snapshot_manifest

    p = tmp_path / "a.flshvec1"
    small_file(p)
    m = snapshot_manifest(p)
    assert m["version"] == 1 and m["config"]["dim"] == 8 and m["num_vectors"] == 100 and m["next_logical_id"] == 100
    secs = m["sections"]
    assert secs["vectors"]["byte_len"] == 100 * 8 * 4 and secs["vectors"]["dtype"] == "f32"
    assert all(s["offset"] % 64 == 0 for s in secs.values())
    assert secs["hnsw_adjacency"]["byte_len"] == 0


def test_rejects_malformed_files(built_lib, tmp_path):
    from fvgb300._lib import FvError
    from fvgb300.index import snapshot_manifest

    p = tmp_path / "a.flshvec1"
    small_file(p)
    raw = p.read_bytes()
    bad = tmp_path / "bad.flshvec1"
    bad.write_bytes(b"NOTFLSH1" + raw[8:])
    with pytest.raises(FvError, match="magic"):
        snapshot_manifest(bad)
    bad.write_bytes(raw[: len(raw) - 100])  # last section cut short
    with pytest.raises(FvError, match="truncated"):
        snapshot_manifest(bad)
    bad.write_bytes(raw[:8] + (10 ** 9).to_bytes(8, "little") + raw[16:])
    with pytest.raises(FvError, match="header"):
        snapshot_manifest(bad)
    bad.write_bytes(raw[:16] + b"!" + raw[17:])  # manifest JSON broken
    with pytest.raises(FvError):
        snapshot_manifest(bad)
    with pytest.raises(FvError):
        snapshot_manifest(tmp_path / "missing.flshvec1")


def test_unknown_manifest_fields_are_ignored(built_lib, tmp_path):
    from fvgb300.index import snapshot_manifest

    p = tmp_path / "a.flshvec1"
    rng = np.random.default_rng(2)
    cfg = {"dim": 4, "max_elements": 10, "m": 16, "ef_construction": 64, "nlist": 0, "m_pq": 0, "metric": 2,
           "future_field": [1, 2, {"x": "y"}]}
    write_snapshot(p, cfg, 10, [("vectors", rng.standard_normal((10, 4)).astype(np.float32))], next_logical_id=12,
                   another={"nested": [True, False, None, -1.5e3, "é\\n"]})
    m = snapshot_manifest(p)
    assert m["config"]["metric"] == 2 and m["config"]["m"] == 16 and m["next_logical_id"] == 12
