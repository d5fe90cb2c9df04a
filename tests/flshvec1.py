"""Test helper: writes FLSHVEC1 snapshot files byte for byte as the
reference's writer lays them out (crates/engine/src/persistence.rs:52-110):
magic, little-endian u64 manifest length, the JSON manifest, zero padding to
64 bytes, then each section zero-padded to a 64-byte offset."""
from __future__ import annotations

import json
import struct

import numpy as np

DTYPES = {np.dtype(np.float32): "f32", np.dtype(np.uint32): "u32", np.dtype(np.uint16): "u16", np.dtype(np.uint8): "u8"}


def _align(v, a=64):
    return (v + a - 1) // a * a


def write_snapshot(path, config, num_vectors, sections, next_logical_id, fp16_padded_dim=0, **extra):
    """sections: list of (name, numpy array) in file order."""
    cursor = 0
    table = {}
    blobs = []
    for name, arr in sections:
        arr = np.ascontiguousarray(arr)
        cursor = _align(cursor)
        table[name] = {"offset": cursor, "byte_len": arr.nbytes, "dtype": DTYPES[arr.dtype], "len": int(arr.size)}
        blobs.append((cursor, arr.tobytes()))
        cursor += arr.nbytes
    manifest = {"version": 1, "config": config, "num_vectors": num_vectors, "entry_point": 0, "cagra_degree": 0,
                "cagra_seeds": [], "rabitq_padded_dim": 0, "fp16_padded_dim": fp16_padded_dim, "sparse_num_docs": 0,
                "sparse_nnz": 0, "next_logical_id": next_logical_id, "sections": table}
    manifest.update(extra)
    head = json.dumps(manifest).encode()
    data_start = _align(16 + len(head))
    with open(path, "wb") as f:
        f.write(b"FLSHVEC1")
        f.write(struct.pack("<Q", len(head)))
        f.write(head)
        f.write(b"\0" * (data_start - 16 - len(head)))
        written = 0
        for off, blob in blobs:
            f.write(b"\0" * (off - written))
            f.write(blob)
            written = off + len(blob)


EMPTY_GRAPH_SECTIONS = [("hnsw_adjacency", np.zeros(0, np.uint32)), ("hnsw_degrees", np.zeros(0, np.uint32)),
                        ("cagra_adjacency", np.zeros(0, np.uint32)), ("rabitq_signs", np.zeros(0, np.float32)),
                        ("rabitq_centroids", np.zeros(0, np.float32)), ("rabitq_bits", np.zeros(0, np.uint32)),
                        ("rabitq_meta", np.zeros(0, np.float32))]
