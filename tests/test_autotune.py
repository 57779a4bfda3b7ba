"""The autotuner's table logic (no GPU): keys bucket the batch size, missing
shapes take the defaults, entries override only the known settings, the
candidate set offers the mixed form only to the jobs it takes, and the
committed table (when present) holds only valid settings."""
import json
import os

from mpsim_gb300 import autotune as A


def test_buckets_and_keys():
    assert A.bucket(1) == 8 and A.bucket(8) == 8 and A.bucket(9) == 16 and A.bucket(5000) > 256
    assert A.key(512, 512, 2, 32) == "d2_m512_n512_b32"
    assert A.key(512, 512, 2, 4) != A.key(512, 512, 2, 400)
    # each bucket is tuned at the smallest batch it covers
    assert [A.bucket(n) for n in A.TUNE_BATCHES] == list(A.BUCKETS)
    assert all(A.bucket(n - 1) != A.bucket(n) for n in A.TUNE_BATCHES[1:])


def test_lookup_defaults_and_override():
    table = {A.key(512, 512, 2, 32): {"precision": "mixed", "lq_off": 1, "block_request": 8,
                                      "ms": {}}}
    got = A.lookup(512, 512, 2, 32, table)
    assert got == {"precision": "mixed", "lq_off": 1, "block_request": 8}
    assert A.lookup(256, 256, 2, 32, table) == A.DEFAULT
    assert A.lookup(512, 512, 2, 4, table) == A.DEFAULT          # other batch bucket


def test_candidates():
    c = A.candidates(512, 512)
    assert ("mixed", 0, 0) in c and ("plain", 0, 8) in c and ("plain", 1, 0) in c
    assert not any(p == "mixed" for p, _, _ in A.candidates(32, 32))   # below 64 columns
    assert not any(p == "mixed" for p, _, _ in A.candidates(128, 256))  # wide
    assert not any(b == 8 for _, _, b in A.candidates(256, 256))       # 8-column blocks: 512/576 rows


def test_committed_table_is_valid():
    if not os.path.exists(A.TABLE_PATH):
        return
    with open(A.TABLE_PATH) as f:
        entries = json.load(f)["entries"]
    assert entries
    for k, e in entries.items():
        assert k.startswith("d") and "_m" in k and "_b" in k
        assert e["precision"] in ("plain", "mixed")
        assert e["lq_off"] in (0, 1) and e["block_request"] in (0, 8, 16)
