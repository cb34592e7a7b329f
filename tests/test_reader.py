"""The C++ t/v/e reader: the parallel path (one thread per core, taken when
every line is a plain record) returns exactly what the sequential scan
returns, which is the reference reader's result (pinned by the oracle's
restatement, IO/graph_reader.cc:12-55), on files with and without the
trailing-whitespace quirk, with CRLF line ends, and on files whose odd lines
send the parallel path back to the sequential scan."""
import numpy as np
import pytest

import fsig_gb300 as F
from oracle import oracle as O


def body(g, labeled=True):
    lines = [f"t {g.num_vertices} {g.num_edges}"]
    lines += [f"v {v} {int(l) if labeled else 0} 0" for v, l in enumerate(g.labels)]
    lines += [f"e {a} {b}" for a, b in np.asarray(g.edges).reshape(-1, 2).tolist()]
    return lines


@pytest.fixture(scope="module")
def graph():
    lab = F.gen_labels(3000, 6, "uniform", seed=11)
    return F.gen_rmat(3000, 20000, seed=11, labels=lab)


CASES = {
    "plain": lambda ls: "\n".join(ls),
    "trailing_newline": lambda ls: "\n".join(ls) + "\n",
    "trailing_spaces": lambda ls: "\n".join(ls) + "  \n\n ",
    "crlf": lambda ls: "\r\n".join(ls) + "\r\n",
    "blank_lines": lambda ls: "\n\n".join(ls),
    "vertex_last": lambda ls: "\n".join([l for l in ls if l[0] != "v"] + [l for l in ls if l[0] == "v"]) + "\n",
    "odd_line": lambda ls: "\n".join(ls[:500] + ["x 1 2"] + ls[500:]) + "\n",
    "split_record": lambda ls: "\n".join(ls[:700] + ["e 1", "2"] + ls[700:]),
    "signed": lambda ls: "\n".join(ls[:50] + ["e +3 4"] + ls[50:]),
}


@pytest.mark.parametrize("case", sorted(CASES))
@pytest.mark.parametrize("labeled", [True, False])
def test_parallel_equals_sequential_and_oracle(graph, tmp_path, case, labeled):
    path = tmp_path / f"{case}.graph"
    path.write_bytes(CASES[case](body(graph)).encode())
    seq = F.read_graph_native(path, labeled, parallel_min_bytes=1 << 40)
    par = F.read_graph_native(path, labeled, parallel_min_bytes=1)
    assert np.array_equal(seq.labels, par.labels)
    assert np.array_equal(seq.edges, par.edges)
    ref = O.read_tve(path, labeled)
    assert np.array_equal(ref["labels"], seq.labels)
    assert ref["E"] == len(seq.edges)


def test_quirk_duplicates_the_last_edge(graph, tmp_path):
    ls = body(graph)
    (tmp_path / "a.graph").write_bytes("\n".join(ls).encode())
    (tmp_path / "b.graph").write_bytes(("\n".join(ls) + "\n").encode())
    a = F.read_graph_native(tmp_path / "a.graph", parallel_min_bytes=1)
    b = F.read_graph_native(tmp_path / "b.graph", parallel_min_bytes=1)
    assert len(b.edges) == len(a.edges) + 1
    assert np.array_equal(b.edges[-1], b.edges[-2])
