"""The FSIG command line (fsig_gb300/csrc/cli.cpp): the reference's argument
convention (main/run.cc:28-64) and output lines, on the golden fixtures."""
import re
import subprocess

import pytest

from conftest import GOLDEN, ROOT

EXE = ROOT / "fsig_gb300" / "_build" / "FSIG"


@pytest.fixture(scope="module")
def exe():
    from fsig_gb300 import _build
    _build.build_all()
    return EXE


def run(exe, *args):
    return subprocess.run([str(exe), *map(str, args)], capture_output=True, text=True, timeout=600)


def test_too_few_arguments(exe):
    p = run(exe, "only_one.graph")
    assert p.returncode == 255
    assert p.stdout.startswith("invalid arguments!")


def test_missing_file_is_an_error_not_a_crash(exe, tmp_path):
    p = run(exe, tmp_path / "absent.graph", tmp_path / "absent_q.graph")
    assert p.returncode == 1
    assert "Error" in p.stdout


@pytest.mark.gpu
@pytest.mark.parametrize("algo,tag", [(1, "#embedding"), (2, "#embeddings"), (3, "#embedding")])
def test_golden_counts_and_hashes(exe, golden, algo, tag):
    data = GOLDEN / golden["graphs"]["cl_zipf16"]["file"]
    rec = golden["oracle_cl_zipf16"]
    names = [n for n in sorted(golden["queries"]) if rec[n]["count"] < 5_000_000][:6]
    for name in names:
        p = run(exe, data, GOLDEN / golden["queries"][name]["file"], algo, 1)
        assert p.returncode == 0, p.stdout + p.stderr
        assert re.search(rf"^{tag}: (\d+)$", p.stdout, re.M).group(1) == str(rec[name]["count"])
        assert int(re.search(r"^hash: (0x[0-9a-f]+)$", p.stdout, re.M).group(1), 16) == rec[name]["hash"]
        assert "time cost(read data):" in p.stdout


@pytest.mark.gpu
def test_output_file_holds_the_embeddings(exe, golden, tmp_path):
    data = GOLDEN / golden["graphs"]["cl_zipf16"]["file"]
    rec = golden["oracle_cl_zipf16"]
    name = min(golden["queries"], key=lambda n: (rec[n]["count"] < 1000, rec[n]["count"]))
    out = tmp_path / "ans.txt"
    p = run(exe, data, GOLDEN / golden["queries"][name]["file"], 1, 1, out, 0)
    assert p.returncode == 0, p.stdout + p.stderr
    lines = out.read_text().splitlines()
    assert len(lines) == rec[name]["count"]
    assert len(set(lines)) == len(lines)
