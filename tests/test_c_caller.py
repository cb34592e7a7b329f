"""A plain C caller of the C ABI (include/fsig.h), built with gcc and linked
against libfsig.so, exercises the host-only entry points -- the t/v/e reader,
reference-exact join orders, refinement classes, status strings -- and, on a
machine without a GPU, fsig_create's refusal (FSIG_ENODEV, no fallback).  Its
output is compared with the Python binding's.  Needs gcc, no GPU."""
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

import fsig_gb300 as F
from conftest import GOLDEN

ROOT = Path(__file__).resolve().parent.parent
BUILD = ROOT / "fsig_gb300" / "_build"

C_SRC = r"""
#include <stdio.h>
#include <stdlib.h>
#include "fsig.h"

int main(int argc, char** argv) {
  /* argv[1]: data graph, argv[2]: query graph */
  fsig_graph_file* g = NULL;
  int rc = fsig_read_graph_file(argv[1], 1, &g);
  if (rc != FSIG_OK) { printf("read %d\n", rc); return 1; }
  uint32_t V = 0; uint64_t E = 0; const int32_t* lab = NULL; const uint32_t* edges = NULL;
  fsig_graph_file_data(g, &V, &lab, &E, &edges);
  unsigned long long lsum = 0, esum = 0;
  for (uint32_t v = 0; v < V; v++) lsum += (unsigned long long)(lab[v] + 1);
  for (uint64_t i = 0; i < 2 * E; i++) esum += edges[i];
  printf("graph %u %llu %llu %llu\n", V, (unsigned long long)E, lsum, esum);
  fsig_free_graph_file(g);

  fsig_graph_file* qf = NULL;
  if (fsig_read_graph_file(argv[2], 1, &qf) != FSIG_OK) return 1;
  uint32_t n = 0; uint64_t m = 0; const int32_t* ql = NULL; const uint32_t* qe = NULL;
  fsig_graph_file_data(qf, &n, &ql, &m, &qe);
  fsig_query q = {n, (uint32_t)m, ql, qe, NULL};
  uint32_t cand[FSIG_MAX_QUERY], order[FSIG_MAX_QUERY], types[FSIG_MAX_QUERY], cls[FSIG_MAX_QUERY];
  uint32_t rcls[FSIG_MAX_QUERY], dom[FSIG_MAX_QUERY];
  for (uint32_t u = 0; u < n; u++) cand[u] = 100 + (u * 37) % 11;
  for (int algo = 1; algo <= 2; algo++) {
    if (fsig_plan_order(&q, algo, cand, order, types, cls) != FSIG_OK) return 1;
    printf("order%d", algo);
    for (uint32_t u = 0; u < n; u++) printf(" %u", order[u]);
    printf("\n");
  }
  if (fsig_refine_classes(&q, rcls, dom) != FSIG_OK) return 1;
  printf("classes");
  for (uint32_t u = 0; u < n; u++) printf(" %u", rcls[u]);
  printf("\n");
  fsig_free_graph_file(qf);

  fsig_query bad = {0, 0, NULL, NULL, NULL};
  printf("empty %d\n", fsig_refine_classes(&bad, rcls, dom));
  printf("status %s\n", fsig_status_string(FSIG_ENODEV));
  fsig_engine* e = NULL;
  rc = fsig_create(0, 0, &e);
  printf("create %d\n", rc);
  if (rc == FSIG_OK) fsig_destroy(e);
  return 0;
}
"""


@pytest.fixture(scope="module")
def c_caller(tmp_path_factory):
    if shutil.which("gcc") is None:
        pytest.skip("gcc not available")
    if not (BUILD / "libfsig.so").exists():
        from fsig_gb300 import _build
        _build.build_all()
    d = tmp_path_factory.mktemp("c_caller")
    src = d / "caller.c"
    src.write_text(C_SRC)
    exe = d / "caller"
    subprocess.run(["gcc", "-std=c11", "-I", str(ROOT / "include"), str(src), "-o", str(exe), "-L", str(BUILD),
                    "-lfsig", f"-Wl,-rpath,{BUILD}"], check=True)
    return exe


def test_c_caller_matches_python(c_caller, golden):
    data = GOLDEN / golden["graphs"]["small_l4"]["file"]
    qname = sorted(golden["queries"])[7]
    qfile = GOLDEN / golden["queries"][qname]["file"]
    out = subprocess.run([str(c_caller), str(data), str(qfile)], capture_output=True, text=True, check=True).stdout
    lines = dict(line.split(" ", 1) for line in out.strip().split("\n"))

    g = F.read_graph_native(data)
    E = len(g.edges)
    assert lines["graph"].split() == [str(g.num_vertices), str(E), str(int((g.labels.astype(np.int64) + 1).sum())),
                                      str(int(g.edges.astype(np.int64).sum()))]
    q = F.read_query(qfile)
    cand = [100 + (u * 37) % 11 for u in range(q.num_vertices)]
    assert [int(x) for x in lines["order1"].split()] == F.plan_order(q, F.ALGO_FSIG, cand)["order"]
    assert [int(x) for x in lines["order2"].split()] == F.plan_order(q, F.ALGO_GSI, cand)["order"]
    assert [int(x) for x in lines["classes"].split()] == F.refine_classes(q)["classes"]
    assert int(lines["empty"]) == F.EQUERY
    assert lines["status"] == "no usable CUDA device"
    import torch
    if not torch.cuda.is_available():
        assert int(lines["create"]) == F.ENODEV
