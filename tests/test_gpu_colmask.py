"""Sparse rounds that skip (word, tile column) items by the per-source column masks.

The masks are a superset kept by the compaction (new edges add bits) and rebuilt with a
full directory build; deletions leave bits behind and clearing the store zeroes them.
Whatever the mask holds, a sparse round must reach every edge of an active source: the
runs below (sparse rounds forced while up to half of the frontier words are non-zero)
must equal the oracle's fixed point after inserts, deletions, re-inserts and a clear,
at 16 tile columns (one mask bit per column) and at 128 (one bit per two columns)."""
import json
import os
import subprocess
import sys
from pathlib import Path

import pytest

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parents[1]

CODE = """
import sys, json, numpy as np
sys.path.insert(0, {root!r})
import cytom_gb300 as cg
from oracle import oracle as orc
scale, vpt = {scale}, {vpt}
n = 1 << scale
ok = []
rng = np.random.default_rng(7)
with cg.Engine(n, vpt, weight_type=cg.WEIGHT_U32) as eng:
    progs = [cg.BFS(eng, start_vertex=0, max_iterations=1000), cg.CC(eng, max_iterations=1000),
             cg.SSSP(eng, start_vertex=1, max_iterations=1000)]
    starts = (0, 0, 1)
    st = orc.Store(n, vpt, True)

    def insert(first, count, seed):
        s, t = orc.rmat(scale, first, count, seed)
        w = orc.edge_weights(s, t, seed + 5)
        eng.insert_edges(s, t, w)
        st.insert(s, t, w)
        eng.do_global_compaction()
        st.compact()

    def check(tag):
        for prog, algo, start in zip(progs, (0, 1, 2), starts):
            stt = prog.execute_algorithm()
            ref, _ = st.run_minprop(algo, start=start, max_iter=1000)
            ok.append([tag, algo, bool(np.array_equal(prog.result(), ref)) and stt["converged"] == 1])

    insert(0, 4 * n, 11)
    check("first")
    insert(4 * n, n // 2, 11)
    check("insert")
    s1, t1, _ = orc.store_edges(st)
    k = rng.choice(len(s1), len(s1) // 3, replace=False)
    assert eng.delete_edges(s1[k], t1[k]) == st.delete(s1[k], t1[k])
    check("delete")
    insert(0, n, 13)
    check("reinsert")
    eng.clear()
    st = orc.Store(n, vpt, True)
    for p in progs:
        p.init_algorithm()
    insert(0, 2 * n, 17)
    check("clear")
    insert(2 * n, n // 4, 17)
    check("after_clear")
print(json.dumps(ok))
"""


@pytest.mark.parametrize("scale,vpt", [(15, 2048), (14, 128)])
def test_sparse_rounds_with_column_masks(scale, vpt):
    env = dict(os.environ, CYTOM_SPARSE="1", CYTOM_SPARSE_DIV="2")
    r = subprocess.run([sys.executable, "-c", CODE.format(root=str(ROOT), scale=scale, vpt=vpt)],
                       capture_output=True, text=True, env=env, timeout=900)
    assert r.returncode == 0, r.stderr[-3000:]
    res = json.loads(r.stdout.strip().splitlines()[-1])
    bad = [x for x in res if not x[2]]
    assert len(res) == 18 and not bad, bad
