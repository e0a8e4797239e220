"""A compiled C++ caller of the C ABI: the binding of INTEGRATION.md, as written there.

The code block under "C++ binding" in INTEGRATION.md is extracted, compiled with g++
against include/cytom_gpu.h and stand-ins for the reference's Config and Edge
(tests/c_caller/harness.cc), linked to libcytom_gpu.so and run on an RMAT edge stream in
batches, one incremental run after each batch -- the reference's EdgeInserter loop. The
BFS levels, CC labels and SSSP distances it writes must equal the oracle's fixed point
bit for bit. The header's own compile check (no GPU) is in test_abi.py."""
import os
import re
import shutil
import subprocess
import struct
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parents[1]


def binding_block() -> str:
    text = (ROOT / "INTEGRATION.md").read_text()
    sec = text[text.index("## C++ binding"):]
    m = re.search(r"```cpp\n(.*?)```", sec, re.S)
    assert m, "no C++ block under 'C++ binding' in INTEGRATION.md"
    return m.group(1)


def build_harness(tmp: Path) -> Path:
    cxx = shutil.which("g++") or shutil.which("c++")
    if not cxx:
        pytest.skip("no C++ compiler")
    (tmp / "binding.inc").write_text(binding_block())
    exe = tmp / "harness"
    lib_dir = ROOT / "cytom_gb300"
    cmd = [cxx, "-std=c++17", "-O1", "-I", str(ROOT / "include"), "-I", str(tmp),
           str(ROOT / "tests" / "c_caller" / "harness.cc"), "-o", str(exe),
           "-L", str(lib_dir), "-lcytom_gpu", f"-Wl,-rpath,{lib_dir}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_integration_binding_compiles_and_matches_oracle(cg, orc, tmp_path):
    cg.load()
    exe = build_harness(tmp_path)
    scale, vpt, batch = 13, 2048, 20000
    n = 1 << scale
    s, t = orc.rmat(scale, 0, 12 * n, 21)
    w = orc.edge_weights(s, t, 23)
    ein = tmp_path / "e.bin"
    with open(ein, "wb") as f:
        f.write(struct.pack("<Q", len(s)))
        f.write(s.tobytes())
        f.write(t.tobytes())
        f.write(w.tobytes())
    st = orc.Store(n, vpt, True)
    st.insert(s, t, w)
    st.compact()
    for name, algo in (("bfs", orc.BFS), ("cc", orc.CC), ("sssp", orc.SSSP)):
        out = tmp_path / f"{name}.bin"
        r = subprocess.run([str(exe), name, str(n), str(vpt), str(batch), str(ein), str(out)],
                           capture_output=True, text=True, timeout=300, env=dict(os.environ))
        assert r.returncode == 0, (name, r.returncode, r.stderr)
        got = np.fromfile(out, np.uint32)
        ref, _ = st.run_minprop(algo, start=0, max_iter=1000)
        assert np.array_equal(got, ref), name
