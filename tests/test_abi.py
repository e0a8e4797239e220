"""CPU tests of the C ABI: the library loads without a GPU and exports every entry
point declared in include/cytom_gpu.h (no compute call is made here)."""
import re
import subprocess
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]


def declared_symbols():
    text = (ROOT / "include" / "cytom_gpu.h").read_text()
    return sorted(set(re.findall(r"^\s*(?:int|void|const char\s*\*)\s*(cytom_\w+)\s*\(", text, re.M)))


def test_header_declares_entry_points():
    syms = declared_symbols()
    for name in ["cytom_create", "cytom_insert_batch", "cytom_compact", "cytom_run",
                 "cytom_get_tiles", "cytom_rmat_generate", "cytom_gridgraph_decode"]:
        assert name in syms


def test_library_exports_every_declared_symbol(cg):
    lib = cg.load()
    for name in declared_symbols():
        assert hasattr(lib, name), name
    out = subprocess.run(["nm", "-D", "--defined-only", str(cg._lib.LIB_PATH)], capture_output=True,
                         text=True).stdout
    exported = set(re.findall(r"\b(cytom_\w+)\b", out))
    assert set(declared_symbols()) <= exported


def test_bindings_cover_header(cg):
    bound = {name for name, _, _ in cg._lib.SIGNATURES}
    assert set(declared_symbols()) <= bound


def test_struct_layouts(cg):
    import ctypes as C
    L = cg._lib
    assert C.sizeof(L.Config) == 40
    assert C.sizeof(L.RmatParams) == 56
    assert C.sizeof(L.JobParams) == 48
    assert C.sizeof(L.RunStats) == 56


def test_cpp_header_compiles():
    # the C++ host mirror and the C header compile as plain C / C++ host code
    r = subprocess.run(["gcc", "-fsyntax-only", "-x", "c", "-std=c11", str(ROOT / "include" / "cytom_gpu.h")],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
