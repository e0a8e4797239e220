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


def test_struct_layouts(cg, tmp_path):
    # every struct of the header has the same size in C (gcc) and in the ctypes binding
    import ctypes as C
    L = cg._lib
    pairs = {"cytom_config": L.Config, "cytom_rmat_params": L.RmatParams, "cytom_job_params": L.JobParams,
             "cytom_run_stats": L.RunStats, "cytom_tune_report": L.TuneReport, "cytom_kernel_stats": L.KernelStats,
             "cytom_fault_injection": L.FaultInjection}
    src = tmp_path / "sizes.c"
    src.write_text('#include <stdio.h>\n#include "cytom_gpu.h"\nint main(void) {\n' +
                   "".join(f'  printf("{k} %zu\\n", sizeof({k}));\n' for k in pairs) + "  return 0;\n}\n")
    exe = tmp_path / "sizes"
    r = subprocess.run(["gcc", "-std=c11", "-I", str(ROOT / "include"), str(src), "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()
    sizes = dict(zip(out[0::2], map(int, out[1::2])))
    for k, cls in pairs.items():
        assert C.sizeof(cls) == sizes[k], (k, C.sizeof(cls), sizes[k])


def test_cpp_header_compiles():
    # the C++ host mirror and the C header compile as plain C / C++ host code
    r = subprocess.run(["gcc", "-fsyntax-only", "-x", "c", "-std=c11", str(ROOT / "include" / "cytom_gpu.h")],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
