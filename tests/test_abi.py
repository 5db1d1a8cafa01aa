"""The C-ABI library: it builds, loads and exports every declared entry point.

CPU only: no call here launches a kernel.  Host-only entry points (meta-path
grammar) are exercised against the oracle's restatement of the reference
grammar.
"""
import ctypes as C
import os

import numpy as np
import pytest


def test_library_exports_every_header_symbol(native):
    lib = native.lib()
    names = native.header_symbols()
    assert len(names) >= 25
    for n in names:
        assert hasattr(lib, n), n


def test_cli_is_built(native):
    assert os.access(native.CLI_PATH, os.X_OK)


PATHS = ["1-3-0-1-2-4-0-0-1", "0-0-1", "12-7-3", "1 3 0", "1-3-0-", "a1-2-3", "0", "1--3-0",
         "2-3-1-4-3-5-1-1-0-0-1-2-2", "1-3", "-1-3-0", "1-3-0-0"]


@pytest.mark.parametrize("s", PATHS)
def test_metapath_grammar_matches_reference(native, oracle_mod, s):
    try:
        ref = oracle_mod.parse_metapath(s)
    except ValueError:
        ref = None
    if ref is None:
        with pytest.raises(ValueError):
            native.MetaPath(s)
        return
    mp = native.MetaPath(s)
    assert mp.vertex_types.tolist() == ref[0].tolist()
    assert mp.edge_types.tolist() == ref[1].tolist()


def test_metapath_to_string(native):
    assert native.MetaPath("1 3 0 1 2").to_string() == "1-3-0-1-2"
    assert native.MetaPath("7").to_string() == "7"


def test_create_without_gpu_reports_cuda_error(native):
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    h = C.c_void_p()
    rc = native.lib().rmcm_create(C.byref(h), None)
    assert rc == native.ECUDA
    assert native.lib().rmcm_status_string(rc) == b"CUDA error"


STRUCTS = [("Opts", "rmcm_opts"), ("Timings", "rmcm_timings"), ("ProductStats", "rmcm_product_stats"),
           ("Tuning", "rmcm_tuning"), ("ServerOpts", "rmcm_server_opts"), ("QueryResult", "rmcm_query_result"),
           ("ServerCounters", "rmcm_server_counters")]


def test_ctypes_mirrors_match_the_header(native, tmp_path):
    """Every ctypes structure of the binding has the size and field offsets
    the C compiler gives the header's struct (compiled here with gcc)."""
    import shutil
    import subprocess
    if shutil.which("gcc") is None:
        pytest.skip("no C compiler")
    lines = ["#include <stddef.h>", "#include <stdio.h>", '#include "resmcm_gpu.h"', "int main(void) {"]
    for py, c in STRUCTS:
        lines.append(f'  printf("{py} sizeof %zu\\n", sizeof({c}));')
        for f, _ in getattr(native, py)._fields_:
            lines.append(f'  printf("{py} {f} %zu\\n", offsetof({c}, {f}));')
    lines += ["  return 0;", "}"]
    src = tmp_path / "abi.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "abi"
    inc = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include")
    subprocess.run(["gcc", "-std=c11", "-I" + inc, str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split("\n")
    want = {}
    for ln in out:
        if ln:
            py, f, v = ln.split()
            want[(py, f)] = int(v)
    for py, _ in STRUCTS:
        cls = getattr(native, py)
        assert C.sizeof(cls) == want[(py, "sizeof")], py
        for f, _ in cls._fields_:
            assert getattr(cls, f).offset == want[(py, f)], (py, f)
