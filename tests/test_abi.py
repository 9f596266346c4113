"""The C ABI library: builds, loads, exports every declared entry point, and its structs
match the Python bindings. CPU only (no compute call needs a GPU here)."""
import ctypes
import os
import re
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INCLUDE = os.path.join(ROOT, "include")


@pytest.fixture(scope="module")
def lib_path():
    from sparqc_gb300 import build
    return build.build()


def declared_functions():
    names = set()
    for f in os.listdir(INCLUDE):
        if not f.endswith(".h"):
            continue
        text = open(os.path.join(INCLUDE, f)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names |= set(re.findall(r"\b(sqc_[a-z0-9_]+)\s*\(", text))
    return names


def test_every_declared_symbol_is_exported(lib_path):
    lib = ctypes.CDLL(lib_path)
    names = declared_functions()
    assert len(names) >= 20
    missing = [n for n in sorted(names) if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binding_lists_every_export():
    from sparqc_gb300 import engine
    assert set(engine.EXPORTS) == declared_functions()


def test_struct_layouts_match(tmp_path, lib_path):
    from sparqc_gb300 import engine
    from sparqc_gb300.gates import GATE_DTYPE
    src = tmp_path / "layout.c"
    src.write_text(r'''
#include <stdio.h>
#include <stddef.h>
#include "sparqc.h"
int main(void) {
    printf("%zu %zu %zu %zu %zu %zu %zu %zu %zu %zu %zu %zu %zu %zu %zu\n", sizeof(sqc_gate), offsetof(sqc_gate, controls),
           offsetof(sqc_gate, lambda), sizeof(sqc_options), sizeof(sqc_hash_table_parameters), sizeof(sqc_stats),
           sizeof(sqc_circuit_desc), sizeof(sqc_batch_options), sizeof(sqc_batch_tuning), sizeof(sqc_batch_stats),
           offsetof(sqc_options, time_passes), sizeof(sqc_server_options), sizeof(sqc_server_stats),
           sizeof(sqc_part_stats), offsetof(sqc_part_stats, amp_updates));
    return 0;
}
''')
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c11", "-I", INCLUDE, str(src), "-o", str(exe)], check=True)
    vals = [int(v) for v in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()]
    assert vals[0] == GATE_DTYPE.itemsize
    assert vals[1] == GATE_DTYPE.fields["controls"][1]
    assert vals[2] == GATE_DTYPE.fields["lambda"][1]
    assert vals[3] == ctypes.sizeof(engine.Options)
    assert vals[4] == ctypes.sizeof(engine.HashTableParameters)
    assert vals[5] == ctypes.sizeof(engine.Stats)
    assert vals[6] == ctypes.sizeof(engine.CircuitDesc)
    assert vals[7] == ctypes.sizeof(engine.BatchOptions)
    assert vals[8] == ctypes.sizeof(engine.BatchTuning)
    assert vals[9] == ctypes.sizeof(engine.BatchStats)
    assert vals[10] == engine.Options.time_passes.offset
    assert vals[11] == ctypes.sizeof(engine.ServerOptions)
    assert vals[12] == ctypes.sizeof(engine.ServerStats)
    assert vals[13] == ctypes.sizeof(engine.PartStats)
    assert vals[14] == engine.PartStats.amp_updates.offset


def test_cpp_dropin_header_compiles(tmp_path):
    src = tmp_path / "t.cpp"
    src.write_text('#include "sparqc_circuit.hpp"\nint main(){ hash_table_parameters hp; (void)hp; return 0; }\n')
    subprocess.run(["g++", "-std=c++17", "-fsyntax-only", "-I", INCLUDE, str(src)], check=True)


def test_no_cpu_fallback_without_gpu(lib_path):
    """Without a usable GPU the engine refuses to create a state instead of computing on the CPU."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from sparqc_gb300 import engine
    with pytest.raises(engine.SparqcError) as e:
        engine.State(10)
    assert e.value.code == engine.ERR_NO_DEVICE


def test_gate_dtype_matches_oracle():
    from oracle.sparse import GATE_DTYPE as O
    from sparqc_gb300.gates import GATE_DTYPE as P
    assert O == P


def test_status_strings(lib_path):
    from sparqc_gb300 import engine
    L = engine.load()
    assert L.sqc_status_string(0) == b"ok"
    assert L.sqc_status_string(3) == b"table full"
