"""The C-ABI library builds, loads and exports every declared entry point
(no compute call: this runs without a GPU)."""
import ctypes as ct
import os
import re
import subprocess

from conftest import ROOT


def declared_symbols():
    names = []
    for h in os.listdir(os.path.join(ROOT, "include")):
        if h.endswith(".h"):
            txt = open(os.path.join(ROOT, "include", h)).read()
            names += re.findall(r"^\s*(?:int|const char\*)\s+(bmc_\w+)\s*\(", txt, re.M)
    return sorted(set(names))


def test_library_exports_header():
    from bmc import _lib

    path = _lib.load().__dict__.get("_name") or _lib.lib_path()
    out = subprocess.run(["nm", "-D", "--defined-only", path], capture_output=True, text=True).stdout
    exported = set(re.findall(r" T (bmc_\w+)", out))
    decl = declared_symbols()
    assert decl, "no declarations found"
    missing = [d for d in decl if d not in exported]
    assert not missing, missing
    # the binding knows every declared symbol
    assert set(decl) <= set(_lib.SIGNATURES)


def test_version_and_error_without_gpu():
    from bmc import _lib

    L = _lib.load()
    a, b = ct.c_int32(), ct.c_int32()
    assert L.bmc_version(ct.byref(a), ct.byref(b)) == 0
    assert (a.value, b.value) == (1, 1)
    # argument validation happens before any device work
    assert L.bmc_scenario_create(None, None) == -1
    assert b"null" in L.bmc_last_error()


def test_struct_layouts_match_header(tmp_path):
    from bmc import _lib

    src = tmp_path / "sz.c"
    src.write_text('#include "bmc.h"\n#include <stdio.h>\nint main(void){printf("%zu %zu %zu %zu\\n",'
                   'sizeof(bmc_step_stats), sizeof(bmc_scenario_desc), sizeof(bmc_feed),'
                   ' sizeof(bmc_model_desc));return 0;}\n')
    exe = tmp_path / "sz"
    subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    sizes = [int(x) for x in subprocess.run([str(exe)], capture_output=True, text=True).stdout.split()]
    assert sizes == [ct.sizeof(_lib.StepStats), ct.sizeof(_lib.ScenarioDesc), ct.sizeof(_lib.Feed),
                     ct.sizeof(_lib.ModelDesc)]
