"""The engine library builds, loads and exports every entry point include/crvgpu.h declares (no GPU needed)."""
import os
import re

from crvgpu import _capi, build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_in_header():
    text = open(os.path.join(ROOT, "include", "crvgpu.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return set(re.findall(r"\b(crv_\w+)\s*\(", text))


def test_library_builds_and_exports_every_declared_symbol():
    path = build.build()
    assert os.path.exists(path)
    L = _capi.load()
    header = declared_in_header()
    assert header, "no entry points found in the header"
    assert header == set(_capi.DECLARED), header ^ set(_capi.DECLARED)
    for name in header:
        assert hasattr(L, name), name
    assert L.crv_version() == 1
    assert _capi.status_string(0) == "ok"
    assert _capi.status_string(3) == "capacity|limit"


def test_struct_sizes_match_header_layout():
    import ctypes
    # CrvStatus: flags, pad, need[16]
    assert ctypes.sizeof(_capi.CrvStatus) == 8 + 16 * 8
    # every double field of CrvParams is 8-byte aligned (no implicit padding surprises between int pairs)
    for name, typ in _capi.CrvParams._fields_:
        off = getattr(_capi.CrvParams, name).offset
        assert off % ctypes.sizeof(typ) == 0, name


def test_workspace_query_without_gpu():
    import ctypes
    from crvgpu.params import make_params
    L = _capi.load()
    P = make_params()
    assert L.crv_response_workspace(ctypes.byref(P), 10, 400, 100000, 64) > 0
    assert L.crv_response_workspace(ctypes.byref(P), -1, 400, 100000, 64) == -1
    assert L.crv_sipm_workspace(ctypes.byref(P), 10, 1000) > 0


def test_pulse_launch_shape_is_validated():
    import pytest
    from crvgpu.pulsefit import DEFAULT_SHAPE, set_shape
    for bad in ((96, 16, 16), (128, 0, 16), (128, 16, 40), (256, 16, 16)):
        with pytest.raises(ValueError):
            set_shape(bad)
    set_shape(DEFAULT_SHAPE)


def test_chain_and_lookup_workspace_queries_without_gpu():
    import ctypes
    from crvgpu.params import make_params
    from crvgpu.resident import ChainCaps
    L = _capi.load()
    P = make_params()
    caps = ChainCaps(events=64, steps=2600, photons=10 ** 6, charges=10 ** 5, slots=10 ** 4, digis=10 ** 4,
                     pulses=10 ** 4, max_steps_per_event=80)
    small = L.crv_chain_workspace(ctypes.byref(P), ctypes.byref(caps.c()))
    big = L.crv_chain_workspace(ctypes.byref(P), ctypes.byref(ChainCaps(**{**caps.as_dict(), "pulses": 10 ** 6}).c()))
    assert 0 < small < big
    bad = caps.c()
    bad.digis = 0                                          # every capacity must be positive
    assert L.crv_chain_workspace(ctypes.byref(P), ctypes.byref(bad)) == -1
    assert L.crv_substeps_workspace(1000) > L.crv_substeps_workspace(10) > 0
    assert L.crv_substeps_workspace(-1) == -1
    assert L.crv_lookup_rows_workspace(1000) > 0 and L.crv_lookup_rows_workspace(-5) == -1


def test_lookup_struct_layouts():
    import ctypes
    # CrvLookup: 9 doubles, 7 edge pointers, 7 + 1 ints, cos phi pointer, 3 tables of 5 pointers + 4 ints, cos theta
    assert ctypes.sizeof(_capi.CrvLookupTable) == 5 * 8 + 4 * 4
    assert ctypes.sizeof(_capi.CrvLookup) == 9 * 8 + 7 * 8 + 8 * 4 + 8 + 3 * (5 * 8 + 4 * 4) + 8
    assert ctypes.sizeof(_capi.CrvSubstepRows) == 15 * 8
    assert ctypes.sizeof(_capi.CrvLookupGroup) == 12 * 8 + 8 + 6 * 4
    assert ctypes.sizeof(_capi.CrvChainCaps) == 7 * 8 + 2 * 4


def test_lookup_file_struct_layouts():
    import ctypes
    assert ctypes.sizeof(_capi.CrvLookupFileInfo) == 4 * 4 + 2 * 8 + 10 * 8 + 2 * 8 + 7 * 8 + 3 * 3 * 8
    assert ctypes.sizeof(_capi.CrvLookupFileTable) == 5 * 8
    assert ctypes.sizeof(_capi.CrvLookupFileOut) == 2 * 8 + 7 * 8 + 3 * 5 * 8


def test_every_struct_matches_the_compiled_header():
    """sizeof and offsetof of every field of every ctypes mirror against the header compiled by the C compiler."""
    import ctypes
    import shutil
    import subprocess
    import tempfile
    import pytest
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    structs = {n: getattr(_capi, n) for n in dir(_capi)
               if n.startswith("Crv") and isinstance(getattr(_capi, n), type)
               and issubclass(getattr(_capi, n), ctypes.Structure)}
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "crvgpu.h"', "int main(void) {"]
    expect = []
    for name, S in sorted(structs.items()):
        lines.append(f'  printf("%zu\\n", sizeof({name}));')
        expect.append((name, "sizeof", ctypes.sizeof(S)))
        for f, _ in S._fields_:
            c_name = f[:-1] if f.endswith("_") else f                  # ctypes spelling of a Python keyword
            lines.append(f'  printf("%zu\\n", offsetof({name}, {c_name}));')
            expect.append((name, f, getattr(S, f).offset))
    lines += ["  return 0;", "}"]
    with tempfile.TemporaryDirectory() as d:
        src, exe = os.path.join(d, "layout.c"), os.path.join(d, "layout")
        open(src, "w").write("\n".join(lines))
        subprocess.run([cc, "-std=c11", "-I", os.path.join(ROOT, "include"), src, "-o", exe], check=True)
        got = [int(v) for v in subprocess.run([exe], check=True, capture_output=True, text=True).stdout.split()]
    assert len(got) == len(expect)
    bad = [(e, g) for e, g in zip(expect, got) if e[2] != g]
    assert not bad, bad[:10]
    assert len(structs) >= 15
