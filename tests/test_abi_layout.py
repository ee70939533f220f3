"""The ctypes bindings (pihm_gpu/*.py) against the C ABI's structs: every
struct the Python side passes across the boundary has the size and field
offsets the C compiler gives it from include/*.h (a field added on one side
only would shift every later field).  Host compilation only, no device."""
import ctypes
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INC = os.path.join(ROOT, "include")


def _pairs():
    from pihm_gpu import batch, deck, land, meshdesc, noah, nvector, solver
    return [
        ("pihm_batch_limits", batch.BatchLimits),
        ("pihm_step_control", batch.StepControlC),
        ("pihm_batch_job", batch.BatchJob),
        ("pihm_batch_info", batch.BatchInfo),
        ("pihm_serve_record", batch.ServeRecord),
        ("pihm_deck_control", deck.DeckControlC),
        ("pihm_land_params", land.LandParamsC),
        ("pihm_forcing_series", land.ForcingSeriesC),
        ("pihm_gpu_mesh", meshdesc.MeshDesc),
        ("pihm_noah_params", noah.NoahParams),
        ("pihm_noah_state", noah.NoahState),
        ("pihm_noah_forcing", noah.NoahForcing),
        ("pihm_nv_coef", nvector.Coef),
        ("pihm_bdf_stats", solver.BdfStats),
    ]


@pytest.fixture(scope="module")
def c_layout(tmp_path_factory):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    pairs = _pairs()
    lines = ['#include <stddef.h>', '#include <stdio.h>', '#include "pihm_gpu.h"', '#include "pihm_nvector.h"',
             '#include "pihm_bdf.h"', '#include "pihm_batch.h"', '#include "pihm_deck.h"', '#include "pihm_land.h"',
             '#include "pihm_noah.h"', 'int main(void) {']
    for cname, py in pairs:
        lines.append(f'  printf("{cname} size %zu\\n", sizeof({cname}));')
        for f in py._fields_:
            lines.append(f'  printf("{cname} {f[0]} %zu\\n", offsetof({cname}, {f[0]}));')
    lines += ["  return 0;", "}"]
    d = tmp_path_factory.mktemp("abi")
    src, exe = d / "layout.c", d / "layout"
    src.write_text("\n".join(lines) + "\n")
    cuda_inc = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "include")
    subprocess.run([cc, "-std=c11", "-I", INC, "-I", cuda_inc, str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    table = {}
    for line in out.splitlines():
        name, field, value = line.split()
        table[(name, field)] = int(value)
    return pairs, table


def test_struct_sizes_and_offsets_match(c_layout):
    pairs, table = c_layout
    for cname, py in pairs:
        assert ctypes.sizeof(py) == table[(cname, "size")], cname
        for f in py._fields_:
            assert getattr(py, f[0]).offset == table[(cname, f[0])], (cname, f[0])
